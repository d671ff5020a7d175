"""The plug-in class on the GPU, configured from JSON, against torchtree itself.

``torchtree_gb300.TreeLikelihoodModel`` is built by torchtree's own JSON
machinery (``process_object`` with ``"type": "torchtree_gb300.TreeLikelihoodModel"``,
core/utils.py:116-203) over torchtree's tree, site-pattern, substitution and
site models, and called like the reference class: ``like()`` runs the GPU
engine and ``backward`` fills the torchtree ``Parameter`` tensors' gradients.
The same objects, built afresh, go through torchtree's own
``TreeLikelihoodModel`` (tree_likelihood.py:281-450) on the CPU in FP64.

* FP64 plug-in: lnL within 1e-10 relative, every gradient within 1e-10 of
  its largest entry (1e-8 for the 61 x 61 codon matrices), unscaled and
  rescaled;
* FP32 plug-in: lnL within 1e-6 relative, gradients within 1e-4 of their
  largest entry.

torchtree comes from its source tree or the copy installed in
``baseline/_ref``; the tests are skipped where neither is present.
"""
import numpy as np
import pytest
import torch

from tests.reference_models import import_torchtree, reference_objects, wide_reference_objects

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torchtree_gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    if not import_torchtree():
        pytest.skip("torchtree not present (neither a source tree nor baseline/_ref)")
    torch.set_default_dtype(torch.float64)
    yield
    torch.set_default_dtype(torch.float32)


def _from_json(dic, precision, clock, tip_states):
    from torchtree.core.utils import process_object

    data = {"id": "like", "type": "torchtree_gb300.TreeLikelihoodModel", "tree_model": "tree",
            "site_model": "site", "substitution_model": "subst", "site_pattern": "sp",
            "precision": precision, "use_tip_states": tip_states}
    if clock is not None:
        data["branch_model"] = "clock"
    return process_object(data, dic)


def _check(got, gots, want, gwant, precision, f64_tol=1e-10):
    ltol, gtol = (1e-10, f64_tol) if precision == "f64" else (1e-6, 1e-4)
    np.testing.assert_allclose(got.detach().numpy(), want.detach().numpy(), rtol=ltol)
    for g, w in zip(gots, gwant):
        np.testing.assert_allclose(g.numpy(), w.numpy(), rtol=gtol, atol=gtol * float(w.abs().max()))


@pytest.mark.parametrize("precision", ["f64", "f32"])
@pytest.mark.parametrize("case,b", [("gtr_weibull", 1), ("gtr_weibull", 2), ("jc69_constant", 1),
                                    ("hky_weibull_clock", 2), ("gtr_weibull_tipstates", 2)])
def test_plugin_class_on_gpu_matches_torchtree(torchtree_gpu, case, b, precision):
    from torchtree.evolution.tree_likelihood import TreeLikelihoodModel as Reference

    from torchtree_gb300 import synthetic
    from torchtree_gb300.model import TreeLikelihoodModel

    wl = synthetic.dna_workload("plugin-gpu", tip_count=40, site_count=800, batch=2, seed=95, shape=0.5,
                                site_model="weibull")
    for rescale in ((False, True) if precision == "f64" else (True,)):
        tree, sp, subst, site, clock, tip_states, leaves = reference_objects(case, wl, b)
        ref = Reference(None, sp, tree, subst, site, clock, False, tip_states)
        ref.rescale = rescale
        want = ref().reshape(-1)
        gwant = torch.autograd.grad(want.sum(), leaves)
        tree, sp, subst, site, clock, tip_states, leaves = reference_objects(case, wl, b)
        dic = {"tree": tree, "sp": sp, "subst": subst, "site": site, "clock": clock}
        like = _from_json(dic, precision, clock, tip_states)
        assert isinstance(like, TreeLikelihoodModel)
        like.rescale = rescale or precision == "f32"
        got = like().reshape(-1)
        assert got.device.type == "cpu"  # returned where the parameters live
        eng = next(iter(like._engines.values()))
        assert eng.device.type == "cuda" and eng.launch_count > 0
        got.sum().backward()
        _check(got, [x.grad for x in leaves], want, gwant, precision)


@pytest.mark.parametrize("precision", ["f64", "f32"])
@pytest.mark.parametrize("kind", ["protein", "codon"])
def test_plugin_class_on_gpu_wide_models(torchtree_gpu, kind, precision):
    from torchtree.evolution.tree_likelihood import TreeLikelihoodModel as Reference

    from torchtree_gb300 import synthetic

    if kind == "protein":
        wl = synthetic.protein_workload("p", tip_count=16, site_count=150, batch=1, seed=710, shape=0.7,
                                        site_model="weibull", branch_mean=0.1)
    else:
        wl = synthetic.codon_workload("c", tip_count=10, site_count=60, batch=1, seed=711, shape=0.7,
                                      site_model="weibull", branch_mean=0.1)
    tree, sp, subst, site, leaves = wide_reference_objects(kind, wl)
    want = Reference(None, sp, tree, subst, site)().reshape(-1)
    gwant = torch.autograd.grad(want.sum(), leaves)
    tree, sp, subst, site, leaves = wide_reference_objects(kind, wl)
    like = _from_json({"tree": tree, "sp": sp, "subst": subst, "site": site}, precision, None, False)
    got = like().reshape(-1)
    got.sum().backward()
    _check(got, [x.grad for x in leaves], want, gwant, precision, f64_tol=1e-8 if kind == "codon" else 1e-10)


@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_plugin_class_with_gamma_site_model(torchtree_gpu, precision):
    """GTR + this package's GammaSiteModel (JSON) through the plug-in on the
    GPU against torchtree's own TreeLikelihoodModel over the same objects on
    the CPU (the reference class accepts any SiteModel), two samples."""
    from torchtree import Parameter
    from torchtree.core.utils import process_object
    from torchtree.evolution.substitution_model import GTR
    from torchtree.evolution.tree_likelihood import TreeLikelihoodModel as Reference

    from oracle import reference as R
    from oracle import reference_arm as RA
    from torchtree_gb300 import synthetic

    wl = synthetic.dna_workload("plugin-gamma", tip_count=60, site_count=900, batch=2, seed=97, shape=0.4,
                                site_model="gamma")
    tips, weights = RA.compress(wl.sequences, wl.data_type)

    def build():
        leaf = lambda a: torch.tensor(np.asarray(a), dtype=torch.float64, requires_grad=True)  # noqa: E731
        bl, ex, pi, shape = leaf(wl.branch_lengths), leaf(wl.exch), leaf(wl.pi), leaf(wl.shape)
        dic = {"tree": R.fixed_tree_class()(wl.topology.postorder, wl.topology.tip_names, Parameter(None, bl)),
               "subst": GTR(None, Parameter(None, ex), Parameter(None, pi)), "sp": R.PatternSource(tips, weights),
               "shape": Parameter("shape", shape)}
        dic["site"] = process_object({"id": "site", "type": "torchtree_gb300.GammaSiteModel", "shape": "shape",
                                      "categories": 4}, dic)
        return dic, [bl, ex, pi, shape]

    dic, leaves = build()
    ref = Reference(None, dic["sp"], dic["tree"], dic["subst"], dic["site"])
    ref.rescale = True
    want = ref().reshape(-1)
    gwant = torch.autograd.grad(want.sum(), leaves)
    dic, leaves = build()
    like = _from_json(dic, precision, None, False)
    like.rescale = True
    got = like().reshape(-1)
    got.sum().backward()
    _check(got, [x.grad for x in leaves], want, gwant, precision)
