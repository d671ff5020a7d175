"""Generate golden vectors by running the reference torchtree itself.

Usage (from the repository root, in a container where the reference source
is available):

    python tests/golden/make_golden.py /path/to/torchtree-source

The reference imports dendropy at module load; ``oracle/_stub/dendropy.py`` stands
in for it (trees are never parsed through dendropy here: post-order triples
come from this package's Newick parser or Yule generator and are handed to
a minimal ``TreeModel``).  Every value written below is computed by the
reference's own classes and functions in FP64: data-type encodings, site
pattern compression, transition matrices, site-model rates, and the
``TreeLikelihoodModel`` log-likelihood with its autograd gradient.
The package under test contributes inputs only (tree, simulated alignment).
"""
from __future__ import annotations

import io
import json
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REPO = HERE.parent.parent


def _setup(ref_root: str):
    sys.path.insert(0, str(REPO / "oracle" / "_stub"))
    sys.path.insert(0, ref_root)
    sys.path.insert(0, str(REPO))


def main(ref_root: str) -> None:
    _setup(ref_root)
    import torch

    torch.set_default_dtype(torch.float64)
    from torchtree import Parameter
    from torchtree.evolution import tree_likelihood as TL
    from torchtree.evolution.alignment import Alignment, Sequence
    from torchtree.evolution.branch_model import StrictClockModel
    from torchtree.evolution.datatype import (AminoAcidDataType, CodonDataType,
                                               GeneralDataType, NucleotideDataType)
    from torchtree.evolution.site_model import ConstantSiteModel, WeibullSiteModel
    from torchtree.evolution.site_pattern import (SitePattern, compress_alignment,
                                                   compress_alignment_states)
    from torchtree.evolution.substitution_model import GTR, HKY, JC69, MG94
    from torchtree.evolution.substitution_model.general import GeneralSymmetricSubstitutionModel
    from torchtree.evolution.taxa import Taxa, Taxon
    from torchtree.evolution.tree_model import TreeModel

    from torchtree_gb300 import synthetic
    from torchtree_gb300.tree import Topology

    out = {}

    # ------------------------------------------------------------ encodings
    nuc, aa = NucleotideDataType(None), AminoAcidDataType(None)
    enc = {"nucleotide": [], "amino_acid": []}
    for o in range(128):
        c = chr(o)
        enc["nucleotide"].append([nuc.encoding(c), list(nuc.partial(c, True)), list(nuc.partial(c, False))])
        enc["amino_acid"].append([aa.encoding(c), list(aa.partial(c, True)), list(aa.partial(c, False))])
    codon = CodonDataType(None, "Universal")
    trips = ["".join(t) for t in __import__("itertools").product("ACGT", repeat=3)]
    trips += ["---", "???", "AN-", "ACN", "TUA", "acg", "RAA"]
    enc["codon_universal"] = {"state_count": codon.state_count,
                              "codes": {t: int(codon.encoding(t)) for t in trips}}
    gen = GeneralDataType(None, ("A", "C", "T", "G"), {"U": "T", "R": ["A", "G"]})
    enc["general_ACTG"] = {c: [int(gen.encoding(c)), list(map(float, gen.partial(c)))] for c in "ACTGURN-"}
    (HERE / "encodings.json").write_text(json.dumps(enc))

    # ------------------------------------------------------------ patterns
    def alignment_of(seqs, names, data_type):
        taxa = Taxa(None, [Taxon(n, {}) for n in names])
        return Alignment(None, [Sequence(n, s) for n, s in zip(names, seqs)], taxa, data_type)

    rng = np.random.default_rng(11)
    chars = np.array(list("ACGTACGTACGTACGTRYKMSWN-?uacgt"))
    pat_cases = []
    small = (["AAG", "AAC", "AAC", "AAT"], list("ABCD"))
    rand_seqs = ["".join(rng.choice(chars, 60)) for _ in range(7)]
    rand_names = [f"s{i}" for i in (3, 0, 6, 1, 5, 2, 4)]  # not sorted: taxa order matters
    for seqs, names in (small, (rand_seqs, rand_names)):
        aln = alignment_of(list(seqs), names, nuc)
        case = {"sequences": list(seqs), "names": names}
        for amb in (False, True):
            parts, w = compress_alignment(aln, None, amb)
            case[f"partials_amb{int(amb)}"] = [p.numpy().tolist() for p in parts]
            case["weights"] = w.tolist()
        states, w2 = compress_alignment_states(aln)
        case["states"] = [s.tolist() for s in states]
        idx = [slice(0, 2), 2] if len(seqs[0]) == 3 else [slice(0, 30), 45, 50, slice(55, 60)]
        parts, w3 = compress_alignment(aln, idx, False)
        case["indices"] = [[i.start, i.stop] if isinstance(i, slice) else i for i in idx]
        case["indexed_partials"] = [p.numpy().tolist() for p in parts]
        case["indexed_weights"] = w3.tolist()
        pat_cases.append(case)
    cod_seqs = ["".join(rng.choice(list("ACGT"), 30)) for _ in range(5)]
    cod_seqs[1] = "---" + cod_seqs[1][3:]
    cod_aln = alignment_of(cod_seqs, [f"c{i}" for i in range(5)], codon)
    parts, w = compress_alignment(cod_aln, None, False)
    states, _ = compress_alignment_states(cod_aln)
    pat_cases.append({"codon": True, "sequences": cod_seqs, "names": [f"c{i}" for i in range(5)],
                      "argmax_partials": [[int(np.argmax(c)) if c.sum() == 1 else -1 for c in p.numpy().T]
                                          for p in parts],
                      "weights": w.tolist(), "states": [s.tolist() for s in states]})
    (HERE / "site_patterns.json").write_text(json.dumps(pat_cases))

    # ------------------------------------------------------ transition, rates
    tr = {}
    r6 = torch.tensor([0.060602, 0.402732, 0.028230, 0.047910, 0.407249, 0.053277])
    pi4 = torch.tensor([0.479367, 0.172572, 0.140933, 0.207128])
    ts = torch.tensor([[0.1], [0.001], [0.5], [2.0]])
    gtr = GTR(None, Parameter(None, r6), Parameter(None, pi4))
    tr["gtr"] = {"rates": r6.tolist(), "pi": pi4.tolist(), "t": ts.squeeze(-1).tolist(),
                 "P": gtr.p_t(ts).squeeze(-3).tolist()}
    hky = HKY(None, Parameter(None, torch.tensor([3.0])), Parameter(None, pi4))
    tr["hky"] = {"kappa": 3.0, "pi": pi4.tolist(), "t": ts.squeeze(-1).tolist(),
                 "P": hky.p_t(ts).squeeze(-3).tolist()}
    jc = JC69(None)
    tr["jc69"] = {"t": ts.squeeze(-1).tolist(), "P": jc.p_t(ts).squeeze(-3).tolist()}
    wb = {}
    for shape in (0.1, 0.5, 1.0, 2.5):
        sm = WeibullSiteModel(None, Parameter(None, torch.tensor([shape])), 4)
        wb[str(shape)] = {"rates": sm.rates().tolist(), "probs": sm.probabilities().tolist()}
    sm = WeibullSiteModel(None, Parameter(None, torch.tensor([0.5])), 4,
                          invariant=Parameter(None, torch.tensor([0.2])))
    wb["0.5+I0.2"] = {"rates": sm.rates().tolist(), "probs": sm.probabilities().tolist()}
    tr["weibull"] = wb
    g20 = GeneralDataType(None, tuple("ACDEFGHIKLMNPQRSTVWY"))
    rates190 = torch.tensor(rng.gamma(1.0, 1.0, 190))
    pi20 = torch.tensor(rng.dirichlet(np.ones(20)))
    gm = GeneralSymmetricSubstitutionModel(None, g20, Parameter(None, torch.arange(190)),
                                           Parameter(None, rates190), Parameter(None, pi20))
    tr["general20"] = {"rates": rates190.tolist(), "pi": pi20.tolist(), "t": [0.05, 0.3],
                       "P": gm.p_t(torch.tensor([[0.05], [0.3]])).squeeze(-3).tolist()}
    pi61 = torch.tensor(rng.dirichlet(np.ones(61)))
    mg = MG94(None, codon, Parameter(None, torch.tensor([1.0])), Parameter(None, torch.tensor([0.4])),
              Parameter(None, torch.tensor([2.5])), Parameter(None, pi61))
    q61 = mg.q()
    tr["mg94"] = {"alpha": 1.0, "beta": 0.4, "kappa": 2.5, "pi": pi61.tolist(),
                  "Q_rows": {str(i): q61[..., i, :].reshape(-1).tolist() for i in (0, 5, 13, 60)},
                  "Q_diag": torch.diagonal(q61, dim1=-2, dim2=-1).reshape(-1).tolist()}
    (HERE / "transition.json").write_text(json.dumps(tr))

    # ---------------------------------------------------------- likelihoods
    class FixedTree(TreeModel):
        """Minimal TreeModel: fixed post-order, branch lengths from a Parameter."""

        def __init__(self, post, names, bl):
            super().__init__(None)
            self._post = [list(map(int, t)) for t in post]
            self._names = list(names)
            self._bl = bl
            self.taxa_count = len(names)

        def branch_lengths(self):
            return self._bl.tensor

        @property
        def postorder(self):
            return self._post

        @property
        def taxa(self):
            return self._names

        def write_newick(self, stream, **kwargs):
            stream.write("();")

        def _sample_shape(self):
            return self._bl.tensor.shape[:-1]

        def handle_model_changed(self, model, obj, index):
            pass

        def handle_parameter_changed(self, variable, index, event):
            self.fire_model_changed()

        @classmethod
        def from_json(cls, data, dic):
            raise NotImplementedError

    def run_model(topo, seqs, bl, subst, site_model, clock=None, amb=False, tip_states=False,
                  rescale=False, params=(), data_type=None):
        names = topo.tip_names
        aln = alignment_of(list(seqs), names, data_type or nuc)
        sp = SitePattern(None, aln)
        blp = Parameter(None, bl)
        tree = FixedTree(topo.postorder, names, blp)
        clock_model = StrictClockModel(None, Parameter(None, clock), tree) if clock is not None else None
        like = TL.TreeLikelihoodModel(None, sp, tree, subst, site_model, clock_model, amb, tip_states)
        like.rescale = rescale
        lnl = like()
        grads = torch.autograd.grad(lnl.sum(), [bl, *params], allow_unused=True)
        return lnl.detach(), grads, like.rescale

    lik = {}
    # tiny (reference known answer -83.329016 with JC69, tree_likelihood tests)
    ref_data = Path(ref_root) / "data"
    tiny_nwk = (ref_data / "tiny.nwk").read_text().strip()
    fasta = {}
    name = None
    for line in (ref_data / "tiny.fa").read_text().splitlines():
        if line.startswith(">"):
            name = line[1:].strip()
            fasta[name] = ""
        elif name:
            fasta[name] += line.strip()
    names = list(fasta)
    topo = Topology.from_newick(tiny_nwk, names)
    ub = torch.tensor(topo.unrooted_branch_lengths(), requires_grad=True)
    jc = JC69(None)
    lnl, (gbl,), _ = run_model(topo, [fasta[n] for n in names], ub, jc, ConstantSiteModel(None))
    lik["tiny_jc69"] = {"newick": tiny_nwk, "names": names, "sequences": [fasta[n] for n in names],
                        "postorder": topo.postorder.tolist(), "branch_lengths": ub.tolist(),
                        "model": "jc69", "site_model": "constant", "lnl": lnl.reshape(-1).tolist(),
                        "grad_branch_lengths": gbl.reshape(-1).tolist()}

    def dna_case(key, wl, sample=slice(None), rescale=False, tip_states=False, amb=False, weibull=True,
                 invariant=None):
        topo = wl.topology
        bl = torch.tensor(wl.branch_lengths[sample], requires_grad=True)
        pi = torch.tensor(wl.pi[sample], requires_grad=True)
        shape = torch.tensor(wl.shape[sample], requires_grad=True)
        if wl.model == "gtr":
            ex = torch.tensor(wl.exch[sample], requires_grad=True)
            subst = GTR(None, Parameter(None, ex), Parameter(None, pi))
        else:
            ex = torch.tensor(wl.exch[sample][..., 1:2], requires_grad=True)  # kappa
            subst = HKY(None, Parameter(None, ex), Parameter(None, pi))
        inv = None
        if invariant is not None:
            inv = torch.tensor(np.full(wl.shape[sample].shape, invariant), requires_grad=True)
        if weibull:
            site = WeibullSiteModel(None, Parameter(None, shape), wl.categories,
                                    invariant=Parameter(None, inv) if inv is not None else None)
        else:
            rates = torch.tensor(synthetic.discrete_gamma_np(float(wl.shape[0, 0]), wl.categories))
            site = ConstantSiteModel(None, Parameter(None, rates))
            site._probability = torch.full((wl.categories,), 1.0 / wl.categories)
        params = [ex, pi, shape] + ([inv] if inv is not None else [])
        lnl, grads, flag = run_model(topo, wl.sequences, bl, subst, site, rescale=rescale,
                                     tip_states=tip_states, amb=amb, params=params)
        rec = {"postorder": topo.postorder.tolist(), "names": topo.tip_names, "sequences": wl.sequences,
               "branch_lengths": bl.tolist(), "model": wl.model, "exch": ex.tolist(), "pi": pi.tolist(),
               "shape": shape.tolist(), "categories": wl.categories,
               "site_model": "weibull" if weibull else "gamma_fixed_rates",
               "rescale": rescale, "tip_states": tip_states, "use_ambiguities": amb,
               "rescaled_after": flag, "lnl": lnl.reshape(-1).tolist(),
               "grad_branch_lengths": grads[0].tolist(), "grad_exch": grads[1].tolist(),
               "grad_pi": grads[2].tolist()}
        if weibull:
            rec["grad_shape"] = grads[3].tolist()
        if inv is not None:
            rec["invariant"] = inv.tolist()
            rec["grad_invariant"] = grads[4].tolist()
        if not weibull:
            rec["category_rates"] = synthetic.discrete_gamma_np(float(wl.shape[0, 0]), wl.categories).tolist()
        lik[key] = rec

    wl1 = synthetic.named_workload("gtr_w4_t69")
    dna_case("gtr_w4_t69", wl1, sample=slice(0, 1))
    dna_case("gtr_w4_t69_rescaled", wl1, sample=slice(0, 1), rescale=True)
    wlb = synthetic.dna_workload("batch3", tip_count=12, site_count=200, batch=3, seed=5, model="hky",
                                 site_model="weibull", shape=0.7, branch_mean=0.08)
    wlb.shape[:, 0] = [0.7, 0.4, 1.3]
    wlb.exch[1, [1, 4]] = 5.0
    dna_case("hky_w4_t12_b3", wlb)
    dna_case("hky_w4_t12_b3_tipstates", wlb, tip_states=True)
    dna_case("hky_w4_t12_b3_rescaled_inv", wlb, rescale=True, invariant=0.15)
    wlg = synthetic.dna_workload("gamma", tip_count=30, site_count=300, batch=1, seed=6, model="gtr",
                                 site_model="gamma", shape=0.3, branch_mean=0.05)
    dna_case("gtr_g4_t30", wlg, weibull=False)
    # ambiguity codes in the tips
    wla = synthetic.dna_workload("amb", tip_count=9, site_count=80, batch=1, seed=8, model="gtr",
                                 site_model="weibull", shape=0.5, branch_mean=0.1)
    arng = np.random.default_rng(9)
    seqs = [list(s) for s in wla.sequences]
    for s in seqs:
        for pos in arng.choice(80, 10, replace=False):
            s[pos] = arng.choice(list("RYKMSWBDHVN-?"))
    wla.sequences = ["".join(s) for s in seqs]
    dna_case("gtr_w4_t9_ambiguities", wla, amb=True)
    dna_case("gtr_w4_t9_no_ambiguities", wla, amb=False)
    # underflow: the unscaled FP64 pass gives -inf, the model switches to rescaling
    wlu = synthetic.dna_workload("underflow", tip_count=700, site_count=40, batch=1, seed=10, model="gtr",
                                 site_model="weibull", shape=1.0, branch_mean=1.0)
    urng = np.random.default_rng(12)
    wlu.sequences = ["".join(urng.choice(list("ACGT"), 40)) for _ in range(700)]
    dna_case("gtr_w4_t700_underflow", wlu)
    # 20-state amino acids (general symmetric model) and 61-state codons (MG94)
    def wide_case(key, wl, sample=slice(None), rescale=False, tip_states=False):
        topo = wl.topology
        bl = torch.tensor(wl.branch_lengths[sample], requires_grad=True)
        pi = torch.tensor(wl.pi[sample], requires_grad=True)
        shape = torch.tensor(wl.shape[sample], requires_grad=True)
        ex = torch.tensor(wl.exch[sample], requires_grad=True)
        if wl.model == "general":
            dtype = aa
            subst = GeneralSymmetricSubstitutionModel(None, aa, Parameter(None, torch.arange(190)),
                                                      Parameter(None, ex), Parameter(None, pi))
        else:  # MG94 with alpha = 1, beta = omega
            dtype = codon
            subst = MG94(None, codon, Parameter(None, torch.ones_like(ex[..., :1])), Parameter(None, ex[..., 1:2]),
                         Parameter(None, ex[..., 0:1]), Parameter(None, pi))
        site = WeibullSiteModel(None, Parameter(None, shape), wl.categories)
        lnl, grads, flag = run_model(topo, wl.sequences, bl, subst, site, rescale=rescale, tip_states=tip_states,
                                     params=[ex, pi, shape], data_type=dtype)
        lik[key] = {"postorder": topo.postorder.tolist(), "names": topo.tip_names, "sequences": wl.sequences,
                    "branch_lengths": bl.tolist(), "model": wl.model, "data_type": wl.data_type,
                    "exch": ex.tolist(), "pi": pi.tolist(), "shape": shape.tolist(), "categories": wl.categories,
                    "site_model": "weibull", "rescale": rescale, "tip_states": tip_states, "use_ambiguities": False,
                    "rescaled_after": flag, "lnl": lnl.reshape(-1).tolist(),
                    "grad_branch_lengths": grads[0].tolist(), "grad_exch": grads[1].tolist(),
                    "grad_pi": grads[2].tolist(), "grad_shape": grads[3].tolist()}

    wlp = synthetic.protein_workload("prot", tip_count=16, site_count=150, batch=2, seed=21, site_model="weibull",
                                     shape=0.6, branch_mean=0.1)
    wide_case("prot_w4_t16_b2", wlp)
    wide_case("prot_w4_t16_b2_tipstates", wlp, tip_states=True)
    wlc = synthetic.codon_workload("codon", tip_count=10, site_count=60, batch=2, seed=22, site_model="weibull",
                                   shape=0.8, branch_mean=0.1)
    wide_case("codon_w4_t10_b2", wlc)
    wide_case("codon_w4_t10_b2_rescaled", wlc, rescale=True)
    # ------------------------------------------------------ time-tree operations
    from types import SimpleNamespace

    from torchtree.evolution.coalescent import ConstantCoalescent
    from torchtree.evolution.tree_height_transform import GeneralNodeHeightTransform
    from torchtree.evolution.tree_model import heights_to_branch_lengths

    tt_cases = {}
    for key, T, seed, hetero in (("isochronous_t12", 12, 31, False), ("heterochronous_t40", 40, 32, True)):
        trng = np.random.default_rng(seed)
        topo = synthetic.yule_topology(T, trng)
        times = trng.uniform(0.0, 2.0, T) if hetero else np.zeros(T)
        times[0] = 0.0
        heights = np.zeros(2 * T - 1)
        heights[:T] = times
        for v, l, r in topo.postorder:
            heights[v] = max(heights[l], heights[r]) + trng.exponential(0.5)
        kids = {int(v): (int(l), int(r)) for v, l, r in topo.postorder}
        pre = []
        stack = [2 * T - 2]
        while stack:  # parent before child (dendropy preorder_node_iter)
            v = stack.pop()
            if v >= T:
                for c in kids[v]:
                    pre.append((v, c))
                    stack.append(c)
        fake = SimpleNamespace(taxa_count=T, postorder=[list(map(int, t)) for t in topo.postorder],
                               preorder=torch.tensor(pre), sampling_times=torch.tensor(times))
        tr = GeneralNodeHeightTransform(fake)
        internal = torch.tensor(heights[T:])
        ratios = tr.inv(internal).detach().clone().requires_grad_()
        h = tr(ratios)
        ld = tr.log_abs_det_jacobian(ratios, h)
        bl = heights_to_branch_lengths(h, tr._bounds, fake.preorder)
        w1 = torch.tensor(trng.normal(size=T - 1))
        w3 = torch.tensor(trng.normal(size=2 * T - 2))
        obj = (h * w1).sum() + 0.7 * ld + (bl * w3).sum()
        (gx,) = torch.autograd.grad(obj, ratios)
        theta = torch.tensor([1.3], requires_grad=True)
        hh = internal.clone().requires_grad_()
        lp = ConstantCoalescent(theta).log_prob(torch.cat((torch.tensor(times), hh)))
        gh, gth = torch.autograd.grad(lp.sum(), [hh, theta])
        tt_cases[key] = {"postorder": topo.postorder.tolist(), "sampling_times": times.tolist(),
                         "internal_heights": internal.tolist(), "ratios": ratios.detach().tolist(),
                         "heights": h.detach().tolist(), "log_det": float(ld), "branch_lengths": bl.detach().tolist(),
                         "w_heights": w1.tolist(), "w_log_det": 0.7, "w_branch_lengths": w3.tolist(),
                         "grad_ratios": gx.tolist(), "theta": 1.3, "coalescent_log_prob": float(lp.reshape(-1)[0]),
                         "coalescent_grad_heights": gh.tolist(), "coalescent_grad_theta": float(gth.reshape(-1)[0])}
    (HERE / "timetree.json").write_text(json.dumps(tt_cases))

    with io.open(HERE / "likelihood.json", "w") as fh:
        json.dump(lik, fh)
    print("wrote", sorted(p.name for p in HERE.glob("*.json")))
    print("tiny lnl", lik["tiny_jc69"]["lnl"], "underflow switched:", lik["gtr_w4_t700_underflow"]["rescaled_after"])


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
