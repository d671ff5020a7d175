"""CPU oracle for the tree-likelihood hot path.

TEST INFRASTRUCTURE ONLY. Nothing in ``torchtree_gb300`` imports this
package; only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline
leg of ``bench.py`` use it, and only as the checker (or, for the baseline,
as the timed CPU restatement of the reference path).

Contents
--------
``likelihood``  FP64 restatement of torchtree's pruning functions,
                transition matrices, rate matrices and site models
                (torch on CPU, gradients by autograd exactly as the
                reference obtains them).
``patterns``    restatement of torchtree's data types (state encodings,
                tip partial vectors) and site-pattern compression
                (pure Python / numpy; integer work, bit-exact).

Parity pin: ``tests/golden/`` holds vectors produced by importing the
reference torchtree 1.0.2 itself (``tests/golden/make_golden.py``) plus the
known answers of the reference's own tests; ``tests/test_oracle_golden.py``
checks this package against all of them.  The discretised-Gamma site model
has no counterpart in the reference: its rates are pinned only by scipy's
``gammaincinv`` and by finite differences ("parity unpinned" for Gamma
rates).
"""
