"""Regenerate the golden fixtures of tests/golden/ with the FP64 CPU oracle.

    python tests/golden/make_golden.py

Fixtures (numpy .npz, a subset of nodes each):
  mg1_faithful.npz   reference deck Mg1, reference operator (shared projector slot)
  mg1_corrected.npz  reference deck Mg1, corrected operator
  mg4_small.npz      4-atom periodic FCC Mg cell, h = 0.85, Rcut = 3.4, 20 Lanczos steps,
                     seed 7 (sqminiapp_gb300.decks.make_fcc_mg_deck)
Each holds the node indices, a_k, b_k (k <= n_qp), lambda, weights, lambda_min/max.
"""
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

SMALL = dict(ncell=1, h=0.85, rcut=3.4, n_qp=20, disp=0.1, seed=7)


def small_deck(dirname):
    from sqminiapp_gb300.decks import make_fcc_mg_deck
    return make_fcc_mg_deck(dirname, "mg4s", **SMALL)


def main():
    import oracle
    from sqminiapp_gb300 import DECK_DIR
    cases = [("mg1_faithful", DECK_DIR, "Mg1", True, np.arange(0, 3366, 97)),
             ("mg1_corrected", DECK_DIR, "Mg1", False, np.arange(0, 3366, 97))]
    tmp = tempfile.mkdtemp()
    d, name, _ = small_deck(tmp)
    cases.append(("mg4_small", d, name, False, np.arange(0, 8000, 61)))
    for tag, ddir, dname, faithful, nodes in cases:
        o = oracle.Oracle(ddir, dname, faithful=faithful)
        nodes = nodes[nodes < o.n_nodes]
        r = o.nodes_and_weights(nodes=nodes, want_ab=True)
        np.savez_compressed(os.path.join(HERE, tag + ".npz"), nodes=nodes, a=r["a"], b=r["b"],
                            lam=r["lambda"], w=r["weights"], lmin=r["lambda_min"],
                            lmax=r["lambda_max"])
        print(tag, len(nodes), "nodes")


if __name__ == "__main__":
    main()
