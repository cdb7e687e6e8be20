"""Regenerate tests/golden/scf_mg4.json: the SCF of the 4-atom bench cell through the CPU
oracle (oracle/scf.py around the FP64 restatement of the reference's per-node path).

    python tests/golden/make_scf_golden.py      # about 10 minutes on 8 cores

Cell: sqminiapp_gb300.decks.CONFIGS["mg4_h0.5_rc6_q30"] with the default seed (the cell of
bench.py's time-to-SCF leg): 4 Mg atoms, 17^3 nodes, 25^3 cubes, 30 Lanczos steps.  SCF: the
deck's mixing (0.3, history 7, Pulay every 2nd iteration), Kerker k_TF = 1, tol 1e-6.
"""
import json
import os
import sys
import tempfile
import time

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))


def main():
    import oracle
    from oracle import scf as oscf
    from sqminiapp_gb300.decks import CONFIGS, DEFAULT_SEED, make_fcc_mg_deck
    with tempfile.TemporaryDirectory() as tmp:
        d, name, _ = make_fcc_mg_deck(tmp, "cell", seed=DEFAULT_SEED, **CONFIGS["mg4_h0.5_rc6_q30"])
        o = oracle.Oracle(d, name, faithful=False)
        t = time.time()
        r = oscf.scf(o, oscf.scf_fields(o), tol=1e-6, maxit=60, mix=0.3, history=7,
                     pulay_every=2, k_tf=1.0)
    out = {"config": "mg4_h0.5_rc6_q30", "seed": DEFAULT_SEED, "tol": 1e-6,
           "iterations": r["iterations"], "converged": bool(r["converged"]),
           "free_energy_per_atom": r["free_energy_per_atom"], "lambda_f": r["lambda_f"],
           "residual": r["residual"], "cpu_seconds": time.time() - t,
           "free_energy_per_atom_history": [float(v) / o.natoms for v in r["free_energy_history"]]}
    with open(os.path.join(HERE, "scf_mg4.json"), "w") as f:
        json.dump(out, f, indent=1)
    print(json.dumps({k: out[k] for k in ("iterations", "free_energy_per_atom", "cpu_seconds")}))


if __name__ == "__main__":
    main()
