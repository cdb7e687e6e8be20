"""Train the learned SCF start (WarmStartMLP) on densities the engine itself converges.

    python -m sqminiapp_gb300.train_warm_start --cells 200 --out model.bin

Training cells: seeded 32-atom FCC Mg cells (2x2x2, side 17 bohr) with Gaussian thermal
displacements (sigma 0.25 bohr), at the discretisation the model will serve (default h = 0.5,
Rcut = 6.5, 40 Lanczos steps: the 108-atom cell's).  Each cell runs the FP32 SCF from the
atomic superposition; its descriptors and rho_SCF - rho_0 become training samples.  The
network is then trained by Adam on the GPU (tensor-core forward and backward kernels).
Prints one JSON line with the cell count, samples, final loss and times.
"""
import argparse
import json
import os
import sys
import tempfile
import time

if __package__ in (None, ""):
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))

from sqminiapp_gb300 import LSDFT, WarmStartMLP  # noqa: E402
from sqminiapp_gb300.decks import make_fcc_mg_deck  # noqa: E402


def main(argv=None):
    p = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    p.add_argument("--cells", type=int, default=200)
    p.add_argument("--first-seed", type=int, default=5000)
    p.add_argument("--ncell", type=int, default=2)
    p.add_argument("--h", type=float, default=0.5)
    p.add_argument("--rcut", type=float, default=6.5)
    p.add_argument("--n-qp", type=int, default=40)
    p.add_argument("--sigma", type=float, default=0.25)
    p.add_argument("--steps", type=int, default=3000)
    p.add_argument("--tiles-per-step", type=int, default=152)
    p.add_argument("--lr", type=float, default=2e-3)
    p.add_argument("--device", type=int, default=0)
    p.add_argument("--out", required=True)
    a = p.parse_args(argv)

    m = WarmStartMLP(device=a.device, seed=a.first_seed)
    t0 = time.perf_counter()
    its = []
    with tempfile.TemporaryDirectory(prefix="sq_train_") as tmp:
        for c in range(a.cells):
            d, name, _ = make_fcc_mg_deck(os.path.join(tmp, "c%d" % c), "cell", ncell=a.ncell, h=a.h,
                                          rcut=a.rcut, n_qp=a.n_qp, disp=a.sigma,
                                          disp_kind="gaussian", seed=a.first_seed + c)
            with LSDFT(d, name, faithful=False, precision=32, device=a.device) as eng:
                r = eng.SCF_LSSGQ(raise_on_maxit=False)
                its.append(r["iterations"])
                m.add_training_cell(eng)
    t_data = time.perf_counter() - t0
    t0 = time.perf_counter()
    # three stages of decreasing learning rate
    n1 = int(0.6 * a.steps)
    n2 = int(0.3 * a.steps)
    m.train(n1, a.tiles_per_step, a.lr)
    m.train(n2, a.tiles_per_step, a.lr * 0.25)
    loss = m.train(a.steps - n1 - n2, a.tiles_per_step, a.lr * 0.05)
    t_train = time.perf_counter() - t0
    m.save(a.out)
    print(json.dumps({"cells": a.cells, "samples": a.cells * round(8.5 * a.ncell / a.h) ** 3,
                      "scf_iterations_mean": sum(its) / len(its), "final_loss": loss,
                      "data_seconds": t_data, "train_seconds": t_train, "out": a.out,
                      "discretisation": {"h": a.h, "rcut": a.rcut, "n_qp": a.n_qp}}), flush=True)


if __name__ == "__main__":
    main()
