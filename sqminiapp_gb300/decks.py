"""Synthetic input decks: seeded FCC magnesium cells in the reference's file format.

A deck is <dir>/<name>.inpt/.ion/.relax plus <dir>/pseudopotential/psd_Mg.pot, read by
the engine exactly as the reference reads its own decks (src/lsdft_readfiles.cc).

Cells: conventional FCC cube (a = 8.5 bohr, 4 atoms at (0,0,0), (1/2,1/2,0), (1/2,0,1/2),
(0,1/2,1/2)) replicated n x n x n, coordinates centred in [-L/2, L/2) (the reference's
convention), every coordinate displaced uniformly in [-d, d] or by a Gaussian of width
sigma.  Random numbers come from numpy's PCG64 raw 64-bit stream, turned into doubles
with 53-bit mantissas and Box-Muller normals here, so a seed gives the same cell on every
machine and numpy version.

Mesh: periodic BOUNDARY_CONDITION 2 with N = round(L/h) points per axis (h = L/N), or the
reference-runnable layout BOUNDARY_CONDITION 1 with N+1 points (h = L/N as well, the last
plane repeating the first).
"""
import math
import os
import shutil

import numpy as np

PSD_MG = os.path.join(os.path.dirname(os.path.abspath(__file__)), "decks", "pseudopotential",
                      "psd_Mg.pot")
A_MG = 8.5
KB_HA_PER_K = 8.617343e-5 / 27.211384523   # src/lsdft_readfiles.cc:40-41
DEFAULT_SEED = 20261203


def beta_of_kelvin(t_kelvin):
    return 1.0 / (KB_HA_PER_K * t_kelvin)


class _Stream:
    def __init__(self, seed):
        self._bg = np.random.PCG64(seed)

    def uniform(self, n):
        raw = self._bg.random_raw(n).astype(np.uint64)
        return (raw >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)

    def normal(self, n):
        m = (n + 1) // 2
        u1 = self.uniform(m)
        u2 = self.uniform(m)
        u1 = np.where(u1 <= 0.0, 1.0 / 9007199254740992.0, u1)
        r = np.sqrt(-2.0 * np.log(u1))
        z = np.concatenate([r * np.cos(2 * math.pi * u2), r * np.sin(2 * math.pi * u2)])
        return z[:n]


def fcc_positions(ncell, a=A_MG):
    basis = np.array([[0, 0, 0], [0.5, 0.5, 0], [0.5, 0, 0.5], [0, 0.5, 0.5]])
    cells = np.array([[i, j, k] for k in range(ncell) for j in range(ncell) for i in range(ncell)])
    pos = (cells[:, None, :] + basis[None, :, :]).reshape(-1, 3) * a
    return pos - 0.5 * a * ncell


def make_fcc_mg_deck(out_dir, name, ncell, h, rcut, n_qp, disp=0.1, disp_kind="uniform",
                     seed=DEFAULT_SEED, lloc=2, temperature_k=1000.0, reference_layout=False,
                     mixing=0.3, mixing_history=7, tol_scf=1e-6):
    """Write an FCC Mg deck; returns (out_dir, name, info dict)."""
    L = A_MG * ncell
    N = int(round(L / h))
    pos = fcc_positions(ncell)
    s = _Stream(seed)
    if disp_kind == "uniform":
        pos = pos + (2.0 * s.uniform(pos.size).reshape(pos.shape) - 1.0) * disp
    elif disp_kind == "gaussian":
        pos = pos + s.normal(pos.size).reshape(pos.shape) * disp
    elif disp_kind != "none":
        raise ValueError("disp_kind must be uniform, gaussian or none")
    os.makedirs(os.path.join(out_dir, "pseudopotential"), exist_ok=True)
    dst = os.path.join(out_dir, "pseudopotential", "psd_Mg.pot")
    if not os.path.exists(dst):
        shutil.copyfile(PSD_MG, dst)
    R = 0.5 * L
    grid = N + 1 if reference_layout else N
    bc = 1 if reference_layout else 2
    beta = beta_of_kelvin(temperature_k)
    with open(os.path.join(out_dir, name + ".inpt"), "w") as f:
        f.write("FD_ORDER: 12\n")
        f.write("CELL: %.16f %.16f %.16f\n" % (R, R, R))
        f.write("FD_GRID: %d %d %d\n" % (grid, grid, grid))
        f.write("BOUNDARY_CONDITION: %d\n" % bc)
        f.write("BETA: %.12f\n" % beta)
        f.write("EXCHANGE_CORRELATION: LDA_PW\n")
        f.write("LANCZOS_DEGREE: %d\n" % n_qp)
        f.write("NTYPE: 1\n")
        f.write("RADIUS_TRUNC: %.12g\n" % rcut)
        f.write("TOL_SCF: %g\n" % tol_scf)
        f.write("MIXING_PARAMETER: %g\n" % mixing)
        f.write("MIXING_HISTORY: %d\n" % mixing_history)
        f.write("PULAY_FREQUENCY: 2\n")
        f.write("PSEUDOPOTENTIAL_LOCAL: %d\n" % lloc)
        f.write("PSEUDOPOTENTIAL_FILE: psd_Mg.pot\n")
        f.write("# synthetic FCC Mg: ncell=%d seed=%d disp=%g (%s) h=%.6f\n"
                % (ncell, seed, disp, disp_kind, L / N))
    with open(os.path.join(out_dir, name + ".ion"), "w") as f:
        f.write("%d\n\nMg 2 %d\n" % (len(pos), len(pos)))
        for p in pos:
            f.write("%.16f %.16f %.16f\n" % tuple(p))
    with open(os.path.join(out_dir, name + ".relax"), "w") as f:
        f.write("Mg %d\n" % len(pos))
        for _ in pos:
            f.write("0 0 0\n")
    return out_dir, name, {"natoms": len(pos), "N": N, "h": L / N, "L": L, "beta": beta}


# The benchmark cells (FCC Mg, periodic), by their sizes.
CONFIGS = {
    "mg4_h0.5_rc6_q30": dict(ncell=1, h=0.5, rcut=6.0, n_qp=30, disp=0.1),
    "mg32_h0.5_rc6.5_q40": dict(ncell=2, h=0.5, rcut=6.5, n_qp=40, disp=0.15),
    "mg108_h0.5_rc6.5_q40": dict(ncell=3, h=0.5, rcut=6.5, n_qp=40, disp=0.25,
                                 disp_kind="gaussian"),
    "mg500_h0.5_rc7_q50": dict(ncell=5, h=0.5, rcut=7.0, n_qp=50, disp=0.2),
    # the uneven batch: three cells of different meshes, cube sizes (25^3, 33^3, 27^3) and
    # Lanczos degrees in one submission
    "uneven_a_mg4_h0.5_rc6_q30": dict(ncell=1, h=0.5, rcut=6.0, n_qp=30, disp=0.2),
    "uneven_b_mg32_h0.45_rc7_q40": dict(ncell=2, h=0.45, rcut=7.0, n_qp=40, disp=0.2),
    "uneven_c_mg108_h0.5_rc6.5_q50": dict(ncell=3, h=0.5, rcut=6.5, n_qp=50, disp=0.2),
}
