"""CPU checks of the SCF closure's oracle (oracle/scf.py) and of the library's host LDA.

The reference declares the SCF pieces without bodies, so these pin the restated method by
its own mathematics: the Poisson solve inverts the FD Laplacian of Create_Laplacian
(src/lsdft_initObjs.cc:308-367) exactly, the LDA potential is the density derivative of the
LDA energy, the pseudocharges carry the valence charge, and the SCF reaches TOL_SCF.
"""
import math

import numpy as np
import pytest


@pytest.fixture(scope="module")
def small_scf(small_cell, oracle_mod):
    from oracle import scf as oscf
    d, name, _ = small_cell
    o = oracle_mod.Oracle(d, name, faithful=False)
    fields = oscf.scf_fields(o)
    return o, fields


def test_lda_exchange_and_derivative():
    from oracle.scf import lda_pw92
    rho = np.logspace(-6, 1, 57)
    eps, v = lda_pw92(rho)
    # v = d(rho eps)/d rho (central differences in log rho)
    h = 1e-5
    ep, _ = lda_pw92(rho * (1 + h))
    em, _ = lda_pw92(rho * (1 - h))
    dnum = (rho * (1 + h) * ep - rho * (1 - h) * em) / (2 * h * rho)
    np.testing.assert_allclose(v, dnum, rtol=1e-8)
    # the correlation part vanishes against exchange at high density; exchange is exact Slater
    ex = -0.75 * (3 * rho / math.pi) ** (1 / 3)
    assert np.all(eps < ex)  # correlation is negative
    # high-density limit: d eps_c / d ln rs -> A = (1 - ln 2) / pi^2 (Gell-Mann-Brueckner)
    rs = np.array([1e-7, 2e-7])
    r = 3 / (4 * math.pi * rs ** 3)
    e, _ = lda_pw92(r)
    ec = e - (-0.75 * (3 * r / math.pi) ** (1 / 3))
    slope = (ec[1] - ec[0]) / math.log(2.0)
    assert slope == pytest.approx((1 - math.log(2)) / math.pi ** 2, rel=2e-3)
    # zero density
    e0, v0 = lda_pw92(np.array([0.0, -1e-3]))
    assert np.all(e0 == 0) and np.all(v0 == 0)


def test_library_host_lda_matches_oracle():
    from oracle.scf import lda_pw92 as oracle_lda
    from sqminiapp_gb300 import lda_pw92
    rho = np.concatenate([np.logspace(-12, 2, 300), [0.0]])
    e1, v1 = lda_pw92(rho)
    e2, v2 = oracle_lda(rho)
    np.testing.assert_allclose(e1, e2, rtol=1e-13, atol=0)
    np.testing.assert_allclose(v1, v2, rtol=1e-13, atol=0)


def test_reference_potential_is_c2():
    from oracle.scf import reference_potential
    rc, z = 0.5, 2.0
    f = lambda r: float(reference_potential(r, rc, z))
    assert f(rc * (1 - 1e-13)) == pytest.approx(-z / rc, rel=1e-11)  # continuous value
    eps = 1e-5
    d_in = (f(rc - eps) - f(rc - 3 * eps)) / (2 * eps)     # one-sided slopes at rc - 2 eps
    d_out = (f(rc + 3 * eps) - f(rc + eps)) / (2 * eps)    # and rc + 2 eps
    assert d_in == pytest.approx(z / rc ** 2, rel=1e-3) and d_out == pytest.approx(z / rc ** 2, rel=1e-3)
    c_in = (f(rc - eps) - 2 * f(rc - 2 * eps) + f(rc - 3 * eps)) / eps ** 2
    assert c_in == pytest.approx(-2 * z / rc ** 3, rel=1e-2)  # second derivative of -z/r
    assert reference_potential(3.0, rc, z) == pytest.approx(-z / 3.0)
    assert np.isfinite(reference_potential(0.0, rc, z))


def test_poisson_inverts_fd_laplacian(small_scf):
    from oracle.scf import poisson
    o, fields = small_scf
    rng = np.random.default_rng(11)
    rho = rng.standard_normal(fields["b"].shape)
    phi = poisson(rho, fields["green"])
    cx, cy, cz = o.fd_coeffs()
    lap = (cx[0] + cy[0] + cz[0]) * phi
    for q in range(1, o.order + 1):
        lap += cx[q] * (np.roll(phi, q, 2) + np.roll(phi, -q, 2))
        lap += cy[q] * (np.roll(phi, q, 1) + np.roll(phi, -q, 1))
        lap += cz[q] * (np.roll(phi, q, 0) + np.roll(phi, -q, 0))
    # -(1/4 pi) Lap phi = (1/2 pi) (-1/2 Lap) phi = rho - mean(rho)
    np.testing.assert_allclose(lap / (2 * math.pi), rho - rho.mean(), atol=1e-11)
    assert abs(phi.mean()) < 1e-12


def test_fields_carry_the_charges(small_scf):
    o, f = small_scf
    ne = o.n_electrons
    assert f["b_total"] == pytest.approx(-ne, rel=1e-4)
    assert np.sum(f["rho0"]) * o.dV == pytest.approx(ne, rel=1e-13)
    assert np.all(f["rho0"] >= 0)
    assert f["e_self"] > 0 and f["e_self_ref"] > 0
    assert abs(f["e_corr"]) < 1e-2 * o.natoms
    # the correction potential vanishes away from the atoms (both potentials are -Z/r there)
    assert np.min(np.abs(f["vc"])) < 1e-6


def test_periodic_pulay_reduces_to_linear_mixing():
    from oracle.scf import periodic_pulay_step
    rng = np.random.default_rng(5)
    x = rng.uniform(0.1, 1.0, (4, 4, 4))
    f = rng.standard_normal((4, 4, 4)) * 0.01
    st = {"dX": [], "dF": [], "x_prev": None}
    np.testing.assert_allclose(periodic_pulay_step(x, f, st, 0, 0.3, 7, 2), x + 0.3 * f)
    # on a linear residual map f(x) = A (x* - x) with SPD A, Pulay steps reach x* quickly
    n = 16
    M = rng.standard_normal((n, n))
    A = 0.2 * np.eye(n) + 0.05 * (M @ M.T) / n
    xs = rng.uniform(0.5, 1.0, n)
    x = np.full(n, 0.75)
    st = {"dX": [], "dF": [], "x_prev": None}
    for k in range(40):
        fk = A @ (xs - x)
        if np.linalg.norm(fk) < 1e-12:
            break
        x = periodic_pulay_step(x, fk, st, k, 0.5, 16, 2)
    assert np.linalg.norm(x - xs) < 1e-8


def test_oracle_scf_converges(small_scf):
    from oracle.scf import scf
    o, fields = small_scf
    r = scf(o, fields, tol=1e-6, maxit=80)
    assert r["converged"], r["residual_history"]
    F = r["free_energy_history"] / o.natoms
    assert abs(F[-1] - F[-2]) < 1e-6
    # the self-consistent density carries the electron count and is non-negative
    assert np.sum(r["rho_out"]) * o.dV == pytest.approx(o.n_electrons, rel=1e-9)
    assert np.all(r["rho_out"] >= -1e-12)
    # restarting from the converged density converges within a few iterations
    r2 = scf(o, fields, tol=1e-6, maxit=6, rho_init=r["rho_out"])
    assert r2["iterations"] <= 4 and r2["converged"]
    assert r2["free_energy_per_atom"] == pytest.approx(r["free_energy_per_atom"], abs=1e-6)


def test_library_scf_fields_match_oracle(small_scf, small_cell):
    """The product's host construction of the fixed SCF fields (scf_setup.cpp, reported
    without a GPU) against the oracle's independent numpy construction."""
    import ctypes
    from sqminiapp_gb300.capi import check, lib
    o, ref = small_scf
    d, name, _ = small_cell
    nx, ny, nz = o.grid
    dp = ctypes.POINTER(ctypes.c_double)
    b = np.zeros(nx * ny * nz)
    rho0 = np.zeros(nx * ny * nz)
    green = np.zeros(nz * ny * (nx // 2 + 1))
    sc = np.zeros(4)
    check(lib().sq_describe_scf_fields(d.encode(), name.encode(), b.ctypes.data_as(dp),
                                       rho0.ctypes.data_as(dp), green.ctypes.data_as(dp),
                                       sc.ctypes.data_as(dp)), "sq_describe_scf_fields")
    shape = ref["b"].shape
    assert np.max(np.abs(b.reshape(shape) - ref["b"])) <= 1e-12 * np.max(np.abs(ref["b"]))
    assert np.max(np.abs(rho0.reshape(shape) - ref["rho0"])) <= 1e-12 * np.max(ref["rho0"])
    np.testing.assert_allclose(green.reshape(ref["green"].shape), ref["green"], rtol=1e-12, atol=0)
    for k, v in zip(("e_self", "e_self_ref", "e_corr", "b_total"), sc):
        assert v == pytest.approx(ref[k], rel=1e-10, abs=1e-12), k
