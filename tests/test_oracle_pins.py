"""Pins of the FP64 CPU oracle (CPU only).

The reference prints no quadrature values, so the oracle is pinned two ways:
* against the counts the reference's own run logs print for its Mg1 deck
  (test/a1.out:12, a2.out:20,29, a4.out:36-63, a4a.out:70-76);
* against independent mathematics (numpy / scipy known answers).
"""
import math

import numpy as np
import pytest


@pytest.fixture(scope="module")
def mg1(deck_dir, oracle_mod):
    return oracle_mod.Oracle(deck_dir, "Mg1", faithful=True)


def test_mg1_grid_and_nodes(mg1):
    # 11 x 18 x 17 = 3366 FD nodes (test/a4a.out:70-76: 891 + 891 + 792 + 792)
    assert mg1.grid == (11, 18, 17)
    assert mg1.n_nodes == 3366 == 891 + 891 + 792 + 792
    assert mg1.nloc == (21, 21, 21)  # 2*ceil(6/h)+1, src/lsdft_readfiles.cc:442-444
    assert mg1.n_qp == 10
    assert mg1.nlm0 == 6             # lmax=2, lloc=1: s + d
    assert mg1.n_electrons == 8


@pytest.mark.parametrize("extra,counts", [
    # the reference's atom loop reads one entry past the 4 atoms (initObjs.cc:3038); the logs
    # match that fifth entry being an atom at the origin
    ([0.0, 0.0, 0.0], {1: [115], 2: [88, 88], 4: [68, 68, 68, 68]}),
    (None, {1: [88], 2: [70, 70], 4: [56, 56, 56, 56]}),
])
def test_local_overlap_counts_match_logs(mg1, extra, counts):
    """AtomOverlap_local[0].Natoms per rank (GetInfluencingAtoms_Local, initObjs.cc:1409-1665).

    Ranks own DMDA blocks of the 11x18x17 grid: 1 rank the whole grid; 2 ranks split y;
    4 ranks split y and z (block sizes 891/891/792/792 in a4a.out)."""
    blocks = {
        1: [((0, 0, 0), (11, 18, 17))],
        2: [((0, 0, 0), (11, 9, 17)), ((0, 9, 0), (11, 9, 17))],
        4: [((0, 0, 0), (11, 9, 9)), ((0, 9, 0), (11, 9, 9)), ((0, 0, 9), (11, 9, 8)),
            ((0, 9, 9), (11, 9, 8))],
    }
    for ranks, expected in counts.items():
        got = [mg1.local_overlap_count(c, d, extra) for c, d in blocks[ranks]]
        assert got == expected


def test_fd_weights_analytic(mg1):
    """-1/2 Laplacian weights of order 2n: c0 = sum 1/p^2 / h^2,
    c_p = (-1)^p (n!)^2 / (p^2 (n-p)! (n+p)!) / h^2 (standard central-difference formula)."""
    n = 6
    cx, cy, cz = mg1.fd_coeffs()
    for c, h in zip((cx, cy, cz), mg1.h):
        assert c[0] == pytest.approx(sum(1.0 / p ** 2 for p in range(1, n + 1)) / h ** 2, rel=1e-15)
        for p in range(1, n + 1):
            w = (-1) ** p * math.factorial(n) ** 2 / (p ** 2 * math.factorial(n - p) * math.factorial(n + p))
            assert c[p] == pytest.approx(w / h ** 2, rel=1e-14)
        # spectral check: the stencil of sin(kx) is k^2/2 sin(kx) to 12th order
        k = 0.3 / h
        sym = c[0] + 2 * sum(c[p] * math.cos(k * p * h) for p in range(1, n + 1))
        assert sym == pytest.approx(0.5 * k * k, rel=1e-8)


def test_spline_is_not_a_knot(oracle_mod):
    """getYD_gen + SplineEvaluate (src/lsdft_tools.cc:15-151) is the not-a-knot cubic spline."""
    from scipy.interpolate import CubicSpline
    rng = np.random.default_rng(0)
    x = np.sort(rng.uniform(0, 5, 40))
    x[0] = 0.0
    y = np.sin(x) + 0.1 * rng.standard_normal(40)
    xq = np.linspace(0, x[-1], 777)
    np.testing.assert_allclose(oracle_mod.spline(x, y, xq),
                               CubicSpline(x, y, bc_type="not-a-knot")(xq), atol=1e-12)


def test_real_spherical_harmonics(oracle_mod):
    """RealSphericalHarmonic (src/lsdft_tools.cc:156-370), l <= 3: orthonormal on the sphere."""
    rng = np.random.default_rng(1)
    v = rng.standard_normal((20000, 3))
    lm = [(l, m) for l in range(4) for m in range(-l, l + 1)]
    Y = np.array([[oracle_mod.ylm(*p, l, m) for (l, m) in lm] for p in v])
    G = 4 * math.pi * (Y.T @ Y) / len(v)  # Monte-Carlo Gram matrix
    np.testing.assert_allclose(G, np.eye(len(lm)), atol=0.06)
    # explicit values
    assert oracle_mod.ylm(0, 0, 2.0, 0, 0) == pytest.approx(0.5 / math.sqrt(math.pi), rel=1e-12)
    assert oracle_mod.ylm(0, 0, 2.0, 1, 0) == pytest.approx(math.sqrt(3 / (4 * math.pi)), rel=1e-12)
    assert oracle_mod.ylm(0, 0, 0, 2, 0) == 0.0  # r < 1e-10: only l = 0 survives


def test_ql_matches_lapack(oracle_mod):
    """TridiagEigenVecSolve_NodesAndWeights (src/lsdft_tools.cc:912-1026): eigenvalues and
    first eigenvector components squared of the tridiagonal (b[n-1] ignored)."""
    rng = np.random.default_rng(2)
    for n in (1, 2, 5, 10, 40, 64):
        a = rng.uniform(-5, 20, n)
        b = rng.uniform(0.1, 8, n)
        lam, w, lo, hi = oracle_mod.ql(a, b)
        T = np.diag(a) + np.diag(b[:n - 1], 1) + np.diag(b[:n - 1], -1)
        ev, V = np.linalg.eigh(T)
        order = np.argsort(lam)
        np.testing.assert_allclose(lam[order], ev, rtol=1e-12, atol=1e-12)
        np.testing.assert_allclose(w[order], V[0] ** 2, atol=1e-12)
        assert lo == pytest.approx(ev[0]) and hi == pytest.approx(ev[-1])
        assert w.sum() == pytest.approx(1.0, abs=1e-13)


def test_gauss_quadrature_small_cube(small_cell, oracle_mod):
    """Corrected operator on a 9^3 cube: the Lanczos Gauss rule integrates e_p^T f(H) e_p of
    the dense truncated Hamiltonian (numpy eigh) - exactly for polynomials of degree < 2 N_qp,
    and to 1e-8 for the smooth exp(-H/4)."""
    d, name, _ = small_cell
    o = oracle_mod.Oracle(d, name, faithful=False)
    assert o.nloc == (9, 9, 9)
    for node in (0, 17, o.n_nodes - 1):
        H = o.dense_hamiltonian(node)
        np.testing.assert_allclose(H, H.T, atol=1e-12)
        ev, V = np.linalg.eigh(H)
        p = H.shape[0] // 2
        wexact = V[p] ** 2
        r = o.nodes_and_weights(nodes=[node], nthreads=1)
        lam, w = r["lambda"][0], r["weights"][0]
        scale = np.max(np.abs(ev))
        for k in range(0, 2 * o.n_qp - 1, 5):
            mq = np.sum(w * (lam / scale) ** k)
            me = np.sum(wexact * (ev / scale) ** k)
            assert mq == pytest.approx(me, rel=1e-9, abs=1e-12)
        f = lambda x: np.exp(-x / 4.0)
        assert np.sum(w * f(lam)) == pytest.approx(np.sum(wexact * f(ev)), rel=1e-8)


def test_fermi_bisection_vs_numpy(oracle_mod):
    rng = np.random.default_rng(3)
    lam = rng.uniform(-2, 5, (300, 12))
    w = rng.dirichlet(np.ones(12), 300)
    beta, ne, dV = 40.0, 170.0, 0.2
    r = oracle_mod.fermi_density_energy(lam, w, beta, ne, dV)
    f = 1 / (1 + np.exp(np.clip(beta * (lam - r["lambda_f"]), -700, 700)))
    assert np.sum(2 * w * f) == pytest.approx(ne, rel=1e-9)
    np.testing.assert_allclose(r["rho"], 2 * np.sum(w * f, axis=1) / dV, rtol=1e-12)
    assert r["e_band"] == pytest.approx(np.sum(2 * w * lam * f), rel=1e-12)
    fs = np.clip(f, 1e-300, 1 - 1e-16)
    ts = np.sum(2 * w * (fs * np.log(fs) + (1 - fs) * np.log1p(-fs))) / beta
    assert r["ts"] == pytest.approx(ts, rel=1e-6, abs=1e-12)


def test_corrected_operator_is_symmetric(deck_dir, oracle_mod):
    o = oracle_mod.Oracle(deck_dir, "Mg1", faithful=False)
    rng = np.random.default_rng(4)
    n = int(np.prod(o.nloc))
    x, y = rng.standard_normal(n), rng.standard_normal(n)
    assert abs(y @ o.matvec(1234, x) - x @ o.matvec(1234, y)) < 1e-9 * abs(y @ o.matvec(1234, x))
