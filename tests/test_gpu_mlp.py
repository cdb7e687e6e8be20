"""GPU learned warm start: descriptor kernel, tensor-core forward and backward kernels against
the numpy oracle (oracle/mlp.py), training, and the gain of the learned SCF start.

Tolerances.  Descriptors: FP32 kernel vs float64, 1e-4 relative to the largest feature.  The
network rounds to BF16 at the same points as the oracle; the remaining differences are FP32
summation order and the occasional BF16 tie broken the other way (one BF16 ulp, 2^-8
relative, in single entries), so outputs agree to 1e-3 of their scale and gradients to 1e-2
of the largest entry of each block.
"""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _params(rng):
    return {"W1": rng.standard_normal((64, 128)) * math.sqrt(2 / 64),
            "b1": rng.standard_normal(128) * 0.1,
            "W2": rng.standard_normal((128, 128)) * math.sqrt(2 / 128),
            "b2": rng.standard_normal(128) * 0.1, "w3": rng.standard_normal(128) * math.sqrt(1 / 128),
            "b3": np.array([0.05])}


def test_forward_matches_oracle():
    from oracle.mlp import forward
    from sqminiapp_gb300 import WarmStartMLP
    rng = np.random.default_rng(10)
    p = _params(rng)
    m = WarmStartMLP(seed=3)
    m.set_params(p)
    x = rng.standard_normal((300, 64)).astype(np.float32)  # 3 tiles, the last one partial
    y = m.forward(x)
    ref = forward({k: v.astype(np.float32).astype(np.float64) for k, v in p.items()}, x)
    assert np.max(np.abs(y - ref)) <= 1e-3 * max(1.0, np.max(np.abs(ref)))


def test_gradients_match_oracle():
    from oracle.mlp import forward_backward
    from sqminiapp_gb300 import WarmStartMLP
    rng = np.random.default_rng(11)
    p = _params(rng)
    m = WarmStartMLP(seed=3)
    m.set_params(p)
    x = rng.standard_normal((333, 64)).astype(np.float32)
    t = rng.standard_normal(333).astype(np.float32)
    loss, g = m.gradients(x, t)
    p64 = {k: v.astype(np.float32).astype(np.float64) for k, v in p.items()}
    lref, gref, _ = forward_backward(p64, x.astype(np.float64), t.astype(np.float64))
    assert loss == pytest.approx(lref, rel=1e-3)
    for k in gref:
        err = np.max(np.abs(g[k] - gref[k]))
        assert err <= 1e-2 * np.max(np.abs(gref[k])), (k, err, np.max(np.abs(gref[k])))


def test_descriptors_match_oracle(small_cell):
    from oracle.mlp import descriptors
    from sqminiapp_gb300 import LSDFT
    d, name, _ = small_cell
    import oracle
    o = oracle.Oracle(d, name, faithful=False)
    pos, _ = o.atoms()
    nx, ny, nz = o.grid
    idx = np.arange(0, nx * ny * nz, 7)
    i, j, k = idx % nx, (idx // nx) % ny, idx // (nx * ny)
    pts = np.stack([i * o.h[0] - o.range[0], j * o.h[1] - o.range[1], k * o.h[2] - o.range[2]], 1)
    ref = descriptors(pts, pos, 2 * np.array(o.range))
    with LSDFT(d, name, faithful=False, precision=32) as eng:
        got = eng.descriptors()[idx]
    assert np.max(np.abs(got - ref)) <= 1e-4 * np.max(np.abs(ref))


def test_training_fits_a_smooth_target():
    """Adam on the tensor-core kernels drives the loss of a learnable target down."""
    from sqminiapp_gb300 import WarmStartMLP
    rng = np.random.default_rng(12)
    m = WarmStartMLP(seed=5)
    x = rng.standard_normal((4096, 64)).astype(np.float32)
    t = (np.tanh(x[:, 0] - 0.5 * x[:, 3]) + 0.3 * x[:, 7] * x[:, 9]).astype(np.float32)
    l0, _ = m.gradients(x, t)
    # train through the gradient kernel: plain SGD steps from the host
    p = m.get_params()
    lr = 0.05
    for _ in range(150):
        loss, g = m.gradients(x, t)
        for k in g:
            p[k] = p[k] - lr * g[k]
        m.set_params({k: p[k] for k in g})
    l1, _ = m.gradients(x, t)
    assert l1 < 0.2 * l0, (l0, l1)


def test_learned_start_beats_atomic_superposition(tmp_path):
    """Trained on converged densities of three seeded 4-atom cells, the network's start
    density is closer to the SCF solution of a fourth cell than the atomic superposition,
    and its SCF needs no more iterations."""
    from sqminiapp_gb300 import LSDFT, WarmStartMLP
    from sqminiapp_gb300.decks import make_fcc_mg_deck
    kw = dict(ncell=1, h=0.85, rcut=3.4, n_qp=20, disp=0.25, disp_kind="gaussian")
    m = WarmStartMLP(seed=7)
    for seed in (101, 102, 103):
        d, name, _ = make_fcc_mg_deck(str(tmp_path / ("c%d" % seed)), "c", seed=seed, **kw)
        with LSDFT(d, name, faithful=False, precision=32) as eng:
            eng.SCF_LSSGQ()
            m.add_training_cell(eng)
    loss = m.train(steps=400, tiles_per_step=16, lr=2e-3)
    assert loss < 0.5
    d, name, _ = make_fcc_mg_deck(str(tmp_path / "test"), "c", seed=999, **kw)
    with LSDFT(d, name, faithful=False, precision=32) as eng:
        base = eng.SCF_LSSGQ()
        rho_scf, _ = eng.scf_density()
        rho_pred = m.predict_density(eng)
        rho0 = eng.scf_fields()["rho0"]
        learned = eng.SCF_LSSGQ(model=m)
    err_pred = np.linalg.norm(rho_pred - rho_scf)
    err_atomic = np.linalg.norm(rho0 - rho_scf)
    assert err_pred < 0.7 * err_atomic, (err_pred, err_atomic)
    assert learned["converged"] == 1
    assert learned["iterations"] <= base["iterations"]
    assert learned["free_energy_per_atom"] == pytest.approx(base["free_energy_per_atom"], abs=1e-5)
    path = tmp_path / "m.bin"
    m.save(path)
    m2 = WarmStartMLP(path=path)
    with LSDFT(d, name, faithful=False, precision=32) as eng:
        np.testing.assert_array_equal(m2.predict_density(eng), rho_pred)


def test_learned_start_highpass_limits(tmp_path):
    """sq_scf_options.learned_highpass: the start keeps the network's correction to the
    superposition scaled by the Kerker symbol k^2/(k^2 + k0^2).  A tiny k0 keeps all of it
    (the plain learned start, up to the k = 0 mode that the electron count fixes), a huge k0
    none (the superposition); every start is non-negative with N_e electrons."""
    import ctypes
    from sqminiapp_gb300 import LSDFT, WarmStartMLP
    from sqminiapp_gb300.capi import check
    from sqminiapp_gb300.decks import make_fcc_mg_deck
    d, name, meta = make_fcc_mg_deck(str(tmp_path), "c", ncell=1, h=0.85, rcut=3.4, n_qp=20,
                                     disp=0.25, disp_kind="gaussian", seed=11)
    rng = np.random.default_rng(12)
    m = WarmStartMLP(seed=9)
    m.set_params(_params(rng))
    with LSDFT(d, name, faithful=False, precision=32) as eng:
        dV = float(np.prod(eng.info.h[:]))

        def start(k0):
            opt = eng._scf_options(None, None, None, None, None, None, None,
                                   learned_highpass=k0)
            check(eng._lib.sq_scf_begin_learned(eng._h, ctypes.byref(opt), m._m), "learned")
            return eng.scf_density()[1].copy()

        plain, low, high, mid = start(0.0), start(1e-6), start(1e6), start(1.0)
        eng.scf_begin()
        rho0 = eng.scf_density()[1].copy()
    ne = rho0.sum() * dV
    for r in (plain, low, high, mid):
        assert np.all(r >= 0.0)
        assert r.sum() * dV == pytest.approx(ne, rel=1e-12)
    scale = np.max(np.abs(plain))
    assert np.max(np.abs(low - plain)) < 1e-6 * scale
    assert np.max(np.abs(high - rho0)) < 1e-6 * scale
    # k0 = 1/bohr keeps part of the correction: strictly between the two
    assert 0 < np.linalg.norm(mid - rho0) < np.linalg.norm(plain - rho0)
