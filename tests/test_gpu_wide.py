"""GPU parity for the large-cube layouts.

Cubes wider than 32 points: the uneven-batch workload's 32-atom cell (side 17 bohr, 38^3
mesh, h = 0.4474 bohr, Rcut = 7 bohr, so 33^3 cubes; 40 Lanczos steps) through the FP32
split-pass kernel on CTA pairs and through the single-pass wide kernel, against the FP64 CPU
oracle, and inside a mixed-cell batch.  Cubes of 29^3: FP64 rows
without zero columns, FP32 planes without zero rows between them (U on chip).

Tolerance: FP32 vectors (unit roundoff 6e-8) over 40 steps, the same 1e-4 relative bound on
the quadrature moments of order <= 3 as the narrow FP32 kernel's parity tests; the first
Lanczos coefficients to 1e-4 relative."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def wide_cell(tmp_path_factory):
    from sqminiapp_gb300.decks import make_fcc_mg_deck
    d = str(tmp_path_factory.mktemp("mg32wide"))
    return make_fcc_mg_deck(d, "mg32w", ncell=2, h=0.45, rcut=7.0, n_qp=40, disp=0.2, seed=23)


def _moments(lam, w):
    return [np.sum(w * lam ** k, axis=1) for k in range(4)]


@pytest.mark.parametrize("kernel", [0, 1])
def test_wide_cube_matches_oracle(wide_cell, oracle_mod, kernel):
    """kernel 0: the split-pass kernel on a CTA pair per node (U on chip); kernel 1: the
    single-pass wide kernel (U in global scratch, compact list)."""
    from sqminiapp_gb300 import LSDFT
    d, name, _ = wide_cell
    o = oracle_mod.Oracle(d, name, faithful=False)
    nodes = np.arange(0, o.n_nodes, 1409)
    rng = np.random.default_rng(12)
    veff = -0.25 + 0.05 * rng.standard_normal(o.n_nodes)
    ref = o.nodes_and_weights(nodes=nodes, veff=veff, want_ab=True)
    with LSDFT(d, name, faithful=False, precision=32, kernel=kernel) as eng:
        assert eng.n_nodes == 38 ** 3
        if kernel == 0:
            assert eng.info.kernel_layout == 16 | 32 and eng.info.kernel_u_on_chip == 1
            assert eng.info.kernel_threads == 384
        else:
            # y gaps + wide (+ the compact list, which this cell's 33^3 lists need in L2)
            assert eng.info.kernel_layout & 3 == 3 and eng.info.kernel_u_on_chip == 0
            assert eng.info.kernel_threads == 576
        full = eng.NodesAndWeights_LSSGQ(veff=veff)
        a, b = eng.lanczos_coefficients(eng.n_nodes)
    np.testing.assert_allclose(a[nodes, :3], ref["a"][:, :3], rtol=1e-3, atol=1e-4)
    np.testing.assert_allclose(b[nodes, :3], ref["b"][:, :3], rtol=1e-3, atol=1e-4)
    for k, (g, e) in enumerate(zip(_moments(full["lambda"][nodes], full["weights"][nodes]),
                                   _moments(ref["lambda"], ref["weights"]))):
        err = np.max(np.abs(g - e) / np.maximum(1.0, np.abs(e)))
        assert err < 1e-4, "moment %d error %.3e" % (k, err)
    for k in ("lambda_min", "lambda_max"):
        np.testing.assert_allclose(full[k][nodes], ref[k], rtol=1e-3, atol=1e-3)
    # every node of the full grid: weights sum to 1
    assert np.allclose(np.sum(full["weights"], axis=1), 1.0, atol=1e-6)
    assert np.all(np.isfinite(full["lambda"]))


def test_wide_cube_rejects_fp64(wide_cell):
    from sqminiapp_gb300 import LSDFT, SqError
    d, name, _ = wide_cell
    with pytest.raises(SqError) as e:
        LSDFT(d, name, faithful=False, precision=64)
    assert "FP32" in str(e.value)


def test_wide_cube_in_mixed_batch(wide_cell, small_cell):
    """A 33^3-cube cell beside a 9^3-cube cell in one batch submission: each gives its
    single-cell result."""
    import torch
    from sqminiapp_gb300 import LSDFT, batch_nodes_and_weights
    cells = [LSDFT(*wide_cell[:2], faithful=False, precision=32),
             LSDFT(*small_cell[:2], faithful=False, precision=32)]
    dev = torch.device("cuda", 0)
    rng = np.random.default_rng(9)
    veffs, outs, refs = [], [], []
    for e in cells:
        v = -0.2 + 0.05 * rng.standard_normal(e.n_nodes)
        refs.append(e.NodesAndWeights_LSSGQ(veff=v))
        veffs.append(torch.from_numpy(v).to(dev))
        outs.append({k: torch.empty(s, dtype=torch.float64, device=dev) for k, s in
                     (("lambda", (e.n_nodes, e.n_qp)), ("weights", (e.n_nodes, e.n_qp)),
                      ("lambda_min", (e.n_nodes,)), ("lambda_max", (e.n_nodes,)))})
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream(dev).cuda_stream
    batch_nodes_and_weights(cells, [v.data_ptr() for v in veffs], None,
                            [{k: t.data_ptr() for k, t in o.items()} for o in outs], stream)
    torch.cuda.synchronize()
    for o, r in zip(outs, refs):
        lam, w = o["lambda"].cpu().numpy(), o["weights"].cpu().numpy()
        for g, e in zip(_moments(lam, w), _moments(r["lambda"], r["weights"])):
            assert np.max(np.abs(g - e) / np.maximum(1.0, np.abs(e))) < 1e-4
    for e in cells:
        e.close()


def test_fp64_unpadded_rows_match_oracle(tmp_path_factory, oracle_mod):
    """29^3 cubes (h = 0.5, Rcut = 7 bohr, the 500-atom workload's cube) in FP64: the x-padded
    rows would need 235 KB of shared memory, so the kernel keeps rows of exactly 29 points and
    bounds-checks x.  FP64 tolerance 1e-9 (summation order only)."""
    from sqminiapp_gb300 import LSDFT
    from sqminiapp_gb300.decks import make_fcc_mg_deck
    d, name, _ = make_fcc_mg_deck(str(tmp_path_factory.mktemp("mg4rc7")), "mg4rc7", ncell=1,
                                  h=0.5, rcut=7.0, n_qp=30, disp=0.2, seed=41)
    o = oracle_mod.Oracle(d, name, faithful=False)
    nodes = np.arange(0, o.n_nodes, 97)
    rng = np.random.default_rng(13)
    veff = -0.25 + 0.05 * rng.standard_normal(o.n_nodes)
    ref = o.nodes_and_weights(nodes=nodes, veff=veff, want_ab=True)
    with LSDFT(d, name, faithful=False, precision=64) as eng:
        assert eng.info.kernel_layout == 4  # rows without zero columns
        full = eng.NodesAndWeights_LSSGQ(veff=veff)
        a, b = eng.lanczos_coefficients(eng.n_nodes)
    np.testing.assert_allclose(a[nodes, :5], ref["a"][:, :5], rtol=1e-9, atol=1e-10)
    np.testing.assert_allclose(b[nodes, :5], ref["b"][:, :5], rtol=1e-9, atol=1e-10)
    for k, (g, e) in enumerate(zip(_moments(full["lambda"][nodes], full["weights"][nodes]),
                                   _moments(ref["lambda"], ref["weights"]))):
        err = np.max(np.abs(g - e) / np.maximum(1.0, np.abs(e)))
        assert err < 1e-9, "moment %d error %.3e" % (k, err)
    with LSDFT(d, name, faithful=False, precision=32) as eng:
        # FP32 (y bounds-checked): no zero rows between z-planes, so that U fits on chip beside P
        assert eng.info.kernel_layout & 7 == 0 and eng.info.kernel_u_on_chip == 1
        f32 = eng.NodesAndWeights_LSSGQ(veff=veff)
    for g, e in zip(_moments(f32["lambda"], f32["weights"]), _moments(full["lambda"], full["weights"])):
        assert np.max(np.abs(g - e) / np.maximum(1.0, np.abs(e))) < 1e-4


@pytest.mark.parametrize("which", ["wide", "small"])
def test_compact_list_matches_full(which, wide_cell, small_cell):
    """The compact projector list (T_l per channel + box coordinates, chi_lm rebuilt while
    streaming) forms the same products as the full list, so the two agree up to the order of
    the FP32 atomic accumulations: 1e-5 relative on the quadrature moments (which the first
    Lanczos coefficients fix)."""
    from sqminiapp_gb300 import LSDFT
    d, name, _ = wide_cell if which == "wide" else small_cell
    out = {}
    for fmt in (1, 2):
        with LSDFT(d, name, faithful=False, precision=32, list_format=fmt) as eng:
            assert bool(eng.info.kernel_layout & 8) == (fmt == 2)
            rng = np.random.default_rng(21)
            veff = -0.2 + 0.05 * rng.standard_normal(eng.n_nodes)
            out[fmt] = eng.NodesAndWeights_LSSGQ(veff=veff)
    for g, e in zip(_moments(out[2]["lambda"], out[2]["weights"]),
                    _moments(out[1]["lambda"], out[1]["weights"])):
        assert np.max(np.abs(g - e) / np.maximum(1.0, np.abs(e))) < 1e-5


def _parity(eng_out, ref, nodes, tol):
    for k, (g, e) in enumerate(zip(_moments(eng_out["lambda"][nodes], eng_out["weights"][nodes]),
                                   _moments(ref["lambda"], ref["weights"]))):
        err = np.max(np.abs(g - e) / np.maximum(1.0, np.abs(e)))
        assert err < tol, "moment %d error %.3e" % (k, err)


@pytest.mark.parametrize("kernel", [0, 1])
def test_fp32_31cube(tmp_path_factory, oracle_mod, kernel):
    """31^3 cubes (h = 0.5, Rcut = 7.5 bohr): the split-pass kernel runs a CTA pair per node
    (kernel 0); the single-pass kernel (kernel 1) keeps P with its y gaps on chip and U in
    global scratch; FP64 fits no single-CTA layout there."""
    from sqminiapp_gb300 import LSDFT, SqError
    from sqminiapp_gb300.decks import make_fcc_mg_deck
    d, name, _ = make_fcc_mg_deck(str(tmp_path_factory.mktemp("mg4rc75")), "mg4rc75", ncell=1,
                                  h=0.5, rcut=7.5, n_qp=30, disp=0.2, seed=43)
    o = oracle_mod.Oracle(d, name, faithful=False)
    nodes = np.arange(0, o.n_nodes, 131)
    veff = np.full(o.n_nodes, -0.2)
    ref = o.nodes_and_weights(nodes=nodes, veff=veff)
    with LSDFT(d, name, faithful=False, precision=32, kernel=kernel) as eng:
        assert eng.cube == (31, 31, 31)
        if kernel == 0:
            assert eng.info.kernel_layout == 16 | 32 and eng.info.kernel_u_on_chip == 1
        else:
            assert eng.info.kernel_layout & 7 == 1 and eng.info.kernel_u_on_chip == 0
        got = eng.NodesAndWeights_LSSGQ(veff=veff)
    _parity(got, ref, nodes, 1e-4)
    with pytest.raises(SqError) as e:
        LSDFT(d, name, faithful=False, precision=64)
    assert "shared memory" in str(e.value)


@pytest.mark.parametrize("precision,tol", [(32, 1e-4), (64, 1e-9)])
def test_faithful_operator_on_large_cube_layouts(precision, tol, tmp_path_factory, oracle_mod):
    """The reference's shared-slot operator through the 29^3 layouts (FP32 planes without y
    gaps, FP64 rows without zero columns) against the faithful oracle."""
    from sqminiapp_gb300 import LSDFT
    from sqminiapp_gb300.decks import make_fcc_mg_deck
    d, name, _ = make_fcc_mg_deck(str(tmp_path_factory.mktemp("mg4rc7f")), "mg4rc7f", ncell=1,
                                  h=0.5, rcut=7.0, n_qp=30, disp=0.2, seed=41)
    o = oracle_mod.Oracle(d, name, faithful=True)
    nodes = np.arange(0, o.n_nodes, 163)
    veff = np.full(o.n_nodes, -0.2)
    ref = o.nodes_and_weights(nodes=nodes, veff=veff)
    with LSDFT(d, name, faithful=True, precision=precision) as eng:
        assert eng.info.kernel_layout == (0 if precision == 32 else 4)
        got = eng.NodesAndWeights_LSSGQ(veff=veff)
    _parity(got, ref, nodes, tol)


def test_faithful_operator_on_wide_cube(wide_cell, oracle_mod):
    """The shared-slot operator on the 33^3 cell (FP32 WIDE, full records)."""
    from sqminiapp_gb300 import LSDFT
    d, name, _ = wide_cell
    o = oracle_mod.Oracle(d, name, faithful=True)
    nodes = np.arange(0, o.n_nodes, 2417)
    veff = np.full(o.n_nodes, -0.2)
    ref = o.nodes_and_weights(nodes=nodes, veff=veff)
    with LSDFT(d, name, faithful=True, precision=32) as eng:
        assert eng.info.kernel_layout == 3
        got = eng.NodesAndWeights_LSSGQ(veff=veff)
    _parity(got, ref, nodes, 1e-4)
