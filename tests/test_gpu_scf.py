"""GPU SCF closure against the FP64 numpy/C++ oracle (oracle/scf.py) on the same deck.

Tolerances.  The fixed fields (pseudocharges, start density, self energies) are FP64 on the
host in both: 1e-12 relative.  The FP64 GPU SCF and the oracle SCF differ in summation order
only, so with both converged to 1e-9 in the density residual their free energies agree to
1e-8 Ha/atom.  The FP32 Lanczos engine must reach the FP64 engine's free energy within
1e-5 Ha/atom, the accuracy target of the mixed-precision engine.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def cell(small_cell, oracle_mod):
    from oracle import scf as oscf
    d, name, _ = small_cell
    o = oracle_mod.Oracle(d, name, faithful=False)
    fields = oscf.scf_fields(o)
    return d, name, o, fields


@pytest.fixture(scope="module")
def oracle_result(cell):
    from oracle import scf as oscf
    _, _, o, fields = cell
    return oscf.scf(o, fields, tol=1e-9, maxit=120)


def test_fields_match_oracle(cell):
    from sqminiapp_gb300 import LSDFT
    d, name, o, ref = cell
    with LSDFT(d, name, faithful=False, precision=64) as eng:
        got = eng.scf_fields()
    for k in ("b", "rho0"):
        g = got[k].reshape(ref[k].shape)
        assert np.max(np.abs(g - ref[k])) <= 1e-12 * np.max(np.abs(ref[k])), k
    for k in ("e_self", "e_self_ref", "e_corr", "b_total"):
        assert got[k] == pytest.approx(ref[k], rel=1e-10, abs=1e-12), k


def test_first_iteration_matches_oracle(cell):
    from oracle import scf as oscf
    from sqminiapp_gb300 import LSDFT
    d, name, o, fields = cell
    ref = oscf.scf(o, fields, tol=1e-30, maxit=1)
    with LSDFT(d, name, faithful=False, precision=64) as eng:
        eng.scf_begin()
        r = eng.scf_step()
        f = eng.scf_fields()
        rho_out, rho_next = eng.scf_density()
    shape = fields["b"].shape
    np.testing.assert_allclose(f["phi"].reshape(shape), ref["phi"], rtol=0, atol=1e-11)
    np.testing.assert_allclose(f["vxc"].reshape(shape), ref["vxc"], rtol=1e-12, atol=1e-14)
    np.testing.assert_allclose(rho_out.reshape(shape), ref["rho_out"], rtol=1e-9, atol=1e-12)
    for k in ("e_band", "e_xc", "e_xc_dc", "e_electrostatic", "ts", "lambda_f", "free_energy"):
        assert r[k] == pytest.approx(ref[k], rel=1e-9, abs=1e-10), k
    assert r["residual"] == pytest.approx(ref["residual"], rel=1e-8)


def test_fp64_scf_matches_oracle(cell, oracle_result):
    from sqminiapp_gb300 import LSDFT
    d, name, o, _ = cell
    ref = oracle_result
    assert ref["converged"]
    with LSDFT(d, name, faithful=False, precision=64) as eng:
        r = eng.SCF_LSSGQ(tol=1e-9, maxit=120)
        rho_out, _ = eng.scf_density()
    assert r["converged"] == 1
    assert abs(r["iterations"] - ref["iterations"]) <= 3
    assert r["free_energy_per_atom"] == pytest.approx(ref["free_energy_per_atom"], abs=1e-8)
    assert r["lambda_f"] == pytest.approx(ref["lambda_f"], abs=1e-7)
    np.testing.assert_allclose(rho_out.reshape(ref["rho_out"].shape), ref["rho_out"], atol=1e-7)


def test_fp32_scf_within_target_of_fp64(cell, oracle_result):
    from sqminiapp_gb300 import LSDFT
    d, name, o, _ = cell
    with LSDFT(d, name, faithful=False, precision=32) as eng:
        r = eng.SCF_LSSGQ(tol=1e-6, maxit=120)
    # FP32 vectors floor the density residual near 1e-5; the engine raises the target to 3e-5
    assert r["tol"] == pytest.approx(3e-5)
    assert r["converged"] == 1
    assert r["free_energy_per_atom"] == pytest.approx(oracle_result["free_energy_per_atom"], abs=1e-5)


def test_warm_start_from_device_density(cell, oracle_result):
    import torch
    from sqminiapp_gb300 import LSDFT
    d, name, o, _ = cell
    rho = torch.from_numpy(np.ascontiguousarray(oracle_result["rho_out"]).reshape(-1)).cuda()
    with LSDFT(d, name, faithful=False, precision=64) as eng:
        torch.cuda.synchronize()
        eng.scf_begin(d_rho_init=rho.data_ptr(), tol=1e-6)
        its = 0
        for its in range(1, 7):
            r = eng.scf_step()
            if r["converged"]:
                break
    assert r["converged"] == 1 and its <= 4
    assert r["free_energy_per_atom"] == pytest.approx(oracle_result["free_energy_per_atom"], abs=1e-6)


def test_density_checkpoint_restart_and_output_echo(cell, oracle_result, tmp_path):
    """An SCF restarted from a .den checkpoint (Read_ElecDens, the reference's READ_DEN_FILE
    warm start) converges at once; the .out echo lists the deck's parameters."""
    from sqminiapp_gb300 import LSDFT, Print_ElecDens, Read_ElecDens
    d, name, o, fields = cell
    shape = fields["b"].shape
    with LSDFT(d, name, faithful=False, precision=64) as eng:
        r1 = eng.SCF_LSSGQ(tol=1e-7, maxit=120)
        rho, _ = eng.scf_density()
        Print_ElecDens(str(tmp_path / "ck"), rho.reshape(shape))
        back = Read_ElecDens(str(tmp_path / "ck"), shape)
        r2 = eng.SCF_LSSGQ(rho_init=back, tol=1e-6, maxit=10)
        eng.write_output_echo(str(tmp_path / "run.out"))
    assert r2["iterations"] <= 4
    assert r2["free_energy_per_atom"] == pytest.approx(r1["free_energy_per_atom"], abs=1e-7)
    text = open(tmp_path / "run.out").read()
    nx, ny, nz = o.grid
    assert "FD_GRID: %d %d %d" % (nx, ny, nz) in text and "EXCHANGE_CORRELATION: LDA_PW" in text


def test_cuda_graph_scf_matches_direct_launches(cell):
    """Replaying the captured graph of an iteration's device part gives the run of direct
    launches (same kernels on the same buffers; only atomic orders inside the Lanczos kernel
    differ, 1e-9 relative on the free energy)."""
    from sqminiapp_gb300 import LSDFT
    d, name, o, _ = cell
    with LSDFT(d, name, faithful=False, precision=64) as eng:
        a = eng.SCF_LSSGQ(tol=1e-8, maxit=120)
        b = eng.SCF_LSSGQ(tol=1e-8, maxit=120, cuda_graph=True)
        c = eng.SCF_LSSGQ(tol=1e-8, maxit=120, cuda_graph=True)  # a fresh capture per run
        t = eng.last_kernel_times()
    assert t[0] > 0.0
    assert a["converged"] == b["converged"] == c["converged"] == 1
    assert abs(a["iterations"] - b["iterations"]) <= 1 and abs(b["iterations"] - c["iterations"]) <= 1
    for r in (b, c):
        assert r["free_energy"] == pytest.approx(a["free_energy"], rel=1e-9)
        np.testing.assert_allclose(r["free_energy_history"][:5], a["free_energy_history"][:5],
                                   rtol=1e-9)


def test_bench_cell_scf_matches_oracle_golden(tmp_path):
    """Full-size SCF of the 4-atom bench cell (17^3 nodes, 25^3 cubes, 30 Lanczos steps)
    against the CPU oracle's run committed in tests/golden/scf_mg4.json (made by
    tests/golden/make_scf_golden.py): FP64 to 1e-8 Ha/atom, FP32 within the 1e-5 target."""
    import json
    import os
    from sqminiapp_gb300 import LSDFT
    from sqminiapp_gb300.decks import CONFIGS, make_fcc_mg_deck
    g = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "scf_mg4.json")))
    d, name, _ = make_fcc_mg_deck(str(tmp_path), "cell", seed=g["seed"], **CONFIGS[g["config"]])
    with LSDFT(d, name, faithful=False, precision=64) as eng:
        r64 = eng.SCF_LSSGQ(tol=g["tol"], maxit=60)
    with LSDFT(d, name, faithful=False, precision=32) as eng:
        r32 = eng.SCF_LSSGQ(maxit=60)
    assert r64["iterations"] == g["iterations"]
    assert r64["free_energy_per_atom"] == pytest.approx(g["free_energy_per_atom"], abs=1e-8)
    assert r64["lambda_f"] == pytest.approx(g["lambda_f"], abs=1e-7)
    assert r32["converged"] == 1
    assert r32["free_energy_per_atom"] == pytest.approx(g["free_energy_per_atom"], abs=1e-5)
