"""The allocation-free Fermi-level entry point against the handle-based one.

sq_fermi_density_energy_noalloc exists for callers that may not allocate device memory (a
host framework that owns the allocator, a fixed memory budget, a stream-ordered pipeline
that cannot take the allocator's synchronisation): it takes only caller buffers and runs on
a static scratch array inside the library.  Here it is called twice in a row through the
C ABI on the same device inputs and must agree with sq_fermi_density_energy_device to the
FP64 tolerance of the other density tests (1e-10 relative).  This file is collected last so
that a failure here does not hide the rest of the suite.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RTOL = 1e-10


def test_noalloc_matches_handle_path(deck_dir):
    import torch
    from sqminiapp_gb300 import LSDFT
    from sqminiapp_gb300.capi import SQ_OK, lib

    dev = torch.device("cuda", 0)
    with LSDFT(deck_dir, "Mg1", faithful=False, precision=64) as eng:
        host = eng.NodesAndWeights_LSSGQ()
        lam = torch.from_numpy(host["lambda"]).to(dev)
        w = torch.from_numpy(host["weights"]).to(dev)
        n, q = lam.shape
        rho_ref = torch.empty(n, dtype=torch.float64, device=dev)
        stream = torch.cuda.current_stream(dev).cuda_stream
        ref = eng.fermi_density_energy_device(lam.data_ptr(), w.data_ptr(), n, eng.n_electrons,
                                              1e-12, rho_ref.data_ptr(), stream)
        beta, dV, ne = eng.beta, eng.dV, eng.n_electrons

    L = lib()
    dp = ctypes.POINTER(ctypes.c_double)
    for call in range(2):
        rho = torch.full((n,), float("nan"), dtype=torch.float64, device=dev)
        out = np.zeros(3)
        st = L.sq_fermi_density_energy_noalloc(
            ctypes.c_void_p(lam.data_ptr()), ctypes.c_void_p(w.data_ptr()), n, q, beta, ne, dV,
            1e-12, 200, ctypes.c_void_p(rho.data_ptr()), out.ctypes.data_as(dp),
            ctypes.c_void_p(stream))
        assert st == SQ_OK, L.sq_last_error_string().decode()
        np.testing.assert_allclose(out[0], ref["lambda_f"], rtol=RTOL, atol=RTOL)
        np.testing.assert_allclose(out[1], ref["e_band"], rtol=RTOL)
        np.testing.assert_allclose(out[2], ref["ts"], rtol=RTOL, atol=1e-14)
        np.testing.assert_allclose(rho.cpu().numpy(), rho_ref.cpu().numpy(), rtol=RTOL, atol=1e-14)


def test_noalloc_rejects_oversize(deck_dir):
    import torch
    from sqminiapp_gb300.capi import SQ_OK, lib

    dev = torch.device("cuda", 0)
    lam = torch.zeros((4, 2), dtype=torch.float64, device=dev)
    w = torch.full((4, 2), 0.5, dtype=torch.float64, device=dev)
    out = np.zeros(3)
    L = lib()
    st = L.sq_fermi_density_energy_noalloc(
        ctypes.c_void_p(lam.data_ptr()), ctypes.c_void_p(w.data_ptr()), 4, 2, 30.0, 4.0, 1.0,
        1e-12, 201, None, out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), None)
    assert st != SQ_OK
    assert "maxit" in L.sq_last_error_string().decode()


def test_noalloc_reports_unconverged_bisection(deck_dir):
    """One bisection step cannot narrow a bracket of several Ha to 1e-12: the call says so
    (SQ_NO_CONVERGENCE) instead of returning the midpoint as converged."""
    import torch
    from sqminiapp_gb300.capi import SQ_NO_CONVERGENCE, SQ_OK, lib

    dev = torch.device("cuda", 0)
    lam = torch.tensor([[-1.0, 0.5], [0.2, 2.0]], dtype=torch.float64, device=dev)
    w = torch.full((2, 2), 0.5, dtype=torch.float64, device=dev)
    out = np.zeros(3)
    L = lib()
    dp = ctypes.POINTER(ctypes.c_double)
    args = (ctypes.c_void_p(lam.data_ptr()), ctypes.c_void_p(w.data_ptr()), 2, 2, 30.0, 2.0,
            1.0, 1e-12)
    st = L.sq_fermi_density_energy_noalloc(*args, 1, None, out.ctypes.data_as(dp), None)
    assert st == SQ_NO_CONVERGENCE, L.sq_last_error_string().decode()
    assert np.isfinite(out[0])
    st = L.sq_fermi_density_energy_noalloc(*args, 200, None, out.ctypes.data_as(dp), None)
    assert st == SQ_OK, L.sq_last_error_string().decode()
