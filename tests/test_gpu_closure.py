"""GPU closure: Fermi level, densities, energies and the electron count against the oracle on
identical quadrature inputs (FP64 throughout, tolerance 1e-10 relative)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def mg1_quadrature(deck_dir):
    from sqminiapp_gb300 import LSDFT
    eng = LSDFT(deck_dir, "Mg1", faithful=False, precision=64)
    q = eng.NodesAndWeights_LSSGQ()
    yield eng, q
    eng.close()


def test_fermi_density_energy_vs_oracle(mg1_quadrature, oracle_mod):
    eng, q = mg1_quadrature
    got = eng.CalculateDensity_lssgq(q["lambda"], q["weights"])
    ref = oracle_mod.fermi_density_energy(q["lambda"], q["weights"], eng.beta, eng.n_electrons,
                                          eng.dV)
    assert got["lambda_f"] == pytest.approx(ref["lambda_f"], abs=1e-10)
    assert got["e_band"] == pytest.approx(ref["e_band"], rel=1e-10)
    assert got["ts"] == pytest.approx(ref["ts"], rel=1e-8, abs=1e-12)
    np.testing.assert_allclose(got["rho"], ref["rho"], rtol=1e-10, atol=1e-14)
    # sum of the densities is the electron count
    assert np.sum(got["rho"]) * eng.dV == pytest.approx(eng.n_electrons, rel=1e-9)


def test_electron_count_and_sharded_bisection(mg1_quadrature):
    import torch
    from sqminiapp_gb300 import sharding
    eng, q = mg1_quadrature
    dev = torch.device("cuda", 0)
    stream = torch.cuda.current_stream(dev).cuda_stream
    full = eng.CalculateDensity_lssgq(q["lambda"], q["weights"])
    lam = torch.from_numpy(q["lambda"]).to(dev)
    w = torch.from_numpy(q["weights"]).to(dev)
    n = lam.shape[0]
    c = eng.electron_count_device(lam.data_ptr(), w.data_ptr(), n, full["lambda_f"], stream)
    assert c == pytest.approx(eng.n_electrons, rel=1e-9)
    # two node ranges, counts summed on the host: the bisection of a two-GPU run
    shards = [sharding.node_range(n, r, 2) for r in range(2)]
    parts = [(lam[b:e].contiguous(), w[b:e].contiguous()) for b, e in shards]

    def local_count(lf):
        return sum(eng.electron_count_device(l.data_ptr(), ww.data_ptr(), l.shape[0], lf, stream)
                   for l, ww in parts)

    lf, _ = sharding.fermi_level(local_count, float(lam.min()), float(lam.max()),
                                 eng.n_electrons, lambda x: x, lambda x: x, lambda x: x)
    assert lf == pytest.approx(full["lambda_f"], abs=1e-10)
