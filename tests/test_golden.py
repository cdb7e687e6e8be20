"""Golden fixtures (tests/golden/make_golden.py): the oracle reproduces them on this host
(CPU), and the CUDA path matches them (GPU) with the tolerances of test_gpu_parity."""
import os
import sys
import tempfile

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def _case(tag, deck_dir):
    g = np.load(os.path.join(HERE, "golden", tag + ".npz"))
    if tag == "mg4_small":
        sys.path.insert(0, os.path.join(HERE, "golden"))
        import make_golden
        d, name, _ = make_golden.small_deck(tempfile.mkdtemp())
        return g, d, name, False
    return g, deck_dir, "Mg1", tag == "mg1_faithful"


@pytest.mark.parametrize("tag", ["mg1_faithful", "mg1_corrected", "mg4_small"])
def test_oracle_reproduces_golden(tag, deck_dir, oracle_mod):
    g, d, name, faithful = _case(tag, deck_dir)
    r = oracle_mod.Oracle(d, name, faithful=faithful).nodes_and_weights(nodes=g["nodes"],
                                                                        want_ab=True)
    np.testing.assert_allclose(r["a"], g["a"], rtol=1e-12, atol=1e-9)
    np.testing.assert_allclose(r["b"], g["b"], rtol=1e-12, atol=1e-9)
    np.testing.assert_allclose(r["weights"], g["w"], rtol=1e-10, atol=1e-12)


def _functionals(lam, w):
    out = [np.sum(w * lam ** k, axis=1) for k in range(4)]
    out.append(np.sum(w / (1 + np.exp(np.clip(30.0 * (lam - 5.0), -700, 700))), axis=1))
    return out


@pytest.mark.gpu
@pytest.mark.parametrize("tag,precision,tol", [
    ("mg1_corrected", 64, 1e-9), ("mg1_corrected", 32, 1e-4),
    ("mg4_small", 64, 1e-9), ("mg4_small", 32, 1e-4), ("mg1_faithful", 64, 1e-8)])
def test_engine_matches_golden(tag, precision, tol, deck_dir):
    from sqminiapp_gb300 import LSDFT
    g, d, name, faithful = _case(tag, deck_dir)
    with LSDFT(d, name, faithful=faithful, precision=precision) as eng:
        r = eng.NodesAndWeights_LSSGQ()
    lam, w = r["lambda"][g["nodes"]], r["weights"][g["nodes"]]
    for k, (a, b) in enumerate(zip(_functionals(lam, w), _functionals(g["lam"], g["w"]))):
        err = np.max(np.abs(a - b) / np.maximum(1.0, np.abs(b)))
        assert err < tol, (k, err)
