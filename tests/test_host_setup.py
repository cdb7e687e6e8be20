"""Host side of the product on the CPU: the library loads and exports the ABI, the deck
readers and the setup agree with the oracle, errors come back as status codes."""
import ctypes
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _describe(deck_dir, name, faithful):
    from sqminiapp_gb300.capi import SqInfo, lib
    info = SqInfo()
    g = np.zeros(32)
    c = np.zeros(24)
    dp = ctypes.POINTER(ctypes.c_double)
    st = lib().sq_describe_deck(deck_dir.encode(), name.encode(), int(faithful),
                                ctypes.byref(info), g.ctypes.data_as(dp), c.ctypes.data_as(dp))
    return st, info, g, c


def test_library_exports_every_declared_symbol():
    from sqminiapp_gb300.capi import SIGNATURES, lib
    header = open(os.path.join(ROOT, "include", "sq_gb300.h")).read()
    declared = set(re.findall(r"\b(sq_\w+)\s*\(", header))
    assert declared, "no declarations found"
    L = lib()
    for name in sorted(declared):
        assert hasattr(L, name), name
    assert declared == set(SIGNATURES), declared ^ set(SIGNATURES)


@pytest.mark.parametrize("faithful", [True, False])
def test_setup_matches_oracle(deck_dir, oracle_mod, faithful):
    st, info, g, c = _describe(deck_dir, "Mg1", faithful)
    assert st == 0
    o = oracle_mod.Oracle(deck_dir, "Mg1", faithful=faithful)
    assert tuple(info.grid) == o.grid and tuple(info.cube) == o.nloc
    assert info.n_nodes == o.n_nodes and info.n_qp == o.n_qp
    assert info.n_images == o.n_images
    np.testing.assert_array_equal(g[:4], o.gamma())          # Gamma_l: same sum, same order
    np.testing.assert_array_equal(c[:3], o.pseudocharge_cutoff()[0])
    assert info.dV == pytest.approx(o.dV, rel=1e-15)
    assert info.n_electrons == o.n_electrons
    assert info.n_lm == 6


def test_synthetic_cells(tmp_path):
    from sqminiapp_gb300.decks import CONFIGS, make_fcc_mg_deck
    d1, n1, m1 = make_fcc_mg_deck(str(tmp_path / "a"), "c", **CONFIGS["mg32_h0.5_rc6.5_q40"])
    d2, n2, m2 = make_fcc_mg_deck(str(tmp_path / "b"), "c", **CONFIGS["mg32_h0.5_rc6.5_q40"])
    assert open(os.path.join(d1, "c.ion")).read() == open(os.path.join(d2, "c.ion")).read()
    st, info, _, _ = _describe(d1, "c", False)
    assert st == 0
    assert tuple(info.grid) == (34, 34, 34) and tuple(info.cube) == (27, 27, 27)
    assert info.n_atoms == 32 and info.n_tables == 32  # periodic images share tables
    assert info.beta == pytest.approx(315.7746, rel=1e-5)  # 1000 K
    d3, _, _ = make_fcc_mg_deck(str(tmp_path / "c"), "c", seed=99, **{
        k: v for k, v in CONFIGS["mg32_h0.5_rc6.5_q40"].items()})
    assert open(os.path.join(d3, "c.ion")).read() != open(os.path.join(d1, "c.ion")).read()


def test_bad_decks_return_status(tmp_path, deck_dir):
    from sqminiapp_gb300.capi import lib
    st, _, _, _ = _describe(str(tmp_path), "missing", False)
    assert st == 1  # SQ_BAD_INPUT
    assert "cannot open" in lib().sq_last_error_string().decode()
    bad = tmp_path / "bad"
    bad.mkdir()
    src = open(os.path.join(deck_dir, "Mg1.inpt")).read()
    (bad / "x.inpt").write_text(src.replace("BOUNDARY_CONDITION: 1", "BOUNDARY_CONDITION: 7"))
    (bad / "x.ion").write_text(open(os.path.join(deck_dir, "Mg1.ion")).read())
    st, _, _, _ = _describe(str(bad), "x", False)
    assert st == 1
    assert "BOUNDARY_CONDITION" in lib().sq_last_error_string().decode()


def test_python_wrapper_fails_loudly_without_library(monkeypatch):
    import sqminiapp_gb300.capi as capi
    monkeypatch.setattr(capi, "_lib", None)
    monkeypatch.setattr(capi, "_LIB", "/nonexistent/libsq_gb300.so")
    with pytest.raises(ImportError):
        capi.lib()


def test_mlp_parameter_count_matches_layout():
    """SQ_MLP_N_PARAMS (the host buffers' size) is the 64-128-128-1 layout's count."""
    import re
    from sqminiapp_gb300 import WarmStartMLP
    n = sum(int(np.prod(s)) for _, s in WarmStartMLP.SHAPES)
    assert n == WarmStartMLP.N_PARAMS == 64 * 128 + 128 + 128 * 128 + 128 + 128 + 1
    hdr = open(os.path.join(ROOT, "include", "sq_gb300.h")).read()
    assert int(re.search(r"#define SQ_MLP_N_PARAMS (\d+)", hdr).group(1)) == n
