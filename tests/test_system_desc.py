"""sq_create's in-memory cell (sq_system_desc) against the deck files it stands for, on the CPU:
sq_describe_system and sq_describe_deck run the same host setup (images, projector tables,
Gamma_l, pseudocharge cutoffs) and must report identical results for the reference's Mg1 deck
(BOUNDARY_CONDITION 1, s+d projectors) and a periodic FCC cell (s+p); invalid descriptions are
refused with SQ_BAD_INPUT, as the deck readers refuse the same values."""
import ctypes

import numpy as np
import pytest

from sqminiapp_gb300.capi import SQ_BAD_INPUT, SQ_OK, SqInfo, lib
from sqminiapp_gb300.system import read_system, to_desc

INFO_FIELDS = [f for f, _ in SqInfo._fields_]


def _describe_deck(d, name, faithful):
    info, gam, cut = SqInfo(), np.zeros(32), np.zeros(24)
    dp = ctypes.POINTER(ctypes.c_double)
    st = lib().sq_describe_deck(d.encode(), name.encode(), faithful, ctypes.byref(info),
                                gam.ctypes.data_as(dp), cut.ctypes.data_as(dp))
    assert st == SQ_OK, lib().sq_last_error_string().decode()
    return info, gam, cut


def _describe_system(sysd, faithful):
    info, gam, cut = SqInfo(), np.zeros(32), np.zeros(24)
    dp = ctypes.POINTER(ctypes.c_double)
    packed = to_desc(sysd)
    st = lib().sq_describe_system(ctypes.byref(packed.desc), faithful, ctypes.byref(info),
                                  gam.ctypes.data_as(dp), cut.ctypes.data_as(dp))
    return st, info, gam, cut


def _same(a, b):
    for f in INFO_FIELDS:
        va, vb = getattr(a, f), getattr(b, f)
        if hasattr(va, "__len__"):
            va, vb = list(va), list(vb)
        assert va == vb, f


@pytest.fixture(scope="module")
def fcc_cell(tmp_path_factory):
    from sqminiapp_gb300.decks import make_fcc_mg_deck
    d = str(tmp_path_factory.mktemp("fccsys"))
    return make_fcc_mg_deck(d, "fcc", ncell=1, h=0.5, rcut=4.0, n_qp=20, disp=0.1, seed=3)


@pytest.mark.parametrize("faithful", [0, 1])
def test_mg1_deck_and_memory_give_the_same_setup(deck_dir, faithful):
    sysd = read_system(deck_dir, "Mg1")
    assert sysd["bc"] == 1 and sysd["n_qp"] == 10 and len(sysd["atom_type"]) == 4
    st, info, gam, cut = _describe_system(sysd, faithful)
    assert st == SQ_OK, lib().sq_last_error_string().decode()
    ref = _describe_deck(deck_dir, "Mg1", faithful)
    _same(info, ref[0])
    np.testing.assert_array_equal(gam, ref[1])
    np.testing.assert_array_equal(cut, ref[2])


def test_periodic_cell_deck_and_memory_give_the_same_setup(fcc_cell):
    d, name, _ = fcc_cell
    sysd = read_system(d, name)
    st, info, gam, cut = _describe_system(sysd, 0)
    assert st == SQ_OK, lib().sq_last_error_string().decode()
    ref = _describe_deck(d, name, 0)
    _same(info, ref[0])
    np.testing.assert_array_equal(gam, ref[1])
    assert info.n_lm == 4  # s + p with PSEUDOPOTENTIAL_LOCAL 2


@pytest.mark.parametrize("edit,msg", [
    (lambda s: s.update(rcut=0.0), "RADIUS_TRUNC"),
    (lambda s: s.update(n_qp=65), "LANCZOS_DEGREE"),
    (lambda s: s.update(fd_order=8), "FD_ORDER"),
    (lambda s: s["types"][0].update(lloc=3), "PSEUDOPOTENTIAL_LOCAL"),
    (lambda s: s["types"][0]["U"].__setitem__(0, None), "wave function"),
    (lambda s: s.update(atom_type=np.array([0, 0, 0, 5], dtype=np.int32)), "atom type"),
    (lambda s: s["types"][0].update(r=s["types"][0]["r"][::-1].copy()), "radial grid"),
])
def test_invalid_descriptions_are_refused(fcc_cell, edit, msg):
    d, name, _ = fcc_cell
    sysd = read_system(d, name)
    edit(sysd)
    st, *_ = _describe_system(sysd, 0)
    assert st == SQ_BAD_INPUT
    assert msg in lib().sq_last_error_string().decode()


@pytest.mark.gpu
@pytest.mark.parametrize("precision,tol", [(64, 1e-12), (32, 1e-6)])
def test_engine_from_memory_matches_engine_from_deck(fcc_cell, precision, tol):
    """sq_create on the in-memory cell and sq_create_from_deck on its files build the same
    engine: the same quadrature on every node (up to the scatter's atomic summation order)."""
    from sqminiapp_gb300 import LSDFT
    d, name, meta = fcc_cell
    rng = np.random.default_rng(2)
    veff = -0.2 + 0.05 * rng.standard_normal(meta["N"] ** 3)
    with LSDFT(None, None, precision=precision, system=read_system(d, name)) as eng:
        a = eng.NodesAndWeights_LSSGQ(veff=veff)
        info = eng.info
    with LSDFT(d, name, precision=precision) as eng:
        b = eng.NodesAndWeights_LSSGQ(veff=veff)
        assert (info.kernel_layout, info.n_images) == (eng.info.kernel_layout, eng.info.n_images)
    for k in range(4):
        np.testing.assert_allclose(np.sum(a["weights"] * a["lambda"] ** k, axis=1),
                                   np.sum(b["weights"] * b["lambda"] ** k, axis=1), rtol=tol, atol=tol)
