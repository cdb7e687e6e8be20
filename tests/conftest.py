import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def deck_dir():
    from sqminiapp_gb300 import DECK_DIR
    return DECK_DIR


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def small_cell(tmp_path_factory):
    """A 4-atom periodic FCC Mg cell, h = 0.85 bohr, Rcut = 3.4 bohr (9^3 cubes)."""
    from sqminiapp_gb300.decks import make_fcc_mg_deck
    d = str(tmp_path_factory.mktemp("mg4small"))
    return make_fcc_mg_deck(d, "mg4s", ncell=1, h=0.85, rcut=3.4, n_qp=20, disp=0.1, seed=7)
