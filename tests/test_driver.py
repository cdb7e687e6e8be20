"""sq_lsdft, the command-line counterpart of the reference's main (src/main.cc): argument
handling and error exits on CPU; the SQ pass, its files and the SCF on the GPU against the
Python binding of the same library."""
import os
import shutil
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
DRIVER = os.path.join(ROOT, "sqminiapp_gb300", "lib", "sq_lsdft")


@pytest.fixture(scope="module")
def driver():
    from sqminiapp_gb300 import build
    build.build()
    assert os.path.exists(DRIVER)
    return DRIVER


def test_usage_and_bad_deck(driver, tmp_path):
    r = subprocess.run([driver], capture_output=True, text=True)
    assert r.returncode == 2 and "usage: sq_lsdft -name NAME" in r.stderr
    r = subprocess.run([driver, "-name"], capture_output=True, text=True)
    assert r.returncode == 2
    r = subprocess.run([driver, "-name", "missing", "-dir", str(tmp_path)], capture_output=True,
                       text=True)
    assert r.returncode == 1 and "missing.inpt" in r.stderr


@pytest.mark.gpu
def test_sq_pass_and_files_match_the_binding(driver, deck_dir, tmp_path):
    from sqminiapp_gb300 import LSDFT, Read_MinMaxLambda
    d = tmp_path / "deck"
    shutil.copytree(deck_dir, d)
    pre = str(tmp_path / "mg1")
    r = subprocess.run([driver, "-name", "Mg1", "-dir", str(d), "-precision", "64",
                        "-lambdas", pre], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert "Time spent in SQ=" in r.stdout and "Total time spent=" in r.stdout
    assert os.path.exists(d / "Mg1.out")
    with LSDFT(str(d), "Mg1", faithful=False, precision=64) as eng:
        ref = eng.NodesAndWeights_LSSGQ()
        shape = eng.grid[::-1]
    lo, hi = Read_MinMaxLambda(pre, shape)
    np.testing.assert_allclose(lo, ref["lambda_min"], rtol=1e-10, atol=1e-12)
    np.testing.assert_allclose(hi, ref["lambda_max"], rtol=1e-10, atol=1e-12)


@pytest.mark.gpu
def test_scf_and_density_file(driver, small_cell, tmp_path):
    from sqminiapp_gb300 import LSDFT, Read_ElecDens
    d, name, _ = small_cell
    pre = str(tmp_path / "rho")
    r = subprocess.run([driver, "-name", name, "-dir", d, "-precision", "64", "-scf", "-den", pre,
                        "-out", str(tmp_path / "run.out")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    line = [x for x in r.stdout.splitlines() if x.startswith("SCF converged")][0]
    f_atom = float(line.split("(")[1].split()[0])
    with LSDFT(d, name, faithful=False, precision=64) as eng:
        res = eng.SCF_LSSGQ()
        rho, _ = eng.scf_density()
        shape = eng.grid[::-1]
    assert f_atom == pytest.approx(res["free_energy_per_atom"], abs=1e-9)
    np.testing.assert_allclose(Read_ElecDens(pre, shape).ravel(), rho, atol=1e-9)
