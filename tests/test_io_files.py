"""The reference's text files written and read by the library (host code, CPU).

Formats: Print_ElecDens / Read_ElecDens (src/lsdft_readfiles.cc:1106-1138, 1242-1289) and
Print_MinMaxLambda / Read_MinMaxLambda (:1294-1381).  The expected text is produced here
with Python's printf-style formatting, which rounds exactly like C's fprintf.
"""
import numpy as np
import pytest


def _expected_den(rho, corner):
    nz, ny, nx = rho.shape
    lines = ["%d %d %d %d %d %d" % (corner[0], corner[1], corner[2], nx, ny, nz)]
    for k in range(nz):
        for j in range(ny):
            for i in range(nx):
                lines.append("%d %d %d %0.16f" % (k + corner[2], j + corner[1], i + corner[0],
                                                  rho[k, j, i]))
    return "\n".join(lines) + "\n"


def test_density_file_format_and_round_trip(tmp_path):
    from sqminiapp_gb300 import Print_ElecDens, Read_ElecDens
    rng = np.random.default_rng(3)
    rho = rng.uniform(0, 0.05, (3, 4, 5))
    rho[0, 0, 0] = 0.0
    corner = (2, 0, 7)
    prefix = str(tmp_path / "gen1")
    Print_ElecDens(prefix, rho, rank=3, corner=corner)
    text = open(prefix + "_3.den").read()
    assert text == _expected_den(rho, corner)
    back = Read_ElecDens(prefix, rho.shape, rank=3, corner=corner)
    # %0.16lf keeps 16 decimals: the read value is the parsed text, exactly
    np.testing.assert_array_equal(back, np.array([float("%0.16f" % v) for v in rho.ravel()]).reshape(rho.shape))
    np.testing.assert_allclose(back, rho, atol=1e-16)


def test_density_file_rejects_other_decomposition(tmp_path):
    from sqminiapp_gb300 import Print_ElecDens, Read_ElecDens, SqError
    rho = np.ones((2, 2, 2))
    prefix = str(tmp_path / "d")
    Print_ElecDens(prefix, rho)
    with pytest.raises(SqError) as e:
        Read_ElecDens(prefix, (2, 2, 2), corner=(1, 0, 0))
    assert e.value.status == 1 and "decomposition" in str(e.value)
    with pytest.raises(SqError):
        Read_ElecDens(str(tmp_path / "missing"), (2, 2, 2))


def test_density_file_read_order_follows_indices(tmp_path):
    """Read_ElecDens stores each line at its own (k, j, i), whatever the line order."""
    from sqminiapp_gb300 import Read_ElecDens
    p = tmp_path / "x_0.den"
    p.write_text("0 0 0 2 1 1\n0 0 1 0.25\n0 0 0 0.75\n")
    np.testing.assert_array_equal(Read_ElecDens(str(tmp_path / "x"), (1, 1, 2)), [[[0.75, 0.25]]])


def test_lambda_file_format_and_round_trip(tmp_path):
    from sqminiapp_gb300 import Print_MinMaxLambda, Read_MinMaxLambda
    rng = np.random.default_rng(4)
    shape = (2, 3, 4)
    lo = rng.uniform(-1, 0, 24)
    hi = rng.uniform(1, 40, 24)
    prefix = str(tmp_path / "gen1")
    Print_MinMaxLambda(prefix, lo, hi, shape)
    lines = open(prefix + "_0.lambdas").read().splitlines()
    assert lines[0] == "0 0 0 4 3 2"
    assert lines[1:] == ["%d %0.16f %0.16f" % (p, lo[p], hi[p]) for p in range(24)]
    a, b = Read_MinMaxLambda(prefix, shape)
    np.testing.assert_allclose(a, lo, atol=1e-16)
    np.testing.assert_allclose(b, hi, atol=1e-15)
