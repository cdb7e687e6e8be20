"""The single-pass Lanczos kernel's on-chip index arithmetic, restated on the CPU for every
cube size the engine accepts, in the layout sq_plan_kernel picks for it with kernel=1 (the same
host code the engine runs; the split-pass kernel has its own restatement in
test_quad_layout.py): every stencil read of P lands either on the right neighbour's slot or, where that
neighbour is outside the cube, on a slot that is never written (a zero pad column, a zero gap
row, or the leading offset) or is masked by a bounds check; every index stays inside the
buffers and fits the 16-bit packing of the projector records.

Formulas (lanczos_kernel.cuh): P index of (x,y,z) = OFF + z*PS + y*pitch + x, with
PS = (ny + 6)*pitch and OFF = 6*pitch when planes are separated by zero gap rows, else
PS = ny*pitch and OFF = 6; U index = (z*ny + y)*upitch + x."""
import numpy as np
import pytest

from sqminiapp_gb300 import plan_kernel
from sqminiapp_gb300.decks import make_fcc_mg_deck

O = 6
YGAP, WIDE, XCLAMP = 1, 2, 4


def layout_of(n, precision, flags):
    pitch = n if flags & XCLAMP else n + O
    upitch = n
    if precision == 32:
        pitch += pitch & 1
        upitch += upitch & 1
    if flags & YGAP:
        ps, off = (n + O) * pitch, O * pitch
    else:
        ps, off = n * pitch, O
    psize = off + n * ps
    return pitch, upitch, ps, off, psize


def check_layout(n, precision, flags):
    pitch, upitch, ps, off, psize = layout_of(n, precision, flags)
    z, y, x = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    idx = off + z * ps + y * pitch + x
    owner = -np.ones(psize + 64, dtype=np.int64)  # slot -> flat cube point, -1 = never written
    owner[idx.ravel()] = np.arange(n ** 3)
    assert idx.max() < psize and idx.min() >= 0
    # 16-bit packing of P and U indices in the projector records
    assert psize < 65536 and upitch * n * n < 65536
    flat = (z * n + y) * n + x
    for d in range(1, O + 1):
        for axis, stride, coord in (("x", 1, x), ("y", pitch, y)):
            for sgn in (-1, 1):
                nb = coord + sgn * d
                inside = (nb >= 0) & (nb < n)
                clamped = (axis == "x" and flags & XCLAMP) or (axis == "y" and not flags & YGAP)
                read = np.where(inside | (not clamped), idx + sgn * d * stride, idx)
                assert read.min() >= 0 and read.max() < psize, (axis, sgn, d)
                got = owner[read]
                want = np.where(inside, flat + sgn * d * (1 if axis == "x" else n), -1)
                if clamped:  # the kernel drops the value of a masked read
                    assert np.all(got[inside] == want[inside]), (axis, sgn, d)
                else:  # an unmasked read outside the cube must hit a zero slot
                    assert np.all(got == want), (axis, sgn, d)
    if precision == 32:  # paired passes: 8-byte alignment of every pair and of the x loads
        assert off % 2 == 0 and pitch % 2 == 0 and ps % 2 == 0 and upitch % 2 == 0
        px = np.arange(0, n, 2)
        i2 = (off + px) // 2
        assert np.all((off + px) % 2 == 0)
        # x loads: pairs i2-3 .. i2+3 of the first and the last row of the cube
        for zz, yy in ((0, 0), (n - 1, n - 1)):
            base = (off + zz * ps + yy * pitch + px) // 2
            assert (2 * (base - 3)).min() >= 0 and (2 * (base + 3) + 1).max() < psize
        # the second point of the last pair of an odd-width row is a pad slot (never written)
        if n % 2:
            assert owner[off + (n - 1) + 1] == -1
        # U pairs: the pair (px, px+1) of row y, plane z stays inside its own row of upitch
        nc = upitch * n * n
        for zz, yy in ((0, 0), (n - 1, n - 1)):
            first = (zz * n + yy) * upitch + px
            assert np.all(first + 1 < (zz * n + yy + 1) * upitch) and (first + 1).max() < nc
    return psize


# (rcut, h, precision) -> cube 2*ceil(rcut/h)+1 from 9 to 33 on a 4-atom cell, and whether
# the planner must accept it.  FP64 cubes of 31^3 and up fit no single-CTA layout.
_CASES = [(4.0, 0.5, 32, True), (4.0, 0.5, 64, True), (6.0, 0.5, 32, True), (6.0, 0.5, 64, True),
          (6.5, 0.5, 32, True), (6.5, 0.5, 64, True), (7.0, 0.5, 32, True), (7.0, 0.5, 64, True),
          (7.5, 0.5, 32, True), (7.5, 0.5, 64, False), (7.0, 8.5 / 19, 32, True),
          (7.0, 8.5 / 19, 64, False), (3.4, 0.85, 32, True), (3.4, 0.85, 64, True),
          (5.0, 0.5, 32, True), (5.0, 0.5, 64, True)]


@pytest.mark.parametrize("rcut,h,precision,fits", _CASES)
def test_kernel_index_arithmetic_stays_in_bounds(rcut, h, precision, fits, tmp_path):
    d, name, _ = make_fcc_mg_deck(str(tmp_path), "c", ncell=1, h=h, rcut=rcut, n_qp=20)
    if not fits:
        with pytest.raises(Exception) as e:
            plan_kernel(d, name, precision=precision, kernel=1)
        assert "does not fit" in str(e.value) or "FP32" in str(e.value)
        return
    p = plan_kernel(d, name, precision=precision, kernel=1)
    n = p.cube[0]
    assert n == 2 * int(np.ceil(rcut / h - 1e-12)) + 1
    flags = p.kernel_layout & 7
    if n > 32:
        assert precision == 32 and flags & WIDE
    psize = check_layout(n, precision, flags)
    # the kernel rounds P up to whole 16-byte vectors before U and the lists
    psize_kernel = (psize + 3) & ~3
    elem = 4 if precision == 32 else 8
    assert elem * psize_kernel < p.kernel_smem_bytes
