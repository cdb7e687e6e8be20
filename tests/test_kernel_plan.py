"""The engine's choice of Lanczos-kernel layout per cell, planned on the host (sq_plan_kernel,
the same code sq_create_from_deck runs before it allocates): on-chip layout flags, U on chip
or in global scratch, projector-list format, threads and shared memory on a GB300."""
import pytest

from sqminiapp_gb300 import GB300_DEVICE, SqError, plan_kernel
from sqminiapp_gb300.decks import CONFIGS, make_fcc_mg_deck

YGAP, WIDE, XCLAMP, COMPACT, QUAD, PAIR = 1, 2, 4, 8, 16, 32


@pytest.fixture(scope="module")
def decks(tmp_path_factory):
    out = {}
    for name in ("mg32_h0.5_rc6.5_q40", "mg500_h0.5_rc7_q50", "uneven_b_mg32_h0.45_rc7_q40",
                 "uneven_a_mg4_h0.5_rc6_q30"):
        d = str(tmp_path_factory.mktemp(name))
        out[name] = make_fcc_mg_deck(d, "c", **CONFIGS[name])[:2]
    return out


def _plan(decks, name, **kw):
    return plan_kernel(*decks[name], **kw)


def test_fp32_layouts(decks):
    smem_max = GB300_DEVICE["smem_optin"]
    # the split-pass kernel wherever it applies: rows of 4*ceil(n/4) floats, P and U on chip,
    # ceil(n/4) threads per row times two z-ranges (the default tile before autotuning)
    p = _plan(decks, "mg32_h0.5_rc6.5_q40")  # 27^3: 7 quads x 27 rows x 2 = 378 -> 384
    assert (p.kernel_layout, p.kernel_u_on_chip, p.kernel_threads) == (QUAD, 1, 384)
    # above 256 threads the launch takes every warp of the register budget (the passes use
    # the threads they need, the list streams and the update all)
    p = _plan(decks, "uneven_a_mg4_h0.5_rc6_q30")  # 25^3: 7 x 25 x 2 = 350 -> 12 warps
    assert (p.kernel_layout, p.kernel_u_on_chip, p.kernel_threads) == (QUAD, 1, 384)
    p = _plan(decks, "mg500_h0.5_rc7_q50")  # 29^3: 8 quads x 29 x 2 = 464 -> 16 warps
    assert (p.kernel_layout, p.kernel_u_on_chip, p.kernel_threads) == (QUAD, 1, 512)
    # 33^3: a pair of CTAs per node, each with half the planes (9 quads x 33 rows, one z-range;
    # 17 planes x 9 quads x 2 y-ranges = 306 threads in the passes), U on chip, 12 warps
    p = _plan(decks, "uneven_b_mg32_h0.45_rc7_q40")
    assert (p.kernel_layout, p.kernel_u_on_chip, p.kernel_threads) == (QUAD | PAIR, 1, 384)
    for name in decks:
        assert 0 < _plan(decks, name).kernel_smem_bytes <= smem_max


def test_single_pass_kernel_layouts(decks):
    p = _plan(decks, "mg32_h0.5_rc6.5_q40", kernel=1)  # 27^3: y gaps, U on chip, 14 warps
    assert (p.kernel_layout, p.kernel_u_on_chip, p.kernel_threads) == (YGAP, 1, 448)
    p = _plan(decks, "uneven_a_mg4_h0.5_rc6_q30", kernel=1)  # 25^3
    assert (p.kernel_layout, p.kernel_u_on_chip) == (YGAP, 1)
    p = _plan(decks, "mg500_h0.5_rc7_q50", kernel=1)  # 29^3: U on chip only without the y gaps
    assert (p.kernel_layout, p.kernel_u_on_chip) == (0, 1)
    p = _plan(decks, "uneven_b_mg32_h0.45_rc7_q40", kernel=1)  # 33^3: wide, U in L2, compact
    assert (p.kernel_layout, p.kernel_u_on_chip, p.kernel_threads) == (YGAP | WIDE | COMPACT, 0, 576)


def test_kernel_option(decks):
    # the split-pass kernel on request, with a chosen tile; refused where it does not apply
    p = _plan(decks, "mg32_h0.5_rc6.5_q40", kernel=2, tile=1)
    assert (p.kernel_layout, p.kernel_threads) == (QUAD, 192)
    for kw in ({"faithful": True}, {"precision": 64}, {"list_format": 2}):
        with pytest.raises(SqError):
            _plan(decks, "mg32_h0.5_rc6.5_q40", kernel=2, **kw)
    assert _plan(decks, "uneven_b_mg32_h0.45_rc7_q40", kernel=2).kernel_layout == QUAD | PAIR
    with pytest.raises(SqError):  # the pair runs one tile only
        _plan(decks, "uneven_b_mg32_h0.45_rc7_q40", kernel=2, tile=1)
    with pytest.raises(SqError):
        _plan(decks, "mg32_h0.5_rc6.5_q40", kernel=3)
    # a tile whose threads exceed the kernel's 512 falls back to the single-pass kernel
    assert _plan(decks, "mg32_h0.5_rc6.5_q40", tile=3).kernel_layout == YGAP


def test_list_format_option(decks):
    assert _plan(decks, "uneven_b_mg32_h0.45_rc7_q40", list_format=1).kernel_layout == QUAD | PAIR
    assert _plan(decks, "uneven_b_mg32_h0.45_rc7_q40", list_format=1,
                 kernel=1).kernel_layout == YGAP | WIDE
    assert _plan(decks, "mg32_h0.5_rc6.5_q40", list_format=2).kernel_layout == YGAP | COMPACT
    assert _plan(decks, "mg32_h0.5_rc6.5_q40", list_format=1).kernel_layout == QUAD
    # the faithful operator and FP64 keep the full records
    assert _plan(decks, "mg32_h0.5_rc6.5_q40", list_format=2, faithful=True).kernel_layout == YGAP
    assert _plan(decks, "mg32_h0.5_rc6.5_q40", list_format=2, precision=64).kernel_layout == 0
    # a small L2 turns the automatic choice to the single-pass kernel with compact records
    small = _plan(decks, "mg32_h0.5_rc6.5_q40", device={"l2_bytes": 16 << 20})
    assert small.kernel_layout == YGAP | COMPACT
    with pytest.raises(SqError):
        _plan(decks, "mg32_h0.5_rc6.5_q40", list_format=3)


def test_fp64_layouts(decks):
    p = _plan(decks, "mg32_h0.5_rc6.5_q40", precision=64)
    assert (p.kernel_layout, p.kernel_u_on_chip, p.kernel_threads) == (0, 0, 448)
    p = _plan(decks, "mg500_h0.5_rc7_q50", precision=64)  # 29^3: rows without zero columns
    assert p.kernel_layout == XCLAMP
    with pytest.raises(SqError) as e:  # 33^3 in FP64 fits no single-CTA layout
        _plan(decks, "uneven_b_mg32_h0.45_rc7_q40", precision=64)
    assert "FP32" in str(e.value)


def test_smaller_shared_memory_moves_u_off_chip(decks):
    # the split-pass kernel moves to a CTA pair per node; the single-pass one keeps P on chip
    # and moves U to global scratch
    p = _plan(decks, "mg32_h0.5_rc6.5_q40", device={"smem_optin": 160 * 1024})
    assert (p.kernel_layout, p.kernel_u_on_chip) == (QUAD | PAIR, 1)
    p = _plan(decks, "mg32_h0.5_rc6.5_q40", device={"smem_optin": 160 * 1024}, kernel=1)
    assert (p.kernel_layout, p.kernel_u_on_chip) == (YGAP, 0)
    p = _plan(decks, "mg32_h0.5_rc6.5_q40", device={"smem_optin": 170 * 1024})
    assert (p.kernel_layout, p.kernel_u_on_chip) == (QUAD, 1)
    with pytest.raises(SqError):
        _plan(decks, "mg32_h0.5_rc6.5_q40", device={"smem_optin": 64 * 1024})
