"""The CTA-pair form of the FP32 split-pass kernel (kernel_layout flags 16 | 32), restated on
the CPU: cubes whose P and U do not fit one CTA run on a cluster of two CTAs per node, the cube
split in z (lanczos_quad.cuh, PairPlanes).

For every cube height the pair form accepts:
  * the two CTAs' owned planes partition [0, nz); each CTA holds P on its owned planes plus
    O = 6 halo planes on the peer's side, so every z-neighbour a pass-A ring loads (|dz| <= 6,
    inside the cube) is held;
  * the update phase's halo writes (owned quads [h0, h1), written at e + dpeer into the peer's
    P) land exactly on the peer's halo planes, each halo quad written once, never on a plane
    the peer owns;
  * pass A (rows over the owned planes, zchunks z-ranges) and pass B (owned planes, ychunks
    y-ranges) each cover every owned quad exactly once within the launch's 384 threads (the
    threads the passes do not need stay idle there);
  * the list of each image splits by owned planes: the two CTAs' z-extents of an image's box
    add up to the single-CTA extent, and U indices (P index - udelta) stay inside U.
The engine's planner picks the pair form for the 33^3 cubes of the uneven-batch cell.
"""
import numpy as np
import pytest

O = 6


def plane_floats(n, pitch):
    return n * pitch + ((pitch - n * pitch) % 32 + 32) % 32


def pair_planes(nz, zsplit, rank):
    """(zo0, zo1, pz0, pz1): owned planes and held planes of P of CTA `rank`."""
    if rank == 0:
        return 0, zsplit, 0, min(nz, zsplit + O)
    return zsplit, nz, max(0, zsplit - O), nz


def pair_threads(n, zsplit, zch, ych):
    nq = (n + 3) // 4
    groups = max(n * zch, max(zsplit, n - zsplit) * ych)
    return max(64, 32 * ((nq * groups + 31) // 32))


HEIGHTS = list(range(14, 41))


@pytest.mark.parametrize("nz", HEIGHTS)
def test_planes_partition_and_halos_hold_the_stencil(nz):
    zs = (nz + 1) // 2
    owned = np.zeros(nz, dtype=int)
    for r in (0, 1):
        zo0, zo1, pz0, pz1 = pair_planes(nz, zs, r)
        owned[zo0:zo1] += 1
        assert pz0 <= zo0 < zo1 <= pz1 and 0 <= pz0 and pz1 <= nz
        for z in range(zo0, zo1):
            for d in range(-O, O + 1):
                if 0 <= z + d < nz:
                    assert pz0 <= z + d < pz1, (nz, r, z, d)
    assert np.all(owned == 1)


@pytest.mark.parametrize("nz", HEIGHTS)
def test_halo_writes_fill_the_peer_halo_once(nz):
    zs = (nz + 1) // 2
    ny, pitch = nz, 4 * ((nz + 3) // 4)
    ps4 = plane_floats(ny, pitch) // 4
    for r in (0, 1):
        zo0, zo1, pz0, pz1 = pair_planes(nz, zs, r)
        qzo0, qzo1, qpz0, qpz1 = pair_planes(nz, zs, r ^ 1)
        h0 = (max(zo0, qpz0) - zo0) * ps4
        h1 = (min(zo1, qpz1) - zo0) * ps4
        dpeer = (zo0 - qpz0) * ps4
        written = np.zeros((qpz1 - qpz0) * ps4, dtype=int)
        for e in range(h0, h1):
            idx = e + dpeer
            assert 0 <= idx < written.size
            written[idx] += 1
            z_peer = qpz0 + idx // ps4
            assert not (qzo0 <= z_peer < qzo1)  # never a plane the peer owns
            assert z_peer == zo0 + e // ps4     # the same global plane
        halo = [z for z in range(qpz0, qpz1) if not (qzo0 <= z < qzo1)]
        for z in range(qpz0, qpz1):
            block = written[(z - qpz0) * ps4:(z - qpz0 + 1) * ps4]
            assert np.all(block == (1 if z in halo else 0)), (nz, r, z)


@pytest.mark.parametrize("n", [33, 35, 37, 38])
@pytest.mark.parametrize("rank", [0, 1])
def test_pair_passes_cover_owned_quads_once(n, rank):
    zs = (n + 1) // 2
    nq = (n + 3) // 4
    zch, ych = 1, 2
    nt = pair_threads(n, zs, zch, ych)
    if nt > 384:
        ych = 1
        nt = pair_threads(n, zs, zch, ych)
    assert nt <= 384
    nt = 384  # the engine launches 12 warps; the threads past nt must stay idle in both passes
    zo0, zo1, _, _ = pair_planes(n, zs, rank)
    nzo = zo1 - zo0
    t = np.arange(nt)
    grp, ql = t // nq, t % nq
    # pass A
    yA, zc = grp % n, grp // n
    zlen = (nzo + zch - 1) // zch
    zb = zo0 + np.minimum(nzo, zc * zlen)
    ze = np.minimum(zo1, zb + zlen)
    act = (zc < zch) & (zb < ze)
    seen = np.zeros((nzo, n, nq), dtype=int)
    for i in np.nonzero(act)[0]:
        seen[zb[i] - zo0:ze[i] - zo0, yA[i], ql[i]] += 1
    assert np.all(seen == 1)
    # pass B
    zB, yc = zo0 + grp % nzo, grp // nzo
    ylen = (n + ych - 1) // ych
    yb = np.minimum(n, yc * ylen)
    ye = np.minimum(n, yb + ylen)
    act = (yc < ych) & (yb < ye)
    seen[:] = 0
    for i in np.nonzero(act)[0]:
        seen[zB[i] - zo0, yb[i]:ye[i], ql[i]] += 1
    assert np.all(seen == 1)


@pytest.mark.parametrize("seed", range(20))
def test_image_boxes_split_by_owned_planes(seed):
    rng = np.random.default_rng(seed)
    n = int(rng.integers(14, 41))
    zs = (n + 1) // 2
    pitch = 4 * ((n + 3) // 4)
    ps = plane_floats(n, pitch)
    Zs = int(rng.integers(-50, 50))
    fz = int(rng.integers(1, 30))
    bz = Zs + int(rng.integers(-fz + 1, n))  # the box meets the cube in z
    full = min(bz + fz, Zs + n) - max(bz, Zs)
    parts = []
    for r in (0, 1):
        zo0, zo1, pz0, _ = pair_planes(n, zs, r)
        za = max(bz, Zs + zo0)
        ez = max(0, min(bz + fz, Zs + zo1) - za)
        parts.append(ez)
        if ez:
            cz0 = za - Zs
            assert zo0 <= cz0 and cz0 + ez <= zo1
            # P index of the box's first and last plane, and the U index = P index - udelta
            udelta = (zo0 - pz0) * ps
            for cz in (cz0, cz0 + ez - 1):
                pidx = (cz - pz0) * ps
                assert 0 <= pidx - udelta < (zo1 - zo0) * ps
    assert sum(parts) == full > 0


def test_engine_plans_a_pair_for_33_cubes(tmp_path):
    from sqminiapp_gb300 import plan_kernel
    from sqminiapp_gb300.decks import CONFIGS, make_fcc_mg_deck
    d, name, _ = make_fcc_mg_deck(str(tmp_path), "c", **CONFIGS["uneven_b_mg32_h0.45_rc7_q40"])
    p = plan_kernel(d, name)
    assert tuple(p.cube) == (33, 33, 33)
    assert p.kernel_layout == 16 | 32 and p.kernel_u_on_chip == 1
    assert pair_threads(33, 17, 1, 2) == 320 <= p.kernel_threads == 384
    ps = plane_floats(33, 36)
    zo0, zo1, pz0, pz1 = pair_planes(33, 17, 0)
    assert p.kernel_smem_bytes > 4 * ps * ((pz1 - pz0) + (zo1 - zo0))
    assert p.kernel_smem_bytes <= 232448
    # FP64 and the faithful operator keep their single-CTA kernels (FP64 33^3: not supported)
    with pytest.raises(Exception):
        plan_kernel(d, name, precision=64)
    assert plan_kernel(d, name, faithful=True).kernel_layout & 32 == 0


@pytest.mark.parametrize("seed", range(6))
def test_pair_step_algebra_matches_one_cta(seed):
    """One Lanczos step split as the pair splits it (FP64 here): each CTA gathers c over the
    list points of its own planes, a_k = CTA 0's stencil partials + CTA 1's + sum Gamma c^2
    with c = c_0 + c_1, the scatter adds chi alpha on each CTA's own planes, and b_k^2 sums
    both CTAs' |w|^2 -- the same a_k, b_k and w as the single-CTA step."""
    rng = np.random.default_rng(seed)
    n, nlm = 15, 4
    zs = (n + 1) // 2
    N = n ** 3
    z_of = np.repeat(np.arange(n), n * n)  # point index (z slowest) -> plane
    own = [z_of < zs, z_of >= zs]
    # local operator: diagonal plus a 7-point-like banded part in the flattened cube
    Hl = np.diag(rng.uniform(0.5, 3.0, N))
    for off in (1, n, n * n):
        band = rng.uniform(-0.5, 0.0, N - off)
        Hl += np.diag(band, off) + np.diag(band, -off)
    m = 3
    chi = [np.where(rng.random((N, 1)) < 0.2, rng.standard_normal((N, nlm)), 0.0) for _ in range(m)]
    gam = [rng.uniform(-1.0, 1.0, nlm) for _ in range(m)]
    P = rng.standard_normal(N)
    U = rng.standard_normal(N)
    tb = 1.7
    inv = 1.0 / tb
    v = P * inv
    # single CTA
    Hv = Hl @ v
    c = [x.T @ v for x in chi]
    a1 = v @ Hv + sum(g @ (cc * cc) for g, cc in zip(gam, c))
    w1 = Hv - tb * U + sum(x @ (g * cc) for x, g, cc in zip(chi, gam, c)) - a1 * v
    b1 = np.sqrt(w1 @ w1)
    # the pair
    cpart = [[x[own[r]].T @ P[own[r]] for x in chi] for r in (0, 1)]   # phase 2 rows
    cx = [(cpart[0][k] + cpart[1][k]) * inv for k in range(m)]
    a_loc = [v[own[r]] @ Hv[own[r]] for r in (0, 1)]                     # passes A and B
    a_nl = sum(g @ (cc * cc) for g, cc in zip(gam, cx))
    a2 = (a_loc[0] + a_loc[1]) + a_nl
    w2 = np.empty(N)
    b2sq = 0.0
    for r in (0, 1):
        sel = own[r]
        Ur = (Hv - tb * U)[sel] + sum(x[sel] @ (g * cc) for x, g, cc in zip(chi, gam, cx))
        w2[sel] = Ur - a2 * v[sel]
        b2sq += w2[sel] @ w2[sel]
    np.testing.assert_allclose(a2, a1, rtol=1e-13)
    np.testing.assert_allclose(np.sqrt(b2sq), b1, rtol=1e-13)
    np.testing.assert_allclose(w2, w1, rtol=1e-12, atol=1e-12)
