"""The split-pass FP32 Lanczos kernel's index arithmetic and stencil algebra, restated on the CPU.

For every cube size the kernel accepts (up to 32 points wide) and every tile it can run with
(threads <= 512), in the thread -> (row, quad, z-range) and (plane, quad, y-range) maps of
lanczos_quad.cuh:
  * the z pass and the y pass each cover every quad of the cube exactly once;
  * every shared-memory read (ring loads, x-neighbour quads and half-quads) lies inside P and
    inside the thread's own row, and every skipped read is a neighbour outside the cube;
  * every read of the quad-aligned Veff copies lies inside its copy, on a 16-byte boundary,
    and holds the value of the cube point it stands for;
  * the two passes, run as the kernel runs them (register rings, predicated x loads, zeroed
    pad points), give the 37-point stencil of the cube with Dirichlet boundary exactly as a
    direct evaluation does (same products, FP64 here).
"""
import numpy as np
import pytest

O = 6
MAX_THREADS = 512


def plane_floats(n, pitch):
    """Floats per z-plane: n rows of pitch plus the pad that makes the stride one row modulo
    the 32 banks (quad_plane_floats in lanczos_quad.cuh)."""
    return n * pitch + ((pitch - n * pitch) % 32 + 32) % 32


def quad_threads(n, tile):
    nq = (n + 3) // 4
    return max(64, 32 * ((nq * n * tile + 31) // 32))


def quad_block(n, tile):
    """Threads the engine launches: the passes' threads, rounded up to every warp of the
    register budget (12 warps up to 384 threads, 16 above) once they pass 256."""
    t = quad_threads(n, tile)
    return t if t <= 256 else (384 if t <= 384 else 512)


@pytest.mark.parametrize("n,h", [(3, 0.85), (5, 0.85), (9, 0.85), (17, 0.5), (27, 0.5)])
@pytest.mark.parametrize("tile", [1, 2, 3, 4])
def test_engine_thread_count(n, h, tile, tmp_path):
    """The engine's thread count for a tile (sq_plan_kernel) is the restated one, and always
    at least two warps: warp 0 builds a node's image list while the others clear P and U.
    Above 256 threads the launch takes every warp of the register budget."""
    from sqminiapp_gb300 import plan_kernel
    from sqminiapp_gb300.decks import make_fcc_mg_deck
    rcut = h * (n - 1) / 2
    d, name, _ = make_fcc_mg_deck(str(tmp_path), "c", ncell=1, h=h, rcut=rcut, n_qp=8)
    if quad_threads(n, tile) > MAX_THREADS:
        return
    p = plan_kernel(d, name, kernel=2, tile=tile)
    assert p.cube[0] == n
    assert p.kernel_threads == quad_block(n, tile) >= quad_threads(n, tile) >= 64


def thread_maps(n, tile):
    """Per thread: pass-A (y, quad, zb, ze, active) and pass-B (z, quad, yb, ye, active)."""
    nq = (n + 3) // 4
    # the launch's threads (those past the passes' need stay idle); the algebra test also
    # runs tiles above the kernel's 512 threads, with exactly the threads they need
    t = np.arange(max(quad_threads(n, tile), quad_block(n, tile)))
    grp, ql = t // nq, t % nq
    ln = (n + tile - 1) // tile
    yA, zc = grp % n, grp // n
    zb = np.minimum(n, zc * ln)
    ze = np.minimum(n, zb + ln)
    actA = (zc < tile) & (zb < ze)
    zB, yc = grp % n, grp // n
    yb = np.minimum(n, yc * ln)
    ye = np.minimum(n, yb + ln)
    actB = (yc < tile) & (yb < ye)
    return nq, ql, (yA, zb, ze, actA), (zB, yb, ye, actB)


CASES = [(n, tile) for n in (9, 13, 17, 21, 25, 27, 29, 31, 32) for tile in (1, 2, 3, 4)
         if quad_threads(n, tile) <= MAX_THREADS]


@pytest.mark.parametrize("n,tile", CASES)
def test_passes_cover_every_quad_once(n, tile):
    nq, ql, (yA, zb, ze, actA), (zB, yb, ye, actB) = thread_maps(n, tile)
    seen = np.zeros((n, n, nq), dtype=int)  # [z][y][quad]
    for i in np.nonzero(actA)[0]:
        seen[zb[i]:ze[i], yA[i], ql[i]] += 1
    assert np.all(seen == 1)
    seen[:] = 0
    for i in np.nonzero(actB)[0]:
        seen[zB[i], yb[i]:ye[i], ql[i]] += 1
    assert np.all(seen == 1)


@pytest.mark.parametrize("n,tile", CASES)
def test_shared_reads_stay_in_the_row(n, tile):
    nq, ql, (yA, zb, ze, actA), _ = thread_maps(n, tile)
    pitch = 4 * nq
    ps = plane_floats(n, pitch)
    assert ps % 4 == 0 and ps >= n * pitch
    nc = n * ps
    for i in np.nonzero(actA)[0]:
        q = ql[i]
        for z in range(zb[i], ze[i]):
            row0 = z * ps + yA[i] * pitch  # first float of the row
            i4 = (z * ps + yA[i] * pitch) // 4 + q
            reads = []
            if q >= 2:  # float2 at x0-6
                reads += [2 * (2 * i4 - 3), 2 * (2 * i4 - 3) + 1]
            if q >= 1:
                reads += list(range(4 * (i4 - 1), 4 * i4))
            if q + 1 < nq:
                reads += list(range(4 * (i4 + 1), 4 * (i4 + 2)))
            if q + 2 < nq:  # float2 at x0+8
                reads += [2 * (2 * i4 + 4), 2 * (2 * i4 + 4) + 1]
            reads = np.array(reads)
            assert np.all((reads >= row0) & (reads < row0 + pitch)), (n, tile, z, q)
            assert nc % 4 == 0 and reads.max() < nc
            # skipped quads are the ones left or right of the row: outside the cube
            x0 = 4 * q
            if q < 2:
                assert x0 - 6 < 0
            if q + 2 >= nq:
                assert x0 + 8 >= n or x0 + 9 >= n


def test_veff_quad_copies_are_aligned_and_right():
    # a small periodic grid: every node's quad reads, through the kernel's indexing
    N, n = 7, 9
    nh = (n - 1) // 2
    EX = EY = EZ = N + 2 * nh
    row = 4 * ((EX + 6 + 3) // 4)
    stride = row * EY * EZ
    rng = np.random.default_rng(0)
    veff = rng.standard_normal((N, N, N))
    cdiag = 1.25
    copies = np.zeros((4, EZ, EY, row))
    for c in range(4):
        for ex in range(EX):
            gx = (ex - nh) % N
            for ey in range(EY):
                for ez in range(EZ):
                    copies[c, ez, ey, ex + c] = cdiag + veff[(ez - nh) % N, (ey - nh) % N, gx]
    flat = copies.reshape(-1)
    nq = (n + 3) // 4
    for I in range(N):
        sh = (4 - (I & 3)) & 3
        assert (I + sh) % 4 == 0
        for J in (0, N - 1):
            for K in (0, N - 1):
                for y in range(n):
                    for z in range(n):
                        for q in range(nq):
                            quad = sh * stride // 4 + ((K + z) * EY + J + y) * (row // 4) + (I + sh) // 4 + q
                            assert (quad + 1) * 4 <= 4 * stride
                            vals = flat[4 * quad:4 * quad + 4]
                            for j in range(4):
                                x = 4 * q + j
                                if x < n:  # a cube point: Veff at global (I+x-nh, J+y-nh, K+z-nh)
                                    want = cdiag + veff[(K + z - nh) % N, (J + y - nh) % N, (I + x - nh) % N]
                                    assert vals[j] == want


def _stencil_direct(v, c):
    n = v.shape[0]
    h = c[0] * v
    for d in range(1, O + 1):
        for ax in range(3):
            a = np.zeros_like(v)
            b = np.zeros_like(v)
            sl = [slice(None)] * 3
            sl2 = [slice(None)] * 3
            sl[ax], sl2[ax] = slice(d, n), slice(0, n - d)
            a[tuple(sl)] = v[tuple(sl2)]   # v(x - d)
            b[tuple(sl2)] = v[tuple(sl)]   # v(x + d)
            h += c[d] * (a + b)
    return h


@pytest.mark.parametrize("n,tile", [(9, 1), (13, 2), (27, 2), (29, 2), (25, 3)])
def test_split_passes_equal_the_direct_stencil(n, tile):
    """Run pass A (z ring, x quads, diagonal, pad zeroing) and pass B (y ring) thread by
    thread on a random cube in the kernel's row-padded layout and compare with the direct
    37-point Dirichlet stencil."""
    rng = np.random.default_rng(n * 7 + tile)
    c = np.concatenate([[-3.0], rng.uniform(-1, 1, O)])
    dv = rng.uniform(0.5, 1.5, (n, n, n))  # cdiag + Veff per point
    v = rng.standard_normal((n, n, n))
    nq, ql, (yA, zb, ze, actA), (zB, yb, ye, actB) = thread_maps(n, tile)
    pitch = 4 * nq
    P = np.zeros((n, n, pitch))
    P[:, :, :n] = v
    U = np.zeros_like(P)
    for i in np.nonzero(actA)[0]:
        q, y = ql[i], yA[i]
        x0 = 4 * q
        ring = {zq: (P[zq, y, x0:x0 + 4] if 0 <= zq < n else np.zeros(4))
                for zq in range(zb[i] - O, ze[i] + O)}
        for z in range(zb[i], ze[i]):
            e = np.zeros(16)  # P[x0-6 .. x0+9] with the kernel's predication
            if q >= 2:
                e[0:2] = P[z, y, x0 - 6:x0 - 4]
            if q >= 1:
                e[2:6] = P[z, y, x0 - 4:x0]
            e[6:10] = ring[z]
            if q + 1 < nq:
                e[10:14] = P[z, y, x0 + 4:x0 + 8]
            if q + 2 < nq:
                e[14:16] = P[z, y, x0 + 8:x0 + 10]
            dvq = np.zeros(4)
            m = min(4, n - x0)
            dvq[:m] = dv[z, y, x0:x0 + m]
            h = dvq * ring[z]
            for d in range(1, O + 1):
                h = h + c[d] * (ring[z - d] + ring[z + d])
                h = h + c[d] * (e[6 - d:10 - d] + e[6 + d:10 + d])
            h[m:] = 0.0  # pad points
            U[z, y, x0:x0 + 4] = h
    for i in np.nonzero(actB)[0]:
        q, z = ql[i], zB[i]
        x0 = 4 * q
        ring = {yq: (P[z, yq, x0:x0 + 4] if 0 <= yq < n else np.zeros(4))
                for yq in range(yb[i] - O, ye[i] + O)}
        for y in range(yb[i], ye[i]):
            h = np.zeros(4)
            for d in range(1, O + 1):
                h = h + c[d] * (ring[y - d] + ring[y + d])
            U[z, y, x0:x0 + 4] += h
    want = _stencil_direct(v, np.concatenate([[0.0], c[1:]])) + dv * v
    np.testing.assert_allclose(U[:, :, :n], want, rtol=1e-12, atol=1e-12)
    assert np.all(U[:, :, n:] == 0.0)


def _gather_pairs(kept, nw):
    """The (image, warp) pairs the kernel's gather loop writes (part[k + w]) and the ones the
    alpha phase reads, restated from lanczos_quad.cuh."""
    n_img = len(kept)
    koff = np.concatenate([[0], np.cumsum(kept)])
    total = int(koff[-1])
    per = (total + nw - 1) // nw
    written = set()
    for w in range(nw):
        r_begin = min(total, w * per)
        r_end = min(total, r_begin + per)
        lo, hi = 0, n_img  # largest k with koff[k] <= r_begin
        while lo < hi:
            mid = (lo + hi + 1) >> 1
            if koff[mid] <= r_begin:
                lo = mid
            else:
                hi = mid - 1
        k = min(lo, max(n_img - 1, 0))
        pos = r_begin
        while pos < r_end:
            kend = min(r_end, koff[k + 1])
            written.add((k, w))
            pos = kend
            k += 1
    read = set()
    for k in range(n_img):
        if koff[k + 1] == koff[k]:
            continue
        for w in range(koff[k] // per, (koff[k + 1] - 1) // per + 1):
            read.add((k, w))
    return written, read, koff, per


@pytest.mark.parametrize("seed", range(40))
def test_gather_partials_cover_every_point_once(seed):
    """Every point of the node's list is summed exactly once into its image's c: the warps'
    ranges tile [0, total), every (image, warp) pair the alpha phase reads was written by that
    warp in the same step, and the partial index k + w never collides or leaves the array."""
    rng = np.random.default_rng(seed)
    n_img = int(rng.integers(1, 120))
    nw = int(rng.integers(2, 17))
    kept = rng.integers(0, 900, n_img) * (rng.random(n_img) > 0.15)
    written, read, koff, per = _gather_pairs(kept, nw)
    assert read <= written
    idx = [k + w for (k, w) in written]
    assert len(set(idx)) == len(idx) and max(idx, default=0) < n_img + 32
    # each point belongs to exactly one warp range and one image: the read pairs cover it once
    total = int(koff[-1])
    covered = np.zeros(total, dtype=int)
    for (k, w) in read:
        lo = max(koff[k], w * per)
        hi = min(koff[k + 1], min(total, w * per + per))
        covered[lo:hi] += 1
    assert np.all(covered == 1)


@pytest.mark.parametrize("n,tile", CASES)
def test_float4_accesses_are_bank_conflict_free(n, tile):
    """Every warp-wide float4 access of the z pass (a row of quads per thread group) and of the
    y pass (a plane per thread group, at one ring row) is served in the minimum four
    wavefronts: within each quarter-warp whose threads work on the same z- (y-) range, the
    eight 16-byte accesses use distinct banks.  (A quarter-warp that straddles two ranges
    reads planes (rows) a range length apart and may pay one extra wavefront.)"""
    nq, ql, (yA, zb, ze, actA), (zB, yb, ye, actB) = thread_maps(n, tile)
    pitch = 4 * nq
    ps = plane_floats(n, pitch)
    nt = len(ql)

    def check(word, active, rng):
        checked = 0
        for q0 in range(0, nt, 8):
            ts = [t for t in range(q0, min(q0 + 8, nt)) if active[t]]
            if len({int(rng[t]) for t in ts}) != 1:
                continue
            banks = [(int(word[t]) + j) % 32 for t in ts for j in range(4)]
            assert len(banks) == len(set(banks)), (n, tile, q0)
            checked += 1
        assert checked >= (np.count_nonzero(active) // 8) * 3 // 4

    # z pass, every thread at the same offset into its z-range (all offsets alike)
    check(zb * ps + yA * pitch + 4 * ql, actA, zb)
    # y pass, every thread at the same offset into its y-range
    check(zB * ps + yb * pitch + 4 * ql, actB, yb)


@pytest.mark.parametrize("planes", list(range(1, 30)))
def test_veff_ring_slots_and_groups(planes):
    """Pass A's Veff ring (lanczos_quad.cuh, kVRingSlots = 4, three planes ahead), restated:
    the prologue commits one group per plane 0..2 (empty past the range), every plane waits
    until at most 2 groups are pending, reads its slot and commits the copy of plane + 3 into
    the slot read one plane earlier.  Every read finds its own plane's copy complete, and no
    copy overwrites a slot before its plane has been read."""
    slots, ahead = 4, 3
    ring = [None] * slots
    groups = []  # (plane or None, slot)
    done = 0     # groups completed so far (in order)

    assigned = [None] * slots  # the plane last issued into each slot

    def commit(plane, slot):
        if plane < planes:
            # the copy may land at once: the slot's previous plane must already have been read
            assert assigned[slot] is None or assigned[slot] in read, "slot reused early"
            assigned[slot] = plane
        groups.append((plane if plane < planes else None, slot))

    read = set()
    for d in range(ahead):
        commit(d, d)
    for i in range(planes):
        # cp.async.wait_group 2: complete the oldest groups until at most 2 are pending
        while len(groups) - done > ahead - 1:
            plane, slot = groups[done]
            if plane is not None:
                assert ring[slot] is None or ring[slot] in read, "slot overwritten unread"
                ring[slot] = plane
            done += 1
        assert ring[i & (slots - 1)] == i
        read.add(i)
        commit(i + ahead, (i + ahead) & (slots - 1))
    assert read == set(range(planes))
