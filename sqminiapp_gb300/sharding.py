"""Node sharding of one cell over several GPUs, one process per GPU.

Every FD node's Lanczos/quadrature is independent (the reference splits the nodes of one
cell over MPI ranks, DMDACreate3d on PETSC_COMM_WORLD, src/lsdft_initObjs.cc:132-133, each
rank looping over its corner block with no communication in the hot loop,
src/lsdft_scf.cc:47-62), so a cell is split into contiguous node ranges (z slowest, so each
range is a z-slab plus partial planes) and each rank runs the SQ pass on its own range.  An
SCF iteration then has three exchanges:
  * the Fermi level: its electron count N_e(lf) is a sum over ranks.  fermi_level_kary
    evaluates k trial levels per round and sums a k-vector over the ranks, so the bracket
    shrinks (k+1)-fold per all-reduce: about 11 rounds for k = 15 instead of about 45 scalar
    all-reduces of a bisection (fermi_level keeps that form too);
  * the band energy and entropy sums (one 2-vector all-reduce);
  * the output density, all-gathered so that every rank runs the same Poisson solve,
    exchange-correlation potential and mixing on the full grid (replicated, identical on
    every rank).
ShardedSCF drives one rank's iteration over a `shard` object (EngineShard: the engine's
sq_scf_shard_* entry points) and a `comm` object (TorchComm: torch.distributed, gloo or
nccl; LocalComm: one rank).
"""
import threading

import numpy as np


def node_range(n_nodes, rank, world):
    """Contiguous node range [begin, end) of `rank` (z-slowest node order, near-equal sizes)."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("bad rank/world")
    return (n_nodes * rank) // world, (n_nodes * (rank + 1)) // world


def fermi_level(local_count, local_min, local_max, n_electrons, allreduce_sum, allreduce_min,
                allreduce_max, tol=1e-12, maxit=400):
    """Bisection for lambda_f with the electron count summed over ranks.

    local_count(lf) -> this rank's 2 sum w f(lambda - lf); local_min/max: extremes of this
    rank's lambdas; allreduce_*: scalar reductions over the ranks.  Returns (lf, iterations).
    """
    lo = allreduce_min(local_min) - 1.0
    hi = allreduce_max(local_max) + 1.0
    it = 0
    for it in range(maxit):
        mid = 0.5 * (lo + hi)
        ne = allreduce_sum(local_count(mid))
        if ne > n_electrons:
            hi = mid
        else:
            lo = mid
        if hi - lo < tol:
            break
    return 0.5 * (lo + hi), it


def torch_reducers(group=None):
    """Scalar all-reduce callables over a torch.distributed group (gloo or nccl)."""
    import torch
    import torch.distributed as dist

    def make(op):
        def red(x):
            backend = dist.get_backend(group)
            dev = torch.device("cuda", torch.cuda.current_device()) if backend == "nccl" else "cpu"
            t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
            dist.all_reduce(t, op=op, group=group)
            return float(t.item())
        return red

    return make(dist.ReduceOp.SUM), make(dist.ReduceOp.MIN), make(dist.ReduceOp.MAX)


def numpy_count(lam, w, beta):
    """Host electron count of quadrature arrays (used where no GPU is present)."""
    def count(lf):
        x = np.clip(beta * (lam - lf), -700.0, 700.0)
        return float(np.sum(2.0 * w / (1.0 + np.exp(x))))
    return count


def fermi_level_kary(local_counts, local_min, local_max, n_electrons, allreduce_sum,
                     allreduce_min, allreduce_max, tol=1e-12, k=15, maxit=64):
    """Fermi level with k trial levels per round: local_counts(levels) -> this rank's counts
    at an array of levels; allreduce_sum sums an array over the ranks.  The bracket
    [lo, hi] keeps count(lo) <= N_e < count(hi) as the bisection does.  Returns
    (lf, rounds)."""
    lo = allreduce_min(local_min) - 1.0
    hi = allreduce_max(local_max) + 1.0
    frac = np.arange(1, k + 1, dtype=np.float64) / (k + 1)
    rounds = 0
    while hi - lo >= tol and rounds < maxit:
        levels = lo + (hi - lo) * frac
        counts = np.asarray(allreduce_sum(np.asarray(local_counts(levels), dtype=np.float64)))
        above = np.nonzero(counts > n_electrons)[0]
        i = int(above[0]) if above.size else k
        new_lo = levels[i - 1] if i > 0 else lo
        new_hi = levels[i] if i < k else hi
        if not (new_lo > lo or new_hi < hi):
            break  # the levels no longer resolve the bracket
        lo, hi = new_lo, new_hi
        rounds += 1
    return 0.5 * (lo + hi), rounds


class LocalComm:
    """One rank: every collective is the identity."""

    rank, world = 0, 1

    def sum(self, x):
        return np.asarray(x, dtype=np.float64)

    def min(self, x):
        return float(x)

    def max(self, x):
        return float(x)

    def gather(self, local, n_total):
        return np.asarray(local, dtype=np.float64).reshape(n_total)


class TorchComm:
    """Collectives over a torch.distributed process group (gloo on CPU tensors, nccl on the
    current device)."""

    def __init__(self, group=None):
        import torch.distributed as dist
        self.dist = dist
        self.group = group
        self.rank = dist.get_rank(group)
        self.world = dist.get_world_size(group)

    def _tensor(self, x):
        import torch
        dev = "cpu"
        if self.dist.get_backend(self.group) == "nccl":
            dev = torch.device("cuda", torch.cuda.current_device())
        return torch.as_tensor(np.atleast_1d(np.asarray(x, dtype=np.float64)), device=dev)

    def _reduce(self, x, op):
        t = self._tensor(x)
        self.dist.all_reduce(t, op=op, group=self.group)
        return t.cpu().numpy()

    def sum(self, x):
        return self._reduce(x, self.dist.ReduceOp.SUM).reshape(np.shape(x))

    def min(self, x):
        return float(self._reduce(x, self.dist.ReduceOp.MIN)[0])

    def max(self, x):
        return float(self._reduce(x, self.dist.ReduceOp.MAX)[0])

    def gather(self, local, n_total):
        """The ranks' node ranges (node_range order) joined into the full array."""
        import torch
        width = max(e - b for b, e in (node_range(n_total, r, self.world) for r in range(self.world)))
        t = self._tensor(np.pad(np.asarray(local, dtype=np.float64), (0, width - len(local))))
        parts = [torch.empty_like(t) for _ in range(self.world)]
        self.dist.all_gather(parts, t, group=self.group)
        out = np.empty(n_total)
        for r, part in enumerate(parts):
            b, e = node_range(n_total, r, self.world)
            out[b:e] = part.cpu().numpy()[:e - b]
        return out


class ThreadComm:
    """Ranks as threads of one process (each with its own engine, e.g. two handles on one
    GPU): collectives meet at a barrier and combine host arrays in rank order.  No GPU work
    waits on another rank; the exchange is on the host."""

    class _Shared:
        def __init__(self, world):
            self.world = world
            self.barrier = threading.Barrier(world)
            self.slots = [None] * world

    def __init__(self, shared, rank):
        self.shared, self.rank, self.world = shared, rank, shared.world

    @classmethod
    def group(cls, world):
        shared = cls._Shared(world)
        return [cls(shared, r) for r in range(world)]

    def _all(self, x):
        sh = self.shared
        sh.slots[self.rank] = np.array(x, dtype=np.float64, copy=True)
        sh.barrier.wait()
        vals = list(sh.slots)
        sh.barrier.wait()
        return vals

    def sum(self, x):
        vals = self._all(x)
        out = np.zeros_like(vals[0])
        for v in vals:
            out = out + v
        return out

    def min(self, x):
        return float(min(v.item() for v in self._all(x)))

    def max(self, x):
        return float(max(v.item() for v in self._all(x)))

    def gather(self, local, n_total):
        vals = self._all(local)
        return np.concatenate(vals).reshape(n_total)


class EngineShard:
    """One rank's part of a sharded SCF on the engine (sq_scf_shard_* of sq_gb300.h); the
    engine's SCF must have been started (LSDFT.scf_begin) with the same options and start
    density on every rank."""

    def __init__(self, engine):
        import ctypes
        self.eng = engine
        self._ct = ctypes
        self.beta = engine.beta
        self.n_nodes = engine.n_nodes
        self.n_electrons = engine.n_electrons
        self.natoms = engine.info.n_atoms

    def _ptr(self, a):
        return a.ctypes.data_as(self._ct.POINTER(self._ct.c_double))

    def sq_pass(self, begin, end):
        from .capi import check
        mm = np.zeros(2)
        check(self.eng._lib.sq_scf_shard_sq(self.eng._h, int(begin), int(end), self._ptr(mm)),
              "sq_scf_shard_sq")
        self._n = end - begin
        return mm[0], mm[1]

    def counts(self, levels):
        from .capi import check
        lv = np.ascontiguousarray(levels, dtype=np.float64)
        out = np.zeros(len(lv))
        check(self.eng._lib.sq_scf_shard_counts(self.eng._h, len(lv), self._ptr(lv),
                                                self._ptr(out)), "sq_scf_shard_counts")
        return out

    def density(self, lf):
        from .capi import check
        rho = np.zeros(self._n)
        sums = np.zeros(2)
        check(self.eng._lib.sq_scf_shard_density(self.eng._h, float(lf), self._ptr(rho),
                                                 self._ptr(sums)), "sq_scf_shard_density")
        return rho, sums

    def finish(self, rho_out, lf, e_band, ts):
        from .capi import SqScfResult, check
        res = SqScfResult()
        rho_out = np.ascontiguousarray(rho_out, dtype=np.float64)
        check(self.eng._lib.sq_scf_shard_finish(self.eng._h, self._ptr(rho_out), float(lf),
                                                float(e_band), float(ts),
                                                self._ct.byref(res)), "sq_scf_shard_finish")
        return res.as_dict()


class ShardedSCF:
    """One rank's SCF iterations over a shard (EngineShard, or any object with sq_pass,
    counts, density, finish, beta, n_nodes, n_electrons) and a comm."""

    def __init__(self, shard, comm, fermi_tol=1e-12, k=15):
        self.shard, self.comm = shard, comm
        self.fermi_tol, self.k = fermi_tol, k
        self.range = node_range(shard.n_nodes, comm.rank, comm.world)
        self.fermi_rounds = []

    def step(self):
        b, e = self.range
        lmin, lmax = self.shard.sq_pass(b, e)
        lf, rounds = fermi_level_kary(self.shard.counts, lmin, lmax, self.shard.n_electrons,
                                      self.comm.sum, self.comm.min, self.comm.max,
                                      tol=self.fermi_tol, k=self.k)
        self.fermi_rounds.append(rounds)
        rho_local, sums = self.shard.density(lf)
        e_band, ent = self.comm.sum(np.asarray(sums, dtype=np.float64))
        rho_out = self.comm.gather(rho_local, self.shard.n_nodes)
        return self.shard.finish(rho_out, lf, float(e_band), float(ent) / self.shard.beta)

    def run(self, maxit=100):
        out = {}
        for _ in range(maxit):
            out = self.step()
            if out.get("converged"):
                break
        return out
