"""Node sharding over several GPUs, one process per GPU.

Every FD node's Lanczos/quadrature is independent (the reference splits nodes over MPI
ranks with no communication in the hot loop, src/lsdft_scf.cc:49,60-80), so a cell is split
into contiguous node ranges and each rank runs sq_nodes_and_weights on its own range.  The
one exchange step is the Fermi level: its bisection needs the global electron count
N_e(lf) = sum over ranks of the local counts, so each bisection step costs one scalar
all-reduce.  The bracket and the update rule are the ones of the single-GPU kernel
(fermi.cu), so a sharded run finds the same lambda_f as an unsharded one.
"""
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
