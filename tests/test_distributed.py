"""Multi-process path on the CPU: world size 2 over gloo (127.0.0.1).

The quadrature of a cell is split into node ranges (one per rank); the Fermi bisection sums
the per-rank electron counts with one scalar all-reduce per step.  The sharded result must
equal the single-process oracle (sqo_fermi_density_energy uses the same bracket and rule).
"""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, lam, w, beta, ne, out):
    import torch.distributed as dist
    from sqminiapp_gb300 import sharding
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        b, e = sharding.node_range(lam.shape[0], rank, world)
        my_l, my_w = lam[b:e], w[b:e]
        s, mn, mx = sharding.torch_reducers()
        lf, it = sharding.fermi_level(sharding.numpy_count(my_l, my_w, beta), my_l.min(),
                                      my_l.max(), ne, s, mn, mx)
        out[rank] = lf
    finally:
        dist.destroy_process_group()


def test_node_ranges_partition():
    from sqminiapp_gb300.sharding import node_range
    for n in (1, 7, 3366, 39304):
        for world in (1, 2, 3, 8):
            ranges = [node_range(n, r, world) for r in range(world)]
            assert ranges[0][0] == 0 and ranges[-1][1] == n
            assert all(ranges[i][1] == ranges[i + 1][0] for i in range(world - 1))


def test_sharded_fermi_level_matches_single_process(oracle_mod):
    rng = np.random.default_rng(5)
    lam = rng.uniform(-1.0, 4.0, (501, 10))
    w = rng.dirichlet(np.ones(10), 501)
    beta, ne = 50.0, 300.0
    ref = oracle_mod.fermi_density_energy(lam, w, beta, ne, 1.0)
    ctx = mp.get_context("spawn")
    out = ctx.Manager().dict()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, lam, w, beta, ne, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    assert out[0] == out[1]
    assert out[0] == pytest.approx(ref["lambda_f"], abs=1e-11)


class OracleShard:
    """One rank's part of a sharded SCF computed by the CPU oracle (the test's stand-in for
    the engine's sq_scf_shard_* calls): SQ pass on the rank's nodes only, the replicated
    potential, mixing and energies of oracle/scf.py on the full grid."""

    def __init__(self, o, fields, mix, history, pulay_every, k_tf, nthreads=2):
        from oracle import scf as S
        self.S, self.o, self.fields = S, o, fields
        self.beta, self.n_nodes, self.n_electrons = o.beta, o.n_nodes, o.n_electrons
        self.shape = fields["b"].shape
        self.x = fields["rho0"].copy()
        self.x *= o.n_electrons / (np.sum(self.x) * o.dV)
        self.state = {"dX": [], "dF": [], "x_prev": None}
        self.mix, self.history, self.every = mix, history, pulay_every
        self.pk = S.kerker(fields["green"], k_tf)
        self.nthreads, self.k = nthreads, 0

    def sq_pass(self, b, e):
        S = self.S
        self.phi = S.poisson(self.x + self.fields["b"], self.fields["green"])
        self.eps, self.vxc = S.lda_pw92(self.x)
        veff = (self.phi + self.vxc).ravel()
        q = self.o.nodes_and_weights(nodes=np.arange(b, e), veff=veff, veff_const=0.0,
                                     nthreads=self.nthreads)
        self.lam, self.w = q["lambda"], q["weights"]
        return float(self.lam.min()), float(self.lam.max())

    def _f(self, lf):
        return 1.0 / (1.0 + np.exp(np.clip(self.beta * (self.lam - lf), -700, 700)))

    def counts(self, levels):
        return np.array([np.sum(2.0 * self.w * self._f(lf)) for lf in levels])

    def density(self, lf):
        f = self._f(lf)
        rho = 2.0 * np.sum(self.w * f, axis=1) / self.o.dV
        with np.errstate(divide="ignore", invalid="ignore"):
            s = np.where((f > 0) & (f < 1), f * np.log(f) + (1 - f) * np.log(1 - f), 0.0)
        return rho, np.array([np.sum(2 * self.w * self.lam * f), np.sum(2 * self.w * s)])

    def finish(self, rho_out, lf, e_band, ts):
        S, fl, x, dV = self.S, self.fields, self.x, self.o.dV
        rho_out = rho_out.reshape(self.shape)
        F = (e_band + np.sum(x * self.eps) * dV - np.sum(x * self.vxc) * dV
             + 0.5 * np.sum((fl["b"] - x) * self.phi) * dV - fl["e_self"] + fl["e_corr"] + ts)
        f = rho_out - x
        err = float(np.linalg.norm(f) / np.linalg.norm(rho_out))
        out = {"free_energy": F, "free_energy_per_atom": F / self.o.natoms, "residual": err,
               "lambda_f": lf, "converged": err < 1e-6}
        if err >= 1e-6:
            self.x = S.periodic_pulay_step(x, f, self.state, self.k, self.mix, self.history,
                                           self.every, self.pk)
            self.x *= self.n_electrons / (np.sum(self.x) * dV)
        self.k += 1
        return out


def _scf_worker(rank, world, port, deck, out):
    import oracle
    import torch.distributed as dist
    from oracle import scf as S
    from sqminiapp_gb300 import sharding
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        o = oracle.Oracle(deck[0], deck[1], faithful=False)
        shard = OracleShard(o, S.scf_fields(o), 0.3, 7, 2, 1.0)
        run = sharding.ShardedSCF(shard, sharding.TorchComm())
        hist = []
        for _ in range(40):
            r = run.step()
            hist.append((r["free_energy_per_atom"], r["residual"], r["lambda_f"]))
            if r["converged"]:
                break
        out[rank] = {"hist": hist, "rounds": run.fermi_rounds, "rho": shard.x.ravel().copy()}
        o.close()
    finally:
        dist.destroy_process_group()


def test_sharded_scf_matches_single_process_oracle(oracle_mod, small_cell):
    """One cell's nodes split over two gloo ranks: the k-level Fermi search, the summed
    energies and the gathered density give the single-process oracle SCF iteration by
    iteration (free energy per atom to 1e-10 Ha, residual and Fermi level alike)."""
    from oracle import scf as S
    d, name, _ = small_cell
    o = oracle_mod.Oracle(d, name, faithful=False)
    ref = S.scf(o, tol=1e-6, maxit=40, mix=0.3, history=7, pulay_every=2, k_tf=1.0)
    o.close()
    ctx = mp.get_context("spawn")
    out = ctx.Manager().dict()
    port = _free_port()
    procs = [ctx.Process(target=_scf_worker, args=(r, 2, port, (d, name), out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=600)
        assert p.exitcode == 0
    h0, h1 = out[0]["hist"], out[1]["hist"]
    assert h0 == h1  # replicated state: bit-identical on both ranks
    assert np.array_equal(out[0]["rho"], out[1]["rho"])
    assert len(h0) == ref["iterations"]
    F = np.array([h[0] for h in h0])
    natoms = ref["free_energy"] / ref["free_energy_per_atom"]
    np.testing.assert_allclose(F, ref["free_energy_history"] / natoms, rtol=0, atol=1e-10)
    np.testing.assert_allclose([h[1] for h in h0], ref["residual_history"], rtol=1e-6, atol=1e-9)
    assert abs(h0[-1][2] - ref["lambda_f"]) < 1e-11
    # the k-level search needs about a quarter of the bisection's all-reduces
    assert max(out[0]["rounds"]) <= 14
