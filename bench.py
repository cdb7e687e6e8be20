#!/usr/bin/env python3
"""Benchmark: node-Lanczos/s of the per-node Spectral Quadrature pass on GB300.

Workload (default): 32 Mg atoms, FCC 2x2x2 periodic cell of side 17 bohr with seeded
+-0.15 bohr displacements, h = 0.5 bohr (34^3 = 39,304 FD nodes), Rcut = 6.5 bohr
(27^3-point cubes), 40 Lanczos steps per node, FP32 vectors with FP64 coefficients,
quadrature, Fermi bisection and sums.  One step = every node's Lanczos + Gauss quadrature
followed by the Fermi-level bisection, node densities and band energy.  Synthetic data:
the cell is generated from a seed; there is no public dataset.

value  = nodes processed per second with the inputs resident in device memory, from CUDA
         events around each step (L2 flushed between steps by writing 256 MiB).
e2e    = the same metric through the host-buffer C ABI (sq_nodes_and_weights +
         sq_fermi_density_energy): Veff uploaded, quadrature and densities read back, every
         step.
roofline: the Lanczos kernel's algorithmic FP32 FLOPs per launch over its CUDA-event time,
         against the device's FP32 FMA peak measured by the library's probe kernel.
cpu_baseline / --impl reference: the FP64 CPU restatement of the reference's per-node path
         (oracle/, one thread per host core) on a bounded sample of the same workload.
scf:     time-to-SCF-convergence (the other half of the headline metric) on the bench's
         32-atom cell: the FP64 engine and the FP32 engine from the atomic-superposition
         density, and the FP32 engine from the learned start (committed model), with their
         free energies per atom.

Multi-GPU (torchrun): one rank per GPU, each rank an independent cell (seed + rank), no
collective on the data path (weak scaling); max time over ranks.
"""
import argparse
import math
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOAD = "mg32_h0.5_rc6.5_q40"
SCF_WORKLOAD = "mg32_h0.5_rc6.5_q40"
WARM_START_MODEL = os.path.join(ROOT, "sqminiapp_gb300", "models", "warm_start_h0.5_rc6.5_q40.bin")
WARM_START_DISCRETISATION = {"h": 0.5, "rcut": 6.5, "n_qp": 40}
METRIC = "node-Lanczos/s"


def parse_args():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=10)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--config", default=WORKLOAD)
    p.add_argument("--cpu-seconds", type=float, default=12.0,
                   help="CPU time budget of the cpu_baseline sample")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--max-nodes", type=int, default=0,
                   help="process only the first N nodes per step (profiling of small cases)")
    p.add_argument("--list-format", type=int, choices=[0, 1, 2], default=0,
                   help="projector-list records of the main workload: 0 automatic, 1 full, "
                        "2 compact")
    p.add_argument("--scf-config", default=SCF_WORKLOAD,
                   help="cell of the time-to-SCF leg ('none' skips it)")
    p.add_argument("--scf-precisions", default="32,64",
                   help="engines timed by the time-to-SCF leg")
    p.add_argument("--scf-model", default=WARM_START_MODEL,
                   help="learned start for the FP32 engine ('none' skips it); used when the cell "
                        "has the discretisation the model was trained at")
    p.add_argument("--scf-learned", choices=["auto", "force"], default="auto",
                   help="force: run the learned start on a cell of another discretisation too")
    p.add_argument("--scf-fp64", choices=["full", "at-fp32-density"], default="full",
                   help="FP64 leg: a full SCF from the atomic start, or one FP64 SCF iteration "
                        "from the FP32 engine's converged density (free energy check for cells "
                        "whose FP64 SCF takes too long)")
    p.add_argument("--scf-mixing", type=float, default=0.5,
                   help="mixing parameter of every time-to-SCF leg (0: the deck's)")
    p.add_argument("--scf-kerker", type=float, default=2.0,
                   help="Kerker k_TF (1/bohr) of every time-to-SCF leg (0: the engine's 1.0)")
    p.add_argument("--batch", choices=["none", "uneven"], default="none",
                   help="uneven: time the three-cell mixed batch (one call per cell vs one "
                        "batched submission)")
    return p.parse_args()


def dist_env():
    return (int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)),
            int(os.environ.get("LOCAL_RANK", 0)))


def make_deck(config, rank):
    from sqminiapp_gb300.decks import CONFIGS, DEFAULT_SEED, make_fcc_mg_deck
    cfg = dict(CONFIGS[config])
    d = tempfile.mkdtemp(prefix="sqbench_r%d_" % rank)
    return make_fcc_mg_deck(d, "cell", seed=DEFAULT_SEED + rank, **cfg), cfg


class ClockSampler:
    """nvidia-smi samples every 200 ms while running (SM clock, limits, throttle reasons)."""
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.rows = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            parts = [s.strip() for s in line.split(",")]
            if len(parts) == 7:
                self.rows.append(parts)

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        sm, smax, reasons = [], [], set()
        for r in self.rows:
            try:
                sm.append(float(r[0]))
                smax.append(float(r[1]))
            except ValueError:
                continue
            for i, n in enumerate(names):
                if r[3 + i].lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def cpu_sample(deck_dir, name, seconds, faithful=False):
    """Time the FP64 oracle on strided node batches until `seconds` of wall time pass."""
    import oracle
    o = oracle.Oracle(deck_dir, name, faithful=faithful)
    threads = os.cpu_count() or 1
    rng = np.random.default_rng(1)
    order = rng.permutation(o.n_nodes)
    batch = threads * 2
    done, t0, pos = 0, time.perf_counter(), 0
    while True:
        nodes = order[pos:pos + batch]
        if len(nodes) == 0:
            break
        o.nodes_and_weights(nodes=nodes, nthreads=threads)
        done += len(nodes)
        pos += len(nodes)
        if time.perf_counter() - t0 > seconds:
            break
    dt = time.perf_counter() - t0
    o.close()
    return done / dt, threads, "%d of %d nodes (random order), %.1f s, %d threads" % (
        done, o.n_nodes, dt, threads)


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    (deck_dir, name, meta), cfg = make_deck(args.config, 0)
    per_step = max(2.0, min(15.0, 150.0 / max(1, args.steps + args.warmup)))
    for _ in range(args.warmup):
        cpu_sample(deck_dir, name, per_step / 4)
    vals, samples = [], []
    t0 = time.perf_counter()
    threads = os.cpu_count() or 1
    for _ in range(args.steps):
        v, threads, s = cpu_sample(deck_dir, name, per_step)
        vals.append(v)
        samples.append(s)
    wall = time.perf_counter() - t0
    value = float(statistics.mean(vals))
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": METRIC,
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": wall * 1e3 / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "fp64", "data": "synthetic (seeded FCC Mg cell)",
        "config": {"workload": args.config, "n_nodes": meta["N"] ** 3, "atoms": meta["natoms"],
                   "grid": [meta["N"]] * 3, "cube": [2 * math.ceil(cfg["rcut"] / meta["h"]) + 1] * 3,
                   "n_qp": cfg["n_qp"], "rcut": cfg["rcut"], "h": meta["h"], "operator": "corrected",
                   "precision": "fp64 (CPU restatement of the reference path)"},
        "cpu_baseline": {"value": value, "unit": METRIC, "cores": threads, "kind": "port",
                         "sample": samples[-1] + "; FP64 restatement of the reference path "
                         "(PETSc/MPI reference not buildable here)"},
        "e2e": {"value": value, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_ours(args):
    import torch
    import torch.distributed as dist
    from sqminiapp_gb300 import LSDFT
    from sqminiapp_gb300.capi import check, lib

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl")
    (deck_dir, name, meta), cfg = make_deck(args.config, rank)
    eng = LSDFT(deck_dir, name, faithful=False, precision=32, device=local,
                list_format=args.list_format)
    n, q = eng.n_nodes, eng.n_qp
    if args.max_nodes > 0:
        n = min(n, args.max_nodes)
    dev = torch.device("cuda", local)
    rng = np.random.default_rng(11 + rank)
    veff_host = (-0.2 + 0.05 * rng.standard_normal(eng.n_nodes)).astype(np.float64)
    veff = torch.from_numpy(veff_host).to(dev)
    lam = torch.empty((n, q), dtype=torch.float64, device=dev)
    wts = torch.empty((n, q), dtype=torch.float64, device=dev)
    lmin = torch.empty(n, dtype=torch.float64, device=dev)
    lmax = torch.empty(n, dtype=torch.float64, device=dev)
    rho = torch.empty(n, dtype=torch.float64, device=dev)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream(dev)
    sptr = stream.cuda_stream

    def step():
        eng.nodes_and_weights_device(veff.data_ptr(), 0.0, 0, n, lam.data_ptr(), wts.data_ptr(),
                                     lmin.data_ptr(), lmax.data_ptr(), sptr)
        return eng.fermi_density_energy_device(lam.data_ptr(), wts.data_ptr(), n, eng.n_electrons,
                                               1e-12, rho.data_ptr(), sptr)

    for _ in range(max(3, args.warmup)):
        step()
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    events = []
    lanczos_ms = []
    t_wall = time.perf_counter()
    for _ in range(args.steps):
        flush.zero_()
        s0 = torch.cuda.Event(enable_timing=True)
        s1 = torch.cuda.Event(enable_timing=True)
        s0.record(stream)
        res = step()
        s1.record(stream)
        events.append((s0, s1))
        lanczos_ms.append(eng.last_kernel_times()[0])
    torch.cuda.synchronize()
    t_wall = time.perf_counter() - t_wall
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    clk = clocks.stop()
    step_ms = [a.elapsed_time(b) for a, b in events]
    total_ms = float(sum(step_ms))
    t = torch.tensor([total_ms], dtype=torch.float64, device=dev)
    if world > 1:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    max_ms = float(t.item())
    value = world * n * args.steps / (max_ms / 1e3)

    # roofline of the dominant kernel
    flops = eng.algorithmic_flops_per_node() * n
    lz_ms = float(np.mean(lanczos_ms))
    achieved = flops / (lz_ms * 1e-3) / 1e12
    peak = np.zeros(1)
    check(lib().sq_measure_fp32_peak(local, peak.ctypes.data_as(
        __import__("ctypes").POINTER(__import__("ctypes").c_double))), "fp32 peak")
    traffic = None  # DRAM bytes per launch from the committed ncu summary, if it covers this workload
    tp = os.path.join(ROOT, "profiles", "lanczos_traffic.txt")
    if os.path.exists(tp):
        kv = dict(line.split(":", 1) for line in open(tp) if ":" in line and not line.startswith("#"))
        if kv.get("workload", "").strip() == args.config and args.max_nodes == 0:
            traffic = float(kv["bytes_per_launch"])

    # e2e through the host-buffer API
    e2e = None
    if not args.no_e2e:
        pin = lambda shape: torch.empty(shape, dtype=torch.float64, pin_memory=True).numpy()
        hv = pin(eng.n_nodes)
        hv[:] = veff_host
        out = {"lambda": pin((n, q)), "weights": pin((n, q)), "lambda_min": pin(n),
               "lambda_max": pin(n)}
        hrho = pin(n)
        eng.NodesAndWeights_LSSGQ(veff=hv, node_end=n, out=out)
        if world > 1:
            dist.barrier()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            eng.NodesAndWeights_LSSGQ(veff=hv, node_end=n, out=out)
            eng.CalculateDensity_lssgq(out["lambda"], out["weights"], rho=hrho)
        e2e_s = time.perf_counter() - t0
        te = torch.tensor([e2e_s], dtype=torch.float64, device=dev)
        if world > 1:
            dist.all_reduce(te, op=dist.ReduceOp.MAX)
        e2e_s = float(te.item())
        e2e = {"value": world * n * args.steps / e2e_s, "unit": METRIC,
               "h2d_bytes_per_step": int(n * 8 + 2 * n * q * 8),
               "d2h_bytes_per_step": int(2 * n * q * 8 + 2 * n * 8 + n * 8)}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        v, cores, sample = cpu_sample(deck_dir, name, args.cpu_seconds)
        cpu = {"value": v, "unit": METRIC, "cores": cores, "kind": "port",
               "sample": sample + "; FP64 restatement of the reference path"}

    scf = None
    if rank == 0 and world == 1 and args.scf_config != "none":
        scf = scf_leg(args, local)
    batch = None
    if rank == 0 and world == 1 and args.batch != "none":
        batch = batch_leg(args, local)

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": max_ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "fp32",
            "data": "synthetic (seeded FCC Mg cell per rank)",
            "config": {"workload": args.config, "n_nodes": n, "atoms": meta["natoms"],
                       "grid": list(eng.grid), "cube": list(eng.cube), "n_qp": q,
                       "rcut": cfg["rcut"], "h": meta["h"], "operator": "corrected",
                       "precision": "fp32 vectors, fp64 coefficients/quadrature/sums",
                       "step": "lanczos+quadrature of all nodes, fermi bisection, density, energy",
                       "l2": "flushed between steps (256 MiB write)",
                       "lambda_f": res["lambda_f"], "e_band": res["e_band"],
                       "kernel_layout": {"flags": eng.info.kernel_layout,
                                         "u_on_chip": bool(eng.info.kernel_u_on_chip),
                                         "threads": eng.info.kernel_threads,
                                         "smem_bytes": eng.info.kernel_smem_bytes}},
            "roofline": {"bound": "fp32", "achieved": achieved, "peak": float(peak[0]),
                         "unit": "TFLOP/s", "frac": achieved / float(peak[0]),
                         "traffic": traffic, "kernel": "lanczos_kernel<float>",
                         "kernel_ms": lz_ms, "flops_per_launch": flops,
                         "peak_kind": "measured FP32 FMA probe"},
            "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": 4 * args.steps,
            "clocks": clk, "wall_s": t_wall, "scf": scf,
        }
        if batch is not None:
            line["batch"] = batch
        print(json.dumps(line), flush=True)
    eng.close()
    if world > 1:
        dist.destroy_process_group()


BATCH_CELLS = {"uneven": ["uneven_a_mg4_h0.5_rc6_q30", "uneven_b_mg32_h0.45_rc7_q40",
                          "uneven_c_mg108_h0.5_rc6.5_q50"]}


def batch_leg(args, local, reps=3):
    """Several independent cells: one sq_nodes_and_weights_device call per cell in a row, and
    one sq_batch_nodes_and_weights submission (FP32, constant Veff -0.2 Ha; device wall clock
    over `reps` repetitions after one untimed run of each form)."""
    import torch
    from sqminiapp_gb300 import LSDFT, batch_nodes_and_weights
    dev = torch.device("cuda", local)
    cells, veffs, outs, names = [], [], [], BATCH_CELLS[args.batch]
    for i, cfg_name in enumerate(names):
        (d, n, _), _ = make_deck(cfg_name, i)
        e = LSDFT(d, n, faithful=False, precision=32, device=local)
        cells.append(e)
        veffs.append(torch.full((e.n_nodes,), -0.2, dtype=torch.float64, device=dev))
        outs.append({k: torch.empty(s, dtype=torch.float64, device=dev) for k, s in
                     (("lambda", (e.n_nodes, e.n_qp)), ("weights", (e.n_nodes, e.n_qp)),
                      ("lambda_min", (e.n_nodes,)), ("lambda_max", (e.n_nodes,)))})
    st = torch.cuda.current_stream(dev).cuda_stream

    def one(e, v, o):
        e.nodes_and_weights_device(v.data_ptr(), 0.0, 0, e.n_nodes, o["lambda"].data_ptr(),
                                   o["weights"].data_ptr(), o["lambda_min"].data_ptr(),
                                   o["lambda_max"].data_ptr(), st)

    def timed(fn):
        fn()
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        for _ in range(reps):
            fn()
        torch.cuda.synchronize(dev)
        return (time.perf_counter() - t0) / reps

    per = [timed(lambda e=e, v=v, o=o: one(e, v, o)) for e, v, o in zip(cells, veffs, outs)]
    seq = timed(lambda: [one(e, v, o) for e, v, o in zip(cells, veffs, outs)])
    bat = timed(lambda: batch_nodes_and_weights(
        cells, [v.data_ptr() for v in veffs], None,
        [{k: t.data_ptr() for k, t in o.items()} for o in outs], st))
    res = {"cells": [{"workload": nm, "nodes": e.n_nodes, "cube": list(e.cube), "n_qp": e.n_qp,
                      "seconds": t, "nodes_per_s": e.n_nodes / t,
                      "kernel_layout": e.info.kernel_layout}
                     for nm, e, t in zip(names, cells, per)],
           "one_call_per_cell_s": seq, "batched_s": bat}
    for e in cells:
        e.close()
    return res


def scf_leg(args, local):
    """Time-to-SCF-convergence of the FP32 and FP64 engines on one cell (host wall clock of
    sq_scf_run from the atomic-superposition start; engine setup timed apart)."""
    from sqminiapp_gb300 import LSDFT
    (deck_dir, name, meta), cfg = make_deck(args.scf_config, 0)
    out = {"workload": args.scf_config, "atoms": meta["natoms"], "start": "atomic superposition",
           "stop": "relative density residual < TOL_SCF (1e-6; 3e-5 floor for FP32 vectors)"}
    # the same mixing for every leg: the deck's history and Pulay period, this parameter and k_TF
    mixing = {"mixing_parameter": args.scf_mixing or None, "kerker_ktf": args.scf_kerker or None}
    out["mixing"] = {"parameter": args.scf_mixing or "deck", "kerker_ktf": args.scf_kerker or 1.0}
    precs = [int(p) for p in args.scf_precisions.split(",") if p]
    if args.scf_fp64 == "at-fp32-density":
        precs = [32] + [p for p in precs if p != 32]  # the FP32 density comes first
    rho32 = None
    for prec in precs:
        t0 = time.perf_counter()
        eng = LSDFT(deck_dir, name, faithful=False, precision=prec, device=local)
        eng.scf_begin()  # builds the pseudocharges / Poisson symbol once per geometry
        setup_s = time.perf_counter() - t0
        if prec == 64 and args.scf_fp64 == "at-fp32-density":
            # one FP64 iteration: the Harris-Foulkes free energy at the FP32 fixed point, equal
            # to the FP64 SCF's to second order in the density difference
            t0 = time.perf_counter()
            r = eng.SCF_LSSGQ(rho_init=rho32, maxit=1, raise_on_maxit=False, **mixing)
            wall = time.perf_counter() - t0
            out["fp64_at_fp32_density"] = {
                "seconds": wall, "setup_seconds": setup_s,
                "free_energy_per_atom": r["free_energy_per_atom"],
                "density_residual": r["residual"],
                "dF_per_atom_vs_fp32": abs(r["free_energy_per_atom"] -
                                           out["fp32"]["free_energy_per_atom"])}
            eng.close()
            continue
        t0 = time.perf_counter()
        r = eng.SCF_LSSGQ(raise_on_maxit=False, **mixing)
        wall = time.perf_counter() - t0
        out["fp%d" % prec] = {"seconds": wall, "setup_seconds": setup_s,
                              "iterations": r["iterations"], "converged": bool(r["converged"]),
                              "free_energy_per_atom": r["free_energy_per_atom"],
                              "residual": r["residual"], "tol": r["tol"],
                              "sq_seconds": r["sq_ms"] / 1e3}
        if prec == 32 and args.scf_fp64 == "at-fp32-density":
            rho32 = eng.scf_density()[0].copy()
        eng.close()
    model_ok = (args.scf_model != "none" and os.path.exists(args.scf_model) and
                (args.scf_learned == "force" or
                 all(cfg[k] == v for k, v in WARM_START_DISCRETISATION.items())))
    if model_ok and 32 in [int(p) for p in args.scf_precisions.split(",") if p]:
        from sqminiapp_gb300 import WarmStartMLP
        model = WarmStartMLP(device=local, path=args.scf_model)
        eng = LSDFT(deck_dir, name, faithful=False, precision=32, device=local)
        eng.scf_begin()
        t0 = time.perf_counter()
        r = eng.SCF_LSSGQ(raise_on_maxit=False, model=model, **mixing)  # descriptors + MLP inside
        wall = time.perf_counter() - t0
        out["fp32_learned"] = {"seconds": wall, "iterations": r["iterations"],
                               "converged": bool(r["converged"]),
                               "free_energy_per_atom": r["free_energy_per_atom"],
                               "residual": r["residual"], "tol": r["tol"],
                               "model": os.path.basename(args.scf_model)}
        eng.close()
        model.close()
        if "fp64" in out:
            out["speedup_fp32_learned_vs_fp64"] = out["fp64"]["seconds"] / wall
            out["dF_per_atom_fp32_learned_vs_fp64"] = abs(r["free_energy_per_atom"] -
                                                          out["fp64"]["free_energy_per_atom"])
    if "fp32" in out and "fp64" in out:
        out["speedup_fp32_vs_fp64"] = out["fp64"]["seconds"] / out["fp32"]["seconds"]
        out["dF_per_atom_fp32_vs_fp64"] = abs(out["fp32"]["free_energy_per_atom"] -
                                              out["fp64"]["free_energy_per_atom"])
    return out


def main():
    args = parse_args()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
