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
parity:  the GPU's quadrature of the nodes the cpu_baseline sample ran, against the oracle's
         (moments of order <= 3, occupations), printed beside the number.
scf:     time-to-SCF-convergence (the other half of the headline metric) on the 108-atom
         cell (51^3 nodes, 27^3 cubes, 40 steps): the FP64 engine and the FP32 engine from
         the atomic-superposition density, and the FP32 engine from the learned start
         (committed model).  Every engine is stopped by the same two criteria, read from its
         per-iteration record: relative density residual < 3e-5, and |dF| < 1e-5 Ha/atom
         between consecutive iterations; the FP64 run continues to its deck tolerance (1e-6)
         and is the reference of the FP32 runs' errors in free energy per atom, Fermi level
         and density.

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
SCF_WORKLOAD = "mg108_h0.5_rc6.5_q40"
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
    p.add_argument("--kernel", type=int, choices=[0, 1, 2], default=0,
                   help="FP32 Lanczos kernel: 0 automatic, 1 single-pass, 2 split-pass")
    p.add_argument("--tile", type=int, default=0,
                   help="split-pass kernel tile (z-/y-ranges per row); 0 autotuned")
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
    p.add_argument("--scf-learned-highpass", type=float, default=0.0,
                   help="learned start: keep the network's correction above this wave vector "
                        "(k^2/(k^2+k0^2), 1/bohr); 0 keeps all of it")
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


def cpu_sample(deck_dir, name, seconds, faithful=False, veff=None):
    """Time the FP64 oracle on strided node batches until `seconds` of wall time pass.
    Returns (nodes/s, threads, description, sampled nodes, oracle results of those nodes)."""
    import oracle
    o = oracle.Oracle(deck_dir, name, faithful=faithful)
    threads = os.cpu_count() or 1
    rng = np.random.default_rng(1)
    order = rng.permutation(o.n_nodes)
    batch = threads * 2
    done, t0, pos = 0, time.perf_counter(), 0
    parts = []
    while True:
        nodes = order[pos:pos + batch]
        if len(nodes) == 0:
            break
        parts.append((nodes, o.nodes_and_weights(nodes=nodes, nthreads=threads, veff=veff)))
        done += len(nodes)
        pos += len(nodes)
        if time.perf_counter() - t0 > seconds:
            break
    dt = time.perf_counter() - t0
    o.close()
    nodes = np.concatenate([p[0] for p in parts])
    res = {k: np.concatenate([p[1][k] for p in parts]) for k in ("lambda", "weights")}
    return done / dt, threads, "%d of %d nodes (random order), %.1f s, %d threads" % (
        done, o.n_nodes, dt, threads), nodes, res


def quadrature_parity(lam, w, ref_lam, ref_w, beta=30.0, mu=None):
    """Largest differences between two Gauss rules per node: moments sum w lambda^k (k <= 3,
    relative to max(1, |moment|)) and the occupation sum w f(lambda - mu) (f Fermi-Dirac at
    beta, mu the median node)."""
    if mu is None:
        mu = float(np.median(ref_lam))
    mom = 0.0
    for k in range(4):
        g = np.sum(w * lam ** k, axis=1)
        e = np.sum(ref_w * ref_lam ** k, axis=1)
        mom = max(mom, float(np.max(np.abs(g - e) / np.maximum(1.0, np.abs(e)))))
    f = lambda L: 1.0 / (1.0 + np.exp(np.clip(beta * (L - mu), -700, 700)))
    occ = float(np.max(np.abs(np.sum(w * f(lam), axis=1) - np.sum(ref_w * f(ref_lam), axis=1))))
    return mom, occ


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
        v, threads, s, _, _ = cpu_sample(deck_dir, name, per_step)
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
                list_format=args.list_format, kernel=args.kernel, tile=args.tile)
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
    sms = torch.cuda.get_device_properties(dev).multi_processor_count
    peak_theory = (sms * 128 * 2 * clk["sm_mhz"] * 1e6 / 1e12) if clk.get("sm_mhz") else None
    traffic = None  # DRAM bytes per launch from the committed ncu summary, if it covers this workload
    tp = os.path.join(ROOT, "profiles", "lanczos_traffic.txt")
    if os.path.exists(tp):
        kv = dict(line.split(":", 1) for line in open(tp) if ":" in line and not line.startswith("#"))
        same_kernel = kv.get("kernel", "lanczos_kernel<float>").strip() == (
            "lanczos_quad_kernel" if eng.info.kernel_layout & 16 else "lanczos_kernel<float>")
        if kv.get("workload", "").strip() == args.config and args.max_nodes == 0 and same_kernel:
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
    parity = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        # the quadrature of the last timed step, checked against the oracle on the nodes the
        # CPU baseline sample runs (same Veff)
        lam_h = lam.cpu().numpy()
        w_h = wts.cpu().numpy()
        v, cores, sample, nodes, ref = cpu_sample(deck_dir, name, args.cpu_seconds,
                                                  veff=veff_host)
        cpu = {"value": v, "unit": METRIC, "cores": cores, "kind": "port",
               "sample": sample + "; FP64 restatement of the reference path"}
        keep = nodes < n
        if np.any(keep):
            mom, occ = quadrature_parity(lam_h[nodes[keep]], w_h[nodes[keep]],
                                         ref["lambda"][keep], ref["weights"][keep])
            parity = {"n_nodes": int(np.count_nonzero(keep)), "max_moment_err": mom,
                      "max_occ_err": occ, "against": "FP64 CPU oracle",
                      "tolerance": {"moment": 1e-4, "occ": 3e-4},
                      "pass": bool(mom < 1e-4 and occ < 3e-4)}

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
                         "traffic": traffic,
                         "kernel": ("lanczos_quad_kernel" if eng.info.kernel_layout & 16
                                    else "lanczos_kernel<float>"),
                         "kernel_ms": lz_ms, "flops_per_launch": flops,
                         "peak_kind": "measured FP32 FMA probe",
                         "peak_theoretical": peak_theory,
                         "frac_theoretical": (achieved / peak_theory) if peak_theory else None,
                         "peak_theoretical_kind": "SMs x 128 FP32 lanes x 2 FLOP x median "
                                                  "sampled SM clock"},
            "cpu_baseline": cpu, "parity": parity, "e2e": e2e, "gpu_launches": 4 * args.steps,
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


RES_STOP = 3e-5   # relative density residual, the FP32 engine's floor-safe tolerance
DF_STOP = 1e-5    # |F_k - F_(k-1)| per atom (Ha), the free-energy accuracy target


def _scf_trace(eng, mixing, tol, model=None, maxit=100, highpass=0.0):
    """One SCF from the atomic superposition (or the learned start), stepped by hand so every
    iteration's host wall time, free energy per atom, residual and Fermi level are recorded.
    The clock starts before the start density is formed (the learned start's descriptors
    and network inference count); the geometry's fixed fields are built before, untimed."""
    eng.scf_begin(tol=tol, **mixing)  # pseudocharges / Poisson symbol of this geometry
    t0 = time.perf_counter()
    if model is not None:
        opt = eng._scf_options(tol, None, mixing.get("mixing_parameter"), None, None, None,
                               mixing.get("kerker_ktf"), learned_highpass=highpass)
        import ctypes
        from sqminiapp_gb300.capi import check
        check(eng._lib.sq_scf_begin_learned(eng._h, ctypes.byref(opt), model._m),
              "sq_scf_begin_learned")
    else:
        eng.scf_begin(tol=tol, **mixing)
    rows = []
    r = {}
    for _ in range(maxit):
        r = eng.scf_step()
        rows.append((time.perf_counter() - t0, r["free_energy_per_atom"], r["residual"],
                     r["lambda_f"], r["sq_ms"] / 1e3))
        if r["converged"]:
            break
    t = np.array([x[0] for x in rows])
    F = np.array([x[1] for x in rows])
    res = np.array([x[2] for x in rows])

    def first(mask):
        i = int(np.argmax(mask)) if np.any(mask) else -1
        return None if i < 0 else {"iterations": i + 1, "seconds": float(t[i]),
                                   "free_energy_per_atom": float(F[i])}

    dF = np.abs(np.diff(F, prepend=np.nan))
    out = {"iterations": len(rows), "converged": bool(r.get("converged")),
           "seconds": float(t[-1]), "free_energy_per_atom": float(F[-1]),
           "residual": float(res[-1]), "tol": r.get("tol"), "lambda_f": float(rows[-1][3]),
           "sq_seconds": float(rows[-1][4]),
           "stop_residual_3e-5": first(res < RES_STOP),
           "stop_dF_1e-5": first(dF < DF_STOP)}
    return out


def scf_leg(args, local):
    """Time-to-SCF-convergence of the FP64 engine, the FP32 engine and the FP32 engine with
    the learned start on one cell, every engine stopped by the same criteria (host wall clock;
    engine setup timed apart)."""
    from sqminiapp_gb300 import LSDFT
    (deck_dir, name, meta), cfg = make_deck(args.scf_config, 0)
    out = {"workload": args.scf_config, "atoms": meta["natoms"], "start": "atomic superposition",
           "stop": {"residual": "relative density residual < %g (every engine)" % RES_STOP,
                    "dF": "|F_k - F_(k-1)| < %g Ha/atom (every engine)" % DF_STOP,
                    "run": "FP64 continues to TOL_SCF (1e-6) and is the error reference; FP32 "
                           "stops at 3e-5, the floor of FP32 Lanczos vectors"}}
    # the same mixing for every leg: the deck's history and Pulay period, this parameter and k_TF
    mixing = {"mixing_parameter": args.scf_mixing or None, "kerker_ktf": args.scf_kerker or None}
    out["mixing"] = {"parameter": args.scf_mixing or "deck", "kerker_ktf": args.scf_kerker or 1.0}
    precs = [int(p) for p in args.scf_precisions.split(",") if p]
    if args.scf_fp64 == "at-fp32-density":
        precs = [32] + [p for p in precs if p != 32]  # the FP32 density comes first
    rho = {}
    for prec in precs:
        t0 = time.perf_counter()
        eng = LSDFT(deck_dir, name, faithful=False, precision=prec, device=local)
        setup_s = time.perf_counter() - t0
        if prec == 64 and args.scf_fp64 == "at-fp32-density":
            # one FP64 iteration: the Harris-Foulkes free energy at the FP32 fixed point, equal
            # to the FP64 SCF's to second order in the density difference
            eng.scf_begin()
            t0 = time.perf_counter()
            r = eng.SCF_LSSGQ(rho_init=rho[32], maxit=1, raise_on_maxit=False, **mixing)
            wall = time.perf_counter() - t0
            out["fp64_at_fp32_density"] = {
                "seconds": wall, "setup_seconds": setup_s,
                "free_energy_per_atom": r["free_energy_per_atom"],
                "density_residual": r["residual"],
                "dF_per_atom_vs_fp32": abs(r["free_energy_per_atom"] -
                                           out["fp32"]["free_energy_per_atom"])}
            eng.close()
            continue
        tr = _scf_trace(eng, mixing, None)
        tr["setup_seconds"] = setup_s
        out["fp%d" % prec] = tr
        rho[prec] = eng.scf_density()[0].copy()
        eng.close()
    model_ok = (args.scf_model != "none" and os.path.exists(args.scf_model) and
                (args.scf_learned == "force" or
                 all(cfg[k] == v for k, v in WARM_START_DISCRETISATION.items())))
    if model_ok and 32 in precs:
        from sqminiapp_gb300 import WarmStartMLP
        model = WarmStartMLP(device=local, path=args.scf_model)
        eng = LSDFT(deck_dir, name, faithful=False, precision=32, device=local)
        tr = _scf_trace(eng, mixing, None, model=model, highpass=args.scf_learned_highpass)
        tr["model"] = os.path.basename(args.scf_model)
        tr["learned_highpass_k0"] = args.scf_learned_highpass
        out["fp32_learned"] = tr
        rho["32L"] = eng.scf_density()[0].copy()
        eng.close()
        model.close()

    def ratio(a, b, key):
        ta, tb = (out.get(a) or {}).get(key), (out.get(b) or {}).get(key)
        return (ta["seconds"] / tb["seconds"]) if ta and tb else None

    if "fp64" in out:
        ref = out["fp64"]
        for leg, rk in (("fp32", 32), ("fp32_learned", "32L")):
            if leg not in out:
                continue
            o = out[leg]
            o["speedup_vs_fp64"] = {
                "residual_3e-5": ratio("fp64", leg, "stop_residual_3e-5"),
                "dF_1e-5": ratio("fp64", leg, "stop_dF_1e-5"),
                "own_tolerances": ref["seconds"] / o["seconds"]}
            # precision errors against the FP64 engine converged to 1e-6
            d = rho[rk] - rho[64]
            o["errors_vs_fp64"] = {
                "free_energy_per_atom": abs(o["free_energy_per_atom"] - ref["free_energy_per_atom"]),
                "lambda_f": abs(o["lambda_f"] - ref["lambda_f"]),
                "rho_rel_l2": float(np.linalg.norm(d) / np.linalg.norm(rho[64])),
                "rho_max_abs": float(np.max(np.abs(d)))}
        # the headline fields of the earlier line format
        if "fp32" in out:
            out["speedup_fp32_vs_fp64"] = out["fp32"]["speedup_vs_fp64"]["residual_3e-5"]
            out["dF_per_atom_fp32_vs_fp64"] = out["fp32"]["errors_vs_fp64"]["free_energy_per_atom"]
        if "fp32_learned" in out:
            out["speedup_fp32_learned_vs_fp64"] = out["fp32_learned"]["speedup_vs_fp64"]["residual_3e-5"]
            out["dF_per_atom_fp32_learned_vs_fp64"] = \
                out["fp32_learned"]["errors_vs_fp64"]["free_energy_per_atom"]
    return out


def main():
    args = parse_args()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
