"""Benchmark: GB energy + force evaluations per second on seeded synthetic
globules (default: GBSW, 50,000 atoms, 32-point Gauss-Legendre x 110-point
Lebedev quadrature, full N^2 pair term).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--workload NAME] [--impl gb300|reference]

A step is one energy + force evaluation of the whole molecule.
* value: evaluations/s with positions resident in HBM (gbx_execute on device
  buffers), timed with CUDA events on the library's execute stream, L2
  flushed (256 MiB write) between timed steps, max over ranks.
* e2e: the same metric through the host-buffer call (gbx_execute_host):
  positions copied host->device and forces/energy device->host every step.
* roofline: the dominant stage, from events the library records around each
  stage on its own stream, against the FP32 pipe (the path has no dense
  contraction; its table gathers and point records stay far below the HBM rate).
* cpu_baseline: the FP64 oracle (a restatement of the reference CPU
  algorithm) on the machine's host cores for the same workload.

Multi-GPU: replicas (the path does not shard on one node here); each rank
evaluates its own copy and value is the sum over ranks.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

from openmmcustomgbintegralforce_gb300.globule import batch_sizes, make_batch, make_globule  # noqa: E402
from openmmcustomgbintegralforce_gb300.spec import GBModel, box_for  # noqa: E402

METRIC = "GB energy+force evals/s at 50k atoms; batched confs/s vs plain; err vs FP64"
UNIT = "evals/s"

# Algorithmic FP32 work per unit, counted op by op from the reference formulas
# (FMA = 2 flops; sqrt / exp / reciprocal counted separately as SFU ops).
# GBSW volume evaluation (CharmmReferenceGBSW.cpp:616-639): delta 3, r^2 5,
# shell bounds 2 -> 10 flops + 1 sqrt; inside the switching shell dr 1,
# dr^2 dr^3 2, cubic 4, product 1 -> +8 flops.
FLOPS_GBSW_EVAL = 10.0
FLOPS_GBSW_SHELL = 8.0
# per quadrature point: point = x + v 3, cell index 6, two weighted sums 4
FLOPS_POINT = 13.0
# GBSW chain rule per listed atom (reduceIntegralForce.cu:45-65 with
# computeGBSWForce.cu:10-25): delta 3, r^2 5, shell bounds 2 -> 10 flops +
# 1 sqrt; inside the shell u 7, du/dr 2, dI/dr 3, factor 1, times delta 3,
# force on i and on the listed atom 6 -> +22 flops; per point as above.
FLOPS_CHAIN_EVAL = 10.0
FLOPS_CHAIN_SHELL = 22.0
# GBMV-I per listed atom (GBMVIntegralTypeI.cpp:158-170): delta 3, r^2 5, r^4 1,
# gamma r^4 1, sum 1 -> 11 flops + exp; chain (:196-222): delta 3, r^2 5,
# r^4 and r^2 terms 2, exp arg 1, factor 4, times delta 3, force on i and on the
# listed atom 6 -> 24 flops + exp.
FLOPS_GBMV1_EVAL = 11.0
FLOPS_GBMV1_CHAIN = 24.0
# GBMV-II per listed atom (GBMVIntegralTypeII.cpp:163-191): delta 3, r^2 5,
# T 2, F = (C/T)^2 1, s1 1, r^2 F^2 3, F delta 6 -> 21 flops + div; chain
# (:221-282): delta 3, r^2 5, T 2, F 1, dF 3, v.delta 5, factor 9, gradient
# 12, force on i and on the listed atom 6 -> 46 flops + 2 div.
FLOPS_GBMV2_EVAL = 21.0
FLOPS_GBMV2_CHAIN = 46.0
# per point beyond FLOPS_POINT: GBMV-I logistic 4 + exp; GBMV-II S 7 +
# logistic 4 + exp; chain factor per point 5
FLOPS_GBMV_POINT = {1: 4.0, 2: 11.0}
FLOPS_GBMV_CHAIN_POINT = 5.0
# unique pair (CharmmReferenceGBSW.cpp:248-282): delta+r^2 8, D 3, exp arg 1,
# f^2 2, 1/f^3 2, energy 3, dG/dr 4 + force 6, dG/dB 2x5 -> 39 flops + exp, rsqrt
FLOPS_PAIR = 39.0


# DRAM bytes (read + write) per step of each stage's kernels, from one ncu
# capture of the same workload and build (the files named in TRAFFIC_SOURCE).
TRAFFIC = {"gbsw50k": {"integrals": 1689.1e6 + 715.5e6, "pair": 3.0e6 + 3.0e6, "chain_rule": 1107.7e6,
                       "lookup_table": 180.0e6 + 146.6e6 + 5.5e6 + 9.6e6},
           "gbmv10k": {"integrals": 404.7e6 + 48.0e6, "chain_rule": 291.8e6, "point_binning": 93.0e6 + 153.1e6,
                       "pair": 0.63e6 + 0.63e6},
           "gbmv1_10k": {"integrals": 211.0e6 + 48.0e6, "chain_rule": 127.1e6, "point_binning": 89.7e6 + 151.1e6,
                         "pair": 0.63e6 + 0.62e6}}
TRAFFIC_SOURCE = {"gbsw50k": "profiles/launches_gbsw50k.md", "gbmv10k": "profiles/launches_gbmv10k.md",
                  "gbmv1_10k": "profiles/launches_gbmv1_10k.md"}


def workloads():
    return {
        "gbsw50k": dict(n=50000, seed=2026, model=GBModel.charmm_gbsw(n_radial=32, lebedev=110),
                        desc="GBSW 50,000-atom globule, 32x110 quadrature, full N^2 pair term"),
        "gbsw50k_cutoff": dict(n=50000, seed=2026, model=GBModel.charmm_gbsw(n_radial=32, lebedev=110, cutoff=2.0),
                               desc="GBSW 50,000-atom globule, 32x110 quadrature, 2.0 nm pair cutoff"),
        "gbsw10k": dict(n=10000, seed=2028, model=GBModel.charmm_gbsw(n_radial=32, lebedev=110),
                        desc="GBSW 10,000-atom globule, 32x110 quadrature (profiling case)"),
        "gbsw10k_cutoff": dict(n=10000, seed=2028, model=GBModel.charmm_gbsw(n_radial=32, lebedev=110, cutoff=1.5),
                               desc="GBSW 10,000-atom globule, 32x110 quadrature, 1.5 nm pair cutoff (profiling case)"),
        "gbsw10k_periodic": dict(n=10000, seed=2028, model=None, periodic_cutoff=1.5,
                                 desc="GBSW 10,000-atom globule in a box 0.5 nm wider than it on every side, "
                                      "32x110 quadrature, CutoffPeriodic 1.5 nm (profiling case)"),
        "gbmv10k": dict(n=10000, seed=2027, model=None, gbmv=2,
                        desc="GBMV-II 10,000-atom globule, 24x50 quadrature"),
        "gbmv1_10k": dict(n=10000, seed=2027, model=None, gbmv=1,
                          desc="GBMV-I 10,000-atom globule, 24x50 quadrature"),
        "gbsw5k_adjoint": dict(n=5000, seed=2029, model=GBModel.charmm_gbsw(), adjoint=True,
                               desc="GBSW 5,000-atom globule, 24x38 quadrature, adjoint (dE/dx, dE/dq, dE/dR, "
                                    "dE/dalpha)"),
        "gbsw1k": dict(n=1000, seed=7, model=GBModel.charmm_gbsw(),
                       desc="GBSW 1,000-atom globule, 24x38 quadrature (reference CPU case)"),
    }


def workload_config(name, w, model, world, jitter_A):
    """The `config` of both arms' JSON lines: the same keys and values."""
    return {"workload": name, "desc": w["desc"], "atoms": w["n"], "quadrature_points": model.n_quad,
            "l2": "flushed (256 MiB write) between steps", "parallelism": "replicas" if world > 1 else "single",
            "jitter_A": jitter_A}


def model_for(w, g):
    if w.get("model") is not None:
        return w["model"]
    if w.get("periodic_cutoff"):
        return GBModel.charmm_gbsw(n_radial=32, lebedev=110, cutoff=w["periodic_cutoff"], periodic=True,
                                   box=box_for(g.positions, margin=0.5))
    box = box_for(g.positions, margin=1.0)
    if w["gbmv"] == 1:
        return GBModel.gbmv1(box=box, lebedev=50)
    return GBModel.gbmv2(box=box, lebedev=50)


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for k, name in enumerate(names):
                if parts[5 + k].lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    path = os.path.join(REPO, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            return json.load(f), "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "sm_max_mhz": 2070.0}, "fallback"


def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl" if args.impl == "gb300" else "gloo")
    return world, rank, local


def replica_value(world: int, ms_max: float) -> float:
    """Whole-job evals/s of `world` independent replicas (weak scaling): every
    rank evaluates one conformation per step, the slowest rank sets the pace."""
    return world * 1000.0 / ms_max


def barrier(world):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


def allmax(world, v):
    if world <= 1:
        return v
    import torch
    import torch.distributed as dist

    t = torch.tensor([v], dtype=torch.float64, device="cuda" if dist.get_backend() == "nccl" else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def oracle_baseline(model, g, sample_s: float = 20.0):
    """Time the FP64 oracle (restated reference algorithm) on host cores."""
    from oracle import oracle as O

    cores = os.cpu_count() or 1
    t0 = time.perf_counter()
    out = O.Oracle(model, nthreads=cores).energy_forces(g.positions, g.charge, g.radius)
    dt = time.perf_counter() - t0
    return out, dt, cores


def run_reference(args, world, rank):
    """Reference arm: the FP64 oracle port of the reference CPU algorithm on
    all host cores, one whole energy + force evaluation per step (the
    reference's own classes need the reference tree, absent on the GPU host,
    and O(N^2) memory: 60 GB at 50k atoms)."""
    if rank != 0:
        return
    from oracle import oracle as O

    w = workloads()[args.workload]
    g = make_globule(w["n"], seed=w["seed"])
    model = model_for(w, g)
    cores = os.cpu_count() or 1
    orc = O.Oracle(model, nthreads=cores)
    times = []
    wall0 = time.perf_counter()
    for k in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        orc.energy_forces(g.positions, g.charge, g.radius)
        dt = time.perf_counter() - t0
        if k >= args.warmup:
            times.append(dt)
    wall = time.perf_counter() - wall0
    ms = 1000.0 * float(np.mean(times))
    v = 1000.0 / ms
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic seeded globule (no dataset)",
            "config": workload_config(args.workload, w, model, world, args.jitter),
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": f"one whole FP64 evaluation per step ({w['n']} atoms, {model.n_quad} points, "
                                       f"OpenMP on {cores} host cores)"},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "wall_s": wall}
    print(json.dumps(line))


BATCH_MOLECULES = 256
BATCH_SEED = 4242


def batch_models(gs):
    """128 GBSW + 128 GBMV-II molecules, 24 x 50 quadrature (alternating)."""
    out = []
    for k, g in enumerate(gs):
        if k % 2 == 0:
            out.append(GBModel.charmm_gbsw(n_radial=24, lebedev=50))
        else:
            out.append(GBModel.gbmv2(box=box_for(g.positions, margin=1.5), n_radial=24, lebedev=50))
    return out


def measure_batched(gs, steps: int):
    """Conformations/s of the batched form (one CUDA graph per call) against
    looping the plain single-molecule path over the same molecules, both with
    device-resident inputs and through host arrays, plus the error of a
    sample against the FP64 oracle."""
    import torch

    from openmmcustomgbintegralforce_gb300._lib import EXEC_ENERGY, EXEC_FORCES, Batch

    models = batch_models(gs)
    sizes = [g.n for g in gs]
    b = Batch(models, sizes)
    for c, g in zip(b.molecules, gs):
        c.set_particle_parameters(g.charge, g.radius)
    X = np.concatenate([g.positions for g in gs])
    E, F = b.execute_host(X)  # checked: sizes every buffer, uploads the positions
    stream = torch.cuda.Stream()
    sptr = stream.cuda_stream
    p, f, e = b.buffers()

    def plain_loop():  # one gbx_execute per molecule on one stream, inputs resident
        for m, c in enumerate(b.molecules):
            c.execute_device(p + 16 * b.offsets[m], f + 24 * b.offsets[m], c.n, e + 8 * m,
                             EXEC_FORCES | EXEC_ENERGY, sptr)

    def timed(fn, k):
        t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        t0.record(stream)
        for _ in range(k):
            fn()
        t1.record(stream)
        torch.cuda.synchronize()
        return t0.elapsed_time(t1) / k

    def host_timed(fn, k):
        t0 = time.perf_counter()
        for _ in range(k):
            fn()
        return 1000.0 * (time.perf_counter() - t0) / k

    def plain_host_loop():  # one host-array call per conformation, as a caller of the plain API
        for c, g in zip(b.molecules, gs):
            c.execute_host(g.positions)

    for _ in range(2):
        plain_loop()
    plain_ms = timed(plain_loop, steps)
    plain_host_loop()
    plain_host_ms = host_timed(plain_host_loop, max(2, steps // 3))
    tune = b.tune()
    b.execute_host(X)  # restores the positions; the tuned graph is captured on the next call
    for _ in range(2):
        b.execute_device(0, sptr)
    batch_ms = timed(lambda: b.execute_device(0, sptr), steps)
    batch_host_ms = host_timed(lambda: b.execute_host(X), max(2, steps // 3))
    E, F = b.execute_host(X)

    # every molecule against its own single-molecule call (the same kernels:
    # identical bits), and a stride-8 sample of them against the FP64 oracle
    mism = 0
    for k, (c, g) in enumerate(zip(b.molecules, gs)):
        Ek, Fk = c.execute_host(g.positions)
        o = b.offsets[k]
        mism += int(not (Ek == E[k] and np.array_equal(Fk, F[o:o + sizes[k]])))
    from oracle import oracle as O

    sample = [k + (k // 8) % 2 for k in range(0, len(gs), 8)]  # every 8th, GBSW and GBMV-II alternating
    errs = []
    for k in sample:
        r = O.Oracle(models[k], nthreads=os.cpu_count() or 1).energy_forces(gs[k].positions, gs[k].charge,
                                                                            gs[k].radius)
        Fk = F[b.offsets[k]:b.offsets[k] + sizes[k]]
        errs.append((abs(E[k] / r["energy"] - 1.0),
                     float(np.sqrt(((Fk - r["forces"]) ** 2).sum() / (r["forces"] ** 2).sum()))))

    # the batched differentiable form: every molecule's energy, dE/dx, dE/dq,
    # dE/dR and dE/dalpha per call, against a loop of gbx_adjoint per molecule
    dev = torch.device("cuda", torch.cuda.current_device())
    M, T = len(gs), b.total
    adj = {k: torch.zeros(n_, dtype=torch.float64, device=dev)
           for k, n_ in (("E", M), ("F", 3 * T), ("q", T), ("R", T), ("a", 2 * M))}

    def batch_adjoint():
        b.adjoint_device(adj["E"].data_ptr(), adj["F"].data_ptr(), adj["q"].data_ptr(), adj["R"].data_ptr(),
                         adj["a"].data_ptr(), 0, sptr)

    def plain_adjoint():
        for m, c in enumerate(b.molecules):
            o = b.offsets[m]
            c.adjoint_device(p + 16 * o, adj["E"].data_ptr() + 8 * m, adj["F"].data_ptr() + 24 * o,
                             adj["q"].data_ptr() + 8 * o, adj["R"].data_ptr() + 8 * o,
                             adj["a"].data_ptr() + 16 * m, 0, sptr)

    batch_adjoint()
    plain_adjoint()
    plain_adj_ms = timed(plain_adjoint, max(2, steps // 3))
    batch_adj_ms = timed(batch_adjoint, max(2, steps // 3))
    A = b.adjoint_host(X)
    adj_err = []
    for k in (0, 1):
        r = O.Oracle(models[k], nthreads=os.cpu_count() or 1).energy_forces(gs[k].positions, gs[k].charge,
                                                                            gs[k].radius, adjoint=True)
        o, n_ = b.offsets[k], sizes[k]
        adj_err.append({"molecule": k, "energy_rel": abs(A["energies"][k] / r["energy"] - 1.0),
                        "force_rel_rms": rel_rms(A["forces"][o:o + n_], r["forces"]),
                        "dEdq_rel_rms": rel_rms(A["dEdq"][o:o + n_], r["dEdq"]),
                        "dEdR_rel_rms": rel_rms(A["dEdR"][o:o + n_], r["dEdR"]),
                        "dEdalpha_rel_max": float(np.abs(A["dEdalpha"][k] / r["dEdalpha"] - 1).max())})
    b.close()
    n = len(gs)
    return {"workload": f"{n} globules, atoms log-uniform in [500, 8000] (total {sum(sizes)}), "
                        f"{(n + 1) // 2} GBSW + {n // 2} GBMV-II, 24x50 quadrature, full N^2",
            "confs_per_s": n * 1000.0 / batch_ms, "ms_per_batch": batch_ms,
            "plain_confs_per_s": n * 1000.0 / plain_ms, "plain_ms_per_loop": plain_ms,
            "speedup_vs_plain": plain_ms / batch_ms, "tune": tune,
            "plain": "one gbx_execute per molecule on one stream (inputs resident, no per-call sync)",
            "host": {"confs_per_s": n * 1000.0 / batch_host_ms, "plain_confs_per_s": n * 1000.0 / plain_host_ms,
                     "speedup_vs_plain": plain_host_ms / batch_host_ms,
                     "plain": "gbx_execute_host per molecule (host positions in, forces and energy out)",
                     "batched": "gbx_batch_execute_host (all positions in, all forces and energies out)"},
            "adjoint": {"confs_per_s": n * 1000.0 / batch_adj_ms, "plain_confs_per_s": n * 1000.0 / plain_adj_ms,
                        "speedup_vs_plain": plain_adj_ms / batch_adj_ms,
                        "batched": "gbx_batch_adjoint (device outputs: energies, forces, dE/dq, dE/dR, dE/dalpha)",
                        "plain": "gbx_adjoint per molecule on one stream", "err_vs_fp64": adj_err},
            "molecules_differing_from_single_calls": mism,
            "err_vs_fp64_sample": {"molecules": sample, "energy_rel_max": max(a for a, _ in errs),
                                   "force_rel_rms_max": max(b_ for _, b_ in errs)}}


# The other BASELINE configurations, measured in the same run as extra keys of
# the line: (workload, timed steps, jitter in A between steps, check vs FP64).
CONFIG_RUNS = {
    "c0_gbsw1k": ("gbsw1k", 50, 0.0),
    "c1_gbmv2_10k_1000_jittered": ("gbmv10k", 1000, 0.01),
    "c1_gbmv1_10k_1000_jittered": ("gbmv1_10k", 1000, 0.01),
    "c2_gbsw50k_cutoff2nm": ("gbsw50k_cutoff", 20, 0.0),
    "c3_gbsw5k_adjoint": ("gbsw5k_adjoint", 20, 0.0),
}


def rel_rms(a, b):
    return float(np.sqrt(((a - b) ** 2).sum() / (b ** 2).sum()))


def stage_roofline(ctx, model, g, n, step, flush, sptr, posq, force, stride, energy, sms, peaks, peak_src):
    """Stage times (CUDA events the library records on its own stream, median
    of 5 calls with L2 flushed before each), each stage's rate in TFLOP/s of
    the reference algorithm's work on this input, and the dominant stage's
    fraction of the FP32 peak."""
    import torch

    from openmmcustomgbintegralforce_gb300._lib import EXEC_CHECK, EXEC_COUNT_WORK, EXEC_ENERGY, EXEC_FORCES, Context

    ctx.set_timing(True)
    stages = []
    for k in range(5):
        flush.fill_(1.0)
        step(EXEC_FORCES | EXEC_ENERGY)
        torch.cuda.synchronize()
        stages.append(ctx.stage_times())
    ctx.set_timing(False)
    stage_ms = {k: float(np.median([s[k] for s in stages])) for k in stages[0]}

    # executed work, and the reference algorithm's work on the same input:
    # its own table, ascending lists, stop at the first burying atom (counted
    # on the device by a reference-table context, outside the timed region)
    step(EXEC_FORCES | EXEC_ENERGY | EXEC_CHECK | EXEC_COUNT_WORK)
    torch.cuda.synchronize()
    executed = ctx.work()
    if model.table_mode == 0 and not model.reference_table:
        rctx = Context(model.replace(reference_table=True), n)
        rctx.set_particle_parameters(g.charge, g.radius)
        rctx.execute_device(posq.data_ptr(), force.data_ptr(), stride, energy.data_ptr(),
                            EXEC_FORCES | EXEC_ENERGY | EXEC_CHECK | EXEC_COUNT_WORK, sptr)
        torch.cuda.synchronize()
        work = rctx.work()
        rctx.close()
    else:
        work = executed

    fp32_peak = sms * 128 * 2 * (peaks.get("sm_max_mhz", 2070.0) * 1e6) / 1e12
    points = float(n) * model.n_quad
    if model.model == 0:
        integral_flops = FLOPS_GBSW_EVAL * work["volume_evals"] + FLOPS_GBSW_SHELL * work["shell_evals"] + \
            FLOPS_POINT * points
        chain_flops = FLOPS_CHAIN_EVAL * work["chain_list_evals"] + FLOPS_CHAIN_SHELL * work["chain_derivative_evals"] + \
            FLOPS_POINT * points
    else:
        ev, ch = (FLOPS_GBMV1_EVAL, FLOPS_GBMV1_CHAIN) if model.model == 1 else (FLOPS_GBMV2_EVAL, FLOPS_GBMV2_CHAIN)
        integral_flops = ev * work["volume_evals"] + (FLOPS_POINT + FLOPS_GBMV_POINT[model.model]) * points
        chain_flops = ch * work["chain_list_evals"] + (FLOPS_POINT + FLOPS_GBMV_CHAIN_POINT) * points
    pair_flops = FLOPS_PAIR * n * (n - 1) / 2.0
    cand = {"integrals": integral_flops / (stage_ms["integrals"] * 1e-3) / 1e12,
            "pair": pair_flops / (stage_ms["pair"] * 1e-3) / 1e12,
            "chain_rule": chain_flops / (stage_ms["chain_rule"] * 1e-3) / 1e12}
    dominant = max(("integrals", "pair", "chain_rule", "lookup_table", "point_binning"), key=lambda k: stage_ms[k])
    achieved = cand.get(dominant)
    return {"bound": "fp32", "kernel": dominant, "achieved": achieved, "peak": fp32_peak, "unit": "TFLOP/s",
            "frac": (achieved / fp32_peak) if achieved else None,
            "peak_source": f"nominal FP32 ({sms} SM x 128 lanes x 2 flop x max SM clock); "
                           f"MEASURED_PEAKS.json ({peak_src}) has no FP32 figure",
            "per_stage_tflops": cand, "per_stage_frac": {k: v / fp32_peak for k, v in cand.items()},
            "stage_ms": stage_ms,
            "work": {"volume_evals": work["volume_evals"], "shell_evals": work["shell_evals"],
                     "points": points, "pairs": n * (n - 1) / 2.0,
                     "chain_list_evals": work["chain_list_evals"],
                     "chain_derivative_evals": work["chain_derivative_evals"],
                     "executed_volume_evals": executed["volume_evals"],
                     "executed_shell_evals": executed["shell_evals"],
                     "note": "volume_evals/shell_evals: the reference algorithm's list work on this input "
                             "(its table, ascending lists, first-burying-atom exit); executed_*: this run's"}}


def measure_config(name, steps, jitter_A, dev, flush):
    """One configuration end to end on device-resident inputs: evals/s from
    CUDA events around each call (L2 flushed between calls; with jitter the
    positions take a fresh N(0, jitter) step before every call, accumulating
    as in MD), e2e through host arrays, and the error of the last
    conformation against the FP64 oracle, whose time is this
    configuration's CPU baseline."""
    import torch

    from openmmcustomgbintegralforce_gb300._lib import EXEC_CHECK, EXEC_ENERGY, EXEC_FORCES, Context
    from oracle import oracle as O

    w = workloads()[name]
    g = make_globule(w["n"], seed=w["seed"])
    model = model_for(w, g)
    n = g.n
    adjoint = bool(w.get("adjoint"))
    ctx = Context(model, n)
    ctx.set_particle_parameters(g.charge, g.radius)
    stream = torch.cuda.Stream(device=dev)
    sptr = stream.cuda_stream
    posq = torch.zeros((n, 4), dtype=torch.float32, device=dev)
    posq[:, :3] = torch.from_numpy(g.positions.astype(np.float32)).to(dev)
    force = torch.zeros(3 * n, dtype=torch.int64, device=dev)
    energy = torch.zeros(1, dtype=torch.float64, device=dev)
    out = {k: torch.zeros(s_, dtype=torch.float64, device=dev) for k, s_ in
           (("energy", 1), ("forces", 3 * n), ("dEdq", n), ("dEdR", n), ("dEdalpha", 2))}
    gen = torch.Generator(device=dev)
    gen.manual_seed(w["seed"])

    def step(flags):
        if adjoint:
            ctx.adjoint_device(posq.data_ptr(), out["energy"].data_ptr(), out["forces"].data_ptr(),
                               out["dEdq"].data_ptr(), out["dEdR"].data_ptr(), out["dEdalpha"].data_ptr(),
                               flags & EXEC_CHECK, sptr)
        else:
            ctx.execute_device(posq.data_ptr(), force.data_ptr(), n, energy.data_ptr(), flags, sptr)

    torch.cuda.synchronize()
    for _ in range(3):
        step(EXEC_FORCES | EXEC_ENERGY | EXEC_CHECK)
    torch.cuda.synchronize()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    launches0 = ctx.launches()
    with torch.cuda.stream(stream):
        for k in range(steps):
            flush.fill_(float(k))
            if jitter_A > 0:
                posq[:, :3] += 0.1 * jitter_A * torch.randn(posq[:, :3].shape, generator=gen, device=dev)
            starts[k].record(stream)
            step(EXEC_FORCES | EXEC_ENERGY)
            ends[k].record(stream)
    torch.cuda.synchronize()
    launches = ctx.launches() - launches0
    ms = float(np.mean([a.elapsed_time(b) for a, b in zip(starts, ends)]))
    x = posq[:, :3].double().cpu().numpy()
    res = {"workload": name, "desc": w["desc"], "atoms": n, "quadrature_points": model.n_quad, "steps": steps,
           "evals_per_s": 1000.0 / ms, "ms_per_step": ms, "gpu_launches_per_step": launches / steps,
           "jitter_A": jitter_A, "l2": "flushed (256 MiB write) between steps"}
    if not adjoint:
        peaks, peak_src = measured_peaks()
        sms = torch.cuda.get_device_properties(dev).multi_processor_count
        rl = stage_roofline(ctx, model, g, n, step, flush, sptr, posq, force, n, energy, sms, peaks, peak_src)
        rl["traffic"] = TRAFFIC.get(name, {}).get(rl["kernel"])
        rl["traffic_source"] = TRAFFIC_SOURCE.get(name)
        res["roofline"] = rl
    if adjoint:
        # host arrays in, every gradient out
        ctx.adjoint(x)
        t = []
        for _ in range(20):
            t0 = time.perf_counter()
            got = ctx.adjoint(x)
            t.append(time.perf_counter() - t0)
        # the median: a single host-side hiccup among a few sub-millisecond calls moved the mean by a quarter
        res["e2e"] = {"evals_per_s": 1.0 / float(np.median(t)), "call": "gbx_adjoint_host",
                      "calls": len(t), "statistic": "median"}
        t0 = time.perf_counter()
        ref = O.Oracle(model, nthreads=os.cpu_count() or 1).energy_forces(x, g.charge, g.radius, adjoint=True)
        dt = time.perf_counter() - t0
        res["err_vs_fp64"] = {"energy_rel": abs(got["energy"] / ref["energy"] - 1.0),
                              "force_rel_rms": rel_rms(got["forces"], ref["forces"]),
                              "dEdq_rel_rms": rel_rms(got["dEdq"], ref["dEdq"]),
                              "dEdR_rel_rms": rel_rms(got["dEdR"], ref["dEdR"]),
                              "dEdalpha_rel_max": float(np.abs(got["dEdalpha"] / ref["dEdalpha"] - 1).max())}
    else:
        ctx.execute_host(x)
        t = []
        for _ in range(5 if n > 20000 else 20):
            t0 = time.perf_counter()
            E, F = ctx.execute_host(x)
            t.append(time.perf_counter() - t0)
        res["e2e"] = {"evals_per_s": 1.0 / float(np.mean(t)), "call": "gbx_execute_host",
                      "h2d_bytes_per_step": n * 16, "d2h_bytes_per_step": n * 3 * 8 + 8}
        t0 = time.perf_counter()
        ref = O.Oracle(model, nthreads=os.cpu_count() or 1).energy_forces(x, g.charge, g.radius)
        dt = time.perf_counter() - t0
        res["err_vs_fp64"] = {"energy_rel": abs(E / ref["energy"] - 1.0),
                              "force_rel_rms": rel_rms(F, ref["forces"])}
    res["err_vs_fp64"]["conformation"] = (f"last of {steps} jittered (N(0, {jitter_A} A) per step, accumulated)"
                                          if jitter_A > 0 else "the workload's globule")
    res["cpu_baseline"] = {"evals_per_s": 1.0 / dt, "cores": os.cpu_count() or 1, "kind": "port",
                           "sample": "the FP64 oracle's evaluation of the checked conformation"}
    ctx.close()
    return res


def measure_custom(dev, flush, steps: int = 50):
    """The compiled-expression path (gbx_create_custom) at the GBMV-II 10k
    configuration: the canonical CHARMM set written as user expressions,
    against the fixed kernels on the same input (the results agree to FP32
    rounding), and a modified set outside it; device evals/s from CUDA events
    around each call (L2 flushed between calls) and e2e through host arrays."""
    import torch

    from openmmcustomgbintegralforce_gb300._lib import EXEC_CHECK, EXEC_ENERGY, EXEC_FORCES, Context, CustomContext
    from openmmcustomgbintegralforce_gb300.expression_sets import CANONICAL, MODIFIED, modified_params

    w = workloads()["gbmv10k"]
    g = make_globule(w["n"], seed=w["seed"])
    model = model_for(w, g)
    n = g.n
    ctxs = {"fixed": Context(model, n), "canonical_expressions": CustomContext(model, n, CANONICAL),
            "modified_expressions": CustomContext(model, n, MODIFIED)}
    ctxs["fixed"].set_particle_parameters(g.charge, g.radius)
    ctxs["canonical_expressions"].set_custom_parameters(np.stack([g.charge, g.radius], axis=1))
    ctxs["modified_expressions"].set_custom_parameters(modified_params(g))
    stream = torch.cuda.Stream(device=dev)
    sptr = stream.cuda_stream
    posq = torch.zeros((n, 4), dtype=torch.float32, device=dev)
    posq[:, :3] = torch.from_numpy(g.positions.astype(np.float32)).to(dev)
    force = torch.zeros(3 * n, dtype=torch.int64, device=dev)
    energy = torch.zeros(1, dtype=torch.float64, device=dev)
    out = {}
    host = {}
    for name, ctx in ctxs.items():
        for _ in range(3):
            ctx.execute_device(posq.data_ptr(), force.data_ptr(), n, energy.data_ptr(),
                               EXEC_FORCES | EXEC_ENERGY | EXEC_CHECK, sptr)
        torch.cuda.synchronize()
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
        with torch.cuda.stream(stream):
            for a, b in ev:
                flush.fill_(1.0)
                a.record(stream)
                ctx.execute_device(posq.data_ptr(), force.data_ptr(), n, energy.data_ptr(), EXEC_FORCES | EXEC_ENERGY,
                                   sptr)
                b.record(stream)
        torch.cuda.synchronize()
        ms = float(np.mean([a.elapsed_time(b) for a, b in ev]))
        ctx.execute_host(g.positions)
        t = []
        for _ in range(10):
            t0 = time.perf_counter()
            host[name] = ctx.execute_host(g.positions)
            t.append(time.perf_counter() - t0)
        out[name] = {"evals_per_s": 1000.0 / ms, "ms_per_step": ms, "e2e_evals_per_s": 1.0 / float(np.mean(t))}
    (E0, F0), (E1, F1) = host["fixed"], host["canonical_expressions"]
    out["canonical_expressions"]["vs_fixed_kernels"] = {"energy_rel": abs(E1 / E0 - 1.0), "force_rel_rms": rel_rms(F1, F0)}
    for c in ctxs.values():
        c.close()
    return {"workload": "gbmv10k through gbx_create_custom", "desc": w["desc"], "atoms": n, **out,
            "parity": "the modified set against the FP64 expression oracle: tests/test_gpu_custom.py"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--workload", default="gbsw50k", choices=sorted(workloads()))
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-batch", action="store_true", help="skip the batched 256-molecule measurement")
    ap.add_argument("--no-configs", action="store_true", help="skip the other configurations' measurements")
    ap.add_argument("--only-expressions", action="store_true",
                    help="measure only the compiled-expression path (GBMV-II 10k) and print its JSON")
    ap.add_argument("--jitter", type=float, default=0.0,
                    help="A: fresh N(0, jitter) position noise before every timed step (MD-like back-to-back "
                         "evaluations); the FP64 error is then taken on the last jittered conformation")
    args = ap.parse_args()
    batch_set = None
    if args.impl == "gb300" and not args.no_batch and not args.only_expressions and int(os.environ.get("RANK", "0")) == 0:
        # generated before any CUDA work, in a spawn-started pool
        batch_set = make_batch(batch_sizes(BATCH_MOLECULES, 500, 8000, seed=BATCH_SEED), seed=BATCH_SEED)
    world, rank, local = dist_setup(args)
    if args.impl == "reference":
        run_reference(args, world, rank)
        return

    import torch

    from openmmcustomgbintegralforce_gb300._lib import EXEC_CHECK, EXEC_COUNT_WORK, EXEC_ENERGY, EXEC_FORCES, Context

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if args.only_expressions:
        flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
        print(json.dumps(measure_custom(dev, flush, steps=args.steps)))
        return
    w = workloads()[args.workload]
    g = make_globule(w["n"], seed=w["seed"])
    model = model_for(w, g)
    n = g.n
    ctx = Context(model, n)
    ctx.set_particle_parameters(g.charge, g.radius)
    stream = torch.cuda.Stream(device=dev)
    sptr = stream.cuda_stream
    stride = ((n + 31) // 32) * 32
    posq = torch.zeros((n, 4), dtype=torch.float32, device=dev)
    posq[:, :3] = torch.from_numpy(g.positions.astype(np.float32)).to(dev)
    force = torch.zeros(3 * stride, dtype=torch.int64, device=dev)
    energy = torch.zeros(1, dtype=torch.float64, device=dev)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    torch.cuda.synchronize()

    def step(flags):
        ctx.execute_device(posq.data_ptr(), force.data_ptr(), stride, energy.data_ptr(), flags, sptr)

    for _ in range(max(args.warmup, 3)):
        step(EXEC_FORCES | EXEC_ENERGY | EXEC_CHECK)
    torch.cuda.synchronize()

    # timed region: device-resident inputs
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    barrier(world)
    torch.cuda.synchronize()
    wall0 = time.perf_counter()
    launches0 = ctx.launches()
    base = posq[:, :3].clone()
    with torch.cuda.stream(stream):
        for k in range(args.steps):
            flush.fill_(float(k))
            if args.jitter > 0:  # outside the timed interval
                posq[:, :3] = base + 0.1 * args.jitter * torch.randn_like(base)
            starts[k].record(stream)
            step(EXEC_FORCES | EXEC_ENERGY)
            ends[k].record(stream)
    torch.cuda.synchronize()
    barrier(world)
    wall = time.perf_counter() - wall0
    launches = ctx.launches() - launches0
    clk = clocks.stop()
    step_ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    ms = allmax(world, float(np.mean(step_ms)))
    value = replica_value(world, ms)

    peaks, peak_src = measured_peaks()
    sms = torch.cuda.get_device_properties(dev).multi_processor_count
    roofline = stage_roofline(ctx, model, g, n, step, flush, sptr, posq, force, stride, energy, sms, peaks, peak_src)
    dominant = roofline["kernel"]
    roofline["traffic"] = TRAFFIC.get(args.workload, {}).get(dominant)
    roofline["traffic_source"] = (("ncu dram__bytes_read.sum + dram__bytes_write.sum per launch, "
                                   + TRAFFIC_SOURCE[args.workload]) if args.workload in TRAFFIC_SOURCE else None)

    # e2e: host buffers through gbx_execute_host (copies inside the timed region)
    for _ in range(2):
        ctx.execute_host(g.positions)
    e2e_times = []
    for k in range(max(3, args.steps // 2)):
        flush.fill_(2.0)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        E_gpu, F_gpu = ctx.execute_host(g.positions)
        e2e_times.append(time.perf_counter() - t0)
    e2e_ms = allmax(world, 1000.0 * float(np.mean(e2e_times)))
    e2e = {"value": world * 1000.0 / e2e_ms, "unit": UNIT, "h2d_bytes_per_step": n * 16,
           "d2h_bytes_per_step": n * 3 * 8 + 8, "ms_per_step": e2e_ms}

    cpu = None
    err = None
    if rank == 0 and not args.no_cpu_baseline:
        out, dt, cores = oracle_baseline(model, g)
        cpu = {"value": 1.0 / dt, "unit": UNIT, "cores": cores, "kind": "port",
               "sample": f"one full FP64 evaluation of the workload ({n} atoms, {model.n_quad} points) "
                         f"with OpenMP on all host cores, {dt:.1f} s"}
        err = {"energy_rel": abs(E_gpu / out["energy"] - 1.0),
               "force_rel_rms": float(np.sqrt(((F_gpu - out["forces"]) ** 2).sum() / (out["forces"] ** 2).sum()))}
    if rank == 0 and args.jitter > 0:
        from oracle import oracle as O

        xj = posq[:, :3].double().cpu().numpy()
        Ej, Fj = ctx.execute_host(xj)
        oj = O.Oracle(model, nthreads=os.cpu_count() or 1).energy_forces(xj, g.charge, g.radius)
        err = {"energy_rel": abs(Ej / oj["energy"] - 1.0),
               "force_rel_rms": float(np.sqrt(((Fj - oj["forces"]) ** 2).sum() / (oj["forces"] ** 2).sum())),
               "conformation": f"last of {args.steps} jittered (N(0, {args.jitter} A))"}

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f32", "data": "synthetic seeded globule (no dataset)",
                "config": workload_config(args.workload, w, model, world, args.jitter),
                "gpu_launches": launches, "gpu_launches_per_step": launches / args.steps, "e2e": e2e, "roofline": roofline, "cpu_baseline": cpu,
                "err_vs_fp64": err, "clocks": clk, "wall_s": wall}
        if batch_set is not None:
            line["batched"] = measure_batched(batch_set, max(3, min(args.steps, 10)))
        if not args.no_configs and world == 1:
            line["configs"] = {k: measure_config(wl, st, jit, dev, flush) for k, (wl, st, jit) in CONFIG_RUNS.items()}
            line["configs"]["f2_compiled_expressions_gbmv2_10k"] = measure_custom(dev, flush)
        print(json.dumps(line))


if __name__ == "__main__":
    main()
