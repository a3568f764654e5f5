#!/usr/bin/env python
"""Benchmark of the GB300 FVM_TVD path: cell-updates/s at 2,097,152 triangles.

Workload: the four-quadrant Riemann problem on [0,1]^2, 1024 x 1024 x 2 jittered
triangles (seed 2, +-0.05h), HLLC flux, minmod reconstruction, SSP-RK3, CFL 0.4,
transmissive boundaries. One step = one SSP-RK3 time step (3 stages) of every
triangle. The headline value is the FP64 drop-in; the mixed form (FP32 faces,
FP64 accumulation/update) is measured in the same run.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

For N > 1 launch with torch.distributed.run: each rank runs its own replica of
the workload on its GPU (the path does not shard here; "replicas only").
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "cfd-2d_gb300")
sys.path.insert(0, PKG)
sys.path.insert(0, ROOT)

METRIC = "cell-updates/s at 2.1M tris, FP64 vs mixed, %HBM peak; adjoint/forward ratio"
UNIT = "cell-updates/s"
N_SIDE = 1024
WORKLOAD = ("four-quadrant Riemann problem on [0,1]^2, 1024x1024x2 = 2,097,152 jittered triangles (seed 2, "
            "+-0.05h), HLLC + minmod + SSP-RK3, CFL 0.4, BOUND_OUTLET all round, STEADY=0")
# algorithmic HBM bytes per cell-update of an ideal fused step (each cell's data
# read once per stage, gradients on chip): FP64 SSP-RK3 and mixed SSP-RK3
STEP_BYTES = {"fp64": 580.0, "mixed": 436.0}
KINDS = ("grad", "flux", "update", "remediate")
FALLBACK_HBM_GBS = 6800.0


def kernel_bytes(kind: str, nc: int, ne: int, fb: int) -> float:
    """Compulsory bytes of one launch of a kernel kind (fb: bytes of a face real).

    grad:   cells W(4) in, G(8) out, faces 12 B, S 8 B; edges nx,ny,l(3) + c1,c2 8 B
    flux:   cells W(4) + G(8) in; edges c1,c2 8 B, nx,ny,l(3), Gauss offsets(8) in, F(4) out
    update: cells faces 12 B, A 32 B in, B 32 B in (stages 2-3), result 32 B out, cfl 8 B,
            flags 4 B, W(4) out; edges F(4) in  (stage 2/3 average: 2/3 of the B read)
    flux_grad (the mixed form's flux kernel that forms the gradients, FP32):
            cells W(4) in, face records 48 B, 1/S 4 B; edges c1,c2 8 B, nx,ny,l(3),
            Gauss offsets(8) in, F(4) out
    """
    if kind == "flux_grad":
        return nc * (4 * fb + 48 + 4) + ne * (8 + 15 * fb)
    if kind == "grad":
        return nc * (12 * fb + 12 + 8) + ne * (3 * fb + 8)
    if kind == "flux":
        return nc * 12 * fb + ne * (8 + 15 * fb)
    if kind == "update":
        return nc * (12 + 32 + 32 * 2 / 3 + 32 + 8 + 4 + 4 * fb) + ne * 4 * fb
    return 0.0


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return FALLBACK_HBM_GBS, "fallback"


def measured_sm_max():
    try:
        return float(json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))["sm_max_mhz"])
    except Exception:
        return 2070.0


def ncu_traffic():
    """Per-launch DRAM bytes of each kernel kind from the committed ncu summary, if any."""
    p = os.path.join(ROOT, "profiles", "ncu_dram_traffic.txt")
    out = {}
    if os.path.exists(p):
        for line in open(p):
            if line.startswith("traffic_bytes_per_launch"):
                _, key, val = line.split()[:3]
                out[key] = float(val)
    return out


def ncu_instr():
    """FP64 / FP32 thread instructions per cell-update of each form, from the committed
    ncu instruction-count summary (one SSP-RK3 step of the 2,097,152-triangle workload)."""
    p = os.path.join(ROOT, "profiles", "ncu_instruction_counts_four_quadrant_2M.md")
    out = {}
    if os.path.exists(p):
        for line in open(p):
            if line.startswith("instr_per_cell_update"):
                _, form, kind, val = line.split()[:4]
                out[(form, kind)] = float(val)
    return out


def ncu_instr_units(name: str):
    """FP64-unit thread instructions per unit (edge / cell) of a method's kernels, from a
    committed ncu summary ("instr_per_unit <method> <kernel> <count> <unit>" lines)."""
    p = os.path.join(ROOT, "profiles", name)
    out = {}
    if os.path.exists(p):
        for line in open(p):
            if line.startswith("instr_per_unit"):
                _, _, kernel, val, unit = line.split()[:5]
                out[kernel] = (float(val), unit)
    return out


def cpu_model():
    try:
        r = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in r.splitlines():
            if line.startswith("Model name:"):
                return line.split(":", 1)[1].strip()
    except Exception:
        pass
    import platform
    return platform.processor() or platform.machine()


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.lines = []
        self.active = False

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                          "-lms", "200", "-i", str(self.gpu)], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            if self.active:
                self.lines.append(line.strip())

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_setup(ngpus):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch
        import torch.distributed as td
        torch.cuda.set_device(local)
        td.init_process_group("nccl")
        dist = td
    return world, rank, local, dist


def reduce_max(dist, x: float) -> float:
    """Max over ranks (NCCL ranks reduce on their GPU, gloo ranks on the host)."""
    if dist is None:
        return x
    import torch
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_rate(world: int, units_per_rank: int, steps: int, ms_max: float) -> float:
    """Whole-job throughput of independent replicas: all ranks' units over the slowest rank's time."""
    return world * units_per_rank * steps / (ms_max * 1e-3)


def barrier(dist):
    if dist is not None:
        dist.barrier()


# ------------------------------------------------------------------ reference arm

def _ref_worker(args):
    """One host process: the oracle (restatement of the reference FVM_TVD) on the workload."""
    n, warm, steps, q = args
    sys.path.insert(0, PKG); sys.path.insert(0, ROOT)
    from cfd2d import cases
    from oracle import pyoracle
    t, m, _ = cases.four_quadrant(n, steps=1)
    o = pyoracle.solver_from_task(t, m, flux="HLLC", recon="MINMOD", scheme="SSPRK3")
    o.step(warm)
    q.put(("ready", m.n_cells))
    a = time.perf_counter()
    o.step(steps)
    q.put(("done", time.perf_counter() - a))


def reference_arm(args, world, rank):
    if rank != 0:
        return
    import multiprocessing as mp
    from oracle import pyoracle
    pyoracle.build()
    ctx = mp.get_context("spawn")
    procs = max(1, (os.cpu_count() or 1))
    procs = min(procs, int(os.environ.get("CFD2D_REF_PROCS", 16)))
    # every process times the same --steps K after --warmup W steps as our arm (each CPU
    # step of the full mesh costs ~1.5 s on one Grace core, so K=20, W=5 is ~40 s)
    steps = max(1, args.steps)
    warm = max(0, args.warmup)
    q = ctx.Queue()
    ps = [ctx.Process(target=_ref_worker, args=((N_SIDE, warm, steps, q),)) for _ in range(procs)]
    for p in ps:
        p.start()
    cells, times = 0, []
    for _ in range(2 * procs):
        kind, v = q.get()
        if kind == "ready":
            cells = v
        else:
            times.append(v)
    for p in ps:
        p.join()
    T = max(times)
    value = procs * cells * steps / T
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": steps, "warmup": warm, "ms_per_step": T / steps * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOAD, "cells": cells, "parallelism": f"{procs} host processes, one "
                       "independent instance each"},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": procs, "kind": "port",
                             "sample": f"{steps} SSP-RK3 step(s) (after {warm} warm-up steps) of the full "
                                       f"2,097,152-triangle workload per process, {procs} processes (the reference "
                                       "cannot run HLLC/minmod/SSP-RK3; the oracle restates it and equals it bit for "
                                       "bit in its own mode)"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------------ our arm

def cpu_baseline_single(seconds: float = 12.0):
    """The oracle on one host core on the same workload, for ~seconds of CPU work."""
    from cfd2d import cases
    from oracle import pyoracle
    pyoracle.build()
    t, m, _ = cases.four_quadrant(N_SIDE, steps=1)
    o = pyoracle.solver_from_task(t, m, flux="HLLC", recon="MINMOD", scheme="SSPRK3")
    a = time.perf_counter()
    k = 0
    while True:
        o.step(1)
        k += 1
        if time.perf_counter() - a >= seconds or k >= 10:
            break
    dt = time.perf_counter() - a
    return {"value": m.n_cells * k / dt, "unit": UNIT, "cores": 1, "kind": "port", "cpu": cpu_model(),
            "sample": f"{k} SSP-RK3 step(s) of the full 2,097,152-triangle workload on one core"}


def fd_check(s, U0, g, ndir, steps=200, every=20, eps=1e-6, seed=4):
    """The FP64 gradient against central finite differences of the FP64 forward (eps 1e-6)
    in ndir seeded unit directions of the 4 N-dimensional initial state; the error of a
    direction is |g.d - fd| / max(|fd|, 1e-3 |g|) (|g| / sqrt(4 N) is the typical size of a
    directional derivative, so the floor keeps near-zero directions from dividing by noise)."""
    rng = np.random.default_rng(seed)
    gn = float(np.linalg.norm(g))
    errs = []
    for _ in range(ndir):
        dvec = rng.standard_normal(U0.shape)
        dvec /= np.linalg.norm(dvec)
        s.set_state(U0 + eps * dvec)
        jp = s.forward(steps, every)
        s.set_state(U0 - eps * dvec)
        jm = s.forward(steps, every)
        fd = (jp - jm) / (2 * eps)
        errs.append(abs(float(np.sum(g * dvec)) - fd) / max(abs(fd), 1e-3 * gn))
    return {"directions": ndir, "eps": eps, "seed": seed, "max_rel_err": max(errs),
            "median_rel_err": float(np.median(errs)), "rel_err": [float("%.3g" % e) for e in errs]}


def adjoint_measure(capi, cases, d, fd_dirs=64):
    """Differentiation workload: 256x256x2 = 131,072-triangle vortex, HLLC + minmod +
    SSP-RK3, 200 steps, J = sum over the box [6,8]x[4,6] of S (p-1)^2, checkpoint
    every 20 steps. For the FP64 form and for the mixed form (FP32 faces in the
    forward and in the adjoint's face work), times a plain 200-step forward, the
    checkpointed forward and the backward sweep (wall clock; each call ends
    synchronised); the mixed gradient is compared with the FP64 one, the FP64 gradient
    with central finite differences in fd_dirs seeded directions."""
    t, m, U0, w, _ = cases.vortex_adjoint(256, steps=200)
    out, grads = {}, {}
    for form in ("fp64", "mixed"):
        t.precision = "MIXED" if form == "mixed" else None
        s = capi.Solver(cases.write_task(t, m, d), mesh=m)
        s.set_objective(0, w, 1.0)
        s.set_state(U0)
        s.step(3)
        s.set_state(U0)
        a = time.perf_counter()
        s.step(200)
        fw = time.perf_counter() - a
        s.set_state(U0)
        a = time.perf_counter()
        J = s.forward(200, 20)
        b = time.perf_counter()
        g, gb = s.backward()
        c = time.perf_counter()
        grads[form] = g
        out[form] = {"J": J, "grad_norm": float(np.linalg.norm(g)), "forward_ms": fw * 1e3,
                     "forward_checkpointed_ms": (b - a) * 1e3, "backward_ms": (c - b) * 1e3,
                     "ratio_backward_over_forward": (c - b) / fw, "ratio_gradient_over_forward": (c - a) / fw}
        if form == "fp64" and fd_dirs > 0:
            out[form]["fd_check"] = fd_check(s, U0, g, fd_dirs)
        s.close()
    t.precision = None
    out["mixed"]["grad_rel_diff_vs_fp64"] = float(np.linalg.norm(grads["mixed"] - grads["fp64"]) /
                                                  np.linalg.norm(grads["fp64"]))
    res = {"workload": "isentropic vortex, 256x256x2 = 131,072 triangles, HLLC + minmod + SSP-RK3, 200 steps, "
                       "J = sum_box S (p-1)^2, checkpoint every 20"}
    res.update(out["fp64"])
    res["mixed"] = out["mixed"]
    return res


COMBINED_N = 4096
ADJOINT_MEMORY = 180e9  # bytes (180 GB, decimal): the combined configuration's device-memory budget


def combined_measure(capi, cases, W, n_side=COMBINED_N, steps=300, every=30, err_steps=30):
    """Scale + mixed precision + adjoint: 4096x4096x2 = 33,554,432 triangles, four-quadrant
    Riemann problem (seed 5, +-0.05h), HLLC + minmod + SSP-RK3, CFL 0.4. The mixed form
    (FP32 faces / FP64 accumulation) runs `steps` steps timed on the device, then the
    checkpointed forward (every `every` steps) and the discrete adjoint (FP32 face work,
    FP64 per-cell sums) of J = sum over cells with centroid in [1/4, 3/4]^2 of S rho^2, with
    the handle's device memory capped at ADJOINT_MEMORY (the store keeps what fits the
    budget). The error is measured after `err_steps` steps against the FP64 solver on the
    same mesh (the FP64 path equals the CPU oracle bit for bit)."""
    d = tempfile.mkdtemp(prefix="cfd2d_comb_")
    a0 = time.perf_counter()
    t, m, _ = cases.four_quadrant(n_side, seed=5, steps=steps, precision="MIXED")
    t.adjoint_memory = ADJOINT_MEMORY
    xy = m.centroids()
    p = m.nodes[m.tris]
    S = 0.5 * np.abs((p[:, 1, 0] - p[:, 0, 0]) * (p[:, 2, 1] - p[:, 0, 1]) -
                     (p[:, 2, 0] - p[:, 0, 0]) * (p[:, 1, 1] - p[:, 0, 1]))
    del p
    w = np.where((xy[:, 0] >= 0.25) & (xy[:, 0] <= 0.75) & (xy[:, 1] >= 0.25) & (xy[:, 1] <= 0.75), S, 0.0)
    del xy, S
    s = capi.Solver(cases.write_task(t, m, d), mesh=m)
    nc = s.n
    s.set_objective(1, w, 0.0)
    U0 = s.state()
    setup_s = time.perf_counter() - a0
    s.step(W)
    s.set_state(U0)
    ms_fw = s.timed_steps(steps)               # plain mixed forward, device time
    s.set_state(U0)
    a = time.perf_counter()
    J = s.forward(steps, every)
    b = time.perf_counter()
    g, _ = s.backward()
    c = time.perf_counter()
    dev_bytes = s.get_info().device_bytes
    s.set_state(U0)
    s.step(err_steps)
    Umx = s.state()
    s.close()
    t.precision = None
    t.adjoint_memory = None
    r = capi.Solver(cases.write_task(t, m, d), mesh=m)
    ms64 = r.timed_steps(err_steps)
    U64 = r.state()
    r.close()
    l1 = lambda x, y: float(np.sum(np.abs(x - y)) / np.sum(np.abs(y)))
    linf = lambda x, y: float(np.max(np.abs(x - y)) / np.max(np.abs(y)))
    hbm, peak_kind = measured_peaks()
    rate = nc * steps / (ms_fw * 1e-3)
    return {
        "workload": f"four-quadrant Riemann problem, {n_side}x{n_side}x2 = {nc:,} triangles (seed 5, +-0.05h), "
                    f"HLLC + minmod + SSP-RK3, CFL 0.4, {steps} steps; J = sum_{{[1/4,3/4]^2}} S rho^2, "
                    f"checkpoint every {every}",
        "cells": nc, "steps": steps, "checkpoint_every": every,
        "value": rate, "unit": UNIT, "ms_per_step": ms_fw / steps, "dtype": "f32 faces / f64 accumulate",
        "roofline_step": {"achieved": rate * STEP_BYTES["mixed"] / 1e9,
                          "frac": rate * STEP_BYTES["mixed"] / 1e9 / hbm, "peak": hbm, "peak_kind": peak_kind,
                          "bytes_per_cell_update": STEP_BYTES["mixed"]},
        "fp64": {"value": nc * err_steps / (ms64 * 1e-3), "ms_per_step": ms64 / err_steps},
        "error_vs_fp64": {"steps": err_steps, "l1_rho": l1(Umx[0], U64[0]), "l1_rhoE": l1(Umx[3], U64[3]),
                          "linf_rho": linf(Umx[0], U64[0]), "linf_rhoE": linf(Umx[3], U64[3])},
        "adjoint": {"J": J, "grad_norm": float(np.linalg.norm(g)), "finite": bool(np.all(np.isfinite(g))),
                    "forward_checkpointed_ms": (b - a) * 1e3, "backward_ms": (c - b) * 1e3,
                    "ratio_backward_over_mixed_forward": (c - b) * 1e3 / ms_fw,
                    "ratio_gradient_over_mixed_forward": (c - a) * 1e3 / ms_fw},
        "device_bytes_with_adjoint": dev_bytes, "device_budget_bytes": ADJOINT_MEMORY,
        "within_budget": bool(dev_bytes <= ADJOINT_MEMORY), "setup_s": setup_s}


def combined_workload(args, capi, cases, world, rank, dist, W, K):
    """The combined configuration on its own line, the FP64 comparison at its full 300 steps."""
    res = combined_measure(capi, cases, W, err_steps=300)
    if rank == 0:
        line = {"metric": "cell-updates/s, 33.5M triangles, mixed forward + mixed discrete adjoint",
                "value": res["value"], "unit": UNIT, "n_gpus": world, "steps": res["steps"], "warmup": W,
                "ms_per_step": res["ms_per_step"], "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": res["dtype"], "data": "synthetic",
                "config": {"workload": res["workload"], "cells": res["cells"],
                           "l2": "no flush: working set far above the 129 MB L2"}}
        line.update({k: v for k, v in res.items() if k not in line and k not in ("workload", "cells")})
        print(json.dumps(line), flush=True)


def batched_measure(capi, cases, W, K, instances=256, forms=("fp64", "mixed"), dist=None):
    """256 isentropic-vortex instances, triangle counts log-uniform in [10k, 400k]
    (seed 3), Mach uniform in [0.1, 0.8], strength uniform in [1, 5], Roe + minmod +
    SSP-RK3, CFL 0.5: per form (FP64, and FP32 faces / FP64 accumulation) one batched
    solver (autotuned launch shapes, one CUDA graph per step) against the same instances
    solved one after another, K steps each; device time from CUDA events."""
    d = tempfile.mkdtemp(prefix="cfd2d_batch_")
    insts = cases.batched_vortices(instances, steps=K)
    out = {}
    for form in forms:
        paths = []
        for k, (t, m, _) in enumerate(insts):
            t.precision = "MIXED" if form == "mixed" else None
            dk = os.path.join(d, f"{form}_{k}")
            os.makedirs(dk)
            paths.append(cases.write_task(t, m, dk))
        a = time.perf_counter()
        b = capi.Batch(paths, meshes=[m for _, m, _ in insts])
        b.set_state(np.concatenate([U0 for _, _, U0 in insts], axis=1), reset_time_step=True)
        create_s = time.perf_counter() - a
        tune_json = os.path.join(d, f"tuning_{form}.json")
        b.autotune(tune_json)
        tuning = json.load(open(tune_json))
        nc = b.n
        b.step(W)
        ms_b = reduce_max(dist, b.timed_steps(K))
        b.close()
        seq_ms = 0.0
        for k, (t, m, U0) in enumerate(insts):
            s = capi.Solver(paths[k], mesh=m)
            s.set_state(U0, reset_time_step=True)
            s.step(W)
            seq_ms += s.timed_steps(K)
            s.close()
        seq_ms = reduce_max(dist, seq_ms)
        out[form] = {"value": nc * K / (ms_b * 1e-3), "ms_per_step": ms_b / K,
                     "sequential": {"value": nc * K / (seq_ms * 1e-3), "ms_per_step_all_instances": seq_ms / K},
                     "speedup_vs_sequential": seq_ms / ms_b, "autotune": tuning, "create_s": create_s}
    out["cells"] = nc
    out["instances"] = instances
    out["steps"] = K
    out["workload"] = (f"{instances} isentropic-vortex instances on [0,10]^2, triangles log-uniform in [10k, 400k] "
                       "(seed 3), Mach U[0.1,0.8], strength U[1,5], Roe + minmod + SSP-RK3, CFL 0.5")
    return out


def batched_workload(args, capi, cases, world, rank, dist, W, K):
    """The batched configuration on its own line (FP64 headline, the mixed form beside it)."""
    res = batched_measure(capi, cases, W, K, args.instances, dist=dist)
    if rank == 0:
        f = res["fp64"]
        print(json.dumps({
            "metric": "aggregate cell-updates/s, 256 uneven vortex instances, batched vs sequential",
            "value": world * f["value"], "unit": UNIT, "n_gpus": world, "steps": K, "warmup": W,
            "ms_per_step": f["ms_per_step"], "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic",
            "config": {"workload": res["workload"], "cells": res["cells"], "instances": res["instances"],
                       "l2": "no flush: the batch's working set (~12 GB) exceeds the 129 MB L2"},
            "sequential": f["sequential"], "speedup_vs_sequential": f["speedup_vs_sequential"],
            "autotune": f["autotune"], "create_s": f["create_s"], "mixed": res.get("mixed"),
            "gpu_launches": K * (3 * 3 + 1)}), flush=True)


IMP_N = 1024
IMP_TAU = 0.002


def implicit_cpu_baseline(n=IMP_N, steps=1):
    """The oracle's FVM_TVD_IMPLICIT on one host core: a bounded sample of the same workload
    (one step of the full mesh, ~10-20 s of CPU work)."""
    from cfd2d import cases
    from oracle import pyoracle
    pyoracle.build()
    t, m, U0 = cases.vortex_implicit(n, tau=IMP_TAU)
    o = pyoracle.implicit_from_task(t, m, U0=U0)
    a = time.perf_counter()
    o.step(steps)
    dt = time.perf_counter() - a
    return {"value": m.n_cells * steps / dt, "unit": UNIT, "cores": 1, "kind": "port", "cpu": cpu_model(),
            "sample": f"{steps} implicit step(s) of the same vortex at {n}x{n}x2 = {m.n_cells} triangles on one core "
                      f"(GMRES iterations {o.info()['iters']})"}


def implicit_workload(args, capi, cases, world, rank, dist, W, K):
    """FVM_TVD_IMPLICIT, the reference's implicit method: isentropic vortex on [0,10]^2,
    1024x1024x2 = 2,097,152 jittered triangles (seed 4), free-stream inlets, unsteady
    TAU 0.002 (CFL ~0.45), per step the Roe-linearised block system assembled from the
    centre states and the Gauss-point fluxes (LAX; GODUNOV reported beside it), solved
    by GMRES (Krylov dimension 30, 20 iterations, 1e-7, the reference's parameters),
    then the update with limits. Device time from CUDA events over the step graphs."""
    n = args.imp_n
    d = tempfile.mkdtemp(prefix="cfd2d_imp_")
    out = {}
    fluxes = ("LAX", "GODUNOV") if args.imp_flux == "both" else (args.imp_flux,)
    for flux in fluxes:
        t, m, U0 = cases.vortex_implicit(n, flux=flux, tau=IMP_TAU)
        dk = os.path.join(d, flux)
        os.makedirs(dk, exist_ok=True)
        s = capi.Solver(cases.write_implicit_task(t, m, dk), mesh=m)
        s.set_state(U0)
        s.step(W)
        barrier(dist)
        ms = reduce_max(dist, s.timed_steps(K))
        st = s.implicit_stats()
        out[flux] = {"ms_per_step": ms / K, "value": world * m.n_cells * K / (ms * 1e-3),
                     "gmres_iterations": st["iters"], "gmres_rel_residual": st["rel"], "status": st["status"]}
        if not args.no_profile:
            prof_ms, prof_n = s.profile_steps(2)
            phases = ["gradients", "fluxes_roe", "assembly", "gmres_update"]
            tot = max(float(prof_ms.sum()), 1e-30)
            out[flux]["phases"] = {k: {"ms_per_step": float(prof_ms[i] / 2), "share": float(prof_ms[i] / tot),
                                       "launches_per_step": int(prof_n[i] // 2)} for i, k in enumerate(phases)}
        cells, bytes_dev = m.n_cells, s.get_info().device_bytes
        if flux == fluxes[0] and not args.no_e2e:
            # end to end through the C ABI with pinned host buffers
            import torch
            nc = m.n_cells
            pin_in = torch.empty((4, nc), dtype=torch.float64).pin_memory()
            pin_out = torch.empty((4, nc), dtype=torch.float64).pin_memory()
            pin_in.copy_(torch.from_numpy(s.state()))
            pi = [pin_in[k].data_ptr() for k in range(4)]
            po = [pin_out[k].data_ptr() for k in range(4)]
            Ke = min(K, 10)
            barrier(dist)
            a = time.perf_counter()
            for _ in range(Ke):
                s.set_state_from(pi)
                s.step(1)
                s.state_into(po)
            e2e_s = reduce_max(dist, (time.perf_counter() - a) / Ke)
            out["e2e"] = {"value": world * nc / e2e_s, "unit": UNIT, "h2d_bytes_per_step": 32 * nc,
                          "d2h_bytes_per_step": 32 * nc, "steps": Ke,
                          "path": "cfd2d_set_state + cfd2d_step(1) + cfd2d_get_state, pinned host buffers"}
        s.close()
    lax = out[fluxes[0]]
    # FP64 operations of the matrix-vector product (64 multiply-adds per cell), the GMRES
    # kernel the step spends most in: achieved rate against GB300's FP64 issue rate
    if rank == 0:
        line = {
            "metric": "implicit-method cell-updates/s at 2.1M triangles (FVM_TVD_IMPLICIT, GMRES per step)",
            "value": lax["value"], "unit": UNIT, "n_gpus": world, "steps": K, "warmup": W,
            "ms_per_step": lax["ms_per_step"], "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic",
            "config": {"workload": f"isentropic vortex on [0,10]^2, {n}x{n}x2 = {cells} jittered triangles (seed 4), "
                                   f"free-stream inlets, {fluxes[0]} flux, unsteady TAU {IMP_TAU}, GMRES (30, 20 iterations, "
                                   "1e-7)", "cells": cells, "device_bytes": bytes_dev,
                       "l2": "no flush: a step streams ~10 GB (Krylov basis 1.4 GB, block matrix 1.1 GB)"},
            "lax": out.get("LAX"), "godunov": out.get("GODUNOV"), "e2e": out.get("e2e"),
        }
        if "phases" in lax:
            line["gpu_launches"] = K * sum(v["launches_per_step"] for v in lax["phases"].values())
        if world == 1 and not args.no_cpu_baseline:
            line["cpu_baseline"] = implicit_cpu_baseline()
        print(json.dumps(line), flush=True)


DG_N = 1024


def rkdg_cpu_baseline(n=DG_N, steps=1):
    """The oracle's FEM_RKDG on one host core: a bounded sample of the same workload
    (one step of the full mesh, ~10-20 s of CPU work)."""
    from cfd2d import cases
    from oracle import pyoracle
    pyoracle.build()
    t, m, pm, U0 = cases.rkdg_vortex(n, flux="GODUNOV")
    o = pyoracle.OracleDG(t, pm)
    o.set_coeffs(U0)
    a = time.perf_counter()
    o.step(steps)
    dt = time.perf_counter() - a
    return {"value": len(pm.tris) * steps / dt, "unit": UNIT, "cores": 1, "kind": "port", "cpu": cpu_model(),
            "sample": f"{steps} FEM_RKDG step(s) of the same vortex at {n}x{n}x2 = {len(pm.tris)} triangles on one core"}


def rkdg_workload(args, capi, cases, world, rank, dist, W, K):
    """FEM_RKDG, the reference's explicit P1 discontinuous Galerkin method: isentropic vortex
    (strength 2) on [0,10]^2, 1024x1024x2 = 2,097,152 jittered triangles (seed 5) as P1
    coefficients, free-stream inlets, 4-point cell and 3-point edge quadrature, GODUNOV flux
    (LAX reported beside it), the reference's two stages, unsteady (TAU from the reference's
    CFL rule). Device time from CUDA events over the step graphs."""
    n = args.dg_n
    d = tempfile.mkdtemp(prefix="cfd2d_dg_")
    out = {}
    fluxes = ("GODUNOV", "LAX") if args.dg_flux == "both" else (args.dg_flux,)
    cells = bytes_dev = 0
    for flux in fluxes:
        t, m, pm, U0 = cases.rkdg_vortex(n, flux=flux)
        dk = os.path.join(d, flux)
        os.makedirs(dk, exist_ok=True)
        with open(os.path.join(dk, "task.xml"), "w") as f:
            f.write(cases.mg.write_rkdg_task_xml(t))
        mesh = cases.mg.Mesh(pm.nodes, pm.tris, m.cell_region, m.bsegs, m.bseg_bnd)
        s = capi.Solver(os.path.join(dk, "task.xml"), mesh=mesh)
        s.set_dg_coeffs(U0)
        s.step(W)
        barrier(dist)
        ms = reduce_max(dist, s.timed_steps(K))
        nc = len(pm.tris)
        out[flux] = {"ms_per_step": ms / K, "value": world * nc * K / (ms * 1e-3), "tau": s.tau}
        if not args.no_profile:
            prof_ms, prof_n = s.profile_steps(2)
            tot = max(float(prof_ms.sum()), 1e-30)
            out[flux]["kernels"] = {k: {"ms_per_step": float(prof_ms[i] / 2), "share": float(prof_ms[i] / tot),
                                        "launches_per_step": int(prof_n[i])}
                                    for i, k in enumerate(["k_dg_edge", "k_dg_cell", "k_dg_tstep"])}
        cells, bytes_dev = nc, s.get_info().device_bytes
        if flux == fluxes[0] and not args.no_e2e:
            import torch
            pin_in = torch.empty((nc, 12), dtype=torch.float64).pin_memory()
            pin_out = torch.empty((nc, 12), dtype=torch.float64).pin_memory()
            pin_in.copy_(torch.from_numpy(s.dg_coeffs()))
            Ke = min(K, 10)
            barrier(dist)
            a = time.perf_counter()
            for _ in range(Ke):
                s.set_dg_coeffs_from(pin_in.data_ptr())
                s.step(1)
                s.dg_coeffs_into(pin_out.data_ptr())
            e2e_s = reduce_max(dist, (time.perf_counter() - a) / Ke)
            out["e2e"] = {"value": world * nc / e2e_s, "unit": UNIT, "h2d_bytes_per_step": 96 * nc,
                          "d2h_bytes_per_step": 96 * nc, "steps": Ke,
                          "path": "cfd2d_dg_set_coeffs + cfd2d_step(1) + cfd2d_dg_get_coeffs, pinned host buffers"}
        s.close()
    main_ = out[fluxes[0]]
    if rank == 0:
        line = {
            "metric": "FEM_RKDG cell-updates/s at 2.1M triangles (P1 discontinuous Galerkin, two stages per step)",
            "value": main_["value"], "unit": UNIT, "n_gpus": world, "steps": K, "warmup": W,
            "ms_per_step": main_["ms_per_step"], "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic",
            "config": {"workload": f"isentropic vortex on [0,10]^2, {n}x{n}x2 = {cells} jittered triangles (seed 5), "
                                   f"P1 coefficients, free-stream inlets, {fluxes[0]} flux, 4-point cell and 3-point edge "
                                   "quadrature, the reference's Runge-Kutta stages", "cells": cells,
                       "device_bytes": bytes_dev, "l2": "no flush: a step streams ~3 GB"},
            "godunov": out.get("GODUNOV"), "lax": out.get("LAX"), "e2e": out.get("e2e"),
        }
        if "kernels" in main_:
            line["gpu_launches"] = K * sum(v["launches_per_step"] for v in main_["kernels"].values())
            # the FP64 unit: ncu-counted FP64-unit instructions per edge / cell against GB300's
            # issue rate (2 per clock and SM at the GPU's maximum SM clock)
            import torch
            instr = ncu_instr_units("ncu_instruction_counts_rkdg_vortex_131k.md")
            sms = torch.cuda.get_device_properties(0).multi_processor_count
            peak = 2.0 * sms * measured_sm_max() * 1e6
            units = {"edge": (3 * n * n + 2 * n), "cell": cells}
            fp = {}
            for kname, key in (("k_dg_edge", "k_dg_edge_godunov"), ("k_dg_cell", "k_dg_cell")):
                if key in instr and fluxes[0] == "GODUNOV":
                    cnt, unit = instr[key]
                    per_launch_ms = main_["kernels"][kname]["ms_per_step"] / 2
                    ach = cnt * units[unit] / (per_launch_ms * 1e-3)
                    fp[kname] = {"fp64_instr_per_" + unit: cnt, "achieved_instr_per_s": ach, "frac": ach / peak}
            if fp:
                line["fp64_unit"] = {"peak_instr_per_s": peak, "kernels": fp,
                                     "source": "profiles/ncu_instruction_counts_rkdg_vortex_131k.md"}
        if world == 1 and not args.no_cpu_baseline:
            line["cpu_baseline"] = rkdg_cpu_baseline(n)
        print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--forms", default="fp64,mixed", help="comma list of fp64, mixed (profiling runs)")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-profile", action="store_true")
    ap.add_argument("--no-combined", action="store_true", help="leave out the 33.5M-triangle combined key")
    ap.add_argument("--no-batched", action="store_true", help="leave out the 256-instance batched key")
    ap.add_argument("--n", type=int, default=N_SIDE, help="squares per side (profiling runs only)")
    ap.add_argument("--workload", default="four_quadrant",
                    choices=["four_quadrant", "batched", "combined", "adjoint", "implicit", "rkdg"],
                    help="four_quadrant: the headline 2.1M-triangle line; batched: 256 uneven vortex instances")
    ap.add_argument("--instances", type=int, default=256)
    ap.add_argument("--adj-n", type=int, default=256, help="squares per side of the adjoint-only run's vortex")
    ap.add_argument("--imp-n", type=int, default=IMP_N, help="squares per side of the implicit workload's vortex")
    ap.add_argument("--imp-flux", default="both", choices=["both", "LAX", "GODUNOV"])
    ap.add_argument("--dg-n", type=int, default=DG_N, help="squares per side of the FEM_RKDG workload's vortex")
    ap.add_argument("--dg-flux", default="both", choices=["both", "LAX", "GODUNOV"])
    args = ap.parse_args()
    world, rank, local, dist = dist_setup(args.gpus)
    if args.impl == "reference":
        reference_arm(args, world, rank)
        return
    W = max(3, args.warmup)
    K = max(1, args.steps)

    from cfd2d import capi, cases
    capi.set_verbosity(0)
    capi.set_device(local)
    import torch

    if args.workload == "batched":
        batched_workload(args, capi, cases, world, rank, dist, W, K)
        return
    if args.workload == "combined":
        combined_workload(args, capi, cases, world, rank, dist, W, K)
        return
    if args.workload == "implicit":
        implicit_workload(args, capi, cases, world, rank, dist, W, K)
        return
    if args.workload == "rkdg":
        rkdg_workload(args, capi, cases, world, rank, dist, W, K)
        return
    if args.workload == "adjoint":  # one checkpointed forward + backward of K steps (profiling runs)
        t, m, U0, w, _ = cases.vortex_adjoint(args.adj_n, steps=K)
        if args.forms.strip() == "mixed":
            t.precision = "MIXED"
        s = capi.Solver(cases.write_task(t, m, tempfile.mkdtemp()), mesh=m)
        s.set_objective(0, w, 1.0)
        s.set_state(U0)
        s.step(W)
        s.set_state(U0)
        a = time.perf_counter()
        s.step(K)
        fw = time.perf_counter() - a
        s.set_state(U0)
        every = max(1, K // 10)
        a = time.perf_counter()
        J = s.forward(K, every)
        b = time.perf_counter()
        g, _ = s.backward()
        c = time.perf_counter()
        if rank == 0:
            print(json.dumps({"profiling_run": True, "workload": "adjoint", "steps": K, "checkpoint_every": every,
                              "J": J, "grad_norm": float(np.linalg.norm(g)), "forward_ms": fw * 1e3,
                              "backward_ms": (c - b) * 1e3, "ratio_backward_over_forward": (c - b) / fw}),
                  flush=True)
        return

    d = tempfile.mkdtemp(prefix="cfd2d_bench_")
    forms = [f.strip() for f in args.forms.split(",") if f.strip()]
    full = forms == ["fp64", "mixed"] and args.n == N_SIDE and not args.no_e2e and not args.no_profile
    t, m, _ = cases.four_quadrant(args.n, steps=K)
    solvers = {}
    for f in forms:
        t.precision = "MIXED" if f == "mixed" else None
        solvers[f] = capi.Solver(cases.write_task(t, m, d), mesh=m)
    nc, ne = m.n_cells, solvers[forms[0]].info.n_edges
    for s in solvers.values():
        s.step(W)
    sampler = ClockSampler(local)
    sampler.start()
    time.sleep(0.5)

    def timed(solver):
        barrier(dist)
        torch.cuda.synchronize()
        sampler.active = True
        ms = solver.timed_steps(K)
        sampler.active = False
        torch.cuda.synchronize()
        barrier(dist)
        return reduce_max(dist, ms)

    ms_of = {f: timed(solvers[f]) for f in forms}
    clocks = sampler.summary()  # the timed region itself (a fraction of a second: one or two samples)
    if not full:
        sampler.stop()
        line = {"profiling_run": True, "forms": forms, "cells": nc, "steps": K, "warmup": W,
                "ms_per_step": {f: ms_of[f] / K for f in forms}}
        if not args.no_profile:  # per-kernel device ms per launch, launched kernel by kernel with events
            line["ms_per_launch"] = {}
            for f in forms:
                ms, cnt = solvers[f].profile_steps(3)
                line["ms_per_launch"][f] = {k: round(float(ms[i] / max(cnt[i], 1)), 5) for i, k in enumerate(KINDS)}
        if rank == 0:
            print(json.dumps(line), flush=True)
        return
    s64, smx = solvers["fp64"], solvers["mixed"]
    ms64, msmx = ms_of["fp64"], ms_of["mixed"]
    # accuracy of the mixed form against the FP64 drop-in after the same W+K steps
    U64, Umx = s64.state(), smx.state()
    l1 = lambda a, b: float(np.sum(np.abs(a - b)) / np.sum(np.abs(b)))
    linf = lambda a, b: float(np.max(np.abs(a - b)) / np.max(np.abs(b)))
    err = {"l1_rho": l1(Umx[0], U64[0]), "l1_rhoE": l1(Umx[3], U64[3]),
           "linf_rho": linf(Umx[0], U64[0]), "linf_rhoE": linf(Umx[3], U64[3]), "steps": W + K}

    # per-kernel device times (kernel-by-kernel launches with events, outside the timed region)
    prof = {}
    for name, s in (("fp64", s64), ("mixed", smx)):
        ms, cnt = s.profile_steps(3)
        prof[name] = {k: {"ms_per_launch": float(ms[i] / max(cnt[i], 1)), "launches": int(cnt[i]),
                          "share": float(ms[i] / max(ms.sum(), 1e-30))} for i, k in enumerate(KINDS)}

    # the configuration's full length: both forms continued to 1000 steps, then compared
    full_steps = 1000
    # the same step graphs for seconds: clock samples under the timed region's load
    sampler.active = True
    for sv in (s64, smx):
        rest = full_steps - sv.get_info().step
        if rest > 0:
            sv.step(rest)
    torch.cuda.synchronize()
    sampler.active = False
    sampler.stop()
    clocks_long = sampler.summary()
    clocks_long["region"] = "timed steps plus the same step graphs continued to 1000 steps (both forms)"
    U64, Umx = s64.state(), smx.state()
    err_full = {"l1_rho": l1(Umx[0], U64[0]), "l1_rhoE": l1(Umx[3], U64[3]),
                "linf_rho": linf(Umx[0], U64[0]), "linf_rhoE": linf(Umx[3], U64[3]),
                "steps": int(s64.get_info().step)}

    # end to end through the C ABI: H2D of the step's input state from pinned memory,
    # one step, D2H of the result into pinned memory, every step
    Ke = min(K, 20)
    pin_in = torch.empty((4, nc), dtype=torch.float64).pin_memory()
    pin_out = torch.empty((4, nc), dtype=torch.float64).pin_memory()
    pin_in.copy_(torch.from_numpy(s64.state()))
    ptr_in = [pin_in[k].data_ptr() for k in range(4)]
    ptr_out = [pin_out[k].data_ptr() for k in range(4)]
    barrier(dist)
    a = time.perf_counter()
    for _ in range(Ke):
        s64.set_state_from(ptr_in)
        s64.step(1)
        s64.state_into(ptr_out)
    e2e_s = reduce_max(dist, (time.perf_counter() - a) / Ke)

    adj = adjoint_measure(capi, cases, d)
    s64.close()
    smx.close()
    comb = combined_measure(capi, cases, W) if not args.no_combined else None
    batch = batched_measure(capi, cases, W, min(K, 20), dist=dist) if not args.no_batched else None

    hbm, peak_kind = measured_peaks()
    traffic = ncu_traffic()
    # dominant kernel of the FP64 drop-in
    dom = max(KINDS, key=lambda k: prof["fp64"][k]["ms_per_launch"] * prof["fp64"][k]["launches"])
    dom_bytes = kernel_bytes(dom, nc, ne, 8)
    dom_ms = prof["fp64"][dom]["ms_per_launch"]
    achieved = dom_bytes / (dom_ms * 1e-3) / 1e9
    value = replica_rate(world, nc, K, ms64)
    value_mx = replica_rate(world, nc, K, msmx)
    step_gbs = nc / (ms64 / K * 1e-3) * STEP_BYTES["fp64"] / 1e9
    step_gbs_mx = nc / (msmx / K * 1e-3) * STEP_BYTES["mixed"] / 1e9
    mx_dom = max(KINDS, key=lambda k: prof["mixed"][k]["ms_per_launch"] * prof["mixed"][k]["launches"])
    # no gradient launches: the mixed flux kernel forms the gradients itself (k_flux_grad)
    mx_kind = "flux_grad" if mx_dom == "flux" and prof["mixed"]["grad"]["launches"] == 0 else mx_dom
    mx_bytes = kernel_bytes(mx_kind, nc, ne, 4)
    mx_ach = mx_bytes / (prof["mixed"][mx_dom]["ms_per_launch"] * 1e-3) / 1e9

    # the FP64 ALU ceiling: ncu-counted FP64 thread instructions per cell-update against
    # GB300's FP64 issue rate (2 per clock and SM) at the clock sampled during the timed runs
    instr = ncu_instr()
    sms = torch.cuda.get_device_properties(local).multi_processor_count
    mhz = clocks.get("sm_mhz") or measured_sm_max()
    fp64_peak = 2.0 * sms * mhz * 1e6
    fp64_ceiling = {"peak_instr_per_s": fp64_peak, "sms": sms, "sm_mhz": mhz,
                    "source": "profiles/ncu_instruction_counts_four_quadrant_2M.md"}
    for form, rate in (("fp64", value / world), ("mixed", value_mx / world)):
        n64 = instr.get((form, "fp64"))
        if n64:
            fp64_ceiling[form] = {"fp64_instr_per_cell_update": n64, "fp32_instr_per_cell_update":
                                  instr.get((form, "fp32")), "achieved_instr_per_s": n64 * rate,
                                  "frac": n64 * rate / fp64_peak}
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": K, "warmup": W,
        "ms_per_step": ms64 / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOAD, "cells": nc, "edges": ne, "form": "FP64 drop-in (headline); mixed below",
                   "l2": "no flush: the step's working set (~0.9 GB FP64, ~0.6 GB mixed) exceeds the 129 MB L2",
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        "roofline": {"bound": "hbm", "kernel": f"k_flux" if dom == "flux" else f"k_{dom}",
                     "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                     "traffic": traffic.get(f"{dom}_fp64"), "algorithmic_bytes_per_launch": dom_bytes,
                     "peak_kind": peak_kind,
                     "note": "FP64 kernels are bound by GB300's FP64 issue rate, not HBM"},
        "roofline_step": {"fp64": {"achieved": step_gbs, "frac": step_gbs / hbm, "bytes_per_cell_update": 580},
                          "mixed": {"achieved": step_gbs_mx, "frac": step_gbs_mx / hbm, "bytes_per_cell_update": 436,
                                    "dominant_kernel": f"k_{mx_kind}", "dominant_achieved": mx_ach,
                                    "dominant_frac": mx_ach / hbm,
                                    "dominant_traffic": traffic.get(f"{mx_kind}_mixed")},
                          "peak": hbm, "unit": "GB/s", "peak_kind": peak_kind},
        "fp64_alu_ceiling": fp64_ceiling,
        "mixed": {"value": value_mx, "unit": UNIT, "ms_per_step": msmx / K, "speedup_vs_fp64": ms64 / msmx,
                  "dtype": "f32 faces / f64 accumulate", "error_vs_fp64": err,
                  "error_vs_fp64_full_length": err_full},
        "adjoint_forward_ratio": adj["ratio_backward_over_forward"],
        "adjoint": adj,
        "kernels": prof,
        "e2e": {"value": world * nc / e2e_s, "unit": UNIT, "h2d_bytes_per_step": 32 * nc,
                "d2h_bytes_per_step": 32 * nc,
                "path": "cfd2d_set_state (pinned H2D) + cfd2d_step(1) + cfd2d_get_state (pinned D2H), FP64",
                "steps": Ke},
        "gpu_launches": K * (3 * 3 + 1),
        "clocks": clocks,
        "clocks_sustained": clocks_long,
    }
    if comb is not None:
        line["combined"] = comb
    if batch is not None:
        line["batched"] = batch
    if world == 1 and rank == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline_single()
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
