#!/usr/bin/env python
"""Throughput of the per-step hot path on GB300.

Workload (BASELINE config "plain VOF advection only, GPU"): a sphere of radius
0.15 centred at (0.35,0.35,0.35) in the unit cube at 256³, FP64 fractions,
advected by the LeVeque 3D deformation field u = U(x) cos(πt/3) (discretely
divergence-free faces) at CFL 0.5 (δt = 1/(4N)).  One step = write the
prescribed face velocity of t_{n+1} (u⁰ keeps t_n) + advect!(flow, intf)
through the C-ABI (three direction-split sweeps with status read-back).

Metric: Mcell-steps/s (interior cells × steps / s).  Inputs exceed L2
(f 137 MB, velocities 2 × 412 MB), so no explicit flush is needed between
steps.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--size 256] [--impl reference]
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import math
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "interfaceadvection.jl_gb300")
for _p in (ROOT, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "Mcell-steps/s"
DevStatusBytes = C.c_byte * 128   # the library's device status block read back once per call
B_BULK_PER_CELL = 41    # vof_bulk: read f, u_d, u0_d (24) + c̄ (1); write f, ρuf_d (16)


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=400)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--size", type=int, default=256)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-seconds", type=float, default=15.0, help="bound of the CPU baseline sample")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-quality", action="store_true", help="skip the 64^3 full-period accuracy run")
    ap.add_argument("--no-e2e", action="store_true", help="skip the host-fed end-to-end pass")
    return ap.parse_args()


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.p = None
        self.gpu = gpu_index
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                       "-i", str(gpu_index), "-lms", "200"], stdout=subprocess.PIPE,
                                      stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.p = None

    def stop(self):
        if self.p is None:
            return None
        self.p.terminate()
        try:
            out, _ = self.p.communicate(timeout=5)
        except Exception:
            self.p.kill()
            out = ""
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.strip().splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            p = json.load(fh)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


# ----------------------------------------------------------------------------------- CPU side
def run_cpu_baseline(N, seconds, threads=None):
    """Time the oracle (C++ OpenMP restatement) on a bounded number of steps of the same workload."""
    import ctypes as C

    import numpy as np
    import torch

    from intfadv import fields, workloads
    from oracle import pyoracle as O

    if threads:
        os.environ["OMP_NUM_THREADS"] = str(threads)
    ng = (N + 2,) * 3
    sdf = workloads.sphere_sdf((0.35, 0.35, 0.35), 0.15, N)
    # initial fraction via the oracle's applyVOF! on host SDF samples
    xc = fields.cell_coords(ng, device="cpu")
    samples = []
    for k in range(7):
        x = [c.clone() for c in xc]
        if k > 0:
            d, s = (k - 1) // 2, (0.01 if (k - 1) % 2 == 0 else -0.01)
            x[d] = x[d] + s
        samples.append(np.asfortranarray(fields.evaluate(sdf, x, ng, device="cpu").numpy()))
    f = O.zeros(ng)
    f[...] = 1.0
    al, nh = O.zeros(ng), O.zeros(ng + (3,))
    arr = (C.c_void_p * 7)(*[s.ctypes.data for s in samples])
    g = O.grid(ng)
    O.lib().orc_apply_vof(C.byref(g), O.ptr(f), O.ptr(al), O.ptr(nh), arr)
    O.lib().orc_bcf(C.byref(g), O.ptr(f))
    del samples
    U = np.asfortranarray(workloads.deformation_field(N, device="cpu").numpy())
    dt = 1.0 / (4 * N)
    u1 = np.asfortranarray(U * workloads.deformation_time_factor(0.0))
    u2 = O.zeros(U.shape)
    steps = 0
    t0 = time.perf_counter()
    while True:
        np.multiply(U, workloads.deformation_time_factor((steps + 1) * dt), out=u2)
        O.advect_vof(f, u1, u2, dt, O.dir_order(steps + 1, 3))
        u1, u2 = u2, u1
        steps += 1
        el = time.perf_counter() - t0
        if el >= seconds or steps >= 200:
            break
    cores = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
    return {"value": N ** 3 * steps / el / 1e6, "unit": METRIC, "cores": cores, "kind": "port",
            "sample": f"{steps} step(s) of the {N}^3 deformation advect! in {el:.1f} s (oracle, OpenMP)"}


# ----------------------------------------------------------------------------------- GPU side
def quality_run(N=64):
    """Full period T=3 at N³ (CFL 0.5): L1 shape error and mass drift."""
    import numpy as np
    import torch

    import intfadv as ia
    from intfadv import workloads
    intf = ia.cVOF((N, N, N), InterfaceSDF=workloads.sphere_sdf((0.35, 0.35, 0.35), 0.15, N))
    f0 = intf.f.clone()
    m0 = intf.mass()
    U = workloads.deformation_field(N)
    dt = 1.0 / (4 * N)
    nsteps = int(round(3.0 / dt))
    u1 = U * workloads.deformation_time_factor(0.0)
    u2 = torch.empty_like(U)
    for s in range(1, nsteps + 1):
        torch.mul(U, workloads.deformation_time_factor(s * dt), out=u2)
        st = ia.advect_vof_raw(intf, intf.f, u1, u2, dt, s)
        if st.code not in (0, 100):
            raise RuntimeError(f"advect status {st.code}")
        u1, u2 = u2, u1
    h3 = (1.0 / N) ** 3
    inner = (slice(1, -1),) * 3
    err = float((intf.f[inner] - f0[inner]).abs().sum()) * h3
    return {"grid": N, "steps": nsteps, "shape_error_L1": err, "mass_drift": abs(intf.mass() - m0) / m0}


def run_gpu(args, rank, world, local_rank):
    import numpy as np
    import torch

    import intfadv as ia
    from intfadv import _lib, workloads

    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    N = args.size
    intf = ia.cVOF((N, N, N), InterfaceSDF=workloads.sphere_sdf((0.35, 0.35, 0.35), 0.15, N), device=dev)
    U = workloads.deformation_field(N, device=dev)
    dt = 1.0 / (4 * N)
    u1 = U * workloads.deformation_time_factor(0.0)
    u2 = torch.empty_like(U)
    m0 = intf.mass()
    step = [0]
    L = _lib.load()

    def one_step():
        step[0] += 1
        s = step[0]
        torch.mul(U, workloads.deformation_time_factor(s * dt), out=u2)
        st = ia.advect_vof_raw(intf, intf.f, u1, u2, dt, s)
        if st.code not in (0, 100):
            raise RuntimeError(f"advect status {st.code}")
        return st

    def swap():
        nonlocal u1, u2
        u1, u2 = u2, u1

    for _ in range(args.warmup):
        one_step()
        swap()
    barrier = (lambda: torch.distributed.barrier()) if world > 1 else (lambda: None)
    # ---- timed region (device-resident inputs)
    clocks = ClockSampler(local_rank)
    barrier()
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record()
    for _ in range(args.steps):
        one_step()
        swap()
    ev1.record()
    torch.cuda.synchronize()
    barrier()
    clk = clocks.stop()
    ms = ev0.elapsed_time(ev1)
    if world > 1:
        t = torch.tensor([ms], device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = float(t.item())
    ms_step = ms / args.steps
    value = world * N ** 3 * args.steps / (ms / 1e3) / 1e6
    launches = args.steps * (1 + 3 * 4)          # status reset + 3 × (bulk + faces + cells + scatter)

    # ---- per-kernel durations (event instrumentation inside the library, same stream)
    T = (C.c_double * 16)()
    Lc = (C.c_int64 * 16)()
    intf.handle.call("ia_timing", 1, None, None, 0)
    for _ in range(max(3, min(args.steps, 10))):
        one_step()
        swap()
    intf.handle.call("ia_timing", 0, T, Lc, 16)
    bulk_ms = T[0] / max(1, Lc[0])
    list_ms = (T[1] + T[9]) / max(1, Lc[1])
    peak, peak_kind = measured_peaks()
    bytes_launch = B_BULK_PER_CELL * N ** 3
    achieved = bytes_launch / (bulk_ms / 1e3) / 1e9

    # ---- end to end through the public API with host buffers
    if args.no_e2e:
        return {"value": value, "ms_per_step": ms_step, "clocks": clk, "launches": launches,
                "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                             "frac": achieved / peak, "traffic": None, "kernel": "vof_bulk"},
                "e2e": None, "mass_drift_after_bench": abs(intf.mass() - m0) / m0}
    hostU = torch.empty(U.shape, dtype=torch.float64, pin_memory=True)
    hostU.copy_(U)
    torch.cuda.synchronize()
    e_steps = max(3, min(args.steps, 10))
    barrier()
    t0 = time.perf_counter()
    for _ in range(e_steps):
        step[0] += 1
        s = step[0]
        u2.copy_(hostU, non_blocking=True)                         # H2D: the step's prescribed velocity
        u2.mul_(workloads.deformation_time_factor(s * dt))
        st = ia.advect_vof_raw(intf, intf.f, u1, u2, dt, s)          # status D2H inside the call
        if st.code not in (0, 100):
            raise RuntimeError(f"advect status {st.code}")
        swap()
    torch.cuda.synchronize()
    barrier()
    e_el = time.perf_counter() - t0
    e2e = world * N ** 3 * e_steps / e_el / 1e6
    h2d = U.numel() * 8
    d2h = C.sizeof(_lib.Status) + C.sizeof(DevStatusBytes)
    drift = abs(intf.mass() - m0) / m0
    return {
        "value": value, "ms_per_step": ms_step, "clocks": clk, "launches": launches,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": None, "kernel": "vof_bulk", "peak_kind": peak_kind,
                     "bytes_per_launch": bytes_launch, "avg_launch_ms": bulk_ms, "list_avg_launch_ms": list_ms},
        "e2e": {"value": e2e, "unit": METRIC, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "mass_drift_after_bench": drift,
    }


def main():
    args = parse()
    rank, world, local_rank = dist_env()
    if world > 1:
        import torch
        torch.distributed.init_process_group("nccl" if args.impl == "ours" else "gloo")
    N = args.size
    cfg = {"workload": f"VOF-only sphere r=0.15 @ (0.35,0.35,0.35), LeVeque deformation, {N}^3, CFL 0.5",
           "grid": [N, N, N], "dtype_fractions": "f64", "l2_flush": "inputs larger than L2 (f 137 MB, u 2x412 MB)",
           "parallelism": f"replicas x{world}"}
    if args.impl == "reference":
        if rank != 0:
            return
        base = run_cpu_baseline(N, args.cpu_seconds)
        line = {"impl": "reference", "metric": METRIC, "value": base["value"], "unit": METRIC, "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": N ** 3 / base["value"] / 1e3,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                "data": "synthetic", "config": cfg,
                "cpu_baseline": base,
                "e2e": {"value": base["value"], "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
                "note": "reference is Julia (not runnable here); arm times the C++ OpenMP restatement (oracle)"}
        print(json.dumps(line), flush=True)
        return
    res = run_gpu(args, rank, world, local_rank)
    if rank == 0:
        cpu = None if args.no_cpu_baseline else run_cpu_baseline(min(N, 256), args.cpu_seconds)
        qual = None if args.no_quality else quality_run(64)
        line = {"metric": METRIC, "value": res["value"], "unit": METRIC, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": res["ms_per_step"], "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": cfg,
                "clocks": res["clocks"], "e2e": res["e2e"], "gpu_launches": res["launches"],
                "roofline": res["roofline"], "cpu_baseline": cpu, "quality": qual,
                "mass_drift_after_bench": res["mass_drift_after_bench"]}
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
