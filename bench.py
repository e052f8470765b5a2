#!/usr/bin/env python
"""Throughput of the per-step hot path of InterfaceAdvection.jl on GB300.

Headline workload (the mixed-precision Poisson rising bubble the metric is
quoted on): a 3D rising bubble at 256 cells per unit
length in a 1x2x1 domain (256x512x256 interior cells), periodic in x/z, walls
in y, one air bubble of radius 0.125 at (0.5,0.5,0.5) in water, density ratio
1000, viscosity ratio 100, Eötvös 10, Morton 1e-3 (gravity 1e-3 in grid units
sets the time scale).  One step = sim_step! = MPFMomStep! through the C-ABI
(RK2 predictor/corrector: CMOM momentum + VOF sweeps, viscosity, surface
tension, two projections, MPCFL), Poisson to L∞ residual 1e-8:
  * value    — mixed precision: FP32 V-cycles inside FP64 defect-correction FCG;
  * fp64_mg  — the same step with FP64 V-cycles (plain FP64 multigrid path).
Secondary line (`vof_only`): the VOF-only sphere in the LeVeque deformation field at 256³.

Metric: Mcell-steps/s = interior cells × steps / s.  All per-step inputs are
larger than L2 (fields of 274 MB each), so no flush is needed between steps.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--size 256] [--impl reference]
                  [--smoother halfsweep|blocked]
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
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
PTOL = 1e-8
B_RBGS_PER_CELL_F32 = 18   # one FP32 red-black half-sweep: L (12) + x read/write (4) + b (2) per cell
# DRAM bytes per cell of that launch from an ncu capture of the same kernel at 160x320x160
# (profiles/kernel_counters_bubble160.md), scaled by the cells of the launch
TRAFFIC_RBGS_PER_CELL_F32 = 22.7
TRAFFIC_VOF_BULK_PER_CELL = 31.1   # vof_bulk, ncu capture at 192³ (profiles/vof_bulk_sphere192.md)
B_BULK_PER_CELL = 33       # vof_bulk: read f, u_d, u0_d (24) + c̄ (1); write ρuf_d (8)
TK = {"vof_bulk": 0, "vof_cells": 1, "ustar": 2, "forcing": 3, "mg_vcycle": 4, "mg_transfer": 6, "krylov": 7,
      "vof_faces": 9, "momflux": 10, "momupdate": 11, "update_project": 12, "mg_fine_rbgs": 13, "nn_precond": 14,
      "mg_fine_first": 15, "other": 8}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--size", type=int, default=256, help="cells per unit length")
    ap.add_argument("--workload", default="bubble", choices=["bubble", "vof"])
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-seconds", type=float, default=20.0, help="bound of the CPU baseline sample")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-secondary", action="store_true", help="skip the FP64-MG and VOF-only side runs")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--smoother", default="halfsweep", choices=["halfsweep", "blocked"],
                    help="FP32 V-cycle smoother of the mixed solver (blocked: relaxation factor 1)")
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
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                       "-i", str(gpu_index), "-lms", "100"], stdout=subprocess.PIPE,
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
        sm, mx, pw, reasons = [], None, [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.strip().splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
                pw.append(float(parts[3]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm),
                "power_w_max": max(pw) if pw else None}


def measured_peak_hbm():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            return float(json.load(fh)["hbm_gbs"]), "of measured"
    except Exception:
        return 6800.0, "of fallback"


# ------------------------------------------------------------------------------------- workloads
def bubble_params(N):
    """Rising bubble in grid units: Eo = ρ g D²/σ = 10, Mo = g μ⁴/(ρ σ³) = 1e-3."""
    G, D, Eo, Mo = 1e-3, 0.25 * N, 10.0, 1e-3
    sigma = G * D * D / Eo
    mu = (Mo * sigma ** 3 / G) ** 0.25
    return dict(dims=(N, 2 * N, N), centre=(N / 2, N / 2, N / 2), radius=0.125 * N, G=G, sigma=sigma, mu=mu,
                lrho=1e-3, lmu=1e-2, perdir=(0, 2))


def make_bubble(N, poisson, device):
    import torch

    import intfadv as ia
    p = bubble_params(N)
    c, r = p["centre"], p["radius"]
    sdf = lambda x: r - torch.sqrt((x[0] - c[0]) ** 2 + (x[1] - c[1]) ** 2 + (x[2] - c[2]) ** 2)
    return ia.TwoPhaseSimulation(p["dims"], (0.0, 0.0, 0.0), float(N), perdir=p["perdir"], λρ=p["lrho"],
                                 λμ=p["lmu"], ν=p["mu"], η=p["sigma"], g=(0.0, -p["G"], 0.0), InterfaceSDF=sdf,
                                 poisson=poisson, poisson_tol=PTOL, poisson_itmx=400, device=device)


# ------------------------------------------------------------------------------------- CPU side
def cpu_bubble_baseline(N, seconds):
    """The oracle (C++ OpenMP restatement; Jacobi-PCG Poisson) on the same bubble at reduced size."""
    import numpy as np

    from oracle.sim import OracleSim
    p = bubble_params(N)
    c, r = p["centre"], p["radius"]
    sdf = lambda x: r - np.sqrt((x[0] - c[0]) ** 2 + (x[1] - c[1]) ** 2 + (x[2] - c[2]) ** 2)
    orc = OracleSim(p["dims"], (0.0, 0.0, 0.0), sdf=sdf, perdir=p["perdir"], lrho=p["lrho"], lmu=p["lmu"],
                    ν=p["mu"], g=(0.0, -p["G"], 0.0), eta=p["sigma"], ptol=PTOL, pitmx=20000)
    cells = p["dims"][0] * p["dims"][1] * p["dims"][2]
    steps, t0 = 0, time.perf_counter()
    while True:
        orc.step()
        steps += 1
        el = time.perf_counter() - t0
        if el >= seconds or steps >= 50:
            break
    cores = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
    return {"value": cells * steps / el / 1e6, "unit": METRIC, "cores": cores, "kind": "port",
            "sample": f"{steps} MPFMomStep! of the rising bubble at {p['dims'][0]}x{p['dims'][1]}x{p['dims'][2]} "
                      f"in {el:.1f} s (oracle, OpenMP, Jacobi-PCG to L-inf 1e-8)"}


def cpu_vof_baseline(N, seconds):
    import numpy as np

    from intfadv import fields, workloads
    from oracle import pyoracle as O
    ng = (N + 2,) * 3
    sdf = workloads.sphere_sdf((0.35, 0.35, 0.35), 0.15, N)
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
    steps, t0 = 0, time.perf_counter()
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


# ------------------------------------------------------------------------------------- GPU side
def timed_steps(sim, steps, barrier, sample_clocks, local_rank):
    import torch

    import intfadv as ia
    clocks = ClockSampler(local_rank) if sample_clocks else None
    barrier()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    its, res = [], []
    e0.record()
    for _ in range(steps):
        st = ia.sim_step(sim)
        its.append(st.poisson_iters[0] + st.poisson_iters[1])
        res.append(max(st.poisson_resid[0], st.poisson_resid[1]))
    e1.record()
    torch.cuda.synchronize()
    barrier()
    return e0.elapsed_time(e1), its, res, (clocks.stop() if clocks else None)


def kernel_times(sim, steps):
    import intfadv as ia
    T, Lc = (C.c_double * 16)(), (C.c_int64 * 16)()
    sim.handle.call("ia_timing", 1, None, None, 0)
    for _ in range(steps):
        ia.sim_step(sim)
    sim.handle.call("ia_timing", 0, T, Lc, 16)
    return {k: {"ms_per_step": T[i] / steps, "launches_per_step": Lc[i] / steps,
                "avg_launch_ms": (T[i] / Lc[i]) if Lc[i] else None} for k, i in TK.items()}


def run_bubble(args, world, local_rank):
    import torch

    import intfadv as ia
    from intfadv import _lib
    dev = torch.device("cuda", local_rank)
    N = args.size
    cells = N * 2 * N * N
    barrier = (lambda: torch.distributed.barrier()) if world > 1 else (lambda: None)
    L = _lib.load()
    sim = make_bubble(N, "mixed", dev)
    # the blocked smoother applies at relaxation factor 1 only
    ia.set_smoother(sim.handle, args.smoother, 1.0 if args.smoother == "blocked" else None)
    for _ in range(args.warmup):
        ia.sim_step(sim)
    n0 = L.ia_launch_count()
    ms, its, res, clk = timed_steps(sim, args.steps, barrier, True, local_rank)
    launches = L.ia_launch_count() - n0
    if world > 1:
        t = torch.tensor([ms], device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = float(t.item())
    value = world * cells * args.steps / (ms / 1e3) / 1e6
    kt = kernel_times(sim, max(2, min(args.steps, 3)))
    peak, peak_kind = measured_peak_hbm()
    fine = kt["mg_fine_rbgs"]
    roof = None
    if fine["avg_launch_ms"]:
        b = B_RBGS_PER_CELL_F32 * cells
        ach = b / (fine["avg_launch_ms"] / 1e3) / 1e9
        roof = {"bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s", "frac": ach / peak,
                "traffic": TRAFFIC_RBGS_PER_CELL_F32 * cells,
                "traffic_note": "ncu dram bytes of the finest-level launch at 160x320x160 (22.7 B/cell), scaled",
                "kernel": "rbgs_pair_k<float> (finest-level red-black Gauss-Seidel half-sweep, mixed V-cycle)",
                "peak_kind": peak_kind, "bytes_per_launch": b, "avg_launch_ms": fine["avg_launch_ms"]}
    e2e = None
    if not args.no_e2e:
        # state kept on the host: each step uploads u and f from pinned memory, runs the step through the
        # public API and downloads u, f, p
        fl, it = sim.flow, sim.intf
        # pinned host state in the fields' own (column-major) layout, so that each copy is one DMA
        pinned = lambda t: torch.empty_strided(t.shape, t.stride(), dtype=t.dtype, pin_memory=True)
        hu = pinned(fl.u).copy_(fl.u)
        hf = pinned(it.f).copy_(it.f)
        hp = pinned(fl.p)
        e_steps = max(2, min(args.steps, 4))
        torch.cuda.synchronize()
        barrier()
        t0 = time.perf_counter()
        # the link copies ~200 GB/s one way and ~340 GB/s both ways at once: the downloads of f and p
        # run on a second stream, beside the next step's upload of u.  Every copy still follows what
        # it depends on: u is uploaded after its download (same stream), f after its download and the
        # next step's kernels after the download of p (the f upload waits for the second stream)
        main, side = torch.cuda.current_stream(), torch.cuda.Stream()
        for _ in range(e_steps):
            fl.u.copy_(hu, non_blocking=True)
            main.wait_stream(side)
            it.f.copy_(hf, non_blocking=True)
            ia.sim_step(sim)
            hu.copy_(fl.u, non_blocking=True)
            side.wait_stream(main)
            with torch.cuda.stream(side):
                hf.copy_(it.f, non_blocking=True)
                hp.copy_(fl.p, non_blocking=True)
        torch.cuda.synchronize()
        barrier()
        el = time.perf_counter() - t0
        nb = fl.u.numel() * 8 + it.f.numel() * 8
        e2e = {"value": world * cells * e_steps / el / 1e6, "unit": METRIC, "h2d_bytes_per_step": nb,
               "d2h_bytes_per_step": nb + fl.p.numel() * 8 + C.sizeof(_lib.Status),
               "note": "state on the host: u, f uploaded and u, f, p downloaded every step around sim_step"}
    out = {"value": value, "ms_per_step": ms / args.steps, "clocks": clk, "launches": launches, "roofline": roof,
           "kernels": kt, "poisson_iters_per_step": statistics.mean(its), "max_resid": max(res), "e2e": e2e,
           "dt": sim.flow.Δt[-1]}
    del sim
    torch.cuda.empty_cache()
    if not args.no_secondary:
        ref = make_bubble(N, "fp64", dev)
        for _ in range(max(1, args.warmup - 1)):
            ia.sim_step(ref)
        k = max(2, min(args.steps, 5))
        ms2, its2, res2, _ = timed_steps(ref, k, barrier, False, local_rank)
        out["fp64_mg"] = {"value": world * cells * k / (ms2 / 1e3) / 1e6, "ms_per_step": ms2 / k,
                          "poisson_iters_per_step": statistics.mean(its2), "max_resid": max(res2),
                          "mg_vcycle_ms_per_step": kernel_times(ref, 2)["mg_vcycle"]["ms_per_step"]}
        out["speedup_vs_fp64_mg"] = value / out["fp64_mg"]["value"]
        del ref
        torch.cuda.empty_cache()
        from intfadv import learned
        if os.path.exists(learned.WEIGHTS):
            # learned preconditioner: the same step with the inner FCG preconditioned by V-cycle + net
            lrn = make_bubble(N, "learned", dev)
            for _ in range(max(1, args.warmup - 1)):
                ia.sim_step(lrn)
            k = max(2, min(args.steps, 5))
            st0 = ia.poisson_stats(lrn.handle)
            ms3, its3, res3, _ = timed_steps(lrn, k, barrier, False, local_rank)
            st1 = ia.poisson_stats(lrn.handle)
            kt3 = kernel_times(lrn, 2)
            out["learned_hybrid"] = {
                "value": world * cells * k / (ms3 / 1e3) / 1e6, "ms_per_step": ms3 / k,
                "poisson_iters_per_step": statistics.mean(its3), "max_resid": max(res3),
                "fallbacks": st1["fallbacks"] - st0["fallbacks"],
                "net_ms_per_step": kt3["nn_precond"]["ms_per_step"],
                "mg_vcycle_ms_per_step": kt3["mg_vcycle"]["ms_per_step"],
                "weights": learned.load_params()[1]}
            del lrn
            torch.cuda.empty_cache()
    return out


def run_vof(args, world, local_rank, steps=200):
    import torch

    import intfadv as ia
    from intfadv import workloads
    dev = torch.device("cuda", local_rank)
    N = args.size
    intf = ia.cVOF((N, N, N), InterfaceSDF=workloads.sphere_sdf((0.35, 0.35, 0.35), 0.15, N), device=dev)
    U = workloads.deformation_field(N, device=dev)
    dt = 1.0 / (4 * N)
    u1 = U * workloads.deformation_time_factor(0.0)
    u2 = torch.empty_like(U)
    m0 = intf.mass()
    s = [0]

    def one():
        nonlocal u1, u2
        s[0] += 1
        torch.mul(U, workloads.deformation_time_factor(s[0] * dt), out=u2)
        st = ia.advect_vof_raw(intf, intf.f, u1, u2, dt, s[0])
        if st.code not in (0, 100):
            raise RuntimeError(f"advect status {st.code}")
        u1, u2 = u2, u1

    for _ in range(5):
        one()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(steps):
        one()
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    T, Lc = (C.c_double * 16)(), (C.c_int64 * 16)()
    intf.handle.call("ia_timing", 1, None, None, 0)
    for _ in range(10):
        one()
    intf.handle.call("ia_timing", 0, T, Lc, 16)
    bulk_ms = T[0] / max(1, Lc[0])
    peak, peak_kind = measured_peak_hbm()
    ach = B_BULK_PER_CELL * N ** 3 / (bulk_ms / 1e3) / 1e9
    return {"workload": f"VOF-only sphere r=0.15, LeVeque deformation, {N}^3, CFL 0.5",
            "value": world * N ** 3 * steps / (ms / 1e3) / 1e6, "ms_per_step": ms / steps,
            "mass_drift": abs(intf.mass() - m0) / m0,
            "roofline": {"bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s", "frac": ach / peak,
                         "traffic": TRAFFIC_VOF_BULK_PER_CELL * N ** 3,
                         "traffic_note": "ncu dram bytes of one launch at 192^3 (31.1 B/cell), scaled",
                         "kernel": "vof_bulk", "peak_kind": peak_kind, "avg_launch_ms": bulk_ms}}


def main():
    args = parse()
    rank, world, local_rank = dist_env()
    if world > 1:
        import torch
        torch.distributed.init_process_group("nccl" if args.impl == "ours" else "gloo")
    N = args.size
    p = bubble_params(N)
    cfg = {"workload": f"3D rising bubble {p['dims'][0]}x{p['dims'][1]}x{p['dims'][2]} (1x2x1, periodic x/z, "
                       f"walls y), r=0.125 at (0.5,0.5,0.5), density ratio 1000, viscosity ratio 100, Eo=10, "
                       f"Mo=1e-3; MPFMomStep! with Poisson to L-inf residual {PTOL}",
           "grid": list(p["dims"]), "poisson": "FP32 V-cycles + FP64 defect-correction FCG (mixed)",
           "l2_flush": "inputs larger than L2 (each field 274 MB)", "parallelism": f"replicas x{world}"}
    if args.workload == "vof":
        cfg = {"workload": f"VOF-only sphere r=0.15, LeVeque deformation, {N}^3, CFL 0.5", "grid": [N, N, N],
               "parallelism": f"replicas x{world}"}
    if args.impl == "reference":
        if rank != 0:
            return
        if args.workload == "vof":
            base = cpu_vof_baseline(N, args.cpu_seconds)
        else:
            base = cpu_bubble_baseline(max(16, N // 4), args.cpu_seconds)
        line = {"impl": "reference", "metric": METRIC, "value": base["value"], "unit": METRIC, "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": None, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": cfg,
                "cpu_baseline": base,
                "e2e": {"value": base["value"], "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
                "note": "the reference is Julia (no toolchain here); this arm times the C++ OpenMP restatement"}
        print(json.dumps(line), flush=True)
        return
    import torch
    torch.cuda.set_device(local_rank)
    if args.workload == "vof":
        res = run_vof(args, world, local_rank)
        if rank == 0:
            cpu = None if args.no_cpu_baseline else cpu_vof_baseline(N, args.cpu_seconds)
            print(json.dumps({"metric": METRIC, "value": res["value"], "unit": METRIC, "n_gpus": world,
                              "steps": 200, "warmup": 5, "ms_per_step": res["ms_per_step"], "higher_is_better": True,
                              "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                              "config": cfg, "roofline": res["roofline"], "cpu_baseline": cpu}), flush=True)
        return
    res = run_bubble(args, world, local_rank)
    if rank == 0:
        vof = None if args.no_secondary else run_vof(args, 1, local_rank)
        cpu = None if args.no_cpu_baseline else cpu_bubble_baseline(max(16, N // 4), args.cpu_seconds)
        line = {"metric": METRIC, "value": res["value"], "unit": METRIC, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": res["ms_per_step"], "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": cfg,
                "clocks": res["clocks"], "e2e": res["e2e"], "gpu_launches": res["launches"],
                "roofline": res["roofline"], "cpu_baseline": cpu,
                "fp64_mg": res.get("fp64_mg"), "speedup_vs_fp64_mg": res.get("speedup_vs_fp64_mg"),
                "learned_hybrid": res.get("learned_hybrid"),
                "poisson_iters_per_step": res["poisson_iters_per_step"], "max_poisson_resid": res["max_resid"],
                "kernels_ms_per_step": {k: v["ms_per_step"] for k, v in res["kernels"].items()},
                "vof_only": vof}
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
