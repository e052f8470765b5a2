#!/usr/bin/env python
"""Throughput of the per-step hot path of InterfaceAdvection.jl on GB300.

Headline workload (the mixed-precision rising bubble the metric is quoted on): a 3D rising bubble at
256 cells per unit length in a 1x2x1 domain (256x512x256 interior cells), periodic in x/z, walls in y,
one air bubble of radius 0.125 at (0.5,0.5,0.5) in water, density ratio 1000, viscosity ratio 100,
Eötvös 10, Morton 1e-3 (gravity 1e-3 in grid units sets the time scale).  One step = sim_step! =
MPFMomStep! through the C-ABI (RK2 predictor/corrector: CMOM momentum + VOF sweeps, viscosity, surface
tension, two projections, MPCFL), Poisson to an L∞ residual of 1e-8 of the dt-scaled system:
  * value          — mixed precision: FP32 V-cycles inside FP64 defect-correction FCG, momentum
                     arithmetic on FP32 pairs (float-float), VOF/PLIC and fields FP64;
  * fp64_mg        — the plain FP64 path: FP64 V-cycles, FP64 momentum arithmetic;
  * fp64_mg_ff     — FP64 V-cycles with the float-float momentum (separates the two gains);
  * learned_hybrid — the mixed path with the inner FCG preconditioned by V-cycle + conv net.
Further measurements in the same line: the headline's mass drift and a steps-matched FP64-oracle
check on a small case, the VOF-only sphere over its full period (C2), a late-time window of the rising
bubble (C3, steps 480-500 from rest), the 512³ bubble swarm (C5), and the oracle on the host cores.

Metric: Mcell-steps/s = interior cells × steps / s.  All per-step inputs are larger than L2 (fields of
274 MB each), so no flush is needed between steps.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--size 256] [--impl reference] [--quick]
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
TK = {"vof_bulk": 0, "vof_cells": 1, "ustar": 2, "forcing": 3, "mg_vcycle": 4, "mg_transfer": 6, "krylov": 7,
      "vof_faces": 9, "momflux": 10, "momupdate": 11, "update_project": 12, "mg_fine_rbgs": 13, "nn_precond": 14,
      "mg_fine_first": 15, "other": 8}

# Roofline candidates: timing family, algorithmic bytes per interior cell of one launch (each field a
# fused launch must read once and write once), the DRAM bytes per cell ncu measured for one launch of
# that kernel, and the kernel name.  The DRAM figures come from single-launch captures at 160x320x160
# (momentum kernels, smoother) and 192³ (vof_bulk), scaled to the cells of a launch here.
ROOF = {
    "momflux": dict(bytes=64, traffic=None, kernel="momflux (CMOM face fluxes of one sweep: read uStar 3, "
                                                   "ρuf_j, f_old; write Φ 3)"),
    # the first two of a stage's three updates also write the next sweep's uStar (24 B) from the new
    # fractions (8 B): 113, 145 and 145 B per cell, 134.3 on average per launch
    "momupdate": dict(bytes=(113 + 2 * 145) / 3, traffic=None,
                      kernel="momupdate (ρu += δt(Φ(I)-Φ(I+δj)+uOld ϕ(ρ̄∂ⱼuⱼ)); in sweeps 1-2 also uStar of the next sweep)"),
    # a finest-level half-sweep runs as one launch or, in the y-slab wavefront, as one launch per slab:
    # its unit is the whole-level half-sweep, 5 per V-cycle at nu = (2, 2) with over-relaxation (2 in the
    # pre-smoothing after the fused first one, 3 in the post-smoothing)
    "mg_fine_rbgs": dict(bytes=18, traffic=15.0, per_vcycle=5,
                         kernel="rbgs_pair_k<float> (finest-level red-black half-sweep)"),
}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--size", type=int, default=256, help="cells per unit length")
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--quick", action="store_true", help="headline only (no side runs, CPU baseline, e2e)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-secondary", action="store_true", help="skip the side runs")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--ref-steps", type=int, default=2, help="oracle steps timed by the reference arm")
    ap.add_argument("--no-coef16", action="store_true",
                    help="FP32 face coefficients in the finest-level smoother of the mixed V-cycle")
    ap.add_argument("--slab-rows", type=int, default=None,
                    help="rows per slab of the finest-level smoothing wavefront (0: whole-level half-sweeps; "
                         "default: the library's, from the L2 size)")
    ap.add_argument("--fine-nu", default=None,
                    help="pre,post smoothings of the finest V-cycle level only (default: the library's)")
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
def make_bubble(N, poisson, device, arith="default"):
    import torch

    import intfadv as ia
    from intfadv import workloads
    p = workloads.bubble_params(N)
    c, r = p["centre"], p["radius"]
    sdf = lambda x: r - torch.sqrt((x[0] - c[0]) ** 2 + (x[1] - c[1]) ** 2 + (x[2] - c[2]) ** 2)
    return ia.TwoPhaseSimulation(p["dims"], (0.0, 0.0, 0.0), float(N), perdir=p["perdir"], λρ=p["lrho"],
                                 λμ=p["lmu"], ν=p["mu"], η=p["sigma"], g=(0.0, -p["G"], 0.0), InterfaceSDF=sdf,
                                 poisson=poisson, poisson_tol=PTOL, poisson_itmx=400, device=device,
                                 momentum_arith=arith)


def make_swarm(N, poisson, device, arith="default"):
    import intfadv as ia
    from intfadv import learned, workloads
    bubbles = workloads.swarm_layout(N=N)
    D = 2 * max(r for _, r in bubbles)
    p = workloads.bubble_params(N, Eo=5.0, D=D)
    return ia.TwoPhaseSimulation((N, N, N), (0.0, 0.0, 0.0), float(N), perdir=(0, 2), λρ=p["lrho"], λμ=p["lmu"],
                                 ν=p["mu"], η=p["sigma"], g=(0.0, -p["G"], 0.0),
                                 InterfaceSDF=learned.bubbles_sdf(bubbles), poisson=poisson, poisson_tol=PTOL,
                                 poisson_itmx=400, device=device, momentum_arith=arith)


# ------------------------------------------------------------------------------------- CPU side
def _omp_threads(n):
    """Set the OpenMP thread count of the oracle (libgomp is shared by the process)."""
    try:
        C.CDLL("libgomp.so.1").omp_set_num_threads(int(n))
    except OSError:
        pass


def cpu_bubble(N, steps, threads=None):
    """The oracle (C++ OpenMP restatement; multigrid-preconditioned CG in the role of WaterLily's
    MultiLevelPoisson) on the rising bubble at N cells per unit length: one MPFMomStep! per step,
    Poisson to the same L∞ tolerance."""
    import numpy as np

    from intfadv import workloads
    from oracle.sim import OracleSim
    cores = threads or (os.cpu_count() or 1)
    _omp_threads(cores)
    p = workloads.bubble_params(N)
    c, r = p["centre"], p["radius"]
    sdf = lambda x: r - np.sqrt((x[0] - c[0]) ** 2 + (x[1] - c[1]) ** 2 + (x[2] - c[2]) ** 2)
    t0 = time.perf_counter()
    orc = OracleSim(p["dims"], (0.0, 0.0, 0.0), sdf=sdf, perdir=p["perdir"], lrho=p["lrho"], lmu=p["lmu"],
                    ν=p["mu"], g=(0.0, -p["G"], 0.0), eta=p["sigma"], ptol=PTOL, pitmx=2000, psolver="mg")
    t_init = time.perf_counter() - t0
    times, iters = [], []
    for _ in range(steps):
        t0 = time.perf_counter()
        orc.step()
        times.append(time.perf_counter() - t0)
        iters.append(int(orc.s.piters))
    _omp_threads(os.cpu_count() or 1)
    cells = p["dims"][0] * p["dims"][1] * p["dims"][2]
    el = sum(times)
    dims = "x".join(str(d) for d in p["dims"])
    return {"value": cells * steps / el / 1e6, "unit": METRIC, "cores": cores, "kind": "port",
            "sample": f"{steps} MPFMomStep! of the rising bubble at {dims} in {el:.1f} s after {t_init:.1f} s of "
                      f"set-up (oracle: C++ OpenMP, {cores} threads; multigrid-preconditioned CG to L-inf {PTOL}, "
                      f"last solve {iters[-1]} iterations)",
            "step_s": times, "grid": list(p["dims"])}


def cpu_vof(N, steps):
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
    t0 = time.perf_counter()
    for s in range(steps):
        np.multiply(U, workloads.deformation_time_factor((s + 1) * dt), out=u2)
        O.advect_vof(f, u1, u2, dt, O.dir_order(s + 1, 3))
        u1, u2 = u2, u1
    el = time.perf_counter() - t0
    return {"value": N ** 3 * steps / el / 1e6, "unit": METRIC, "cores": os.cpu_count() or 1, "kind": "port",
            "sample": f"{steps} advect! steps of the {N}^3 deformation sphere in {el:.1f} s (oracle, OpenMP)"}


def oracle_check(device, N=24, steps=5):
    """A steps-matched FP64-oracle comparison on a small rising bubble (the headline's physics at
    N cells per unit length, N x 2N x N, the headline's solver and arithmetic); both sides solve the
    pressure to L-inf 1e-12 so that the comparison measures the step, not the solver tolerance."""
    import numpy as np
    import torch

    import intfadv as ia
    from intfadv import workloads
    from oracle.sim import OracleSim
    p = workloads.bubble_params(N)
    c, r = p["centre"], p["radius"]
    sdf_t = lambda x: r - torch.sqrt((x[0] - c[0]) ** 2 + (x[1] - c[1]) ** 2 + (x[2] - c[2]) ** 2)
    sdf_n = lambda x: r - np.sqrt((x[0] - c[0]) ** 2 + (x[1] - c[1]) ** 2 + (x[2] - c[2]) ** 2)
    kw = dict(perdir=p["perdir"], ν=p["mu"], g=(0.0, -p["G"], 0.0))
    sim = ia.TwoPhaseSimulation(p["dims"], (0.0, 0.0, 0.0), float(N), λρ=p["lrho"], λμ=p["lmu"], η=p["sigma"],
                                InterfaceSDF=sdf_t, poisson="mixed", poisson_tol=1e-12, poisson_itmx=500,
                                device=device, **kw)
    orc = OracleSim(p["dims"], (0.0, 0.0, 0.0), sdf=sdf_n, lrho=p["lrho"], lmu=p["lmu"], eta=p["sigma"], ptol=1e-12,
                    pitmx=5000, psolver="mg", **kw)
    for _ in range(steps):
        ia.sim_step(sim)
        orc.step()
    torch.cuda.synchronize()
    ef = float(np.abs(sim.intf.f.cpu().numpy() - orc.f).max())
    eu = float(np.abs(sim.flow.u.cpu().numpy() - orc.u).max()) / float(np.abs(orc.u).max())
    return {"case": f"rising bubble {N}x{2 * N}x{N} (the headline's physics), {steps} steps, mixed solver with "
                    f"float-float momentum vs the FP64 oracle, both to L-inf 1e-12",
            "max_abs_err_f": ef, "max_rel_err_u": eu}


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
    v0 = ia.poisson_stats(sim.handle)["vcycles"]
    sim.handle.call("ia_timing", 1, None, None, 0)
    for _ in range(steps):
        ia.sim_step(sim)
    sim.handle.call("ia_timing", 0, T, Lc, 16)
    vc = (ia.poisson_stats(sim.handle)["vcycles"] - v0) / steps
    out = {k: {"ms_per_step": T[i] / steps, "launches_per_step": Lc[i] / steps,
               "avg_launch_ms": (T[i] / Lc[i]) if Lc[i] else None} for k, i in TK.items()}
    out["_vcycles_per_step"] = vc
    return out


def probe_peaks():
    from intfadv import _lib
    L = _lib.load()
    a, b = C.c_double(), C.c_double()
    if L.ia_probe_fma_rates(C.byref(a), C.byref(b)) != 0:
        return None
    return {"fp64_fma_per_s": a.value, "fp32_fma_per_s": b.value,
            "how": "8 independent FMA chains per thread, 8 blocks of 256 threads per SM, CUDA events"}


def rooflines(kt, cells, peak, peak_kind):
    """Roofline of each candidate kernel from its live CUDA-event time: algorithmic bytes of one unit
    (one pass over the grid) ÷ the time per unit, the family's event time per step over its units per
    step (launches, or whole-level half-sweeps for the slab-launched smoother); the dominant one
    (largest time per step) is the line's `roofline`."""
    out = {}
    for fam, spec in ROOF.items():
        k = kt.get(fam)
        if not k or not k["avg_launch_ms"]:
            continue
        units = spec["per_vcycle"] * kt["_vcycles_per_step"] if "per_vcycle" in spec else k["launches_per_step"]
        if not units:
            continue
        unit_ms = k["ms_per_step"] / units
        b = spec["bytes"] * cells
        ach = b / (unit_ms / 1e3) / 1e9
        out[fam] = {"bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s", "frac": ach / peak,
                    "traffic": (spec["traffic"] * cells) if spec["traffic"] else None, "kernel": spec["kernel"],
                    "peak_kind": peak_kind, "bytes_per_launch": b, "avg_launch_ms": unit_ms,
                    "launches_per_unit": k["launches_per_step"] / units, "ms_per_step": k["ms_per_step"]}
    dom = max(out, key=lambda f: out[f]["ms_per_step"]) if out else None
    return dom, out


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
    if args.no_coef16:
        ia.set_poisson_coef16(sim.handle, False)
    if args.slab_rows is not None:
        ia.set_poisson_slab_rows(sim.handle, args.slab_rows)
    if args.fine_nu:
        n1, n2 = (int(v) for v in args.fine_nu.split(","))
        _lib.check(sim.handle.call("ia_poisson_mg_fine", C.c_int32(n1), C.c_int32(n2)), "ia_poisson_mg_fine")
    m0 = sim.intf.mass()
    for _ in range(args.warmup):
        ia.sim_step(sim)
    n0 = L.ia_launch_count()
    ms, its, res, clk = timed_steps(sim, args.steps, barrier, True, local_rank)
    launches = L.ia_launch_count() - n0
    m1 = sim.intf.mass()
    if world > 1:
        t = torch.tensor([ms], device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = float(t.item())
    value = world * cells * args.steps / (ms / 1e3) / 1e6
    kt = kernel_times(sim, max(2, min(args.steps, 3)))
    peak, peak_kind = measured_peak_hbm()
    dom, roofs = rooflines(kt, cells, peak, peak_kind)
    out = {"value": value, "ms_per_step": ms / args.steps, "clocks": clk, "launches": launches,
           "roofline": roofs.get(dom), "rooflines": roofs, "kernels": kt,
           "poisson_iters_per_step": statistics.mean(its), "max_resid": max(res), "dt": sim.flow.Δt[-1],
           "mass_drift": {"value": abs(m1 - m0) / m0, "steps": args.warmup + args.steps + 0,
                          "note": "|Σf - Σf₀|/Σf₀ over the warm-up and timed steps from the initial state"}}
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
        e_steps = args.steps
        # flat views of the dense fields and their pinned copies (same strides), cut into chunks of ~100 MB
        def flat(t):
            dense = 1
            for d in sorted(range(t.dim()), key=lambda d: t.stride(d)):
                assert t.size(d) == 1 or t.stride(d) == dense, "e2e chunks need a dense field"
                dense *= t.size(d)
            return t.as_strided((t.numel(),), (1,), t.storage_offset())
        def chunks(dv, hv, n=8):
            dv, hv = flat(dv), flat(hv)
            step = (dv.numel() + n - 1) // n
            return [(dv[a:a + step], hv[a:a + step]) for a in range(0, dv.numel(), step)]
        state = chunks(fl.u, hu) + chunks(it.f, hf)
        torch.cuda.synchronize()
        barrier()
        t0 = time.perf_counter()
        # the link copies ~200 GB/s one way and ~340 GB/s both ways at once.  After a step, p and then u
        # and f go down chunk by chunk on one stream; each chunk goes back up for the next step on a
        # second stream as soon as its own download has landed, so the two directions overlap.  The next
        # step's kernels wait for both streams (its input is uploaded and p, which it rewrites, is down).
        main, down, up = torch.cuda.current_stream(), torch.cuda.Stream(), torch.cuda.Stream()
        up.wait_stream(main)
        with torch.cuda.stream(up):
            fl.u.copy_(hu, non_blocking=True)
            it.f.copy_(hf, non_blocking=True)
        for s in range(e_steps):
            main.wait_stream(up)
            main.wait_stream(down)
            ia.sim_step(sim)
            down.wait_stream(main)
            with torch.cuda.stream(down):
                hp.copy_(fl.p, non_blocking=True)
            for dv, hv in state:
                with torch.cuda.stream(down):
                    hv.copy_(dv, non_blocking=True)
                    ev = torch.cuda.Event()
                    ev.record(down)
                if s + 1 < e_steps:
                    up.wait_event(ev)
                    with torch.cuda.stream(up):
                        dv.copy_(hv, non_blocking=True)
        torch.cuda.synchronize()
        barrier()
        el = time.perf_counter() - t0
        nb = fl.u.numel() * 8 + it.f.numel() * 8
        e2e = {"value": world * cells * e_steps / el / 1e6, "unit": METRIC, "h2d_bytes_per_step": nb,
               "d2h_bytes_per_step": nb + fl.p.numel() * 8 + C.sizeof(_lib.Status),
               "steps": e_steps,
               "note": "state on the host: u, f uploaded and u, f, p downloaded every step around sim_step "
                       "(in chunks, each chunk's upload after its own download, both directions at once)"}
    out["e2e"] = e2e
    del sim
    torch.cuda.empty_cache()
    if args.no_secondary or args.quick:
        return out
    # the comparison runs over the same window of the same run as the headline: the same warm-up steps
    # from the same initial state, then the same number of timed steps
    k = args.steps
    for key, arith in (("fp64_mg", "fp64"), ("fp64_mg_ff", "ff")):
        ref = make_bubble(N, "fp64", dev, arith)
        for _ in range(args.warmup):
            ia.sim_step(ref)
        ms2, its2, res2, _ = timed_steps(ref, k, barrier, False, local_rank)
        out[key] = {"value": world * cells * k / (ms2 / 1e3) / 1e6, "ms_per_step": ms2 / k, "steps": k,
                    "warmup": args.warmup,
                    "poisson_iters_per_step": statistics.mean(its2), "max_resid": max(res2),
                    "momentum_arith": arith, "mg_vcycle_ms_per_step": kernel_times(ref, 2)["mg_vcycle"]["ms_per_step"]}
        del ref
        torch.cuda.empty_cache()
    out["speedup_vs_fp64_mg"] = value / out["fp64_mg"]["value"]
    from intfadv import learned
    if os.path.exists(learned.WEIGHTS):
        # learned preconditioner: the same step with the inner FCG preconditioned by V-cycle + net
        lrn = make_bubble(N, "learned", dev)
        for _ in range(args.warmup):
            ia.sim_step(lrn)
        st0 = ia.poisson_stats(lrn.handle)
        ms3, its3, res3, _ = timed_steps(lrn, k, barrier, False, local_rank)
        st1 = ia.poisson_stats(lrn.handle)
        kt3 = kernel_times(lrn, 2)
        out["learned_hybrid"] = {
            "value": world * cells * k / (ms3 / 1e3) / 1e6, "ms_per_step": ms3 / k, "steps": k,
            "warmup": args.warmup,
            "poisson_iters_per_step": statistics.mean(its3), "max_resid": max(res3),
            "fallbacks": st1["fallbacks"] - st0["fallbacks"],
            "net_ms_per_step": kt3["nn_precond"]["ms_per_step"],
            "mg_vcycle_ms_per_step": kt3["mg_vcycle"]["ms_per_step"],
            "weights": learned.load_params()[1]}
        del lrn
        torch.cuda.empty_cache()
    return out


def run_bubble_late(args, local_rank, total=500, window=20):
    """C3 as configured: 500 steps from rest; the last `window` steps timed (deformed bubble)."""
    import torch

    import intfadv as ia
    dev = torch.device("cuda", local_rank)
    N = args.size
    cells = N * 2 * N * N
    sim = make_bubble(N, "mixed", dev)
    m0 = sim.intf.mass()
    t0 = time.perf_counter()
    for _ in range(total - window):
        ia.sim_step(sim)
    ms, its, res, _ = timed_steps(sim, window, lambda: None, False, local_rank)
    el = time.perf_counter() - t0
    out = {"workload": f"rising bubble {N}x{2 * N}x{N}, steps {total - window + 1}-{total} of a run from rest",
           "value": cells * window / (ms / 1e3) / 1e6, "ms_per_step": ms / window,
           "poisson_iters_per_step": statistics.mean(its), "max_resid": max(res),
           "mass_drift": abs(sim.intf.mass() - m0) / m0, "all_steps_wall_s": el, "t": sum(sim.flow.Δt[:-1])}
    del sim
    torch.cuda.empty_cache()
    return out


def run_swarm(args, local_rank, N=512, steps=100, fp64_steps=10):
    """C5: 512³ unit cube, 64 bubbles r ∈ U[0.02, 0.05] (seed 5), Eö 5: the mixed path over the
    configured 100 steps (all timed), and the plain FP64 path over its first steps."""
    import torch

    import intfadv as ia
    dev = torch.device("cuda", local_rank)
    cells = N ** 3
    out = {"workload": f"bubble swarm {N}^3, 64 bubbles r in U[0.02,0.05] (seed 5), Eo=5, density ratio 1000, "
                       f"viscosity ratio 100, periodic x/z, walls y"}
    for key, poisson, arith, k in (("mixed", "mixed", "default", steps), ("fp64_mg", "fp64", "fp64", fp64_steps)):
        sim = make_swarm(N, poisson, dev, arith)
        m0 = sim.intf.mass()
        ms, its, res, _ = timed_steps(sim, k, lambda: None, False, local_rank)
        out[key] = {"value": cells * k / (ms / 1e3) / 1e6, "ms_per_step": ms / k, "steps": k,
                    "poisson_iters_per_step": statistics.mean(its), "max_resid": max(res),
                    "mass_drift": abs(sim.intf.mass() - m0) / m0}
        if key == "mixed":
            kt = kernel_times(sim, 2)
            peak, peak_kind = measured_peak_hbm()
            dom, roofs = rooflines(kt, cells, peak, peak_kind)
            out["roofline"] = roofs.get(dom)
        del sim
        torch.cuda.empty_cache()
    out["speedup_vs_fp64_mg"] = out["mixed"]["value"] / out["fp64_mg"]["value"]
    return out


def run_vof(args, world, local_rank):
    """C2: the sphere in the LeVeque deformation field over its full period T=3 at CFL 0.5 (12 N steps),
    all timed; L1 shape error Σ|f - f₀|Δx³ against the initial sphere and the mass drift."""
    import torch

    import intfadv as ia
    from intfadv import workloads
    dev = torch.device("cuda", local_rank)
    N = args.size
    intf = ia.cVOF((N, N, N), InterfaceSDF=workloads.sphere_sdf((0.35, 0.35, 0.35), 0.15, N), device=dev)
    f0 = intf.f.clone()
    U = workloads.deformation_field(N, device=dev)
    dt = 1.0 / (4 * N)
    steps = 12 * N                              # T = 3 at Δt = 1/(4N)
    u1 = U * workloads.deformation_time_factor(0.0)
    u2 = torch.empty_like(U)
    m0 = intf.mass()
    s = [0]
    codes = set()

    def one():
        nonlocal u1, u2
        s[0] += 1
        torch.mul(U, workloads.deformation_time_factor(s[0] * dt), out=u2)
        st = ia.advect_vof_raw(intf, intf.f, u1, u2, dt, s[0])
        codes.add(st.code)
        u1, u2 = u2, u1

    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(steps):
        one()
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    inner = (slice(1, -1),) * 3
    l1 = float((intf.f[inner] - f0[inner]).abs().sum()) / N ** 3
    drift = abs(intf.mass() - m0) / m0
    T, Lc = (C.c_double * 16)(), (C.c_int64 * 16)()
    intf.handle.call("ia_timing", 1, None, None, 0)
    for _ in range(10):
        one()
    intf.handle.call("ia_timing", 0, T, Lc, 16)
    bulk_ms = T[0] / max(1, Lc[0])
    peak, peak_kind = measured_peak_hbm()
    ach = 33 * N ** 3 / (bulk_ms / 1e3) / 1e9
    return {"workload": f"VOF-only sphere r=0.15 at (0.35,0.35,0.35), LeVeque deformation, {N}^3, CFL 0.5, "
                        f"full period T=3 ({steps} advect! steps, all timed)",
            "value": world * N ** 3 * steps / (ms / 1e3) / 1e6, "ms_per_step": ms / steps, "steps": steps,
            "l1_shape_error": l1, "mass_drift": drift, "status_codes": sorted(codes),
            "roofline": {"bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s", "frac": ach / peak,
                         "traffic": 31.1 * N ** 3, "kernel": "vof_bulk (read f, u_d, u⁰_d, c̄; write ρuf_d: 33 B)",
                         "peak_kind": peak_kind, "avg_launch_ms": bulk_ms}}


def main():
    args = parse()
    rank, world, local_rank = dist_env()
    if world > 1:
        import torch
        torch.distributed.init_process_group("nccl" if args.impl == "ours" else "gloo")
    N = args.size
    dims = (N, 2 * N, N)
    cfg = {"workload": f"3D rising bubble {dims[0]}x{dims[1]}x{dims[2]} (1x2x1, periodic x/z, walls y), r=0.125 at "
                       f"(0.5,0.5,0.5), density ratio 1000, viscosity ratio 100, Eo=10, Mo=1e-3; MPFMomStep! with "
                       f"Poisson to L-inf residual {PTOL}",
           "grid": list(dims), "poisson": "FP32 V-cycles + FP64 defect-correction FCG (mixed)",
           "momentum_arith": "float-float (FP32 pairs); VOF, PLIC, fields and defect correction FP64",
           "l2_flush": "inputs larger than L2 (each field 274 MB)", "parallelism": f"replicas x{world}"}
    if args.impl == "reference":
        if rank != 0:
            return
        base = cpu_bubble(N, args.ref_steps)
        line = {"impl": "reference", "metric": METRIC, "value": base["value"], "unit": METRIC, "n_gpus": world,
                "steps": args.ref_steps, "warmup": 0, "ms_per_step": 1e3 * statistics.mean(base["step_s"]),
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                "data": "synthetic", "config": cfg, "cpu_baseline": base,
                "e2e": {"value": base["value"], "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
                "note": f"the reference is Julia (no toolchain here); this arm times the C++ OpenMP restatement of "
                        f"its step (multigrid-preconditioned CG in the role of MultiLevelPoisson) on the same "
                        f"{dims[0]}x{dims[1]}x{dims[2]} grid, {args.ref_steps} steps whatever --steps says"}
        print(json.dumps(line), flush=True)
        return
    import torch
    torch.cuda.set_device(local_rank)
    res = run_bubble(args, world, local_rank)
    if rank == 0:
        quick = args.quick or args.no_secondary
        extra = {}
        if not quick:
            extra["oracle_check"] = oracle_check(torch.device("cuda", local_rank))
            extra["vof_only"] = run_vof(args, 1, local_rank)
            extra["rising_bubble_late"] = run_bubble_late(args, local_rank)
            extra["swarm"] = run_swarm(args, local_rank)
            extra["measured_fma_peaks"] = probe_peaks()
        cpu = None if (quick or args.no_cpu_baseline) else cpu_bubble(N, 1)
        cpu1 = None if (quick or args.no_cpu_baseline) else cpu_bubble(max(16, N // 4), 2, threads=1)
        line = {"metric": METRIC, "value": res["value"], "unit": METRIC, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": res["ms_per_step"], "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64 fields; f32-pair momentum; f32 V-cycles",
                "data": "synthetic", "config": cfg, "clocks": res["clocks"], "e2e": res["e2e"],
                "gpu_launches": res["launches"], "roofline": res["roofline"], "rooflines": res["rooflines"],
                "cpu_baseline": cpu, "cpu_baseline_1core": cpu1,
                "mass_drift": res["mass_drift"], "fp64_mg": res.get("fp64_mg"), "fp64_mg_ff": res.get("fp64_mg_ff"),
                "speedup_vs_fp64_mg": res.get("speedup_vs_fp64_mg"), "learned_hybrid": res.get("learned_hybrid"),
                "poisson_iters_per_step": res["poisson_iters_per_step"], "max_poisson_resid": res["max_resid"],
                "kernels_ms_per_step": {k: v["ms_per_step"] for k, v in res["kernels"].items() if not k.startswith("_")},
                "vcycles_per_step": res["kernels"].get("_vcycles_per_step"), **extra}
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
