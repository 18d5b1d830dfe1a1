"""Benchmark of the upwind DG transport sweep on the 3D chive workload.

Workload: 64^3 hexes of [0,1]^3 with interior vertices jittered by U[-0.1h, 0.1h]
(seeded; at +-0.2h every seed tried gives a cyclic S12 upwind graph, which
allium rejects), trilinear DG (p = 1, 8 DOF/cell), level-symmetric S12 (168
directions), one group, sigma_t log-uniform in [0.1, 100] per cell, vacuum
boundaries, q uniform in [0, 1] per cell.  A step is one InverseAdvectionOperator
Mult (one full sweep of every cell, angle and group).  The metric is swept
cell-angle-group DOF per second = G * Nw * Ndof / sweep time.

  value     FP64 sweep with q and psi resident in HBM (CUDA events), in the
            library's default mode: the first Mult after (re)assembly stores
            the inverse of every local system, later Mults apply them (two
            different sources alternate over the timed steps); the uncached
            FP64 sweep and the first Mult are reported beside it
  e2e       the same Mult through the C ABI with pinned host buffers, the
            host->device copy of q and the device->host copy of psi inside the
            timed region (wall clock around the synchronous call)
  fp32      the FP32 sweep (FP32 storage and local solves), resident in HBM

`--impl reference` times the CPU restatement of the reference sweep (OpenMP,
all host cores) on a sample of the same workload (8 of the 168 directions,
one per octant, on the full mesh).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

SEED = 20261203
JITTER = 0.1   # +-0.2h makes every tried seed's S12 upwind graph cyclic (the reference rejects cyclic graphs)
CELLS = (64, 64, 64)
ORDER = 1
SN = 12
METRIC = "swept cell-angle-group DOF/s"
UNIT = "DOF*angle*group/s"


def workload(cells=CELLS):
    from allium_gb300 import mesh as M
    from allium_gb300 import quadrature as Q
    mesh = M.cartesian(cells, jitter=JITTER, seed=SEED)
    quad = Q.level_symmetric(SN, 3)
    rng = np.random.default_rng(SEED + 1)
    sigma = 10.0 ** rng.uniform(-1.0, 2.0, size=(1, mesh.num_elements))
    q = rng.uniform(0.0, 1.0, size=(1, mesh.num_elements))
    return mesh, quad, sigma, q


def config(levels=None, cells=CELLS):
    if tuple(cells) != CELLS:
        return {"workload": f"profiling case: {cells[0]}^3 jittered hex mesh, p=1, S12, 1 group", "levels": levels}
    c = {"workload": "chive 3D sweep: 64^3 hex mesh of [0,1]^3, interior vertices jittered +-0.1h (seed 20261203; +-0.2h gives a cyclic S12 upwind graph), "
                     "p=1 Gauss-Lobatto DG (8 DOF/cell), level-symmetric S12 (168 directions), 1 group, "
                     "sigma_t log-uniform [0.1,100] per cell, vacuum boundaries, q ~ U[0,1] per cell",
         "cells": 64 ** 3, "dofs_per_cell": 8, "angles": 168, "groups": 1,
         "psi_entries": 64 ** 3 * 8 * 168,
         "l2_policy": "inputs larger than L2 (q and psi are 2.8 GB each in FP64)"}
    if levels is not None:
        c["levels"] = levels
    return c


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def fp64_fma_peak(reps=3):
    """FP64 multiply-add rate of this GPU (G DFMA/s), measured with the library's
    probe kernel: every SM full of threads running independent FMA chains."""
    import ctypes as C
    import torch
    from allium_gb300 import _lib
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    blocks, threads, iters = sms * 8, 256, 4096
    sink = torch.empty(blocks * threads, dtype=torch.float64, device="cuda")
    st = torch.cuda.current_stream()
    run = lambda: _lib.check(_lib.lib().allium_fp64_fma_probe(blocks, threads, iters, C.c_void_p(sink.data_ptr()),
                                                               C.c_void_p(st.cuda_stream)))
    run()
    torch.cuda.synchronize()
    best = 0.0
    for _ in range(reps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        run()
        e1.record(st)
        e1.synchronize()
        best = max(best, blocks * threads * 8.0 * iters / (e0.elapsed_time(e1) * 1e-3) / 1e9)
    return {"gdfma_s": best, "tflops": 2e-3 * best, "blocks": blocks, "threads": threads,
            "fma_per_thread": 8 * iters}


def traffic_per_entry():
    """DRAM bytes per swept entry of the FP64 sweep kernel from the committed
    ncu summary (profiles/sweep_fp64_traffic.json), or None."""
    path = os.path.join(ROOT, "profiles", "sweep_fp64_traffic.json")
    try:
        with open(path) as f:
            return float(json.load(f)["dram_bytes_per_entry"])
    except Exception:
        return None


class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons during the timed region."""

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in self.lines:
            parts = [p.strip() for p in l.split(",")]
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
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


def cpu_sweep_sample(threads, steps, warmup, ndir=8):
    """CPU restatement of Mult_Upwind (OpenMP) on the workload mesh with ndir of
    the 168 directions (one per octant for ndir = 8).  Returns DOF*angle*group/s
    per step."""
    from oracle.oracle import OracleSweep
    from allium_gb300 import quadrature as Q
    mesh, quad, sigma, q = workload()
    pick = [i * (quad.size // 8) for i in range(ndir)]
    sub = Q.AngularQuadrature(3, quad.omega[pick].copy(), quad.weights[pick].copy())
    o = OracleSweep(mesh, ORDER, sub, sigma)
    src = o.form_source(q_cell=q)
    psi = np.empty_like(src)
    for _ in range(warmup):
        o.mult(src, psi, threads=threads)
    rates = []
    for _ in range(steps):
        t0 = time.perf_counter()
        o.mult(src, psi, threads=threads)
        rates.append(o.psi_size / (time.perf_counter() - t0))
    return rates, o.psi_size


def cpu_trt_sweep_rate(groups=2, steps=3):
    """CPU oracle sweep rate (DOF*angle*group/s, all cores) on the TRT wave's
    mesh and quadrature (128 x 128, p = 1, S8) with `groups` of its 32 groups:
    the cost per group is the same, so the rate carries over."""
    from oracle.oracle import OracleSweep
    from allium_gb300 import mesh as M
    from allium_gb300 import quadrature as Q
    mesh = M.cartesian((128, 128))
    quad = Q.level_symmetric(8, 2)
    sig = np.ones((groups, mesh.num_elements))
    o = OracleSweep(mesh, 1, quad, sig)
    src = np.random.default_rng(SEED).random(o.psi_size)
    psi = np.empty_like(src)
    o.mult(src, psi, threads=os.cpu_count() or 1)
    rates = []
    for _ in range(steps):
        t0 = time.perf_counter()
        o.mult(src, psi, threads=os.cpu_count() or 1)
        rates.append(o.psi_size / (time.perf_counter() - t0))
    return statistics.median(rates)


def cpu_extrapolated(line, rate3d, n3d):
    """CPU time to tolerance of the solver sections, extrapolated as FP64
    sweeps x CPU sweep time (the all-core oracle restatement of Mult_Upwind;
    Krylov vector work excluded, so a lower bound): the C2 solve on the 3D
    workload and the 200-step TRT wave, beside the GPU times."""
    out = {"kind": "extrapolated: FP64 sweeps x measured CPU sweep time (lower bound)",
           "cores": os.cpu_count()}
    t = line.get("time_to_tolerance")
    if t:
        sweeps = t["fp64_gmres"]["fp64_sweeps"]
        cpu_s = sweeps * n3d / rate3d
        out["c2_fp64_gmres"] = {"seconds": cpu_s, "fp64_sweeps": sweeps, "cpu_sweep_rate": rate3d,
                                "gpu_seconds": t["fp64_gmres"]["seconds"],
                                "gpu_speedup": cpu_s / t["fp64_gmres"]["seconds"]}
    tr = line.get("trt_marshak")
    if tr:
        rate2d = cpu_trt_sweep_rate()
        sweeps = tr["fp64"]["fp64_sweeps"]
        cpu_s = sweeps * tr["psi_entries"] / rate2d
        out["c4_trt_fp64"] = {"seconds": cpu_s, "fp64_sweeps": sweeps, "cpu_sweep_rate": rate2d,
                              "gpu_seconds": tr["fp64"]["seconds"], "gpu_speedup": cpu_s / tr["fp64"]["seconds"]}
    return out


def solve_section(L, mesh, quad, sigma, src, maxiter=400, fp64_setup_s=0.0, fused_setup_s=0.0):
    """Time to a 1e-8 relative residual of T phi = b on the 3D workload with
    sigma_s / sigma_t ~ U[0.5, 0.999] per cell: FP64 GMRES(30) with the FP64
    sweep against FP32-inner / FP64-outer refinement (the fused FP32 operator
    with double-float residuals and no FP64 sweep; and the earlier form whose
    outer residuals are FP64 sweeps), each without and with MIP-DSA as the
    right preconditioner.  fp64_setup_s / fused_setup_s: the one-off setup of
    each arm (the FP64 factor pass; the fused schedule and FP32 cell tables),
    added in the *_with_setup figures."""
    import torch
    from allium_gb300.solvers import SchurOperator, refine, refine_fused, solve_gmres, true_residual
    rng = np.random.default_rng(SEED + 2)
    sigma_s = sigma * rng.uniform(0.5, 0.999, size=sigma.shape)
    # operator setup shared by both: stored FP64 and FP32 local inverses
    f = src.float()
    L.MultF32(f, f)
    L.ToNodeLayoutF32(src, f)      # the node-layout inner sweep's FP32 copy of the inverses
    L.MultF32Nodes(f, f)
    torch.cuda.synchronize()
    del f
    out = {}
    op = SchurOperator(L, sigma_s)
    plain = solve_gmres(op, src, tol=1e-8, restart=30, maxiter=maxiter)
    b = op.rhs(src)
    out["fp64_gmres"] = {"seconds": plain.seconds, "iterations": plain.iterations, "converged": plain.converged,
                         "fp64_sweeps": plain.sweeps64, "residual": true_residual(op, b, plain.phi)}
    op2 = SchurOperator(L, sigma_s)
    ir = refine(op2, src, tol=1e-8, inner_tol=1e-4, restart=30)
    out["fp32_inner_fp64_outer"] = {"seconds": ir.seconds, "outer": ir.iterations,
                                    "inner_iterations": getattr(ir, "inner_iterations", None),
                                    "converged": ir.converged, "fp64_sweeps": ir.sweeps64, "fp32_sweeps": ir.sweeps32,
                                    "residual": true_residual(op2, b, ir.phi)}
    out["speedup"] = plain.seconds / ir.seconds if ir.seconds > 0 else None
    out["phi_rel_diff"] = float((torch.max(torch.abs(ir.phi - plain.phi)) / torch.max(torch.abs(plain.phi))).item())
    # the fused FP32 operator with double-float residuals: no FP64 sweep at all
    refine_fused(L, sigma_s, src, tol=1e-8)   # warm-up (graphs of its buffers)
    torch.cuda.synchronize()
    fr = refine_fused(L, sigma_s, src, tol=1e-8, inner_tol=1e-4, restart=30)
    del fr.psi
    out["fp32_fused_refinement"] = {
        "seconds": fr.seconds, "outer": fr.iterations, "inner_iterations": fr.inner_iterations,
        "converged": fr.converged, "fp64_sweeps": fr.sweeps64, "fp32_sweeps": fr.sweeps32,
        "double_float_residuals": fr.residuals_df, "history": fr.history, "residual": true_residual(op2, b, fr.phi),
        "phi_rel_diff_vs_fp64_gmres": float((torch.max(torch.abs(fr.phi - plain.phi))
                                             / torch.max(torch.abs(plain.phi))).item())}
    out["fused_speedup"] = plain.seconds / fr.seconds
    out["setup_seconds"] = {"fp64_factor_pass": fp64_setup_s, "fused_schedule_and_tables": fused_setup_s}
    out["fused_speedup_with_setup"] = (plain.seconds + fp64_setup_s) / (fr.seconds + fused_setup_s)
    torch.cuda.empty_cache()
    # MIP-DSA as the right preconditioner of both (inexact block-Jacobi CG inside)
    from allium_gb300.dsa import DSAPreconditioner
    t0 = time.perf_counter()
    dsa = DSAPreconditioner(L, sigma_s, cg_tol=1e-4, cg_maxiter=50, vcycle=False)
    torch.cuda.synchronize()
    setup_s = time.perf_counter() - t0
    op3 = SchurOperator(L, sigma_s)
    pd = solve_gmres(op3, src, tol=1e-8, restart=30, maxiter=maxiter, prec=dsa)
    out["fp64_gmres_dsa"] = {"seconds": pd.seconds + setup_s, "setup_seconds": setup_s, "iterations": pd.iterations,
                             "converged": pd.converged, "fp64_sweeps": pd.sweeps64,
                             "residual": true_residual(op3, b, pd.phi)}
    op4 = SchurOperator(L, sigma_s)
    ird = refine(op4, src, tol=1e-8, inner_tol=1e-4, restart=30, prec=dsa)
    out["fp32_inner_fp64_outer_dsa"] = {"seconds": ird.seconds + setup_s, "outer": ird.iterations,
                                        "inner_iterations": getattr(ird, "inner_iterations", None),
                                        "converged": ird.converged, "fp64_sweeps": ird.sweeps64,
                                        "fp32_sweeps": ird.sweeps32, "residual": true_residual(op4, b, ird.phi)}
    out["cg_iterations"] = dsa.K.cg_iterations
    out["speedup_best_vs_fp64_gmres"] = plain.seconds / min(ir.seconds, out["fp64_gmres_dsa"]["seconds"],
                                                            out["fp32_inner_fp64_outer_dsa"]["seconds"])
    out["problem"] = ("3D workload, sigma_s/sigma_t ~ U[0.5,0.999] per cell, tol 1e-8 on ||b - T phi||/||b||; "
                      "plain FP64 GMRES(30) is the reference arm of the speedups")
    return out


def trt_section(steps):
    """Multigroup Marshak wave (linearized TRT): 128 x 128 quads of [0,1]^2, p = 1,
    S8, 32 log-spaced groups over [1e-2, 10], sigma_g = 10 nu_g^-3 T^-1/2 per cell
    (explicit in each step), c_v = 1, a = c = 1, T0 = 1e-3, Planck inflow at T = 1
    on x = 0, backward Euler dt = 1e-3; each step's Schur system solved to 1e-8
    by FP64 GMRES and by FP32-inner / FP64-outer refinement, the same steps."""
    import torch
    from allium_gb300.trt import marshak_wave
    out = {"problem": "multigroup Marshak wave, 128x128 quads, p=1, S8 (40 directions), 32 groups, dt=1e-3, "
                      "tol 1e-8 per step, no DSA", "steps": steps}
    T = {}
    for method in ("fp64", "ir"):   # warm-up on a small instance (library kernels, torch, graphs)
        w = marshak_wave(cells=16, method=method)
        for _ in range(3):
            w.step()
        del w
    for method in ("fp64", "ir"):
        s = marshak_wave(method=method)
        torch.cuda.synchronize()
        secs, its, s64, s32, conv = 0.0, [], 0, 0, True
        for _ in range(steps):
            r = s.step()
            secs += r.seconds
            its.append(r.iterations)
            s64 += r.sweeps64
            s32 += r.sweeps32
            conv = conv and r.converged
        T[method] = s.T.clone()
        psi_entries = s.L.width
        out[method] = {"seconds": secs, "ms_per_step": 1e3 * secs / steps, "krylov_iterations": int(np.sum(its)),
                       "max_iterations": int(np.max(its)), "fp64_sweeps": s64, "fp32_sweeps": s32, "converged": conv,
                       "T_max": float(s.T.max().item()),
                       "launch": {k: {kk: s.tuned[k][kk] for kk in ("schedule", "block")}
                                  for k in ("fp64", "fp32") if k in s.tuned}}
        del s
        torch.cuda.empty_cache()
    out["psi_entries"] = psi_entries
    out["speedup"] = out["fp64"]["seconds"] / out["ir"]["seconds"]
    out["T_rel_diff"] = float((torch.max(torch.abs(T["ir"] - T["fp64"])) / torch.max(torch.abs(T["fp64"]))).item())
    return out


def gemm_section(reps=20):
    """The MLP's BF16 GEMMs on the tcgen05 kernel against the mma.sync kernel
    (CUDA events, best of two rounds of `reps`): a hidden layer's forward
    product over the wave's 16384 cells, its weight gradient (K = 16384, split
    over blocks) and a 4096^3 product, where the tensor pipe rather than memory
    bounds the kernel (its TFLOP/s against the measured cuBLAS BF16 rate)."""
    import torch
    from allium_gb300.mlp import gemm, tc_status
    g = torch.Generator(device="cpu").manual_seed(5)
    st = torch.cuda.current_stream()
    out = {}
    peak = None
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peak = float(json.load(f)["bf16_tflops"])
    except Exception:
        peak = 1900.0
    cases = {"layer_forward": (16384, 256, 256, False, True),
             "weight_gradient": (256, 256, 16384, True, False),
             "square_4096": (4096, 4096, 4096, False, True)}
    for name, (M, N, K, ta, tb) in cases.items():
        A = torch.randn((K, M) if ta else (M, K), generator=g).to("cuda", torch.bfloat16)
        B = torch.randn((N, K) if tb else (K, N), generator=g).to("cuda", torch.bfloat16)
        C = torch.empty((M, N), dtype=torch.float32, device="cuda")
        res = {"M": M, "N": N, "K": K}
        for tc in (True, False):
            fn = lambda: gemm(A, B, out=C, transA=ta, transB=tb, tc=tc)
            for _ in range(3):
                fn()
            torch.cuda.synchronize()
            best = float("inf")
            for _ in range(2):
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(st)
                for _ in range(reps):
                    fn()
                e1.record(st)
                e1.synchronize()
                best = min(best, e0.elapsed_time(e1) / reps)
            ref = C.clone() if tc else ref
            res["tc_ms" if tc else "mma_sync_ms"] = best
        tc_status()
        res["rel_diff"] = float((torch.max(torch.abs(C - ref)) / torch.max(torch.abs(ref))).item())
        res["tc_tflops"] = 2.0 * M * N * K / (res["tc_ms"] * 1e-3) / 1e12
        res["mma_sync_tflops"] = 2.0 * M * N * K / (res["mma_sync_ms"] * 1e-3) / 1e12
        res["tc_frac_of_measured_bf16"] = res["tc_tflops"] / peak
        out[name] = res
        del A, B, C, ref
    out["note"] = ("tc: k_gemm_tc (tcgen05.mma, TMEM accumulator, cp.async.bulk.tensor operands, operands made "
                   "K-major first where a transpose is needed, included in the time); mma_sync: k_gemm_bf16; "
                   "fractions of the measured cuBLAS BF16 burst rate")
    return out


def learned_section(steps=200, train_steps=50, epochs=20):
    """Learned initial iterate on the multigroup Marshak wave: steps 1..train_steps
    plain (their (state -> next moments) pairs recorded), then a per-cell MLP
    (4 layers x 256, BF16 tensor-core GEMMs, FP32 accumulation, Adam) trained on
    them corrects the linear extrapolation 2 phi_n - phi_{n-1}, which becomes
    the initial iterate of every later step's FP64 GMRES solve (to 1e-8).  The
    same later steps are also run from phi_n (plain) and from the extrapolation
    alone, three runs of the same problem side by side."""
    import torch
    from allium_gb300.mlp import LearnedInitialIterate
    from allium_gb300.trt import marshak_wave
    runs = {k: marshak_wave(method="fp64") for k in ("plain", "extrapolated", "learned")}
    li = LearnedInitialIterate(runs["learned"], width=256, layers=4, seed=0)
    ex = LearnedInitialIterate(runs["extrapolated"], width=16, layers=2, seed=0)   # only its extrapolate()
    out = {"problem": "multigroup Marshak wave of the TRT section, FP64 GMRES to 1e-8 per step",
           "steps": steps, "train_steps": train_steps}
    its = {k: 0 for k in runs}
    secs = {k: 0.0 for k in runs}
    train_s = 0.0
    for n in range(steps):
        for name, s in runs.items():
            before = (s.phi(), s.T.clone(), s.sigma.clone())
            if n < train_steps:
                r = s.step()
                if name == "learned" and n > 0:
                    li.record(*before, s.phi())
                elif name == "extrapolated":
                    ex.last = before[0].clone()
                continue
            t0 = time.perf_counter()
            if name == "learned":
                if li.stats is None:
                    out["final_loss"] = li.train(epochs=epochs)
                    torch.cuda.synchronize()
                    train_s = time.perf_counter() - t0
                    t0 = time.perf_counter()
                guess = li.predict(*before)
            elif name == "extrapolated":
                guess = ex.extrapolate(before[0])
            else:
                guess = None
            torch.cuda.synchronize()
            pred_s = time.perf_counter() - t0
            r = s.step(phi0=guess)
            its[name] += r.iterations
            secs[name] += r.seconds + pred_s
    for k in runs:
        out[k] = {"krylov_iterations": its[k], "seconds": secs[k]}
    out["learned"]["train_seconds"] = train_s
    out["learned"]["correction_gain"] = li.gain
    out["learned"]["samples"] = sum(x.shape[0] for x in li.X)
    out["iteration_ratio_vs_plain"] = its["plain"] / max(its["learned"], 1)
    out["iteration_ratio_vs_extrapolated"] = its["extrapolated"] / max(its["learned"], 1)
    out["speedup_incl_training"] = secs["plain"] / (secs["learned"] + train_s)
    out["T_rel_diff"] = float((torch.max(torch.abs(runs["learned"].T - runs["plain"].T))
                               / torch.max(runs["plain"].T)).item())
    return out


def batch_section(count):
    """Batched uneven problems: `count` independent one-group 2D problems
    (side U{16..256}, p U{1,2,3}, S4..S12, sigma_t 10^U[-1, log10 50] per cell,
    c U[0.3, 0.99], q = 1, vacuum), each to a 1e-8 relative residual: one union
    handle per (order, S_N) group, four groups built and solved at a time on
    their own streams, by FP32-inner / FP64-outer refinement with
    DSA-preconditioned GMRES, against the same method on one handle per
    problem."""
    import gc
    import torch
    from allium_gb300.batch import ProblemGroup, random_problems, solve_batched
    probs = random_problems(count, seed=SEED + 7)
    warm = random_problems(6, seed=1, sides=(8, 16))
    solve_batched(warm, "ir", workers=4)
    out = {"problems": count, "entries": int(sum(p.mesh.num_elements * (p.order + 1) ** 2 * (p.sn * (p.sn + 2) // 2)
                                              for p in probs))}
    res, groups = solve_batched(probs, method="ir", tol=1e-8, workers=4)
    out["batched_ir"] = {"seconds": res.seconds, "setup_seconds": res.setup_seconds, "groups": res.groups,
                         "concurrent_groups": 4,
                         "outer_per_group": res.iterations, "converged": res.converged,
                         "fp64_sweeps": res.sweeps64, "fp32_sweeps": res.sweeps32}
    del groups
    gc.collect()
    torch.cuda.empty_cache()
    setup = solve = 0.0
    conv = True
    for p in probs:
        a = time.perf_counter()
        g = ProblemGroup([p])
        torch.cuda.synchronize()
        b = time.perf_counter()
        c = g.solve_ir(tol=1e-8)[3]
        torch.cuda.synchronize()
        setup += b - a
        solve += time.perf_counter() - b
        conv = conv and c
        del g
    out["one_by_one_ir"] = {"seconds": solve, "setup_seconds": setup, "converged": conv}
    out["batching_speedup"] = (solve + setup) / (res.seconds + res.setup_seconds)
    out["note"] = ("refinement with DSA-preconditioned GMRES is the batched method: source iteration with the "
                   "same DSA needs 18-36 iterations per group and runs about 3x longer")
    return out


def sharded_section(mesh, quad, sigma, q, rank, world, barrier, max_over_ranks):
    """The C2 solve with the directions split over the ranks (run under
    torchrun, N > 1): AngleShardedGMRES to 1e-8, each rank a handle over its
    slice of the S12 directions, one NCCL allreduce of the FP64 moments per
    application of T.  Strong scaling of one problem, reported beside the
    weak-scaled headline."""
    import torch
    from allium_gb300.sharded import AngleShardedGMRES
    rng = np.random.default_rng(SEED + 2)
    sigma_s = sigma * rng.uniform(0.5, 0.999, size=sigma.shape)
    t0 = time.perf_counter()
    solver = AngleShardedGMRES(mesh, ORDER, quad, sigma, sigma_s, rank, world)
    barrier()
    setup_s = max_over_ranks(time.perf_counter() - t0)
    solver.solve(q, tol=1e-8)        # warm-up: factor pass of each slice handle, graphs
    barrier()
    t0 = time.perf_counter()
    phi, it, conv = solver.solve(q, tol=1e-8)
    torch.cuda.synchronize()
    seconds = max_over_ranks(time.perf_counter() - t0)
    out = {"seconds": seconds, "setup_seconds": setup_s, "iterations": it, "converged": bool(conv),
           "directions_per_rank": solver.a1 - solver.a0, "ranks": world,
           "exchange": "one NCCL allreduce of G*Ndof FP64 moments per application of T",
           "scaling": "strong (one problem split by direction)"}
    del solver
    torch.cuda.empty_cache()
    return out


def warm_solver_libraries():
    """Untimed: one pass of every solver path on a 24x24 problem and a few
    training steps of the cell network.  On a fresh
    machine the first call into cuSOLVER (GMRES's least squares), cuSPARSE and
    a few torch kernels loads and initialises those libraries, seconds per
    library; none of that belongs in a solver's time."""
    import torch
    from allium_gb300 import mesh as M
    from allium_gb300 import quadrature as Q
    from allium_gb300.dsa import DSAPreconditioner
    from allium_gb300.solvers import SchurOperator, refine, solve_gmres, source_iteration
    from allium_gb300.sweep import FormTransportSource, InverseAdvectionOperator
    mesh = M.cartesian((24, 24))   # 625 vertices: one aggregation level below the vertex space
    ne = mesh.num_elements
    sig_t, sig_s, q = np.ones((1, ne)), np.full((1, ne), 0.9), np.ones((1, ne))
    L = InverseAdvectionOperator(mesh, 1, Q.level_symmetric(4, 2), sig_t)
    src = torch.from_numpy(FormTransportSource(L, q)).cuda()
    for vcycle in (False, True):
        dsa = DSAPreconditioner(L, sig_s, cg_tol=1e-6, cg_maxiter=20, vcycle=vcycle)
        source_iteration(SchurOperator(L, sig_s), src, tol=1e-6, dsa=dsa)
        solve_gmres(SchurOperator(L, sig_s), src, tol=1e-6, restart=30, maxiter=40, prec=dsa)
        refine(SchurOperator(L, sig_s), src, tol=1e-6, inner_tol=1e-3, restart=30, prec=dsa)
    from allium_gb300.mlp import CellMLP
    net = CellMLP(8, 4, width=256, layers=4, seed=0)
    X = torch.randn(4096, 8, device="cuda")
    Y = torch.randn(4096, 4, device="cuda")
    for _ in range(3):
        net.train_step(X[torch.randperm(4096, device="cuda")].contiguous(), (Y - Y.mean(0)) / Y.std(0))
    net.forward(X)
    torch.cuda.synchronize()


def chive2d_section(cpu=True):
    """The 2D chive configuration: 64x64 quads, p = 1, S8, sigma_t = 1,
    sigma_s = 0.9, q = 1, vacuum; source iteration to 1e-8 relative change of
    phi on the GPU (FP64 sweep), and the CPU oracle doing the same iteration."""
    import torch
    from allium_gb300 import mesh as M
    from allium_gb300 import quadrature as Q
    from allium_gb300.solvers import SchurOperator, source_iteration
    from allium_gb300.sweep import FormTransportSource, InverseAdvectionOperator
    mesh = M.cartesian((64, 64))
    quad = Q.level_symmetric(8, 2)
    ne = mesh.num_elements
    sig_t, sig_s, q = np.ones((1, ne)), np.full((1, ne), 0.9), np.ones((1, ne))
    L = InverseAdvectionOperator(mesh, 1, quad, sig_t)
    src = torch.from_numpy(FormTransportSource(L, q)).cuda()
    from allium_gb300.dsa import DSAPreconditioner
    source_iteration(SchurOperator(L, sig_s), src, tol=1e-8)   # warm-up (graphs, factors)
    res = source_iteration(SchurOperator(L, sig_s), src, tol=1e-8)
    out = {"gpu_si": {"seconds": res.seconds, "iterations": res.iterations, "converged": res.converged}}
    t0 = time.perf_counter()
    dsa = DSAPreconditioner(L, sig_s, cg_tol=1e-10, cg_maxiter=200, vcycle=True)
    torch.cuda.synchronize()
    setup_s = time.perf_counter() - t0
    acc = source_iteration(SchurOperator(L, sig_s), src, tol=1e-8, dsa=dsa)
    out["gpu_si_mip_dsa"] = {"seconds": acc.seconds + setup_s, "setup_seconds": setup_s,
                             "iterations": acc.iterations, "converged": acc.converged,
                             "cg_iterations": dsa.K.cg_iterations,
                             "phi_rel_diff_vs_si": float((torch.max(torch.abs(acc.phi - res.phi))
                                                          / torch.max(torch.abs(res.phi))).item())}
    if cpu:
        from oracle.oracle import OracleSweep
        o = OracleSweep(mesh, 1, quad, sig_t)
        src_h = o.form_source(q_cell=q)
        t0 = time.perf_counter()
        phi = np.zeros(o.ndof)
        it = 0
        for it in range(1, 5001):
            psi = o.scattering_source(sig_s, phi, src_h)
            o.mult(psi, psi, threads=os.cpu_count() or 1)
            new = o.moments(psi)
            change = np.linalg.norm(new - phi) / np.linalg.norm(new)
            phi = new
            if change < 1e-8:
                break
        cpu_s = time.perf_counter() - t0
        out["cpu_si"] = {"seconds": cpu_s, "iterations": it, "cores": os.cpu_count(), "kind": "port"}
        out["phi_rel_diff_gpu_vs_cpu"] = float(np.max(np.abs(res.phi.cpu().numpy() - phi)) / np.max(np.abs(phi)))
        out["speedup_vs_cpu"] = cpu_s / res.seconds
    return out


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    rates, size = cpu_sweep_sample(threads, args.steps, max(1, args.warmup))
    v = statistics.median(rates)
    sample = f"full 64^3 mesh, 8 of 168 S12 directions (one per octant): {size} DOF*angle per sweep"
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": size / v * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": config(),
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def _timed(stream, steps, fn):
    """Average ms per call of fn(i) over `steps` calls, CUDA events on `stream`."""
    import torch
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for i in range(steps):
        fn(i)
    e1.record(stream)
    e1.synchronize()
    return e0.elapsed_time(e1) / steps


def run_gpu(args):
    import torch
    from allium_gb300.sweep import FormTransportSource, InverseAdvectionOperator

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    cells = (args.cells,) * 3
    mesh, quad, sigma, q = workload(cells)
    L = InverseAdvectionOperator(mesh, ORDER, quad, sigma)   # runs on torch's current stream
    stream = torch.cuda.current_stream()
    N = L.width
    src_host = FormTransportSource(L, q)
    # two different sources, alternated over the timed steps
    srcs = [torch.from_numpy(src_host).cuda(), torch.from_numpy(src_host[::-1].copy()).cuda()]
    psi = torch.empty_like(srcs[0])

    def barrier():
        torch.cuda.synchronize()
        if dist:
            dist.barrier()

    def max_over_ranks(x):
        if not dist:
            return x
        t = torch.tensor([x], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())

    clk = ClockSampler(local).__enter__()   # sampled across all timed regions below

    # --- FP64 without the factor cache (every Mult refactors, as the reference does)
    L.SetFactorCache(0)
    for i in range(args.warmup):
        L.Mult(srcs[i % 2], psi)
    barrier()
    ms_plain = max_over_ranks(_timed(stream, max(3, args.steps // 10), lambda i: L.Mult(srcs[i % 2], psi)))

    # --- FP64 with the factor cache: the first Mult factors, later ones reuse
    L.SetFactorCache(1)
    barrier()
    ms_first = max_over_ranks(_timed(stream, 1, lambda i: L.Mult(srcs[0], psi)))
    # launch configuration chosen by the autotuner (schedule, threads per block)
    from allium_gb300.autotune import autotune
    tuned = autotune(L, reps=3, schedules=None if args.schedule == "auto" else
                     ([0] if args.schedule == "levels" else [1]))
    for i in range(args.warmup):
        L.Mult(srcs[i % 2], psi)
    barrier()
    ms = max_over_ranks(_timed(stream, args.steps, lambda i: L.Mult(srcs[i % 2], psi)))
    barrier()
    value = world * N / (ms * 1e-3)
    # the same cached FP64 sweep as one persistent dataflow launch
    L.SetSchedule(1)
    for i in range(args.warmup):
        L.Mult(srcs[i % 2], psi)
    barrier()
    ms_flow = _timed(stream, max(3, args.steps // 5), lambda i: L.Mult(srcs[i % 2], psi))
    L.SetSchedule(tuned["fp64"]["schedule"])
    L.Mult(srcs[0], psi)
    L.synchronize()

    # --- FP32 sweep, resident
    f_src = srcs[0].float()
    f_psi = torch.empty_like(f_src)
    for _ in range(args.warmup):
        L.MultF32(f_src, f_psi)
    L.synchronize()
    ms32 = _timed(stream, args.steps, lambda i: L.MultF32(f_src, f_psi))
    err32 = float((torch.max(torch.abs(f_psi.double() - psi)) / torch.max(torch.abs(psi))).item())
    # FP32 sweep on the node-major layout (the inner-iteration layout)
    L.ToNodeLayoutF32(srcs[0], f_src)
    for _ in range(args.warmup):
        L.MultF32Nodes(f_src, f_psi)
    L.synchronize()
    ms32n = _timed(stream, args.steps, lambda i: L.MultF32Nodes(f_src, f_psi))
    back = torch.empty_like(psi)
    L.FromNodeLayoutF32(f_psi, back)
    err32n = float((torch.max(torch.abs(back - psi)) / torch.max(torch.abs(psi))).item())
    del f_src, f_psi, back

    # --- fused FP32 inner operator: phi = D L^-1 (D^T S x / sum w) on the fused layout
    nd = L.G * L.ndof
    t0 = time.perf_counter()
    fused_levels = L.FusedLevels()          # schedule setup (unit levels, records)
    iso = torch.rand(nd, dtype=torch.float32, device="cuda")
    fz_psi = torch.empty(N, dtype=torch.float32, device="cuda")
    fz_phi = torch.empty(nd, dtype=torch.float64, device="cuda")
    L.FusedMultF32(iso, None, fz_psi, phi=fz_phi, phi_mode=1)   # FP32 cell tables, graph capture
    torch.cuda.synchronize()
    fused_setup_s = time.perf_counter() - t0
    for _ in range(args.warmup):
        L.FusedMultF32(iso, None, fz_psi, phi=fz_phi, phi_mode=1)
    L.synchronize()
    ms_fused = _timed(stream, args.steps, lambda i: L.FusedMultF32(iso, None, fz_psi, phi=fz_phi, phi_mode=1))
    ms_fused_nophi = _timed(stream, args.steps, lambda i: L.FusedMultF32(iso, None, fz_psi))
    ms_fused_phi32 = _timed(stream, args.steps, lambda i: L.FusedMultF32(iso, None, fz_psi, phi=fz_phi, phi_mode=3))
    # accuracy of the fused sweep on the headline source against the FP64 sweep
    fz_src = torch.empty(N, dtype=torch.float32, device="cuda")
    L.ToFusedLayout(srcs[0], fz_src)
    L.FusedMultF32(None, fz_src, fz_psi)
    back = torch.empty_like(psi)
    L.FromFusedLayout(fz_psi, None, back)
    L.Mult(srcs[0], psi)
    L.synchronize()
    err_fused = float((torch.max(torch.abs(back - psi)) / torch.max(torch.abs(psi))).item())
    # double-float residual and moments
    hi_t = fz_psi.clone()
    lo_t = torch.zeros_like(hi_t)
    iso_lo = torch.zeros_like(iso)
    r32 = torch.empty_like(fz_psi)
    ms_resid = _timed(stream, max(3, args.steps // 4), lambda i: L.TransportResidualDF(iso, iso_lo, hi_t, lo_t, r32))
    ms_mom_df = _timed(stream, max(3, args.steps // 4), lambda i: L.MomentsDF(hi_t, lo_t, fz_phi))
    del fz_src, back, hi_t, lo_t, r32, fz_psi
    torch.cuda.empty_cache()

    # --- e2e through the C ABI with pinned host buffers (copies inside the timed region)
    h_srcs = [s.cpu().pin_memory() for s in srcs]
    h_psi = torch.empty_like(h_srcs[0]).pin_memory()
    from allium_gb300.autotune import autotune_pipeline
    pipe = autotune_pipeline(L, h_srcs[0], h_psi)   # untimed: picks the slices and compute streams
    for i in range(max(args.warmup, 2)):   # warm-up over both pinned sources (a fresh buffer's first copy is slower)
        L.Mult(h_srcs[i % 2], h_psi)
    barrier()
    t0 = time.perf_counter()
    call_s = []
    for i in range(args.steps):
        tc = time.perf_counter()
        L.Mult(h_srcs[i % 2], h_psi)   # returns with psi in host memory
        call_s.append(time.perf_counter() - tc)
    e2e_s = max_over_ranks((time.perf_counter() - t0) / args.steps)
    e2e = world * N / e2e_s
    clk.__exit__(None, None, None)
    L.Mult(h_srcs[(args.steps - 1) % 2], h_psi)
    L.Mult(srcs[(args.steps - 1) % 2], psi)
    L.synchronize()
    assert torch.equal(h_psi, psi.cpu()), "host and device paths disagree"

    sharded = None
    if world > 1:
        sharded = sharded_section(mesh, quad, sigma, q, rank, world, barrier, max_over_ranks)

    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return

    peak, peak_kind = measured_peaks()
    fp64_peak = fp64_fma_peak()
    alg_bytes = 16.0 * N + 8.0 * mesh.num_elements * (1 + 3 * 8)
    achieved = alg_bytes / (ms * 1e-3) / 1e9
    tpe = traffic_per_entry()
    roof = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "traffic": (tpe * N if tpe is not None else None), "peak_kind": peak_kind,
            "kernel": ("k_sweep_cached_level<3,1> (FP64 sweep from stored local inverses)"
                       if tuned["fp64"]["schedule"] == 0 else
                       "k_flow<3,1,double,cached> (persistent dataflow FP64 sweep from stored local inverses)"),
            "algorithmic_bytes_per_launch": alg_bytes,
            "launch": ("one Mult = the CUDA graph of all wavefront-level launches" if tuned["fp64"]["schedule"] == 0
                       else "one Mult = one persistent launch")}
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": config(L.num_levels, cells),
            "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": 8 * N, "d2h_bytes_per_step": 8 * N,
                    "ms_per_step": e2e_s * 1e3,
                    "call_ms": {"median": 1e3 * float(np.median(call_s)), "min": 1e3 * min(call_s),
                                "p90": 1e3 * float(np.percentile(call_s, 90)), "max": 1e3 * max(call_s),
                                "slow_calls_over_1p5x_median": int(sum(c > 1.5 * np.median(call_s) for c in call_s))},
                    "pipeline": {"chunks": pipe["best"]["chunks"], "compute_streams": pipe["best"]["streams"],
                                 "taper": pipe["best"]["taper"],
                                 "trials_ms": {f"{t['chunks']}x{t['streams']}t{t['taper']}": round(t["ms"], 2)
                                               for t in pipe["trials"]}}},
            "gpu_launches": args.steps * (L.num_levels if tuned["fp64"]["schedule"] == 0 else 2),
            "roofline": roof,
            # the kernel's own bound: GB300's FP64 pipe, its multiply-add rate measured in
            # this run (fp64_fma_peak); per (cell, angle) node of the p = 1 hex sweep: 64 DFMA
            # for inv(A) b plus 20 per inflow face (F u and its scaling), 3 inflow faces on average
            "fp64_pipe": {"achieved_gdfma_s": (N / 8) * (64 + 3 * 20) / (ms * 1e-3) / 1e9,
                          "peak_gdfma_s": fp64_peak["gdfma_s"], "peak_kind": "measured",
                          "peak_probe": fp64_peak,
                          "frac": (N / 8) * (64 + 3 * 20) / (ms * 1e-3) / 1e9 / fp64_peak["gdfma_s"]},
            # the same bound in the units of a flop roofline: flops executed per DOF*angle
            # (2 per DFMA) against the reference algorithm's (per-node assembly and LU,
            # about 211 for 3D p = 1), whose work the stored inverses avoid
            "compute_roofline": {"executed_flops_per_unit": 2.0 * (64 + 3 * 20) / 8,
                                 "reference_algorithm_flops_per_unit": 211,
                                 "achieved_tflops": N * 2.0 * (64 + 3 * 20) / 8 / (ms * 1e-3) / 1e12,
                                 "peak_tflops": 2e-3 * fp64_peak["gdfma_s"], "peak_kind": "measured FP64 FMA rate",
                                 "frac": N * 2.0 * (64 + 3 * 20) / 8 / (ms * 1e-3) / 1e12 / (2e-3 * fp64_peak["gdfma_s"]),
                                 "reference_algorithm_equivalent_tflops": N * 211 / (ms * 1e-3) / 1e12},
            "fp64_uncached": {"value": N / (ms_plain * 1e-3), "ms_per_step": ms_plain,
                              "note": "every Mult assembles and factors all local systems (pivoted LU), as the reference does"},
            "fp64_first_mult_ms": ms_first,
            "autotune": {"fp64": tuned["fp64"], "fp32_nodes": tuned.get("fp32"),
                         "trials": len(tuned["trials"])},
            "fp64_dataflow_launch_ms": ms_flow,
            "factor_cache_bytes": N * 8 * 8,
            "fp32": {"value": N / (ms32 * 1e-3), "unit": UNIT, "ms_per_step": ms32,
                     "max_rel_err_vs_fp64": err32,
                     "roofline_frac": (8.0 * N / (ms32 * 1e-3) / 1e9) / peak,
                     "note": "allium's RIGHT layout, local systems rebuilt and solved in FP32 each sweep"},
            "fp32_nodes": {"value": N / (ms32n * 1e-3), "unit": UNIT, "ms_per_step": ms32n,
                           "max_rel_err_vs_fp64": err32n,
                           "roofline_frac": (8.0 * N / (ms32n * 1e-3) / 1e9) / peak,
                           "note": "node-major layout (the refinement's inner sweep), from an FP32 copy of the stored inverses"},
            "fp32_fused": {
                "value": N / (ms_fused * 1e-3), "unit": UNIT, "ms_per_step": ms_fused,
                "ms_without_moments": ms_fused_nophi, "ms_fp32_moments": ms_fused_phi32,
                "max_rel_err_vs_fp64": err_fused,
                "levels": fused_levels[0], "unit_levels": bool(fused_levels[1]), "setup_seconds": fused_setup_s,
                "roofline": {"bound": "hbm", "unit": "GB/s", "peak": peak, "peak_kind": peak_kind,
                             "algorithmic_bytes_per_entry": 8,
                             "achieved": 8.0 * N / (ms_fused * 1e-3) / 1e9,
                             "frac": 8.0 * N / (ms_fused * 1e-3) / 1e9 / peak},
                "kernels": "k_fused_level<3,1> once per level + k_moments_f32, one CUDA graph",
                "note": ("the inner operator phi = D L^-1 (D^T S x / sum w) of the refinement: per-cell source "
                         "in registers, FP32 local solves, moments in double-float; 8 B per entry is the "
                         "FP32 sweep's algorithmic traffic (read q, write psi)")},
            "sharded_c2": sharded,
            "double_float_residual_ms": ms_resid,
            "double_float_moments_ms": ms_mom_df,
            "clocks": clk.summary()}
    if not args.no_solve:
        warm_solver_libraries()
        line["time_to_tolerance"] = solve_section(L, mesh, quad, sigma, srcs[0],
                                                  fp64_setup_s=max(0.0, (ms_first - ms) * 1e-3),
                                                  fused_setup_s=fused_setup_s)
        line["chive_2d"] = chive2d_section(cpu=not args.no_cpu)
        line["trt_marshak"] = trt_section(args.trt_steps)
        line["learned_iterate"] = learned_section(args.trt_steps, min(50, args.trt_steps // 4))
        line["mlp_gemm"] = gemm_section()
        if args.batch_problems > 0:
            # the 64^3 handle (stored inverses, FP32 copies, fused tables) is not
            # needed any more: release it before the batched problems' handles
            del L, srcs, psi
            import gc
            gc.collect()
            torch.cuda.synchronize()
            torch.cuda.empty_cache()
            line["batched_uneven"] = batch_section(args.batch_problems)
    if not args.no_cpu and tuple(cells) == CELLS:
        rates, size = cpu_sweep_sample(os.cpu_count() or 1, 3, 1)
        line["cpu_baseline"] = {"value": statistics.median(rates), "unit": UNIT, "cores": os.cpu_count(),
                                "kind": "port",
                                "sample": f"full 64^3 mesh, 8 of 168 S12 directions (one per octant), {size} DOF*angle per sweep, median of 3"}
        rates1, size1 = cpu_sweep_sample(1, 3, 1, ndir=1)
        line["cpu_baseline_1thread"] = {"value": statistics.median(rates1), "unit": UNIT, "cores": 1, "kind": "port",
                                        "sample": f"full 64^3 mesh, 1 of 168 S12 directions, {size1} DOF*angle per sweep, median of 3"}
        try:
            line["cpu_time_to_tolerance"] = cpu_extrapolated(line, statistics.median(rates), N)
        except Exception as exc:   # a reported estimate, never a reason to lose the line
            line["cpu_time_to_tolerance"] = {"error": repr(exc)}
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--cells", type=int, default=CELLS[0], help="cells per axis (smaller cases for profiling)")
    ap.add_argument("--no-solve", action="store_true", help="skip the time-to-tolerance solves")
    ap.add_argument("--trt-steps", type=int, default=200, help="time steps of the multigroup TRT section")
    ap.add_argument("--schedule", default="auto", choices=["auto", "levels", "dataflow"],
                    help="sweep schedule: chosen by the autotuner, or fixed (for profiler runs, whose "
                         "serialised launches would skew the tuner)")
    ap.add_argument("--batch-problems", type=int, default=256, help="problems of the batched section (0 skips it)")
    ap.add_argument("--gemm", action="store_true", help="only the MLP GEMM comparison (one JSON line)")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    elif args.gemm:
        print(json.dumps({"mlp_gemm": gemm_section()}), flush=True)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
