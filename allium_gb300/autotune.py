"""Launch-configuration autotuner for one sweep handle.

The knobs are the schedule (wavefront levels, one launch per level captured
in a CUDA graph, or the persistent dataflow kernel with per-node completion
flags) and the threads per block of the thread-per-node level kernels, for
the FP64 sweep and the FP32 sweep (node-major layout) separately, the order
of the FP32 inverse copy that the node-major sweep reads, and the
shape of the pinned-host-buffer pipeline (direction slices, compute streams).  Each
candidate is timed with CUDA events over a few Mults after one untimed call
(which captures its graph and, for FP64, builds the factor cache once), the
fastest is kept and set on the handle.  Every candidate computes each node
with the same arithmetic, so tuning changes speed only.
"""
from __future__ import annotations

import torch


def _time(fn, reps):
    fn()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        fn()
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps


def autotune(L, reps=3, blocks=(32, 64, 128), fp32=True, schedules=None):
    """Pick (schedule, FP64 block) on FP64 Mults and the FP32 node-layout block
    on FP32 Mults; returns {"fp64": {...}, "fp32": {...}, "trials": [...]}.
    schedules restricts the schedules tried (0 levels, 1 dataflow)."""
    dev = torch.device("cuda")
    src = torch.rand(L.width, dtype=torch.float64, device=dev)
    psi = torch.empty_like(src)
    if schedules is None:
        schedules = [0]
        if L.order <= 1 and not getattr(L, "has_reflective", False):
            schedules.append(1)
    trials = []
    best = None
    for sch in schedules:
        L.SetSchedule(sch)
        for b in (blocks if sch == 0 else (blocks[-1],)):
            L.SetBlockSize(64, b)
            ms = _time(lambda: L.Mult(src, psi), reps)
            trials.append({"precision": 64, "schedule": sch, "block": b, "ms": ms})
            if best is None or ms < best["ms"]:
                best = trials[-1]
    L.SetSchedule(best["schedule"])
    L.SetBlockSize(64, best["block"])
    out = {"fp64": best, "trials": trials}
    if fp32 and L.order <= 1 and not getattr(L, "has_reflective", False):
        f = torch.empty(L.width, dtype=torch.float32, device=dev)
        L.ToNodeLayoutF32(src, f)
        g = torch.empty_like(f)
        best32 = None
        for layout in (0, 1):
            L.SetF32InverseLayout(layout)
            for b in blocks:
                L.SetBlockSize(32, b)
                ms = _time(lambda: L.MultF32Nodes(f, g), reps)
                trials.append({"precision": 32, "schedule": best["schedule"], "block": b, "layout": layout, "ms": ms})
                if best32 is None or ms < best32["ms"]:
                    best32 = trials[-1]
        L.SetF32InverseLayout(best32["layout"])
        L.SetBlockSize(32, best32["block"])
        out["fp32"] = best32
    L.synchronize()
    return out


def autotune_pipeline(L, h_src, h_psi, reps=3,
                      shapes=((8, 4, 1), (8, 4, 0), (8, 4, 2), (8, 3, 1), (10, 4, 2), (6, 4, 1), (12, 4, 2))):
    """Pick the (slices, compute streams, end taper) of the pinned-host-buffer
    Mult: each shape is timed on the host clock (the call returns once psi is
    back in host memory) after two untimed calls, median of `reps`; the
    fastest is set on the handle.  Returns {"best": {...}, "trials": [...]}."""
    import time
    trials = []
    for chunks, streams, taper in shapes:
        L.SetPipeline(chunks, streams, taper)
        L.Mult(h_src, h_psi)
        L.Mult(h_src, h_psi)
        ts = []
        for _ in range(reps):
            t0 = time.perf_counter()
            L.Mult(h_src, h_psi)
            ts.append(time.perf_counter() - t0)
        ts.sort()
        trials.append({"chunks": chunks, "streams": streams, "taper": taper, "ms": 1e3 * ts[len(ts) // 2]})
    best = min(trials, key=lambda t: t["ms"])
    L.SetPipeline(best["chunks"], best["streams"], best["taper"])
    return {"best": best, "trials": trials}
