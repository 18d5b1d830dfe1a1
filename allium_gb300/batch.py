"""Many independent transport problems solved together on one GPU.

Problems that share the DG order and the angular quadrature are placed in one
handle over the disjoint union of their meshes (mesh.disjoint_union).  Their
upwind graphs have no common edge, so the union's wavefront levels are the
levelwise union of every problem's levels: one launch per level sweeps that
level of all problems of the group at once, and the launch sequence is
captured once per group as a CUDA graph.  Each group is solved by source
iteration with MIP-DSA (the chive method, exe/chive.cpp:704-735) or by
FP32-inner / FP64-outer refinement with DSA-preconditioned GMRES inside, and
convergence is judged per problem: the group stops when every one of its
problems has met the tolerance on its own norms.

The problem distribution of random_problems is the batched-uneven workload:
structured quad meshes of [0,1]^2 with side U{16..256}, order U{1,2,3},
level-symmetric S4..S12, sigma_t = 10^U[-1, log10 50] per cell, scattering
ratio U[0.3, 0.99] per problem, q = 1, vacuum boundaries.
"""
from __future__ import annotations

import math
import time
from dataclasses import dataclass, field

import numpy as np
import torch

from . import mesh as M
from . import quadrature as Q
from .dsa import DSAPreconditioner
from .solvers import SchurOperator, gmres
from .sweep import DiscreteToMoment, FormTransportSource, InverseAdvectionOperator, ScatteringSource


@dataclass
class TransportProblem:
    mesh: M.Mesh
    order: int
    sn: int
    sigma_t: np.ndarray     # [Ne]
    sigma_s: np.ndarray     # [Ne]
    q: np.ndarray           # [Ne] isotropic source density per cell


def random_problems(count=256, seed=20261203, sides=(16, 256), orders=(1, 2, 3), sns=(4, 6, 8, 10, 12)):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        side = int(rng.integers(sides[0], sides[1] + 1))
        p = int(rng.choice(orders))
        sn = int(rng.choice(sns))
        mesh = M.cartesian((side, side))
        ne = mesh.num_elements
        st = 10.0 ** rng.uniform(-1.0, math.log10(50.0), size=ne)
        c = rng.uniform(0.3, 0.99)
        out.append(TransportProblem(mesh, p, sn, st, c * st, np.ones(ne)))
    return out


class ProblemGroup:
    """Problems with one (order, S_N) in one union handle."""

    def __init__(self, problems, cg_tol=1e-4, cg_maxiter=100, vcycle=True):
        self.problems = problems
        p0 = problems[0]
        self.order, self.sn = p0.order, p0.sn
        mesh, eoff = M.disjoint_union([p.mesh for p in problems])
        self.mesh = mesh
        quad = Q.level_symmetric(self.sn, mesh.dim)
        st = np.concatenate([p.sigma_t for p in problems])[None, :]
        ss = np.concatenate([p.sigma_s for p in problems])[None, :]
        qc = np.concatenate([p.q for p in problems])[None, :]
        self.L = InverseAdvectionOperator(mesh, self.order, quad, st)
        self.D = DiscreteToMoment(self.L)
        self.sigma_s = ss
        n = self.L.n
        dev = torch.device("cuda")
        self.dof_off = eoff * n
        counts = np.diff(self.dof_off)
        self.pid = torch.from_numpy(np.repeat(np.arange(len(problems)), counts)).to(dev)
        self.q = torch.from_numpy(FormTransportSource(self.L, qc)).to(dev)
        self.op = SchurOperator(self.L, ss)
        self.dsa = DSAPreconditioner(self.L, ss, cg_tol=cg_tol, cg_maxiter=cg_maxiter, vcycle=vcycle)
        self.entries = self.L.width

    def norms(self, v):
        """Per-problem 2-norms of a moment vector."""
        acc = torch.zeros(len(self.problems), dtype=v.dtype, device=v.device)
        acc.index_add_(0, self.pid, v * v)
        return torch.sqrt(acc)

    def solve_si(self, tol=1e-8, maxiter=2000):
        """Source iteration with DSA; per-problem relative change below tol."""
        op, L, D = self.op, self.L, self.D
        phi = torch.zeros(op.n, dtype=torch.float64, device=self.q.device)
        new = torch.empty_like(phi)
        it = 0
        while it < maxiter:
            ScatteringSource(L, op.sigma_s, phi, self.q, op.psi)
            L.Mult(op.psi, op.psi)
            op.sweeps64 += 1
            D.Mult(op.psi, new)
            r = new - phi
            self.dsa(r, r)
            torch.add(phi, r, out=new)
            it += 1
            change = (self.norms(new - phi) / self.norms(new)).max().item()
            phi, new = new, phi
            if change < tol:
                return phi, it, True
        return phi, it, False

    def solve_ir(self, tol=1e-8, inner_tol=1e-4, restart=30, max_outer=20):
        """FP32-inner / FP64-outer refinement; per-problem residual below tol."""
        op = self.op
        b = op.rhs(self.q)
        bn = self.norms(b)
        phi = torch.zeros_like(b)
        r = b.clone()
        w = torch.empty_like(b)
        outer = inner = 0
        while outer < max_outer:
            rn = self.norms(r)
            if (rn / bn).max().item() <= tol:
                return phi, outer, inner, True
            scale = (1.0 / torch.clamp(rn, min=1e-300))[self.pid]
            d, it, _ = gmres(op.apply32, r * scale, tol=inner_tol, restart=restart, maxiter=500, prec=self.dsa)
            inner += it
            phi += d / scale
            op.apply(phi, w)
            torch.sub(b, w, out=r)
            outer += 1
        return phi, outer, inner, (self.norms(r) / bn).max().item() <= tol


@dataclass
class BatchResult:
    seconds: float
    setup_seconds: float
    groups: int
    problems: int
    entries: int
    iterations: list = field(default_factory=list)
    converged: bool = True
    sweeps64: int = 0
    sweeps32: int = 0


def group_problems(problems):
    keys = {}
    for i, p in enumerate(problems):
        keys.setdefault((p.order, p.sn), []).append(i)
    return [idx for _, idx in sorted(keys.items())]


def solve_batched(problems, method="si", tol=1e-8, workers=1):
    """Build one union handle per (order, S_N) group and solve every group.

    workers > 1 solves that many groups at a time, each on its own CUDA stream
    from its own host thread: a group's handle, DSA and Krylov vectors live on
    the stream that was current when the group was built, and the level launches
    of a small group leave most of the GPU idle, so concurrent groups fill it.
    The groups are built one after another (their setup holds the GIL for most
    of its host work, and one at a time keeps the peak memory down)."""
    t0 = time.perf_counter()
    idx = group_problems(problems)
    streams = [torch.cuda.Stream() for _ in idx] if workers > 1 else [torch.cuda.current_stream() for _ in idx]

    def build(k):
        with torch.cuda.stream(streams[k]):
            g = ProblemGroup([problems[j] for j in idx[k]])
        g.stream = streams[k]
        return g

    groups = [build(k) for k in range(len(idx))]   # one at a time: lower peak memory
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    res = BatchResult(0.0, t1 - t0, len(groups), len(problems), sum(g.entries for g in groups))

    def run(g):
        with torch.cuda.stream(g.stream):
            if method == "si":
                g.phi, it, conv = g.solve_si(tol=tol)
            else:
                g.phi, it, _, conv = g.solve_ir(tol=tol)
            g.stream.synchronize()
        return it, conv

    if workers > 1:
        from concurrent.futures import ThreadPoolExecutor
        # largest groups first, so that the small ones fill in around them
        order = sorted(range(len(groups)), key=lambda k: -groups[k].entries)
        with ThreadPoolExecutor(max_workers=workers) as ex:
            futs = {k: ex.submit(run, groups[k]) for k in order}
            results = [futs[k].result() for k in range(len(groups))]
    else:
        results = [run(g) for g in groups]
    for g, (it, conv) in zip(groups, results):
        res.iterations.append(it)
        res.converged = res.converged and conv
        res.sweeps64 += g.op.sweeps64
        res.sweeps32 += g.op.sweeps32
    torch.cuda.synchronize()
    res.seconds = time.perf_counter() - t1
    return res, groups
