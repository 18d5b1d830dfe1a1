"""Angle-sharded source iteration across ranks (one GPU per rank).

Within one Mult every direction is an independent sweep (src/sweep.cpp:157-175
builds one upwind graph per angle), so the directions of the quadrature are
split into contiguous slices, one per rank.  A rank sweeps only its slice and
contributes its partial scalar flux sum_{a in slice} w_a psi_a; one allreduce
(sum) of the FP64 moments per iteration gives every rank the full phi, which
the next iteration's scattering source needs.  That allreduce is the only
exchange: psi stays sharded.

The isotropic scattering source of a slice handle divides by the slice's weight
sum; scaling sigma_s by (slice weight sum / full weight sum) makes it divide by
the full sum, as the unsharded D^T does (src/transport_op.cpp:33-89).

Ranks talk through torch.distributed (NCCL between GPUs; gloo for the CPU
tests and for ranks that share one GPU, where the moments pass through host
memory).  The sweep side is a backend object with source(q_cell),
scatter(sigma_s, phi, q), mult(psi) and moments(psi); GPUBackend wraps the
library's handle.

AngleShardedSI is source iteration; AngleShardedGMRES is GMRES on the
scalar-flux system T phi = b (the Krylov option of exe/chive.cpp:704-735) with
the same single exchange per application of T.
"""
from __future__ import annotations

import numpy as np
import torch

from .quadrature import AngularQuadrature


def angle_slice(num_angles, rank, world):
    """Contiguous, balanced slice of directions owned by rank."""
    a0 = (num_angles * rank) // world
    a1 = (num_angles * (rank + 1)) // world
    return a0, a1


def sub_quadrature(quad, a0, a1):
    return AngularQuadrature(quad.dim, np.ascontiguousarray(quad.omega[a0:a1]),
                             np.ascontiguousarray(quad.weights[a0:a1]))


class GPUBackend:
    """The library's sweep handle over one slice of directions."""

    def __init__(self, mesh, order, quad, sigma_t):
        from .sweep import DiscreteToMoment, InverseAdvectionOperator
        self.L = InverseAdvectionOperator(mesh, order, quad, sigma_t)
        self.D = DiscreteToMoment(self.L)
        self.psi = torch.empty(self.L.width, dtype=torch.float64, device="cuda")
        self.phi_size = self.L.G * self.L.ndof

    def source(self, q_cell):
        from .sweep import FormTransportSource
        return torch.from_numpy(FormTransportSource(self.L, q_cell)).cuda()

    def scatter(self, sigma_s, phi, q):
        from .sweep import ScatteringSource
        ScatteringSource(self.L, sigma_s, phi, q, self.psi)
        return self.psi

    def mult(self, psi):
        self.L.Mult(psi, psi)
        return psi

    def moments(self, psi):
        out = torch.empty(self.phi_size, dtype=torch.float64, device=psi.device)
        self.D.Mult(psi, out)
        return out


def allreduce_sum(t, group=None):
    """In-place sum of t over the ranks of group.  gloo reduces host tensors:
    a CUDA tensor goes through a host copy there (ranks that share one GPU, or
    a CPU-only world)."""
    import torch.distributed as dist
    if t.is_cuda and dist.get_backend(group) == "gloo":
        h = t.cpu()
        dist.all_reduce(h, op=dist.ReduceOp.SUM, group=group)
        t.copy_(h)
    else:
        dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
    return t


class AngleShardedSI:
    """Source iteration phi <- D L^{-1} (D^T M_s phi + q) with directions
    split over the ranks of `group` (torch.distributed).

    group_shards > 1 also splits the groups: the world is a grid of
    group_shards x (world / group_shards) ranks, rank = ig * na + ia with ia
    the direction slice and ig the group slice.  Within-group scattering does
    not couple groups, so the moment allreduce runs only among the na ranks of
    one group slice; the convergence test sums the squared norms over all
    ranks.  Every rank must construct the solver (the sub-communicators are
    created collectively)."""

    def __init__(self, mesh, order, quad, sigma_t, sigma_s, rank, world, backend=GPUBackend, group=None,
                 group_shards=1):
        import torch.distributed as dist
        sigma_t = np.ascontiguousarray(sigma_t, dtype=np.float64)
        sigma_s = np.ascontiguousarray(sigma_s, dtype=np.float64)
        G = sigma_t.shape[0]
        if group_shards < 1 or world % group_shards or group_shards > G:
            raise ValueError("group_shards must divide the world size and not exceed the group count")
        na = world // group_shards
        ia, ig = rank % na, rank // na
        self.na, self.ng = na, group_shards
        self.a0, self.a1 = angle_slice(quad.size, ia, na)
        self.g0, self.g1 = angle_slice(G, ig, group_shards)
        sub = sub_quadrature(quad, self.a0, self.a1)
        scale = float(np.sum(sub.weights) / np.sum(quad.weights))
        self.sigma_s = sigma_s[self.g0:self.g1] * scale
        self.b = backend(mesh, order, sub, np.ascontiguousarray(sigma_t[self.g0:self.g1]))
        self.world_group = group
        if group_shards == 1:
            self.group = group
        else:
            # one communicator per group slice, created by every rank in the same order
            self.group = None
            for k in range(group_shards):
                g = dist.new_group(ranks=[k * na + j for j in range(na)])
                if k == ig:
                    self.group = g

    def solve(self, q_cell, tol=1e-8, maxiter=1000):
        """Returns (phi of this rank's groups [g1 - g0] x Ndof, iterations, converged)."""
        import torch.distributed as dist
        q_cell = np.ascontiguousarray(q_cell, dtype=np.float64)[self.g0:self.g1]
        q = self.b.source(q_cell)
        phi = None
        it = 0
        change = float("inf")
        while it < maxiter:
            zero = torch.zeros(self.b.phi_size, dtype=torch.float64, device=q.device) if phi is None else phi
            psi = self.b.scatter(self.sigma_s, zero, q)
            psi = self.b.mult(psi)
            new = self.b.moments(psi)
            allreduce_sum(new, self.group)   # the one exchange
            it += 1
            if self.ng == 1:
                change = (torch.linalg.norm(new - zero) / torch.linalg.norm(new)).item()
            else:
                # every rank of a group slice holds the same moments: the world sums
                # count each slice na times, which cancels in the ratio
                sq = torch.stack([torch.sum((new - zero) ** 2), torch.sum(new * new)])
                allreduce_sum(sq, self.world_group)
                change = float(torch.sqrt(sq[0] / sq[1]).item())
            phi = new
            if change < tol:
                break
        return phi, it, change < tol


class AngleShardedGMRES(AngleShardedSI):
    """GMRES on T phi = (I - D L^{-1} D^T S) phi = D L^{-1} q = b with the
    directions (and optionally the groups) split over the ranks.

    T x = x - sum_r D_r L_r^{-1} D_r^T S x: each rank sweeps its slice and one
    allreduce of the moments over the direction slices of its group slice
    completes the product, as in source iteration.  After that exchange every
    rank of a group slice holds the same Krylov vectors (the group slice's part
    of phi), so inner products need a second reduction only across group
    slices: reduce() sums the partial dot products over the world and divides
    by the number of ranks holding each slice.  With group_shards = 1 every
    rank repeats the same small Hessenberg work and no dot product is
    exchanged."""

    def _reduce(self, t):
        allreduce_sum(t, self.world_group)
        t /= self.na
        return t

    def apply(self, x, out):
        psi = self.b.scatter(self.sigma_s, x, None)
        psi = self.b.mult(psi)
        part = self.b.moments(psi)
        allreduce_sum(part, self.group)
        torch.sub(x, part, out=out)
        self.sweeps += 1
        return out

    def solve(self, q_cell, tol=1e-8, restart=30, maxiter=1000):
        """Returns (phi of this rank's groups [g1 - g0] x Ndof, iterations, converged)."""
        from .solvers import gmres
        q_cell = np.ascontiguousarray(q_cell, dtype=np.float64)[self.g0:self.g1]
        self.q = self.b.source(q_cell)
        self.sweeps = 0
        b = self.b.moments(self.b.mult(self.q.clone()))
        allreduce_sum(b, self.group)
        phi, it, hist = gmres(self.apply, b, tol=tol, restart=restart, maxiter=maxiter,
                              reduce=self._reduce if self.ng > 1 else None)
        return phi, it, hist[-1] <= tol


class AngleShardedRefinement:
    """The mixed-precision refinement with no FP64 sweep (solvers.refine_fused)
    with the directions split over the ranks of `group`.

    Each rank's handle sweeps its slice of the directions in FP32; every moment
    vector a sweep produces (the right-hand side, each inner GMRES product, the
    correction of phi, each projection of the residual) is completed by one
    allreduce, so the GMRES work in moment space is repeated identically on every
    rank.  The transport residual r = q + D^T S phi - L psi needs no exchange:
    it is local to each direction once phi is complete.  sigma_s is scaled by
    the slice's share of the weight sum, as in AngleShardedSI."""

    def __init__(self, mesh, order, quad, sigma_t, sigma_s, rank, world, group=None):
        from .sweep import InverseAdvectionOperator
        self.a0, self.a1 = angle_slice(quad.size, rank, world)
        sub = sub_quadrature(quad, self.a0, self.a1)
        scale = float(np.sum(sub.weights) / np.sum(quad.weights))
        self.sigma_s = np.ascontiguousarray(sigma_s, dtype=np.float64) * scale
        self.L = InverseAdvectionOperator(mesh, order, sub, np.ascontiguousarray(sigma_t, dtype=np.float64))
        self.group = group

    def solve(self, q_cell, tol=1e-8, inner_tol=1e-4):
        """Returns the SolveResult of refine_fused; phi is the full scalar flux."""
        from .solvers import refine_fused
        from .sweep import FormTransportSource
        q = torch.from_numpy(FormTransportSource(self.L, np.ascontiguousarray(q_cell, dtype=np.float64))).cuda()
        return refine_fused(self.L, self.sigma_s, q, tol=tol, inner_tol=inner_tol,
                            allreduce=lambda t: allreduce_sum(t, self.group))
