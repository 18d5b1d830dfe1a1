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
tests).  The sweep side is a backend object with source(q_cell),
scatter(sigma_s, phi, q), mult(psi) and moments(psi); GPUBackend wraps the
library's handle.
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


class AngleShardedSI:
    """Source iteration phi <- D L^{-1} (D^T M_s phi + q) with directions
    split over the ranks of `group` (torch.distributed)."""

    def __init__(self, mesh, order, quad, sigma_t, sigma_s, rank, world, backend=GPUBackend, group=None):
        self.a0, self.a1 = angle_slice(quad.size, rank, world)
        sub = sub_quadrature(quad, self.a0, self.a1)
        scale = float(np.sum(sub.weights) / np.sum(quad.weights))
        self.sigma_s = np.ascontiguousarray(sigma_s, dtype=np.float64) * scale
        self.b = backend(mesh, order, sub, sigma_t)
        self.group = group

    def solve(self, q_cell, tol=1e-8, maxiter=1000):
        import torch.distributed as dist
        q = self.b.source(q_cell)
        phi = None
        it = 0
        change = float("inf")
        while it < maxiter:
            zero = torch.zeros(self.b.phi_size, dtype=torch.float64, device=q.device) if phi is None else phi
            psi = self.b.scatter(self.sigma_s, zero, q)
            psi = self.b.mult(psi)
            new = self.b.moments(psi)
            dist.all_reduce(new, op=dist.ReduceOp.SUM, group=self.group)   # the one exchange
            it += 1
            change = (torch.linalg.norm(new - zero) / torch.linalg.norm(new)).item()
            phi = new
            if change < tol:
                break
        return phi, it, change < tol
