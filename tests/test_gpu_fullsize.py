"""The benchmark workload at full size against the CPU oracle.

The 64^3 jittered hex mesh, p = 1, S12 (168 directions), the benchmark's cross
sections and source (bench.workload()): 352 M swept entries, too many for the
oracle in a test, so the comparison takes one direction per octant (8 of 168,
the directions of the CPU baseline sample).  Every direction sweeps
independently, so the GPU handle over all 168 directions and an oracle over the
8 compute the same numbers for them.  Levels bit for bit; the FP64 sweep
within 1e-12 relative (max norm), the fused FP32 sweep within 2e-5."""
import numpy as np
import pytest

import bench
from allium_gb300 import quadrature as Q
from allium_gb300.sweep import FormTransportSource, InverseAdvectionOperator
from oracle.oracle import OracleSweep
from tests.helpers import rel_err

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def test_headline_workload_full_size():
    mesh, quad, sigma, q = bench.workload()
    ne, nw = mesh.num_elements, quad.size
    L = InverseAdvectionOperator(mesh, 1, quad, sigma)
    pick = [i * (nw // 8) for i in range(8)]
    sub = Q.AngularQuadrature(3, quad.omega[pick].copy(), quad.weights[pick].copy())
    o = OracleSweep(mesh, 1, sub, sigma)
    # wavefront levels of the picked directions, bit for bit
    nl, lev_o = o.levels()
    assert nl > 0
    lev = L.levels().reshape(ne, nw)[:, pick]
    assert np.array_equal(lev, lev_o.reshape(ne, 8))
    # FormTransportSource and the FP64 sweep (stored-inverse path after its first Mult)
    src = FormTransportSource(L, q)
    src_o = o.form_source(q_cell=q)
    ndof = L.ndof
    assert rel_err(src.reshape(nw, ndof)[pick], src_o.reshape(8, ndof)) < 1e-12
    ref = o.mult(src_o).reshape(8, ndof)
    d = torch.from_numpy(src).cuda()
    psi = torch.empty_like(d)
    for _ in range(2):   # the factoring Mult, then the cached one
        L.Mult(d, psi)
        L.synchronize()
        got = psi.view(nw, ndof)[pick].cpu().numpy()
        assert rel_err(got, ref) < 1e-12
    # the fused FP32 sweep (unit-level schedule) on the same source
    f_src = torch.empty(L.width, dtype=torch.float32, device="cuda")
    L.ToFusedLayout(d, f_src)
    L.FusedMultF32(None, f_src, f_src)
    back = torch.empty_like(d)
    L.FromFusedLayout(f_src, None, back)
    L.synchronize()
    assert rel_err(back.view(nw, ndof)[pick].cpu().numpy(), ref) < 2e-5
