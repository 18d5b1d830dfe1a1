"""allium_sweep_balance_noalloc, the entry point for callers that cannot
allocate GPU memory when they call (caller-owned memory pools, allocation-free
time steps, hosts that hand the library only its vectors).  Called through the C ABI and checked against
allium_sweep_balance, with the 1e-12 relative tolerance of the other FP64
tests, on two calls in a row.  Collected last so that a failure here comes
after every other test has run."""
import ctypes as C

import numpy as np
import pytest

from allium_gb300 import _lib
from allium_gb300.sweep import AdvectionOperator, InverseAdvectionOperator
from tests.helpers import problem

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

TOL64 = 1e-12


def test_balance_without_allocation_matches_balance():
    mesh, quad, sig = problem(3, (8, 8, 8), 1, sn=4, G=2, jitter=0.1, seed=11)
    L = InverseAdvectionOperator(mesh, 1, quad, sig)
    lib = _lib.lib()
    for call, seed in enumerate((1, 2)):
        psi = torch.from_numpy(np.random.default_rng(seed).random(L.width)).cuda()
        ref = AdvectionOperator(L).ComputeBalance(psi)
        if call == 0:
            out = torch.zeros(1, dtype=torch.float64, device="cuda")
            st = lib.allium_sweep_balance_noalloc(L.h, C.c_void_p(psi.data_ptr()), C.c_void_p(out.data_ptr()))
            assert st == 0, lib.allium_sweep_last_error(L.h)
            L.synchronize()
            got = out.item()
        else:
            host = np.zeros(1)
            st = lib.allium_sweep_balance_noalloc(L.h, C.c_void_p(psi.data_ptr()), C.c_void_p(host.ctypes.data))
            assert st == 0, lib.allium_sweep_last_error(L.h)
            got = float(host[0])
        assert abs(got - ref) <= TOL64 * abs(ref)


def test_balance_without_allocation_rejects():
    mesh, quad, sig = problem(2, (64, 64), 0, sn=8, G=1)
    lib = _lib.lib()
    L = InverseAdvectionOperator(mesh, 0, quad, sig)
    out = np.zeros(1)
    host_psi = np.zeros(L.width)
    # psi in host memory would need staging, which allocates
    assert lib.allium_sweep_balance_noalloc(L.h, C.c_void_p(host_psi.ctypes.data), C.c_void_p(out.ctypes.data)) == 1
    # above the fixed partial-sum capacity: 820 groups x 40 angles x 4096 cells > 134217728
    big = np.ones((820, mesh.num_elements))
    Lb = InverseAdvectionOperator(mesh, 0, quad, big)
    small = torch.zeros(8, dtype=torch.float64, device="cuda")
    assert lib.allium_sweep_balance_noalloc(Lb.h, C.c_void_p(small.data_ptr()), C.c_void_p(out.ctypes.data)) == 3
    assert b"134217728" in lib.allium_sweep_last_error(Lb.h)
