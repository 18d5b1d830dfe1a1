"""The direction-sharded solvers with the library's GPU handle: two ranks in
two processes that share one GPU, each sweeping half of the directions
through GPUBackend, with gloo carrying the moment allreduce through host
memory (no kernel of one rank waits for the other).  Source iteration and
GMRES both equal the unsharded GPU solve to 1e-12 relative with the same
iteration count; the sharded mixed-precision refinement (FP32 sweeps, no FP64
sweep) reaches the FP64 solution to 1e-8."""
import os
import socket

import numpy as np
import pytest

from tests.helpers import problem

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _case():
    mesh, quad, sigma = problem(3, (6, 5, 4), 1, sn=6, G=2, jitter=0.1, seed=11)
    rng = np.random.default_rng(12)
    ss = sigma * rng.uniform(0.5, 0.95, size=sigma.shape)
    q = rng.uniform(0.0, 1.0, size=sigma.shape)
    return mesh, quad, sigma, ss, q


def _worker(rank, world, port, path, method):
    import torch.distributed as dist
    from allium_gb300.sharded import AngleShardedGMRES, AngleShardedSI
    torch.cuda.set_device(0)
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    mesh, quad, sigma, ss, q = _case()
    cls = AngleShardedSI if method == "si" else AngleShardedGMRES
    solver = cls(mesh, 1, quad, sigma, ss, rank, world)
    phi, it, conv = solver.solve(q, tol=1e-13, maxiter=500)
    torch.cuda.synchronize()
    np.save(f"{path}.{rank}.npy", np.concatenate([phi.cpu().numpy(), [solver.a0, solver.a1, it, conv]]))
    dist.destroy_process_group()


def _unsharded(method):
    from allium_gb300.solvers import SchurOperator, solve_gmres, source_iteration
    from allium_gb300.sweep import FormTransportSource, InverseAdvectionOperator
    mesh, quad, sigma, ss, q = _case()
    L = InverseAdvectionOperator(mesh, 1, quad, sigma)
    src = torch.from_numpy(FormTransportSource(L, q)).cuda()
    op = SchurOperator(L, ss)
    if method == "si":
        res = source_iteration(op, src, tol=1e-13, maxiter=500)
    else:
        res = solve_gmres(op, src, tol=1e-13, restart=30, maxiter=500)
    return res.phi.cpu().numpy(), res.iterations, quad.size


@pytest.mark.parametrize("method", ["si", "gmres"])
def test_two_ranks_share_one_gpu(tmp_path, method):
    mp = pytest.importorskip("torch.multiprocessing")
    ref, it_ref, nw = _unsharded(method)
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    path = str(tmp_path / "phi")
    mp.spawn(_worker, args=(2, port, path, method), nprocs=2, join=True)
    rs = [np.load(f"{path}.{r}.npy") for r in range(2)]
    assert [(int(r[-4]), int(r[-3])) for r in rs] == [(0, nw // 2), (nw // 2, nw)]
    assert np.array_equal(rs[0][:-4], rs[1][:-4])   # both ranks hold the same reduced moments
    for r in rs:
        assert r[-1] == 1.0 and int(r[-2]) == it_ref
        assert np.max(np.abs(r[:-4] - ref)) < 1e-12 * np.max(np.abs(ref))


def _refine_worker(rank, world, port, path):
    import torch.distributed as dist
    from allium_gb300.sharded import AngleShardedRefinement
    torch.cuda.set_device(0)
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    mesh, quad, sigma, ss, q = _case()
    solver = AngleShardedRefinement(mesh, 1, quad, sigma, ss, rank, world)
    res = solver.solve(q, tol=1e-10)
    torch.cuda.synchronize()
    np.save(f"{path}.{rank}.npy", np.concatenate([res.phi.cpu().numpy(), [res.iterations, res.converged]]))
    dist.destroy_process_group()


def test_two_ranks_refinement_without_fp64_sweeps(tmp_path):
    mp = pytest.importorskip("torch.multiprocessing")
    ref, _, _ = _unsharded("gmres")
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    path = str(tmp_path / "phi")
    mp.spawn(_refine_worker, args=(2, port, path), nprocs=2, join=True)
    rs = [np.load(f"{path}.{r}.npy") for r in range(2)]
    assert np.array_equal(rs[0], rs[1])   # the moment-space work is the same on both ranks
    assert rs[0][-1] == 1.0
    assert np.max(np.abs(rs[0][:-2] - ref)) < 1e-8 * np.max(np.abs(ref))
