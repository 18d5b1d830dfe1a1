"""The angle-sharded source iteration and GMRES on two to four CPU ranks
(gloo): each rank sweeps its slice of the directions with the oracle standing
in for its GPU, one allreduce of the moments per application of the operator
(and, with group slices, of the Krylov inner products); the result equals the
unsharded iteration to 1e-10 relative."""
import os
import socket

import numpy as np
import pytest
import torch

from tests.helpers import problem


class OracleBackend:
    def __init__(self, mesh, order, quad, sigma_t):
        from oracle.oracle import OracleSweep
        self.o = OracleSweep(mesh, order, quad, sigma_t)
        self.phi_size = self.o.G * self.o.ndof

    def source(self, q_cell):
        return torch.from_numpy(self.o.form_source(q_cell=q_cell))

    def scatter(self, sigma_s, phi, q):
        qn = np.zeros(self.o.G * self.o.Nw * self.o.ndof) if q is None else q.numpy()
        return torch.from_numpy(self.o.scattering_source(sigma_s, phi.numpy(), qn))

    def mult(self, psi):
        return torch.from_numpy(self.o.mult(psi.numpy()))

    def moments(self, psi):
        return torch.from_numpy(self.o.moments(psi.numpy()))


def _case():
    mesh, quad, sigma = problem(2, (6, 5), 1, sn=6, G=2, seed=9)
    return mesh, quad, sigma, 0.8 * sigma, np.ones((2, mesh.num_elements))


def _worker(rank, world, port, path, group_shards=1, method="si"):
    import torch.distributed as dist
    from allium_gb300.sharded import AngleShardedGMRES, AngleShardedSI
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    mesh, quad, sigma, ss, q = _case()
    cls = AngleShardedSI if method == "si" else AngleShardedGMRES
    solver = cls(mesh, 1, quad, sigma, ss, rank, world, backend=OracleBackend, group_shards=group_shards)
    phi, it, conv = solver.solve(q, tol=1e-12, maxiter=500)
    np.save(f"{path}.{rank}.npy", np.concatenate([phi.numpy(), [solver.g0, solver.g1, it, conv]]))
    dist.destroy_process_group()


def _unsharded():
    from oracle.oracle import OracleSweep
    mesh, quad, sigma, ss, q = _case()
    o = OracleSweep(mesh, 1, quad, sigma)
    src = o.form_source(q_cell=q)
    phi = np.zeros(o.G * o.ndof)
    for it in range(1, 501):
        new = o.moments(o.mult(o.scattering_source(ss, phi, src)))
        done = np.linalg.norm(new - phi) / np.linalg.norm(new) < 1e-12
        phi = new
        if done:
            break
    return phi.reshape(o.G, -1), it


@pytest.mark.parametrize("world,group_shards", [(2, 2), (4, 2)])
def test_angle_and_group_sharded_si(tmp_path, world, group_shards):
    # ranks on a (group slice x direction slice) grid: 2 ranks = one group each,
    # all directions; 4 ranks = 2 group slices x 2 direction slices
    mp = pytest.importorskip("torch.multiprocessing")
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    path = str(tmp_path / "phi")
    mp.spawn(_worker, args=(world, port, path, group_shards), nprocs=world, join=True)
    ref, it_ref = _unsharded()
    na = world // group_shards
    for r in range(world):
        res = np.load(f"{path}.{r}.npy")
        g0, g1, it, conv = int(res[-4]), int(res[-3]), int(res[-2]), res[-1]
        assert conv == 1.0 and it == it_ref
        got = res[:-4].reshape(g1 - g0, -1)
        assert np.max(np.abs(got - ref[g0:g1])) < 1e-10 * np.max(np.abs(ref))
        assert (g0, g1) == ((r // na), (r // na) + 1)


@pytest.mark.parametrize("world", [2, 3])
def test_angle_sharded_si(tmp_path, world):
    # 2 ranks: even halves of the 24 directions; 3 ranks: slices of 8
    mp = pytest.importorskip("torch.multiprocessing")
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    path = str(tmp_path / "phi")
    mp.spawn(_worker, args=(world, port, path), nprocs=world, join=True)
    rs = [np.load(f"{path}.{r}.npy") for r in range(world)]
    r0 = rs[0]
    assert all(np.array_equal(r0, r) for r in rs[1:])   # every rank holds the same reduced moments
    assert r0[-1] == 1.0
    r0 = np.concatenate([r0[:-4], r0[-2:]])   # drop the group range (all groups here)
    # the unsharded iteration with the full quadrature
    from oracle.oracle import OracleSweep
    mesh, quad, sigma, ss, q = _case()
    o = OracleSweep(mesh, 1, quad, sigma)
    src = o.form_source(q_cell=q)
    phi = np.zeros(o.G * o.ndof)
    for it in range(1, 501):
        new = o.moments(o.mult(o.scattering_source(ss, phi, src)))
        done = np.linalg.norm(new - phi) / np.linalg.norm(new) < 1e-12
        phi = new
        if done:
            break
    assert it == int(r0[-2])
    assert np.max(np.abs(r0[:-2] - phi)) < 1e-10 * np.max(np.abs(phi))


def _unsharded_gmres():
    from allium_gb300.solvers import gmres
    from oracle.oracle import OracleSweep
    mesh, quad, sigma, ss, q = _case()
    o = OracleSweep(mesh, 1, quad, sigma)
    src = o.form_source(q_cell=q)
    zero = np.zeros(src.size)
    b = torch.from_numpy(o.moments(o.mult(src)))

    def apply(x, out):
        out.copy_(x - torch.from_numpy(o.moments(o.mult(o.scattering_source(ss, x.numpy(), zero)))))
        return out

    phi, it, hist = gmres(apply, b, tol=1e-12, restart=30, maxiter=500)
    return phi.numpy().reshape(o.G, -1), it


@pytest.mark.parametrize("world,group_shards", [(2, 1), (3, 1), (4, 2)])
def test_angle_sharded_gmres(tmp_path, world, group_shards):
    # direction slices (one Krylov space repeated on every rank) and a 2 x 2
    # grid whose Krylov vectors are split by group (inner products reduced)
    mp = pytest.importorskip("torch.multiprocessing")
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    path = str(tmp_path / "phi")
    mp.spawn(_worker, args=(world, port, path, group_shards, "gmres"), nprocs=world, join=True)
    ref, it_ref = _unsharded_gmres()
    for r in range(world):
        res = np.load(f"{path}.{r}.npy")
        g0, g1, it, conv = int(res[-4]), int(res[-3]), int(res[-2]), res[-1]
        assert conv == 1.0 and it == it_ref
        got = res[:-4].reshape(g1 - g0, -1)
        assert np.max(np.abs(got - ref[g0:g1])) < 1e-10 * np.max(np.abs(ref))
