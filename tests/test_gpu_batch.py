"""Batched independent problems: a union handle sweeps every problem of a
group exactly as its own handle does (same arithmetic per node, bit for bit),
and the batched DSA-accelerated solves reach each problem's own solution."""
import numpy as np
import pytest

from allium_gb300 import mesh as M
from allium_gb300 import quadrature as Q
from allium_gb300.batch import ProblemGroup, random_problems, solve_batched
from allium_gb300.solvers import SchurOperator, solve_gmres
from allium_gb300.sweep import FormTransportSource, InverseAdvectionOperator

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("order,sn", [(1, 4), (2, 6), (3, 4)])
def test_union_sweep_equals_separate_sweeps(order, sn):
    probs = [p for p in random_problems(12, seed=3, sides=(6, 20), orders=(order,), sns=(sn,))]
    g = ProblemGroup(probs)
    rng = np.random.default_rng(0)
    src = rng.random(g.L.width)
    out = np.empty_like(src)
    g.L.Mult(src, out)
    n, Nw = g.L.n, g.L.Nw
    src = src.reshape(Nw, -1)
    out = out.reshape(Nw, -1)
    assert g.L.num_levels == max(InverseAdvectionOperator(p.mesh, order, Q.level_symmetric(sn, 2),
                                                          p.sigma_t[None, :]).num_levels for p in probs)
    for k, p in enumerate(probs):
        a, b = g.dof_off[k], g.dof_off[k + 1]
        L = InverseAdvectionOperator(p.mesh, order, Q.level_symmetric(sn, 2), p.sigma_t[None, :])
        s = np.ascontiguousarray(src[:, a:b]).reshape(-1)
        o = np.empty_like(s)
        L.Mult(s, o)
        assert np.array_equal(o.reshape(Nw, -1), out[:, a:b])


@pytest.mark.parametrize("method", ["si", "ir"])
def test_batched_solves_match_single_solves(method):
    probs = random_problems(8, seed=5, sides=(8, 24))
    res, groups = solve_batched(probs, method=method, tol=1e-9)
    assert res.converged and res.problems == 8
    for g in groups:
        phi = g.phi
        for k, p in enumerate(g.problems):
            L = InverseAdvectionOperator(p.mesh, p.order, Q.level_symmetric(p.sn, 2), p.sigma_t[None, :])
            q = torch.from_numpy(FormTransportSource(L, p.q[None, :])).cuda()
            ref = solve_gmres(SchurOperator(L, p.sigma_s[None, :]), q, tol=1e-11, restart=60).phi
            a, b = g.dof_off[k], g.dof_off[k + 1]
            err = torch.max(torch.abs(phi[a:b] - ref)).item() / torch.max(torch.abs(ref)).item()
            assert err < 1e-6


def test_concurrent_groups_match_sequential_groups():
    # four groups built and solved at a time, each on its own stream from its own
    # host thread: the same iterations and answers as one group after another
    probs = random_problems(12, seed=6, sides=(8, 24))
    seq, g1 = solve_batched(probs, method="ir", tol=1e-9, workers=1)
    con, g4 = solve_batched(probs, method="ir", tol=1e-9, workers=4)
    assert seq.converged and con.converged and seq.iterations == con.iterations
    for a, b in zip(g1, g4):
        err = torch.max(torch.abs(a.phi - b.phi)).item() / torch.max(torch.abs(a.phi)).item()
        assert err < 1e-9
