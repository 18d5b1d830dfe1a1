"""Host side of the batched-problem driver (CPU): the uneven problem
distribution and the grouping by (order, S_N) that decides which problems share
a union handle."""
import numpy as np

from allium_gb300 import mesh as M
from allium_gb300.batch import group_problems, random_problems


def test_random_problems_distribution():
    probs = random_problems(64, seed=3)
    assert len(probs) == 64
    for p in probs:
        side = int(round(np.sqrt(p.mesh.num_elements)))
        assert side * side == p.mesh.num_elements and 16 <= side <= 256
        assert p.order in (1, 2, 3) and p.sn in (4, 6, 8, 10, 12)
        assert np.all(p.sigma_t >= 0.1 - 1e-12) and np.all(p.sigma_t <= 50.0 + 1e-9)
        c = p.sigma_s / p.sigma_t
        assert np.allclose(c, c[0]) and 0.3 <= c[0] <= 0.99
        assert np.all(p.q == 1.0)
    # seeded: the same problems again
    again = random_problems(64, seed=3)
    assert all(a.order == b.order and a.sn == b.sn and np.array_equal(a.sigma_t, b.sigma_t)
               for a, b in zip(probs, again))


def test_group_problems_partition():
    probs = random_problems(80, seed=5)
    groups = group_problems(probs)
    flat = sorted(i for g in groups for i in g)
    assert flat == list(range(80))                       # every problem exactly once
    keys = [(probs[g[0]].order, probs[g[0]].sn) for g in groups]
    assert len(set(keys)) == len(keys)                    # one group per (order, S_N)
    for g in groups:
        assert len({(probs[i].order, probs[i].sn) for i in g}) == 1
    assert keys == sorted(keys)


def test_union_offsets_of_a_group():
    probs = random_problems(6, seed=1, sides=(8, 16))
    mesh, eoff = M.disjoint_union([p.mesh for p in probs])
    assert eoff[0] == 0 and eoff[-1] == mesh.num_elements
    assert np.array_equal(np.diff(eoff), [p.mesh.num_elements for p in probs])
