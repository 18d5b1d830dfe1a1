"""Host-side logic of the solvers that needs no GPU: splitting a psi-sized
RIGHT source q[(g Nw + a) Ndof + i] into its per-cell isotropic part."""
from types import SimpleNamespace

import pytest

torch = pytest.importorskip("torch")

from allium_gb300.solvers import split_isotropic


def _iso(G, Nw, ndof, seed=0):
    g = torch.Generator().manual_seed(seed)
    cell = torch.rand((G, 1, ndof), generator=g, dtype=torch.float64)
    return cell, cell.expand(G, Nw, ndof).contiguous().reshape(-1)


def test_isotropic_source_is_split():
    L = SimpleNamespace(G=2, Nw=5, ndof=7)
    cell, q = _iso(2, 5, 7)
    q_iso, rest = split_isotropic(L, q)
    assert rest is None
    assert torch.equal(q_iso, cell.reshape(-1))


@pytest.mark.parametrize("where", [0, 17, 69])
def test_one_direction_differs(where):
    L = SimpleNamespace(G=2, Nw=5, ndof=7)
    _, q = _iso(2, 5, 7, seed=1)
    q[where] += 1e-12
    q_iso, rest = split_isotropic(L, q)
    assert q_iso is None and rest is q


def test_nan_is_not_isotropic():
    L = SimpleNamespace(G=1, Nw=3, ndof=2)
    q = torch.full((6,), float("nan"), dtype=torch.float64)
    q_iso, rest = split_isotropic(L, q)
    assert q_iso is None and rest is q
