"""Host logic of the pinned-host-buffer pipeline autotuner: every shape is
tried, timed by the host clock (median of the timed calls after two untimed
ones), and the fastest is left set on the handle.  A fake handle stands in for
the GPU: its Mult sleeps for a time that depends on the shape set last."""
import time

import pytest

pytest.importorskip("torch")

from allium_gb300.autotune import autotune_pipeline


class FakeHandle:
    def __init__(self, cost_ms):
        self.cost_ms = cost_ms
        self.shape = None
        self.calls = []

    def SetPipeline(self, chunks, streams, taper=0):
        self.shape = (chunks, streams, taper)

    def Mult(self, src, psi):
        self.calls.append(self.shape)
        time.sleep(self.cost_ms.get(self.shape, 6.0) * 1e-3)


def test_fastest_shape_is_kept():
    shapes = ((8, 4, 1), (8, 4, 0), (6, 4, 1), (12, 4, 2))
    L = FakeHandle({(6, 4, 1): 1.0})
    out = autotune_pipeline(L, None, None, reps=3, shapes=shapes)
    assert L.shape == (6, 4, 1)
    assert (out["best"]["chunks"], out["best"]["streams"], out["best"]["taper"]) == (6, 4, 1)
    assert [(t["chunks"], t["streams"], t["taper"]) for t in out["trials"]] == list(shapes)
    # two untimed and three timed calls per shape
    for s in shapes:
        assert L.calls.count(s) == 5
    best_ms = out["best"]["ms"]
    assert all(t["ms"] > best_ms for t in out["trials"] if (t["chunks"], t["streams"], t["taper"]) != (6, 4, 1))


def test_median_ignores_one_slow_call():
    """One slow timed call of the best shape (a host hiccup) does not move the
    choice: the median of three is taken."""
    class Hiccup(FakeHandle):
        def Mult(self, src, psi):
            self.calls.append(self.shape)
            n = self.calls.count(self.shape)
            ms = self.cost_ms.get(self.shape, 6.0)
            if self.shape == (8, 4, 0) and n == 3:
                ms = 40.0
            time.sleep(ms * 1e-3)

    L = Hiccup({(8, 4, 0): 1.0})
    out = autotune_pipeline(L, None, None, reps=3, shapes=((8, 4, 1), (8, 4, 0)))
    assert L.shape == (8, 4, 0) and out["best"]["ms"] < 5.0
