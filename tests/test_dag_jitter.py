"""The benchmark's +-0.1h jitter instead of the configuration's +-0.2h, as a
measured fact: at +-0.2h the S12 upwind graph of the 64^3 hex mesh has a cycle
for every seed tried (9 seeds; the reference rejects such graphs,
src/sweep.cpp:205-208).  At +-0.1h cycles still occur at 64^3 (seeds 1, 2) but
the benchmark's seed gives an acyclic graph of 220 levels.  The 64^3 results
come from tests/golden/make_dag_jitter.py (the CPU oracle's Kahn levels, about
15 s per mesh); on a 16^3 mesh +-0.2h is cyclic and +-0.1h acyclic, live."""
import json
import os

import pytest

from tests.golden.make_dag_jitter import BENCH_SEED, levels

HERE = os.path.dirname(os.path.abspath(__file__))


def test_recorded_64_cubed_results():
    with open(os.path.join(HERE, "golden", "dag_jitter.json")) as f:
        d = json.load(f)
    assert d["cells"] == 64 and d["sn"] == 12 and d["directions"] == 168
    wide = [r for r in d["results"] if r["jitter_h"] == 0.2]
    narrow = [r for r in d["results"] if r["jitter_h"] == 0.1]
    assert len(wide) >= 8 and all(not r["acyclic"] and r["levels"] == -1 for r in wide)
    assert any(r["seed"] == BENCH_SEED for r in wide)
    bench_run = [r for r in narrow if r["seed"] == BENCH_SEED]
    assert bench_run and bench_run[0]["acyclic"] and bench_run[0]["levels"] == 220
    assert all(r["acyclic"] == (r["levels"] > 0) for r in d["results"])


@pytest.mark.parametrize("seed", [1, 2, 3, 4])
def test_small_mesh_same_behaviour(seed):
    assert levels(16, 0.2, seed) == -1
    assert levels(16, 0.1, seed) > 0
