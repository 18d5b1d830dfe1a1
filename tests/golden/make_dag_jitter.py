"""Writes dag_jitter.json: whether the S12 upwind graph of the 64^3 hex mesh of
the benchmark stays acyclic when its interior vertices are jittered by +-0.2h
(the configuration's stated jitter) and by +-0.1h (the benchmark's), over
several seeds, using the CPU oracle's Kahn levels (-1 = a cycle, which the
reference rejects: src/sweep.cpp:205-208).  Recorded: +-0.2h cyclic for every
seed; +-0.1h cyclic for seeds 1 and 2, acyclic (220 levels) for the benchmark's.  Run from the repository root:
    python tests/golden/make_dag_jitter.py [cells]
"""
import json
import os
import sys
import time

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

from allium_gb300 import mesh as M  # noqa: E402
from allium_gb300 import quadrature as Q  # noqa: E402
from oracle.oracle import OracleSweep  # noqa: E402

BENCH_SEED = 20261203


def levels(cells, jitter, seed, sn=12):
    mesh = M.cartesian((cells,) * 3, jitter=jitter, seed=seed)
    quad = Q.level_symmetric(sn, 3)
    o = OracleSweep(mesh, 1, quad, np.ones((1, mesh.num_elements)))
    nl, _ = o.levels()
    return int(nl)


def main():
    cells = int(sys.argv[1]) if len(sys.argv) > 1 else 64
    runs = [(0.2, s) for s in list(range(1, 9)) + [BENCH_SEED]] + [(0.1, BENCH_SEED), (0.1, 1), (0.1, 2)]
    out = {"cells": cells, "order": 1, "sn": 12, "directions": 168, "results": []}
    for jit, seed in runs:
        t0 = time.time()
        nl = levels(cells, jit, seed)
        out["results"].append({"jitter_h": jit, "seed": seed, "levels": nl, "acyclic": nl >= 0})
        print(jit, seed, nl, f"{time.time() - t0:.0f}s", flush=True)
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "dag_jitter.json")
    with open(path, "w") as f:
        json.dump(out, f, indent=1)


if __name__ == "__main__":
    main()
