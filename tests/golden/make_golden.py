"""Writes tests/golden/lsquad.json from allium's level-symmetric tables.

Run with the path of a reference checkout (read only):
    python tests/golden/make_golden.py <reference root>
The fixture keeps, for each order N, the directions and weights exactly as the
reference's LevelSymmetricQuadrature builds them (src/angular_quadrature.cpp:
98-147): all rows in 3D; in 2D the first half with weights doubled.  The tests
compare the library's own level-symmetric generator against it.
"""
import json
import os
import sys

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "lsquad.json")


def read(ref, n):
    with open(os.path.join(ref, "data", "lsquad", f"LS_{n}.txt")) as f:
        lines = f.read().split("\n")
    head = lines[0]
    total = int(head.split("Total Directions =")[1].split()[0])
    rows = [[float(x) for x in l.split()] for l in lines[1:] if l.strip()]
    assert len(rows) == total
    return rows


def main():
    if len(sys.argv) != 2:
        sys.exit("usage: make_golden.py <reference root>")
    ref = sys.argv[1]
    out = {}
    for n in range(2, 13, 2):   # the orders the library generates
        rows = read(ref, n)
        out[str(n)] = {
            "3": {"omega": [r[:3] for r in rows], "weights": [r[3] for r in rows]},
            "2": {"omega": [r[:2] for r in rows[: len(rows) // 2]], "weights": [2 * r[3] for r in rows[: len(rows) // 2]]},
        }
    with open(OUT, "w") as f:
        json.dump(out, f)
    print("wrote", OUT)


if __name__ == "__main__":
    main()
