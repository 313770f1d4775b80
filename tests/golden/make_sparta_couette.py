"""Extract the SPARTA Couette solution that ships with the reference's tests
into tests/golden/sparta_couette.json (the JSON is committed).

Usage: python tests/golden/make_sparta_couette.py <reference>/test/data/external

Source files (reference repository, test/data/external): in.Couette (the
SPARTA input: 50 cells over 5e-4 m, Ar VHS d = 4.11e-10 m, omega = 0.81,
diffuse walls at 300 K moving at -/+500 m/s, nrho 5e22, fnum 5e14 (1,000
particles per cell), dt 2.59e-9 s, 50,000 steps, grid and wall quantities
averaged over steps 14,001-50,000), avg_seed_12345.grid.50000 (per cell:
temp, press, n, nrho, u, v) and boundary_seed_12345.grid.50000 (per wall:
nflux, mflux, press, shx, shy, shz, ke).  The reference's
test/test_1D_couette.jl:115-118 notes that its Couette solution, averaged
over the same steps, was compared with this one.
"""
import json
import os
import sys

if len(sys.argv) != 2:
    sys.exit("usage: make_sparta_couette.py <directory holding in.Couette and the *.grid.50000 files>")
SRC = sys.argv[1]
OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "sparta_couette.json")


def read_grid(path):
    lines = open(path).read().splitlines()
    i = next(k for k, ln in enumerate(lines) if ln.startswith("ITEM: CELLS"))
    rows = [ln.split() for ln in lines[i + 1:] if ln.strip()]
    return [[float(x) for x in r[1:7]] for r in sorted(rows, key=lambda r: int(r[0]))]


def read_boundary(path):
    rows = [ln.split() for ln in open(path).read().splitlines() if ln.strip() and not ln.startswith("#")]
    rows = [r for r in rows if len(r) == 8]
    return [[float(x) for x in r[1:8]] for r in rows[:2]]


def main():
    cells = read_grid(os.path.join(SRC, "avg_seed_12345.grid.50000"))
    walls = read_boundary(os.path.join(SRC, "boundary_seed_12345.grid.50000"))
    assert len(cells) == 50 and len(walls) == 2
    out = {"source": "reference test/data/external (SPARTA, seed 12345)",
           "setup": {"L": 5e-4, "n_cells": 50, "T_wall": 300.0, "v_wall": 500.0, "nrho": 5e22, "ppc": 1000,
                     "dt": 2.59e-9, "n_steps": 50000, "avg_from": 14001},
           "cell_columns": ["temp", "press", "n", "nrho", "u", "v"], "cells": cells,
           "wall_columns": ["nflux", "mflux", "press", "shx", "shy", "shz", "ke"], "walls": walls}
    with open(OUT, "w") as f:
        json.dump(out, f, indent=1)
    print(OUT)


if __name__ == "__main__":
    main()
