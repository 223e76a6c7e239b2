"""Generates the golden fixture of the tabulated 2-/3-body terms from the
UNMODIFIED reference (its chimesFF.cpp built with -DTABULATION, the option its
LAMMPS pair style uses).

The tabulated parameter set is regenerated wherever it is needed by
``synth.write_tabulated_param_file`` with the arguments in ``meta.json`` (the
tables are several MB, so they are not stored); the fixture holds the cluster
queries, the reference's results for them (compute_2B_tab / compute_3B_tab:
energy, forces, stress, force_scalar_in at 17 significant digits) and SHA-256
digests of the tables the reference read, so a test can tell whether its
regenerated tables are byte-identical.

Run from the repository root where the reference sources are available:
    python tests/golden/make_tab_golden.py
"""

from __future__ import annotations

import hashlib
import json
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

from chimes_calculator_gb300 import synth  # noqa: E402
from oracle import oracle  # noqa: E402

OUT = os.path.join(HERE, "tabulated")
# generator arguments of the tabulated set: 2 elements, 2B order 12, 3B order 8
# (tabulated), 4B order 4 (Chebyshev); 2B grids 0.5 A + k * 0.005 A, 3B grids
# 0.8 A + k * 0.1 A
META = {"spec": {"elements": ["C", "N"], "orders": [12, 8, 4], "seed": 3001},
        "tab": {"r0_2": 0.5, "step2": 0.005, "r0_3": 0.8, "step3": 0.1, "seed": 3002},
        "queries": {"n2": 160, "n3": 160, "seed": 3003}}


def tab_spec():
    m = META["spec"]
    return synth.spec_c2(elements=tuple(m["elements"]), orders=tuple(m["orders"]), seed=m["seed"])


def write_tab_set(directory: str) -> str:
    return synth.write_tabulated_param_file(os.path.join(directory, "tab.txt"), tab_spec(), **META["tab"])


def table_digests(directory: str) -> dict:
    out = {}
    for name in sorted(os.listdir(directory)):
        if name.endswith(".energy") or name.endswith(".force"):
            with open(os.path.join(directory, name), "rb") as f:
                out[name] = hashlib.sha256(f.read()).hexdigest()
    return out


def make_queries(param_file: str) -> list:
    """Cluster queries inside the tables' ranges (the reference exits on a
    2-body distance at or below a table's second grid point): random 2-body
    distances, exact 2-body grid points (the interval-start branch of
    get_tab_2B), 3-body distances below and past the 3-body cutoffs."""
    q = META["queries"]
    rng = np.random.default_rng(q["seed"])
    d = os.path.dirname(param_file)
    nt = len(META["spec"]["elements"])
    lines = []

    def unit():
        v = rng.normal(size=3)
        return v / np.linalg.norm(v)

    grid = np.loadtxt(os.path.join(d, "tab_2b.type_0.dat.energy"), skiprows=1)[:, 0]
    for k in range(q["n2"]):
        t = rng.integers(0, nt, size=2)
        r = float(grid[2 + rng.integers(0, len(grid) - 4)]) if k % 4 == 0 else float(rng.uniform(0.6, 5.2))
        dr = unit() * r
        lines.append("2 %d %d %r %r %r %r" % (t[0], t[1], r, float(dr[0]), float(dr[1]), float(dr[2])))
    for k in range(q["n3"]):
        t = rng.integers(0, nt, size=3)
        rr = rng.uniform(0.9, 4.3 if k % 3 == 0 else 3.95, size=3)
        drs = np.concatenate([unit() * r for r in rr])
        lines.append("3 %d %d %d " % tuple(t) + " ".join(repr(float(v)) for v in rr) + " " +
                     " ".join(repr(float(v)) for v in drs))
    return lines


def main():
    if oracle.build_reference_tab() is None:
        raise SystemExit("reference sources unavailable: cannot generate the tabulated fixture")
    os.makedirs(OUT, exist_ok=True)
    with tempfile.TemporaryDirectory() as d:
        pfile = write_tab_set(d)
        lines = make_queries(pfile)
        qfile = os.path.join(OUT, "queries.txt")
        with open(qfile, "w") as f:
            f.write("\n".join(lines) + "\n")
        rows = oracle.run_reference_tab(pfile, qfile, os.path.join(d, "ref.out"))
        with open(os.path.join(OUT, "ref_out.txt"), "w") as f:
            for r in rows:
                f.write(" ".join(repr(float(v)) for v in r) + "\n")
        meta = dict(META)
        meta["table_sha256"] = table_digests(d)
        with open(os.path.join(OUT, "meta.json"), "w") as f:
            json.dump(meta, f, indent=1)
    print("wrote", OUT)


if __name__ == "__main__":
    main()
