"""Generates the per-cluster golden fixtures under tests/golden/clusters/ from
the UNMODIFIED reference (its chimesFF.cpp, default build).

For a few of the golden parameter sets it draws clusters of 1-4 atoms from the
case's configuration (atoms near a random centre, with their displacement
vectors), writes them as a query file and runs the reference's own
chimesFF::compute_1B / compute_2B / compute_3B / compute_4B -- the overloads
that return force_scalar_in -- through oracle/ref_cluster_driver.cpp.  The
fixture holds the queries, the type names of the parameter set and the
reference's results per query (energy, forces, stress, force_scalar_in at 17
significant digits, get_badness after the call).  The GPU tests run the
library's drop-in C++ class and per-cluster C interface on the same queries.

Run from the repository root where the reference sources are available:
    python tests/golden/make_cluster_golden.py
"""

from __future__ import annotations

import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)
sys.path.insert(0, os.path.join(REPO, "tests"))

from oracle import oracle  # noqa: E402

OUT = os.path.join(HERE, "clusters")
# golden case -> (clusters of 2, 3, 4 atoms, reach of the draw for each order, seed)
CASES = {
    "penalty": ((120, 0, 0), (1.6, 0.0, 0.0), 5101),     # short pairs: penalty and damping below rin
    "c2_small": ((80, 120, 120), (5.5, 4.2, 3.3), 5102),
    "triclinic": ((60, 80, 80), (5.0, 4.2, 3.2), 5103),  # cubic cutoff, SPECIFIC cutoffs, energy offsets
    "ref_hn3": ((60, 100, 100), (5.5, 4.2, 3.3), 5104),  # a fitted force field with SPECIAL cutoffs
}


def draw(cfg, nb, count, reach, rng):
    """Clusters of nb atoms near a random centre: (type names, dx[P], dr[P][3])."""
    pos, cell = cfg.pos, cfg.cell
    inv = np.linalg.inv(cell)
    pairs = [(i, j) for i in range(nb) for j in range(i + 1, nb)]
    out = []
    tries = 0
    while len(out) < count and tries < 100000:
        tries += 1
        i0 = int(rng.integers(len(pos)))
        d = (pos - pos[i0]) @ inv
        d -= np.round(d)
        r = np.sqrt(((d @ cell) ** 2).sum(1))
        near = np.where((r > 0) & (r < reach))[0]
        if len(near) < nb - 1:
            continue
        ids = np.concatenate([[i0], rng.choice(near, size=nb - 1, replace=False)])
        p = [d[k] @ cell for k in ids]
        dr = np.array([p[j] - p[i] for i, j in pairs])
        dx = np.sqrt((dr ** 2).sum(1))
        out.append(([cfg.types[k] for k in ids], dx, dr))
    return out


def main():
    from conftest import Golden
    if not os.path.isdir(oracle.REFROOT):
        raise SystemExit("reference sources unavailable: cannot generate the per-cluster fixtures")
    subprocess.run(["make", "-s", "-C", os.path.join(REPO, "oracle"), "refcl", "REFROOT=" + oracle.REFROOT],
                   check=True)
    drv = os.path.join(REPO, "oracle", "_ref", "ref_cluster_driver")
    for case, (counts, reaches, seed) in CASES.items():
        g = Golden(case)
        o = oracle.Oracle(g.params)
        names = sorted(set(g.cfg.types))
        tidx = {n: int(o.type_indices([n])[0]) for n in names}
        rng = np.random.default_rng(seed)
        lines, qnames = [], []
        for n in names:                                   # compute_1B of every type present
            lines.append("1 %d" % tidx[n])
            qnames.append([n])
        for nb, count, reach in zip((2, 3, 4), counts, reaches):
            for tn, dx, dr in draw(g.cfg, nb, count, reach, rng):
                t = [tidx[n] for n in tn]
                lines.append(" ".join([str(nb)] + [str(v) for v in t] + [repr(float(v)) for v in dx] +
                                      [repr(float(v)) for v in dr.reshape(-1)]))
                qnames.append(tn)
        d = os.path.join(OUT, case)
        os.makedirs(d, exist_ok=True)
        with open(os.path.join(d, "queries.txt"), "w") as f:
            f.write("\n".join(lines) + "\n")
        with tempfile.TemporaryDirectory() as tmp:
            out = os.path.join(tmp, "out.txt")
            subprocess.run([drv, g.params, os.path.join(d, "queries.txt"), out], check=True, capture_output=True)
            with open(out) as f:
                res = f.read()
        with open(os.path.join(d, "ref_out.txt"), "w") as f:
            f.write(res)
        with open(os.path.join(d, "meta.json"), "w") as f:
            json.dump({"case": case, "type_names": qnames, "counts": counts, "seed": seed}, f)
        print(case, len(lines), "queries")


if __name__ == "__main__":
    main()
