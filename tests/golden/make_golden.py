"""Generates the golden fixtures under tests/golden/ from the UNMODIFIED
reference calculator.

Each case is a seeded synthetic parameter file (ChIMES text format) plus a
periodic configuration.  The reference's own serial_chimes_interface::calculate
is compiled from the reference sources by oracle/Makefile (target ``ref``) and
run on every case; its energy, forces and stress are stored at 17 significant
digits together with the sizes and SHA-256 digests of its cluster lists
(neighlist_2b/3b/4b in the reference's order).  The GPU tests compare against
these files; the reference itself is not needed where the tests run.

Besides the small seeded cases it writes:
  * the 12/10/4 recipe of the large workloads: a cut-down 3072-atom box of the
    32768-atom two-element configuration at the same density (``c3_cut``), the
    full 32768-atom configuration (``c3_full``: energy, stress, list digests,
    every 16th atom's force and force sums; the configuration is regenerated
    from its seed and checked by digest), four three-element configurations
    of the batched workload's extremes (8 and 512 atoms at 0.05 and 0.12
    atoms/A^3) and each of the serving workload's three parameter sets on one
    configuration;
  * the reference's own regression inputs (serial_interface/tests: HN3
    2+3+4-body with SPECIAL cutoffs and energy offsets, CO2400K with
    replication, the rotated TiO2 cell, CHON), with the reference's parameter
    files stored gzipped and its configurations verbatim (``ref_*``).

Run from the repository root where the reference sources are available
(REFROOT, default the reference checkout the oracle's Makefile uses):
    python tests/golden/make_golden.py [case ...]
"""

from __future__ import annotations

import gzip
import hashlib
import json
import os
import shutil
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

from chimes_calculator_gb300 import synth  # noqa: E402
from oracle import oracle  # noqa: E402


def lists_digest(l2, l3, l4):
    out = {}
    for name, a in (("l2", l2), ("l3", l3), ("l4", l4)):
        a = np.ascontiguousarray(np.asarray(a, dtype="<i4"))
        out[name] = {"n": int(a.shape[0]), "sha256": hashlib.sha256(a.tobytes()).hexdigest()}
    return out


def tri_cell(a, b, c, alpha, beta, gamma):
    """Lattice vectors (rows) of a triclinic cell, then rotated off-axis."""
    al, be, ga = np.radians([alpha, beta, gamma])
    va = np.array([a, 0.0, 0.0])
    vb = np.array([b * np.cos(ga), b * np.sin(ga), 0.0])
    cx = c * np.cos(be)
    cy = c * (np.cos(al) - np.cos(be) * np.cos(ga)) / np.sin(ga)
    vc = np.array([cx, cy, np.sqrt(c * c - cx * cx - cy * cy)])
    th = 0.37
    R = np.array([[np.cos(th), -np.sin(th), 0.1], [np.sin(th), np.cos(th), -0.2], [0.05, 0.15, 1.0]])
    q, _ = np.linalg.qr(R)
    return np.stack([va, vb, vc]) @ q.T


def lattice_config(elements, L, reps, jitter, seed):
    """Diamond-like crystal (8-site cubic basis) with a small seeded jitter."""
    rng = np.random.default_rng(seed)
    basis = np.array([[0, 0, 0], [0, .5, .5], [.5, 0, .5], [.5, .5, 0],
                      [.25, .25, .25], [.25, .75, .75], [.75, .25, .75], [.75, .75, .25]])
    pts = []
    for i in range(reps):
        for j in range(reps):
            for k in range(reps):
                pts.extend((basis + [i, j, k]) / reps)
    frac = np.array(pts)
    cell = np.diag([L, L, L])
    pos = frac @ cell + rng.normal(0, jitter, size=frac.shape)
    types = [elements[i % len(elements)] for i in range(len(pos))]
    return synth.Config(types, pos, cell)


def cases():
    """name -> (ParamSpec, Config, small)"""
    C = {}
    C["c1"] = (synth.spec_c1(), synth.config_c1(), False)
    C["c2"] = (synth.spec_c2(), synth.config_c2(), False)
    C["c2_small"] = (synth.spec_c2(seed=2002), synth.config_c2(n_atoms=200, box=12.6, seed=2102), False)
    # triclinic, cubic fcut, SPECIFIC cutoffs, energy offsets, explicit penalty settings
    spec = synth.ParamSpec(elements=["C", "N"], orders=(10, 6, 4), rin=(0.8, 1.0), rout=(4.2, 4.8), lam=(1.2, 1.6),
                           fcut=("CUBIC",), s3max={0: [4.0, 4.0, 4.0], 1: [4.1, 3.9, 3.9], 2: [3.8, 3.8, 4.2],
                                                   3: [4.0, 4.0, 4.0]},
                           s4max={0: [3.0] * 6, 1: [3.1, 3.1, 2.9, 3.1, 2.9, 2.9], 2: [3.0] * 6,
                                  3: [3.2, 3.0, 3.0, 3.0, 3.0, 2.8], 4: [3.0] * 6},
                           s3min=0.7, energy_offsets=[-12.5, -7.25], penalty=(0.02, 5.0e3), seed=2003)
    cell = tri_cell(11.0, 12.0, 11.5, 78.0, 96.0, 105.0)
    C["triclinic"] = (spec, synth.random_config(150, cell, ["C", "N"], 1.0, seed=2103), False)
    # box smaller than twice the cutoff: multi-image and self-image clusters
    spec = synth.ParamSpec(elements=["C", "N", "O"], orders=(8, 5, 3), rin=0.9, rout=4.5, lam=1.4,
                           fcut=("TERSOFF", 0.5), s3max=4.0, s4max=3.0, seed=2004)
    C["smallbox"] = (spec, synth.random_config(20, np.diag([6.0, 6.5, 7.0]), ["C", "N", "O"], 1.1, seed=2104),
                     False)
    # replication of a tiny crystalline cell (small = true)
    spec = synth.ParamSpec(elements=["C"], orders=(12, 6, 0), rin=1.0, rout=4.0, lam=1.3,
                           fcut=("TERSOFF", 0.5), s3max=3.6, seed=2005)
    C["replicate"] = (spec, lattice_config(["C"], 3.57, 1, 0.03, seed=2105), True)
    # excluded many-body types
    spec = synth.ParamSpec(elements=["C", "N"], orders=(12, 6, 3), rin=0.9, rout=5.0, lam=1.4,
                           fcut=("TERSOFF", 0.5), s3max=4.0, s4max=3.2, excluded3=(1,), excluded4=(2,), seed=2006)
    C["excluded"] = (spec, synth.random_config(120, np.diag([11.0, 11.0, 11.0]), ["C", "N"], 1.0, seed=2106),
                     False)
    # penalty region and distances below the inner cutoff
    spec = synth.ParamSpec(elements=["C"], orders=(12, 5, 0), rin=1.1, rout=4.5, lam=1.4, fcut=("TERSOFF", 0.5),
                           s3max=3.5, penalty=(0.15, 1.0e3), seed=2007)
    C["penalty"] = (spec, synth.random_config(60, np.diag([8.5, 8.5, 8.5]), ["C"], 0.95, seed=2107), False)
    # published-style expanded coefficient lists (every permutation listed)
    spec = synth.ParamSpec(elements=["C", "N"], orders=(12, 6, 3), rin=0.9, rout=5.0, lam=(1.3, 1.6),
                           fcut=("TERSOFF", 0.5), s3max=4.0, s4max=3.2, expand=True, seed=2008)
    C["expanded"] = (spec, synth.random_config(128, np.diag([11.2, 11.2, 11.2]), ["C", "N"], 1.0, seed=2108), False)
    # 4B cutoff larger than 3B cutoff: the valid_3mer carry-over of the reference's enumeration
    spec = synth.ParamSpec(elements=["C", "N"], orders=(10, 5, 3), rin=0.9, rout=5.0, lam=1.4,
                           fcut=("TERSOFF", 0.5), s3max=3.0, s4max=3.6, seed=2009)
    C["rc4_gt_rc3"] = (spec, synth.random_config(100, np.diag([10.0, 10.0, 10.0]), ["C", "N"], 1.0, seed=2109),
                       False)
    # 2B only
    spec = synth.ParamSpec(elements=["C", "N", "O"], orders=(16, 0, 0), rin=0.8, rout=6.0, lam=(1.2, 1.8),
                           fcut=("CUBIC",), seed=2010)
    C["twobody"] = (spec, synth.random_config(90, np.diag([10.0, 11.0, 12.0]), ["C", "N", "O"], 1.0, seed=2110),
                    False)
    return C


C3_DENSITY = 32768 / (70.0 * 70.0 * 72.0)
# atoms kept for the full-size case's force comparison: every FORCE_STRIDE-th
FORCE_STRIDE = 16


def cycled(cfg, elements):
    """Types assigned cyclically so every element (and most type tuples) occurs."""
    return synth.Config([elements[i % len(elements)] for i in range(cfg.n_atoms)], cfg.pos, cfg.cell)


def recipe_cases():
    """The 12/10/4 parameter recipe of the full-size, batched and serving
    workloads: name -> (ParamSpec, Config, small, extra)."""
    C = {}
    n = 3072
    L = (n / C3_DENSITY / (72.0 / 70.0)) ** (1.0 / 3.0)
    C["c3_cut"] = (synth.spec_c3(), synth.config_c3(n_atoms=n, box=(L, L, L * 72.0 / 70.0), seed=3103), False, {})
    C["c3_full"] = (synth.spec_c3(), synth.config_c3(), False,
                    {"large": True, "params_from": "c3_cut", "config_from": "config_c3"})
    spec4 = synth.spec_c4()
    for k, (n, rho) in enumerate(((8, 0.05), (8, 0.12), (512, 0.05), (512, 0.12))):
        L = (n / rho) ** (1.0 / 3.0)
        cfg = synth.random_config(n, np.diag([L, L, L]), ["C", "N", "O"], 1.0, seed=3400 + k)
        C["c4_n%d_rho%03d" % (n, int(round(rho * 100)))] = (spec4, cycled(cfg, ["C", "N", "O"]), False,
                                                             {} if k == 0 else {"params_from": "c4_n8_rho005"})
    for k, spec in enumerate(synth.specs_c5()):
        n = (96, 300, 240)[k]
        L = (n / 0.09) ** (1.0 / 3.0)
        cfg = synth.random_config(n, np.diag([L, L * 1.05, L * 0.95]), spec.elements, 1.0, seed=3500 + k)
        C["c5_set%d" % k] = (spec, cycled(cfg, list(spec.elements)), False, {})
    return C


# the reference's own regression inputs (serial_interface/tests/test_list.dat)
REF_FIELDS = {
    "ref_hn3": ("published_params.HN3.2+3+4b.Tersoff.special.offsets.txt", "HN3.2gcc_3000K.OUTCAR_#000.xyz", False),
    "ref_co2400k": ("published_params.CO2400K.2+3+4b.Tersoff.special.offsets.txt", "CO.9GPa_2400K.OUTCAR_#000.xyz",
                    True),
    "ref_tio2_arbrot": ("validated_params.TiO2.2+3b.Tersoff.txt", "TiO2.unitcell_arbrot_#000.xyz", False),
    "ref_chon": ("test_params.CHON.txt", "CHON.testfile_#000.xyz", False),
}


def write_expected(d, name, small, res, lst, timing, n_atoms, extra):
    out = {
        "case": name,
        "small": bool(small),
        "n_atoms": n_atoms,
        "energy": repr(res["energy"]),
        "stress": [repr(float(v)) for v in res["stress"]],
        "lists": lists_digest(*lst),
        "reference_seconds": timing["best_s"],
    }
    F = np.asarray(res["force"])
    if extra.get("large"):
        idx = np.arange(0, n_atoms, FORCE_STRIDE)
        out["force_index"] = {"start": 0, "stride": FORCE_STRIDE}
        out["force"] = [[repr(float(v)) for v in row] for row in F[idx]]
        out["force_sum"] = [repr(float(v)) for v in F.sum(axis=0)]
        out["force_sumsq"] = repr(float((F * F).sum()))
    else:
        out["force"] = [[repr(float(v)) for v in row] for row in F]
    for k in ("large", "params_from", "config_from", "config_sha256", "source"):
        if k in extra:
            out[k] = extra[k]
    with open(os.path.join(d, "expected.json"), "w") as f:
        json.dump(out, f, indent=0)
    print(name, n_atoms, "E=%.10f" % res["energy"], {k: v["n"] for k, v in out["lists"].items()},
          "%.3fs" % timing["best_s"])


def gzip_copy(src, dst):
    """Deterministic gzip (no name, fixed mtime) so regenerating leaves git clean."""
    with open(src, "rb") as f:
        data = f.read()
    with open(dst, "wb") as raw:
        with gzip.GzipFile(filename="", mode="wb", fileobj=raw, mtime=0, compresslevel=9) as g:
            g.write(data)


def main(names):
    C = cases()
    R = recipe_cases()
    names = names or (list(C) + list(R) + list(REF_FIELDS))
    if oracle.build_reference() is None:
        raise SystemExit("reference sources unavailable: cannot generate golden fixtures")
    with tempfile.TemporaryDirectory() as scratch:
        for name in names:
            d = os.path.join(HERE, name)
            os.makedirs(d, exist_ok=True)
            extra = {}
            if name in REF_FIELDS:
                ff, xyz, small = REF_FIELDS[name]
                base = os.path.join(oracle.REFROOT, "serial_interface", "tests")
                pfile = os.path.join(scratch, name + ".params.txt")
                shutil.copyfile(os.path.join(base, "force_fields", ff), pfile)
                gzip_copy(pfile, os.path.join(d, "params.txt.gz"))
                xfile = os.path.join(d, "config.xyz")
                shutil.copyfile(os.path.join(base, "configurations", xyz), xfile)
                n_atoms = synth.read_xyz(xfile).n_atoms
                extra["source"] = "serial_interface/tests: force_fields/%s, configurations/%s" % (ff, xyz)
            else:
                spec, cfg, small = C[name] if name in C else R[name][:3]
                extra = {} if name in C else dict(R[name][3])
                n_atoms = cfg.n_atoms
                if "params_from" in extra:
                    pfile = os.path.join(HERE, extra["params_from"], "params.txt")
                else:
                    pfile = synth.write_param_file(os.path.join(d, "params.txt"), spec)
                if "config_from" in extra:
                    # too large to commit: regenerated from its seed, pinned by digest
                    text = cfg.xyz_text()
                    extra["config_sha256"] = hashlib.sha256(text.encode()).hexdigest()
                    xfile = os.path.join(scratch, name + ".xyz")
                    with open(xfile, "w") as f:
                        f.write(text)
                else:
                    xfile = cfg.write_xyz(os.path.join(d, "config.xyz"))
            res, lst, timing = oracle.run_reference(pfile, xfile, small, os.path.join(scratch, name),
                                                    lists=True, time_reps=1)
            write_expected(d, name, small, res, lst, timing, n_atoms, extra)


if __name__ == "__main__":
    main(sys.argv[1:])
