"""The drop-in C++ and per-cluster C surfaces, executed on the GPU.

tests/dropin_check.cpp is a program written against the reference's own
interfaces -- serial_chimes_interface::calculate
(serial_interface/src/serial_chimes_interface.h:97-103), chimesFF::compute_1B
/ compute_2B / compute_3B / compute_4B with and without force_scalar_in and
get_badness (chimesFF/src/chimesFF.h:152-192), chimes_compute_{2,3,4}b_props
and their _fromf90 forms (chimesFF/api/chimescalc_C.cpp:86-318).  It is
compiled here against include/ and libchimescalc.so and run on the GPU; its
output is compared with fixtures the reference made (tests/golden/*/expected.json
and tests/golden/clusters/, see make_cluster_golden.py): energies 1e-10
relative, forces, stress and force scalars 1e-9, badness exactly, and the
accumulate / overwrite semantics of each call."""

import json
import os
import subprocess

import numpy as np
import pytest

from conftest import E_REL_TOL, F_ABS_TOL, GOLDEN, REPO, S_ABS_TOL

pytestmark = pytest.mark.gpu

CLUSTERS = os.path.join(GOLDEN, "clusters")


@pytest.fixture(scope="module")
def dropin_exe(native_lib, tmp_path_factory):
    exe = str(tmp_path_factory.mktemp("dropin") / "dropin_check")
    lib_dir = os.path.dirname(native_lib._name)
    subprocess.run(["g++", "-O1", "-std=c++11", "-I", os.path.join(REPO, "include"),
                    os.path.join(REPO, "tests", "dropin_check.cpp"), "-o", exe, "-L", lib_dir, "-lchimescalc",
                    "-Wl,-rpath," + lib_dir], check=True)
    return exe


def _run(exe, *args):
    p = subprocess.run([exe, *map(str, args)], capture_output=True, text=True)
    assert p.returncode == 0, p.stdout + p.stderr


@pytest.mark.parametrize("name", ["c2_small", "triclinic", "smallbox", "replicate", "penalty", "c4_n8_rho012",
                                  "ref_tio2_arbrot", "ref_chon"])
def test_serial_interface_class(golden, dropin_exe, tmp_path, name):
    """serial_chimes_interface::calculate adds energy and forces into the
    caller's values and overwrites the stress; get_badness reports the
    configuration's short pairs.  With replication (small = true) the
    reference divides the whole energy sum, the caller's incoming value
    included, by (n_replicates + 1)^3 (serial_chimes_interface.cpp:1105)."""
    from oracle.oracle import Oracle
    g = golden[name]
    o = Oracle(g.params)
    scale = 1.0
    if g.small:   # the oracle restates the reference's accumulation: energy 2 in, zero forces
        r2 = o.calculate(g.cfg.pos, g.cfg.types, g.cfg.cell, small=True, energy=2.0)
        scale = (r2["energy"] - g.energy) / 2.0
    out = tmp_path / "out.txt"
    _run(dropin_exe, "serial", g.params, g.xyz, int(g.small), out)
    rows = out.read_text().split("\n")
    e = float(rows[0])
    s = np.array([float(v) for v in rows[1].split()])
    n = g.cfg.n_atoms
    f = np.array([[float(v) for v in r.split()] for r in rows[2:2 + n]])
    badness = int(rows[2 + n])
    assert abs(e - (2.0 * scale + g.energy)) <= E_REL_TOL * max(1.0, abs(g.energy))
    assert g.force_error(f - 0.1) <= F_ABS_TOL
    assert np.abs(s - g.stress).max() <= S_ABS_TOL
    assert badness == o.calculate(g.cfg.pos, g.cfg.types, g.cfg.cell, small=g.small)["badness"]
    if name == "penalty":
        assert badness > 0


def _ref_rows(case):
    with open(os.path.join(CLUSTERS, case, "queries.txt")) as f:
        queries = [ln.split() for ln in f if ln.strip()]
    with open(os.path.join(CLUSTERS, case, "ref_out.txt")) as f:
        ref = [[float(v) for v in ln.split()] for ln in f if ln.strip()]
    assert len(queries) == len(ref)
    return queries, ref


def _split(row, nb):
    npair = nb * (nb - 1) // 2
    e = row[0]
    f = np.array(row[1:1 + 3 * nb])
    s = np.array(row[1 + 3 * nb:7 + 3 * nb])
    rest = row[7 + 3 * nb:]
    return e, f, s, np.array(rest[:npair if nb > 1 else 0]), rest[npair if nb > 1 else 0:]


@pytest.mark.parametrize("case", sorted(os.listdir(CLUSTERS)))
def test_chimesFF_methods(golden, dropin_exe, tmp_path, case):
    """chimesFF::compute_1B..4B (both overloads) on the reference's own
    per-cluster results, force_scalar_in and get_badness included."""
    g = golden[case]
    queries, ref = _ref_rows(case)
    out = tmp_path / "out.txt"
    _run(dropin_exe, "clusters", g.params, os.path.join(CLUSTERS, case, "queries.txt"), out)
    got = [[float(v) for v in ln.split()] for ln in out.read_text().split("\n") if ln.strip()]
    assert len(got) == len(ref)
    seen = set()
    for q, a, b in zip(queries, got, ref):
        nb = int(q[0])
        ea, fa, sa, fsa, tail_a = _split(a, nb)
        eb, fb, sb, fsb, tail_b = _split(b, nb)
        assert abs(ea - eb) <= E_REL_TOL * max(1.0, abs(eb)), (case, q[:4])
        assert np.abs(fa - fb).max() <= F_ABS_TOL, (case, q[:4])
        assert np.abs(sa - sb).max() <= S_ABS_TOL, (case, q[:4])
        if nb > 1:
            assert np.abs(fsa - fsb).max() <= 1e-9 * max(1.0, np.abs(fsb).max()), (case, q[:4])
        assert int(tail_a[0]) == int(tail_b[0]), "badness"          # get_badness after the call
        assert int(tail_a[1]) == 1, "overload without force_scalar_in differs"
        seen.add((nb, eb != 0.0, int(tail_b[0])))
    if case == "penalty":
        assert {(2, True, 1), (2, True, 2)} <= seen


@pytest.mark.parametrize("case", ["c2_small", "ref_hn3"])
def test_per_cluster_c_abi(golden, dropin_exe, tmp_path, case):
    """chimes_compute_{2,3,4}b_props and the _fromf90 forms add energy, forces
    and the six packed stress components into the caller's values and leave
    stress[6..8] as they were (the 4-body wrapper's copy-in/assign-back,
    chimescalc_C.cpp:290-317, has the same effect)."""
    g = golden[case]
    queries, ref = _ref_rows(case)
    out = tmp_path / "out.txt"
    _run(dropin_exe, "capi", g.params, os.path.join(CLUSTERS, case, "queries.txt"), out)
    got = [[float(v) for v in ln.split()] for ln in out.read_text().split("\n") if ln.strip()]
    multi = [(q, r) for q, r in zip(queries, ref) if int(q[0]) >= 2]
    assert len(got) == len(multi)
    counts = {2: 0, 3: 0, 4: 0}
    for (q, r), a in zip(multi, got):
        nb = int(q[0])
        eb, fb, sb, _, _ = _split(r, nb)
        w = 1 + 3 * nb + 9
        for form in range(2):
            row = a[form * w:(form + 1) * w]
            e, f, s = row[0], np.array(row[1:1 + 3 * nb]), np.array(row[1 + 3 * nb:])
            assert abs(e - (1.0 + eb)) <= E_REL_TOL * max(1.0, abs(eb)), (case, q[:4], form)
            assert np.abs(f - (0.25 + fb)).max() <= F_ABS_TOL, (case, q[:4], form)
            assert np.abs(s[:6] - (0.5 + sb)).max() <= S_ABS_TOL, (case, q[:4], form)
            assert np.all(s[6:] == 0.5), (case, q[:4], form)
        counts[nb] += eb != 0.0
    assert min(counts.values()) > 5, counts
