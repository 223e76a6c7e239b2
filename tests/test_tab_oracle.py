"""Tabulated 2-/3-body terms (the reference's TABULATION build, used by its
LAMMPS pair style), host side: the oracle's restatement of compute_2B_tab /
compute_3B_tab against the reference's own results (golden fixture, and the
reference built here when its sources exist), the product's parser on
tabulated files and the errors it reports, and the parameter cache."""

import ctypes
import json
import os
import shutil
import subprocess
import sys

import numpy as np
import pytest

from chimes_calculator_gb300 import synth
from oracle.oracle import REFROOT

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden", "tabulated")
sys.path.insert(0, os.path.join(HERE, "golden"))
import make_tab_golden as mtg  # noqa: E402

REF_EXAMPLE = os.path.join(REFROOT, "etc", "lmp", "tests", "example-tabulate")


def _queries():
    with open(os.path.join(GOLD, "queries.txt")) as f:
        return [ln.split() for ln in f if ln.strip()]


def _oracle_rows(o, queries):
    rows = []
    for t in queries:
        if t[0] == "2":
            e, f, st, fs = o.compute_2b_tab(float(t[3]), [float(v) for v in t[4:7]], [int(t[1]), int(t[2])])
            rows.append(np.concatenate([[e], f, st, [fs]]))
        else:
            e, f, st, fs = o.compute_3b_tab([float(v) for v in t[4:7]], [float(v) for v in t[7:16]],
                                            [int(v) for v in t[1:4]])
            rows.append(np.concatenate([[e], f, st, fs]))
    return rows


@pytest.fixture(scope="module")
def tab_set(tmp_path_factory):
    d = tmp_path_factory.mktemp("tab")
    return mtg.write_tab_set(str(d))


def test_oracle_reproduces_reference_fixture(tab_set):
    """compute_2B_tab / compute_3B_tab of the oracle against the reference's
    results stored in the fixture: bit for bit when the regenerated tables are
    byte-identical to the ones the reference read, else within 1e-12."""
    from oracle.oracle import Oracle
    meta = json.load(open(os.path.join(GOLD, "meta.json")))
    same_tables = mtg.table_digests(os.path.dirname(tab_set)) == meta["table_sha256"]
    o = Oracle(tab_set)
    assert o.tab_flags()[:2] == (1, 1)
    ref = [np.array([float(v) for v in ln.split()]) for ln in open(os.path.join(GOLD, "ref_out.txt"))]
    got = _oracle_rows(o, _queries())
    assert len(got) == len(ref) == 320
    assert o.tab_flags()[2] == 0
    nonzero = 0
    for a, b in zip(got, ref):
        if same_tables:
            assert np.array_equal(a, b)
        else:
            assert np.allclose(a, b, rtol=1e-12, atol=1e-12)
        nonzero += bool(np.any(b[1:7] != 0))
    assert nonzero > 250   # most queries lie inside the cutoffs


def test_oracle_matches_live_reference(tmp_path):
    """The reference built here (-DTABULATION) on another seeded set with
    finer 3-body grids, bit for bit."""
    from oracle import oracle
    if oracle.build_reference_tab() is None:
        pytest.skip("reference sources not present")
    spec = synth.spec_c2(elements=("C", "N", "O"), orders=(10, 6, 0), seed=3101)
    p = synth.write_tabulated_param_file(str(tmp_path / "t.txt"), spec, step2=0.01, step3=0.07, r0_3=0.75,
                                         seed=3102)
    rng = np.random.default_rng(3103)
    lines = []
    for k in range(200):
        t = rng.integers(0, 3, size=2)
        r = float(rng.uniform(0.55, 5.1))
        v = rng.normal(size=3)
        v = v / np.linalg.norm(v) * r
        lines.append("2 %d %d %r %r %r %r" % (t[0], t[1], r, float(v[0]), float(v[1]), float(v[2])))
    for k in range(200):
        t = rng.integers(0, 3, size=3)
        rr = rng.uniform(0.8, 4.2, size=3)
        v = rng.normal(size=9)
        lines.append("3 %d %d %d " % tuple(t) + " ".join(repr(float(x)) for x in np.concatenate([rr, v])))
    q = tmp_path / "q.txt"
    q.write_text("\n".join(lines) + "\n")
    ref = oracle.run_reference_tab(p, str(q), str(tmp_path / "out.txt"))
    got = _oracle_rows(oracle.Oracle(p), [ln.split() for ln in lines])
    for a, b in zip(got, ref):
        assert np.array_equal(a, b)


def test_oracle_matches_reference_on_its_example_table(tmp_path):
    """The reference's own tabulated 2-body table (its LAMMPS example), read
    here at test time: the oracle and the reference agree bit for bit over
    the table's range, grid points included."""
    from oracle import oracle
    if not os.path.isdir(REF_EXAMPLE) or oracle.build_reference_tab() is None:
        pytest.skip("reference sources not present")
    for ext in (".energy", ".force"):
        shutil.copy(os.path.join(REF_EXAMPLE, "chimes_scan_2b.type_0.dat" + ext), tmp_path)
    spec = synth.ParamSpec(elements=["C"], orders=(12, 0, 0), rin=1.0, rout=3.15, lam=1.25, fcut=("CUBIC",),
                           penalty=(0.1, 1.0e4), seed=3201)
    text = synth.build_param_text(spec).replace("PAIRTYPE PARAMS: 0 C C",
                                                "PAIRTYPE PARAMS: 0 C C TABULATED chimes_scan_2b.type_0.dat")
    p = tmp_path / "p.txt"
    p.write_text(text)
    grid = np.loadtxt(tmp_path / "chimes_scan_2b.type_0.dat.energy", skiprows=1)[:, 0]
    rng = np.random.default_rng(3202)
    rs = list(rng.uniform(grid[1] + 1e-6, 3.2, size=300)) + list(grid[2:-1:37])
    lines = []
    for r in rs:
        v = rng.normal(size=3)
        v = v / np.linalg.norm(v) * r
        lines.append("2 0 0 %r %r %r %r" % (float(r), float(v[0]), float(v[1]), float(v[2])))
    q = tmp_path / "q.txt"
    q.write_text("\n".join(lines) + "\n")
    ref = oracle.run_reference_tab(str(p), str(q), str(tmp_path / "out.txt"))
    got = _oracle_rows(oracle.Oracle(str(p)), [ln.split() for ln in lines])
    for a, b in zip(got, ref):
        assert np.array_equal(a, b)


def test_oracle_flags_distances_outside_the_table(tab_set):
    from oracle.oracle import Oracle
    o = Oracle(tab_set)
    o.compute_2b_tab(0.3, [0.3, 0.0, 0.0], [0, 0])      # below the first grid point
    assert o.tab_flags()[2] & 1
    e, f, st, fs = o.compute_2b_tab(7.0, [7.0, 0.0, 0.0], [0, 0])   # past the outer cutoff: nothing
    assert e == 0.0 and not f.any() and o.tab_flags()[2] == 0


# --------------------------------------------------------------------------
# product parser (host only)
# --------------------------------------------------------------------------
@pytest.fixture
def lib(native_lib):
    native_lib.ck_set_error_mode(1)
    return native_lib


def _check(lib, path):
    orders = (ctypes.c_int * 3)()
    nt = ctypes.c_int()
    cuts = (ctypes.c_double * 3)()
    rc = lib.ck_check_params(str(path).encode(), orders, ctypes.byref(nt), cuts)
    return rc, lib.ck_last_error().decode()


def test_tabulated_file_parses(lib, tab_set):
    rc, err = _check(lib, tab_set)
    assert rc == 0, err


def _variant(tmp_path, tab_set, edit):
    d = tmp_path / "v"
    shutil.copytree(os.path.dirname(tab_set), d)
    p = d / "tab.txt"
    edit(d, p)
    return p


@pytest.mark.parametrize("case,msg", [
    ("mixture", "tabulated or not tabulated"),
    ("missing_table", "could not open file"),
    ("length_mismatch", "differ in length"),
    ("not_ascending", "strictly ascending"),
    ("tiny_3b", "at least 2 grid points"),
    ("bad_row", "unexpected number of items"),
])
def test_tabulated_file_errors(lib, tmp_path, tab_set, case, msg):
    def edit(d, p):
        text = p.read_text()
        if case == "mixture":
            p.write_text(text.replace("PAIRTYPE PARAMS: 1 C N TABULATED tab_2b.type_1.dat", "PAIRTYPE PARAMS: 1 C N"))
        elif case == "missing_table":
            os.remove(d / "tab_3b.type_2.dat.force")
        elif case == "length_mismatch":
            f = d / "tab_2b.type_0.dat.force"
            rows = f.read_text().split("\n")
            f.write_text("\n".join([str(int(rows[0]) - 1)] + rows[1:-2]) + "\n")
        elif case == "not_ascending":
            f = d / "tab_2b.type_2.dat.energy"
            rows = f.read_text().split("\n")
            rows[5], rows[6] = rows[6], rows[5]
            f.write_text("\n".join(rows))
        elif case == "tiny_3b":
            for ext in (".energy", ".force"):
                f = d / ("tab_3b.type_1.dat" + ext)
                rows = f.read_text().split("\n")
                f.write_text("\n".join(["5"] + rows[1:6]) + "\n")
        elif case == "bad_row":
            f = d / "tab_3b.type_0.dat.force"
            rows = f.read_text().split("\n")
            rows[3] = " ".join(rows[3].split()[:4])
            f.write_text("\n".join(rows))
    rc, err = _check(lib, _variant(tmp_path, tab_set, edit))
    assert rc != 0 and msg in err, err


def test_tabulated_parameter_cache_round_trip(lib, tab_set, tmp_path):
    """The binary parameter cache keeps the tables: it packs into the same
    device image as the text file (tests/factored_check.cpp compares them)."""
    here = HERE
    csrc = os.path.join(os.path.dirname(here), "chimes_calculator_gb300", "csrc")
    exe = str(tmp_path / "factored_check")
    subprocess.run(["g++", "-O1", "-std=c++17", "-ffp-contract=off", "-I" + csrc,
                    os.path.join(here, "factored_check.cpp"), os.path.join(csrc, "ck_params.cpp"), "-o", exe],
                   check=True)
    cache = str(tmp_path / "tab.ckpc")
    assert lib.ck_convert_params(tab_set.encode(), cache.encode()) == 0, lib.ck_last_error()
    out = subprocess.run([exe, tab_set, cache], capture_output=True, text=True)
    # (the tabulated 3-body types have no coefficient lists, so only 4-body tuples are checked)
    assert out.returncode == 0 and out.stdout.strip().splitlines()[-1].startswith("ok"), out.stdout + out.stderr
    rc, err = _check(lib, cache)
    assert rc == 0, err
