"""Tabulated 2-/3-body terms on the GPU (the reference's TABULATION build):
the pair-style path (ck_nl_compute) against the oracle's restatement of
pair_chimes.cpp with compute_2B_tab / compute_3B_tab, and the per-cluster
entry (chimesFF::compute_2B_tab / compute_3B_tab) against the reference's own
results in the golden fixture."""

import json
import os
import sys

import numpy as np
import pytest

from conftest import E_REL_TOL, F_ABS_TOL, MIXED_E_REL_TOL, MIXED_F_ABS_TOL
from chimes_calculator_gb300 import synth

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden", "tabulated")
sys.path.insert(0, os.path.join(HERE, "golden"))
import make_tab_golden as mtg  # noqa: E402

SKIN = 1.0


@pytest.fixture(scope="module")
def tab_dir(tmp_path_factory):
    d = tmp_path_factory.mktemp("gtab")
    p = mtg.write_tab_set(str(d))
    return p


@pytest.fixture(scope="module")
def only2(tmp_path_factory):
    d = tmp_path_factory.mktemp("gtab2")
    return synth.write_tabulated_param_file(str(d / "t2.txt"), mtg.tab_spec(), tab3=False, seed=41)


@pytest.fixture(scope="module")
def only3(tmp_path_factory):
    d = tmp_path_factory.mktemp("gtab3")
    return synth.write_tabulated_param_file(str(d / "t3.txt"), mtg.tab_spec(), tab2=False, step3=0.1, seed=42)


def _setup(params, n_atoms=200, box=12.6, seed=5):
    from oracle.oracle import Oracle
    o = Oracle(params)
    cfg = synth.random_config(n_atoms, np.diag([box, box, box]), ["C", "N"], 1.0, seed=seed)
    ti = o.type_indices(cfg.types)
    nl = synth.lammps_neighbors(cfg, ti, max(o.max_cutoffs) + SKIN, seed=seed)
    return o, nl


def _close(a, b):
    assert abs(a["energy"] - b["energy"]) <= E_REL_TOL * max(1.0, abs(b["energy"]))
    assert np.abs(a["force"] - b["force"]).max() <= F_ABS_TOL
    assert np.abs(a["virial"] - b["virial"]).max() <= 1e-9 * max(1.0, np.abs(b["virial"]).max())


@pytest.mark.parametrize("which", ["both", "only2", "only3"])
@pytest.mark.parametrize("precision", [0, 1])
def test_pair_style_matches_oracle(native_lib, tab_dir, only2, only3, which, precision):
    from chimes_calculator_gb300 import Calculator
    params = {"both": tab_dir, "only2": only2, "only3": only3}[which]
    o, nl = _setup(params)
    ref = o.lammps_compute(nl, SKIN, rebuild=True)
    c = Calculator(precision=precision)
    c.load_params(params)
    assert c.tabulated() == (which != "only3", which != "only2")
    r = c.nl_compute(nl, SKIN, rebuild=True, per_atom=True)
    # tabulated terms are looked up in FP64 in either precision form; the
    # Chebyshev terms beside them follow the mixed budget in precision 1
    etol, ftol = (E_REL_TOL, F_ABS_TOL) if precision == 0 else (MIXED_E_REL_TOL, MIXED_F_ABS_TOL)
    assert abs(r["energy"] - ref["energy"]) <= etol * max(1.0, abs(ref["energy"]))
    assert np.abs(r["force"] - ref["force"]).max() <= ftol
    if precision == 0:
        _close(r, ref)
        assert np.abs(r["eatom"] - ref["eatom"]).max() <= 1e-9
        assert np.abs(r["vatom"] - ref["vatom"]).max() <= 1e-9 * max(1.0, np.abs(ref["vatom"]).max())
    for a, b in zip(c.nl_lists(), o.lammps_lists()):
        assert np.array_equal(a, b)


def test_pair_style_reuses_lists_with_tables(native_lib, tab_dir):
    from chimes_calculator_gb300 import Calculator
    o, nl = _setup(tab_dir, seed=9)
    c = Calculator()
    c.load_params(tab_dir)
    o.lammps_compute(nl, SKIN, rebuild=True)
    c.nl_compute(nl, SKIN, rebuild=True)
    rng = np.random.default_rng(1)
    moved = synth.NeighborData(**{**nl.__dict__, "x": nl.x + rng.uniform(-0.15, 0.15, nl.x.shape)})
    for _ in range(2):
        ref = o.lammps_compute(moved, SKIN, rebuild=False)
        r = c.nl_compute(moved, SKIN, rebuild=False)
        _close(r, ref)


def _gold_rows():
    with open(os.path.join(GOLD, "queries.txt")) as f:
        q = [ln.split() for ln in f if ln.strip()]
    ref = [np.array([float(v) for v in ln.split()]) for ln in open(os.path.join(GOLD, "ref_out.txt"))]
    return q, ref


def test_per_cluster_tab_matches_reference_fixture(native_lib, tab_dir):
    """compute_2B_tab / compute_3B_tab per cluster against the reference's
    results: bit for bit when the regenerated tables are byte-identical to the
    ones the reference read, else within 1e-12."""
    from chimes_calculator_gb300 import Calculator
    meta = json.load(open(os.path.join(GOLD, "meta.json")))
    exact = mtg.table_digests(os.path.dirname(tab_dir)) == meta["table_sha256"]
    c = Calculator()
    c.load_params(tab_dir)
    q, ref = _gold_rows()
    for nb in (2, 3):
        rows = [(t, r) for t, r in zip(q, ref) if int(t[0]) == nb]
        P = 1 if nb == 2 else 3
        typ = np.array([[int(v) for v in t[1:1 + nb]] for t, _ in rows])
        dx = np.array([[float(v) for v in t[1 + nb:1 + nb + P]] for t, _ in rows])
        dr = np.array([[float(v) for v in t[1 + nb + P:1 + nb + 4 * P]] for t, _ in rows])
        out = c.clusters(nb, dx, dr, typ, tab=True)
        got = np.concatenate([out["energy"][:, None], out["force"].reshape(len(rows), -1), out["stress"],
                              out["fscal"]], axis=1)
        want = np.array([r for _, r in rows])
        if exact:
            assert np.array_equal(got, want)
        else:
            assert np.allclose(got, want, rtol=1e-12, atol=1e-12)


def test_errors(native_lib, tab_dir):
    from chimes_calculator_gb300 import Calculator, ChimesError
    c = Calculator()
    c.load_params(tab_dir)
    # a 2-body distance below the table: the reference prints and exits
    with pytest.raises(ChimesError, match="outside the tabulated range"):
        c.clusters(2, [[0.3]], [[[0.3, 0.0, 0.0]]], [[0, 0]], tab=True)
    # the Chebyshev entry on a tabulated term, and the serial interface, refuse the set
    with pytest.raises(ChimesError, match="tabulated"):
        c.clusters(2, [[2.0]], [[[2.0, 0.0, 0.0]]], [[0, 0]])
    cfg = synth.random_config(20, np.diag([9.0, 9.0, 9.0]), ["C", "N"], 1.0, seed=3)
    with pytest.raises(ChimesError, match="tabulated"):
        c.evaluate(cfg.pos, c.type_indices(cfg.types), cfg.cell)
    # the context stays usable
    out = c.clusters(2, [[2.0]], [[[2.0, 0.0, 0.0]]], [[0, 0]], tab=True)
    assert np.isfinite(out["energy"]).all()
