"""The oracle (C restatement of the reference) against the reference's own
outputs: the committed golden fixtures (generated by the compiled reference,
tests/golden/make_golden.py) and -- where the reference tree is present -- the
reference's own regression fixtures and a fresh reference build."""

import os

import numpy as np
import pytest

from conftest import golden_names, list_digest

from oracle.oracle import REFROOT, Oracle



@pytest.mark.parametrize("name", golden_names(large=False))
def test_oracle_matches_reference_golden(golden, name):
    g = golden[name]
    o = Oracle(g.params)
    r = o.calculate(g.cfg.pos, g.cfg.types, g.cfg.cell, small=g.small)
    # the restatement keeps the reference's operation order: agreement to the last bits
    assert abs(r["energy"] - g.energy) <= 1e-12 * max(1.0, abs(g.energy))
    assert np.abs(r["force"] - g.force).max() <= 1e-12
    assert np.abs(r["stress"] - g.stress).max() <= 1e-14
    l2, l3, l4 = o.lists()
    for key, arr in (("l2", l2), ("l3", l3), ("l4", l4)):
        assert arr.shape[0] == g.lists[key]["n"]
        assert list_digest(arr) == g.lists[key]["sha256"], key


def test_oracle_accumulates_like_reference(golden):
    """calculate adds into the caller's energy and forces (calculate_chimes_instance :93-95)."""
    g = golden["c1"]
    o = Oracle(g.params)
    f0 = np.full((g.cfg.n_atoms, 3), 0.25)
    r = o.calculate(g.cfg.pos, g.cfg.types, g.cfg.cell, energy=3.0, force=f0)
    assert abs(r["energy"] - (g.energy + 3.0)) < 1e-10
    assert np.abs(r["force"] - (g.force + 0.25)).max() < 1e-12


def _ref_cases():
    base = os.path.join(REFROOT, "serial_interface", "tests")
    return [
        ("published_params.liqC.2+3b.cubic.txt", "liqC.2.5gcc_6000K.OUTCAR_#000.xyz", False),
        ("published_params.liqC.2b.cubic.txt", "liqC.2.5gcc_6000K.OUTCAR_#000.xyz", False),
        ("validated_params.TiO2.2+3b.Tersoff.txt", "TiO2.unitcell_arbrot_#000.xyz", False),
        ("published_params.liqCO.2+3b.cubic.txt", "diam.8_#000.xyz", True),
        ("published_params.CO2400K.2+3+4b.Tersoff.special.offsets.txt", "CO.9GPa_2400K.OUTCAR_#000.xyz", True),
        ("published_params.HN3.2+3+4b.Tersoff.special.offsets.txt", "HN3.2gcc_3000K.OUTCAR_#000.xyz", False),
        ("test_params.CHON.txt", "CHON.testfile_#000.xyz", False),
    ], base


def _expected_dat(base, ff, xyz):
    p = os.path.join(base, "expected_output", "%s.%s.dat" % (ff, xyz))
    if not os.path.exists(p):
        return None
    vals = [float(v) for v in open(p).read().split()]
    return vals


@pytest.mark.skipif(not os.path.isdir(REFROOT), reason="reference tree not present")
def test_oracle_against_reference_regression_fixtures():
    """The reference's own golden outputs (serial_interface/tests/expected_output,
    compared at its 1e-3 absolute tolerance, compare.sh:29) on its own inputs."""
    from chimes_calculator_gb300 import synth
    cases, base = _ref_cases()
    checked = 0
    for ff, xyz, small in cases:
        exp = _expected_dat(base, ff, xyz)
        if exp is None:
            continue
        cfg = synth.read_xyz(os.path.join(base, "configurations", xyz))
        r = Oracle(os.path.join(base, "force_fields", ff)).calculate(cfg.pos, cfg.types, cfg.cell, small=small)
        s = r["stress"] * 6.9479   # GPa, as the reference's debug.dat (examples/cpp/main.cpp:132-149)
        got = [r["energy"], s[0], s[4], s[8], s[1], s[2], s[5]] + list(r["force"].reshape(-1))
        assert len(got) == len(exp)
        assert np.abs(np.array(got) - np.array(exp)).max() < 1e-3, (ff, xyz)
        checked += 1
    assert checked >= 3


@pytest.mark.skipif(not os.path.isdir(REFROOT), reason="reference tree not present")
def test_oracle_bit_exact_against_reference_build(tmp_path):
    """Fresh reference build on the reference's own fixtures: identical results and cluster lists."""
    from oracle.oracle import build_reference, run_reference
    from chimes_calculator_gb300 import synth
    if build_reference() is None:
        pytest.skip("reference could not be compiled")
    cases, base = _ref_cases()
    for ff, xyz, small in cases[:5]:
        p = os.path.join(base, "force_fields", ff)
        x = os.path.join(base, "configurations", xyz)
        ref, lst, _ = run_reference(p, x, small, str(tmp_path / "r"), lists=True)
        cfg = synth.read_xyz(x)
        o = Oracle(p)
        r = o.calculate(cfg.pos, cfg.types, cfg.cell, small=small)
        assert r["energy"] == ref["energy"], ff
        assert np.array_equal(r["force"], ref["force"]), ff
        assert np.array_equal(r["stress"], ref["stress"]), ff
        for a, b in zip(o.lists(), lst):
            assert np.array_equal(a, b), ff
