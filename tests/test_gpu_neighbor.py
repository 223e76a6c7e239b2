"""Pair-style path (ck_nl_compute): the GPU form of LAMMPS pair_style chimesFF
on a LAMMPS-style neighbour list against the oracle's restatement of
pair_chimes.cpp -- the same 3-/4-body cluster lists in the same order,
energy, per-atom forces (ghosts included) and virial; lists reused between
rebuilds; the mixed form within its budget."""

import numpy as np
import pytest

from conftest import E_REL_TOL, F_ABS_TOL, MIXED_E_REL_TOL, MIXED_F_ABS_TOL
from chimes_calculator_gb300 import synth

pytestmark = pytest.mark.gpu

SKIN = 1.0


def _setup(g, seed=7):
    from oracle.oracle import Oracle
    o = Oracle(g.params)
    ti = o.type_indices(g.cfg.types)
    nl = synth.lammps_neighbors(g.cfg, ti, max(o.max_cutoffs) + SKIN, seed=seed)
    return o, nl


def _calc(g, precision=0, factored=True):
    from chimes_calculator_gb300 import Calculator
    c = Calculator(precision=precision)
    c.set_contraction(factored)
    c.load_params(g.params)
    return c


def _close(a, b, etol, ftol):
    assert abs(a["energy"] - b["energy"]) <= etol * max(1.0, abs(b["energy"]))
    assert np.abs(a["force"] - b["force"]).max() <= ftol
    assert np.abs(a["virial"] - b["virial"]).max() <= 1e-9 * max(1.0, np.abs(b["virial"]).max())


@pytest.mark.parametrize("factored", [True, False], ids=["factored", "per_coef"])
@pytest.mark.parametrize("name", ["c1", "c2_small", "triclinic", "smallbox", "excluded", "penalty"])
def test_matches_pair_style_oracle(golden, native_lib, name, factored):
    g = golden[name]
    o, nl = _setup(g)
    ref = o.lammps_compute(nl, SKIN)
    c = _calc(g, factored=factored)
    r = c.nl_compute(nl, SKIN)
    _close(r, ref, E_REL_TOL, F_ABS_TOL)
    for a, b in zip(c.nl_lists(), o.lammps_lists()):
        assert np.array_equal(a, b)


@pytest.mark.parametrize("name", ["c2_small", "smallbox"])
def test_per_atom_energy_and_virial(golden, native_lib, name):
    g = golden[name]
    o, nl = _setup(g)
    ref = o.lammps_compute(nl, SKIN)
    r = _calc(g).nl_compute(nl, SKIN, per_atom=True)
    _close(r, ref, E_REL_TOL, F_ABS_TOL)
    assert np.abs(r["eatom"] - ref["eatom"]).max() <= 1e-9
    assert np.abs(r["vatom"] - ref["vatom"]).max() <= 1e-9 * max(1.0, np.abs(ref["vatom"]).max())


def test_lists_reused_until_rebuild(golden, native_lib):
    g = golden["c2_small"]
    o, nl = _setup(g, seed=3)
    c = _calc(g)
    o.lammps_compute(nl, SKIN, rebuild=True)
    c.nl_compute(nl, SKIN, rebuild=True)
    rng = np.random.default_rng(0)
    moved = synth.NeighborData(**{**nl.__dict__, "x": nl.x + rng.uniform(-0.2, 0.2, nl.x.shape)})
    ref = o.lammps_compute(moved, SKIN, rebuild=False)
    r = c.nl_compute(moved, SKIN, rebuild=False)
    _close(r, ref, E_REL_TOL, F_ABS_TOL)
    for a, b in zip(c.nl_lists(), o.lammps_lists()):
        assert np.array_equal(a, b)


def test_mixed_within_budget(golden, native_lib):
    g = golden["c2"]
    o, nl = _setup(g)
    ref = o.lammps_compute(nl, SKIN)
    r = _calc(g, precision=1).nl_compute(nl, SKIN)
    assert abs(r["energy"] - ref["energy"]) <= MIXED_E_REL_TOL * abs(ref["energy"])
    assert np.abs(r["force"] - ref["force"]).max() <= MIXED_F_ABS_TOL


def test_rejects_bad_neighbour_index(golden, native_lib):
    from chimes_calculator_gb300 import ChimesError
    g = golden["c1"]
    o, nl = _setup(g)
    bad = synth.NeighborData(**{**nl.__dict__, "neigh": nl.neigh.copy()})
    bad.neigh[5] = len(nl.x) + 3
    with pytest.raises(ChimesError):
        _calc(g).nl_compute(bad, SKIN)
