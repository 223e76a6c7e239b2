"""The oracle's restatement of the LAMMPS pair style (pair_chimes.cpp) on
synthetic LAMMPS-style neighbour lists agrees with the oracle's serial
calculate when every ghost's force is folded back to its owner (boxes of at
least twice the cutoff, so no atom meets its own image): the two reference
drivers evaluate the same clusters."""

import numpy as np
import pytest

from chimes_calculator_gb300 import synth


@pytest.mark.parametrize("name", ["c1", "c2_small", "triclinic"])
def test_pair_style_restatement_matches_serial(golden, name):
    from oracle.oracle import Oracle
    g = golden[name]
    o = Oracle(g.params)
    ti = o.type_indices(g.cfg.types)
    skin = 1.0
    nl = synth.lammps_neighbors(g.cfg, ti, max(o.max_cutoffs) + skin, seed=5)
    r = o.lammps_compute(nl, skin)
    ref = o.calculate(g.cfg.pos, g.cfg.types, g.cfg.cell, small=False)
    F = np.zeros((g.cfg.n_atoms, 3))
    np.add.at(F, nl.owner, r["force"])
    vol = abs(np.linalg.det(g.cfg.cell))
    st = ref["stress"] * vol
    vir = np.array([st[0], st[4], st[8], st[1], st[2], st[5]])
    assert abs(r["energy"] - ref["energy"]) <= 1e-11 * abs(ref["energy"])
    assert np.abs(F - ref["force"]).max() <= 1e-10
    assert np.abs(r["virial"] - vir).max() <= 1e-9 * max(1.0, np.abs(vir).max())
    # per-atom shares add up to the totals
    assert abs(r["eatom"].sum() - r["energy"]) <= 1e-10 * max(1.0, abs(r["energy"]))
    assert np.abs(r["vatom"].sum(axis=0) - r["virial"]).max() <= 1e-9 * max(1.0, np.abs(r["virial"]).max())


def test_pair_style_lists_are_reused_until_rebuild(golden):
    from oracle.oracle import Oracle
    g = golden["c2_small"]
    o = Oracle(g.params)
    ti = o.type_indices(g.cfg.types)
    skin = 1.0
    nl = synth.lammps_neighbors(g.cfg, ti, max(o.max_cutoffs) + skin, seed=1)
    o.lammps_compute(nl, skin, rebuild=True)
    l3, l4 = o.lammps_lists()
    moved = synth.NeighborData(**{**nl.__dict__, "x": nl.x + 0.01})
    o.lammps_compute(moved, skin, rebuild=False)
    m3, m4 = o.lammps_lists()
    assert np.array_equal(l3, m3) and np.array_equal(l4, m4)
