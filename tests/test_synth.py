"""Seeded workload generator: orbit counts, determinism, and that its
parameter files parse in both the oracle and the product parser."""

import numpy as np
import pytest

from chimes_calculator_gb300 import synth


def test_orbit_counts():
    # multisets of 3 powers in [0,7] with at most one zero: C(10,3) - 8 = 112
    assert len(synth.power_orbits((0, 0, 0), 8, 2)) == 112
    assert len(synth.power_orbits((0, 0, 0), 10, 2)) == 210
    # no symmetry with three distinct atoms: every tuple is its own orbit
    assert len(synth.power_orbits((0, 1, 2), 10, 2)) == 972
    total = sum(len(o) for o in synth.power_orbits((0, 0, 1, 1), 4, 3))
    assert total == 4 ** 6 - 1 - 6 * 3 - 15 * 9     # sextets with >= 3 nonzero powers


def test_generator_is_deterministic():
    a = synth.build_param_text(synth.spec_c2())
    b = synth.build_param_text(synth.spec_c2())
    assert a == b
    c1 = synth.config_c1()
    c2 = synth.config_c1()
    assert np.array_equal(c1.pos, c2.pos) and c1.types == c2.types


def test_minimum_image_rejection():
    cfg = synth.config_c1()
    f = cfg.pos @ np.linalg.inv(cfg.cell)
    d = f[:, None, :] - f[None, :, :]
    d -= np.round(d)
    r = np.sqrt(((d @ cfg.cell) ** 2).sum(-1))
    r[np.arange(len(r)), np.arange(len(r))] = 99
    assert r.min() >= 1.2


def test_params_parse_in_oracle_and_product(tmp_path, native_lib):
    import ctypes
    from oracle.oracle import Oracle
    p = synth.write_param_file(str(tmp_path / "p.txt"), synth.spec_c3())
    o = Oracle(p)
    assert o.orders == (12, 10, 4)
    orders = (ctypes.c_int * 3)()
    nt = ctypes.c_int()
    cuts = (ctypes.c_double * 3)()
    native_lib.ck_set_error_mode(1)
    assert native_lib.ck_check_params(p.encode(), orders, ctypes.byref(nt), cuts) == 0
    assert tuple(orders) == (12, 10, 4) and nt.value == 2
    assert tuple(cuts) == pytest.approx(o.max_cutoffs)
