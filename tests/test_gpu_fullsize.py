"""Full-size workloads (too large for the oracle in test time) checked through
size-independent properties: zero net force (every cluster term is a sum of
equal-and-opposite pair forces), FP64 against the mixed path, invariance
under a rigid translation of all atoms, and list counts against the pair
density."""

import numpy as np
import pytest

from conftest import MIXED_E_REL_TOL, MIXED_F_ABS_TOL

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def c3(tmp_path_factory):
    from chimes_calculator_gb300 import synth
    d = tmp_path_factory.mktemp("c3")
    p = synth.write_param_file(str(d / "p.txt"), synth.spec_c3())
    return p, synth.config_c3()


def test_c3_fp64_vs_mixed_and_momentum(c3, native_lib):
    from chimes_calculator_gb300 import FP64, MIXED, Calculator
    p, cfg = c3
    out = {}
    for prec in (FP64, MIXED):
        c = Calculator(precision=prec)
        c.load_params(p)
        out[prec] = c.evaluate(cfg.pos, cfg.types, cfg.cell)
        counts = c.counts()
    r64, r32 = out[FP64], out[MIXED]
    assert np.abs(r64["force"].sum(axis=0)).max() < 1e-9 * cfg.n_atoms
    assert abs(r32["energy"] - r64["energy"]) <= MIXED_E_REL_TOL * abs(r64["energy"])
    assert np.abs(r32["force"] - r64["force"]).max() <= MIXED_F_ABS_TOL
    s = r64["stress"].reshape(3, 3)
    assert np.allclose(s, s.T, atol=0)
    # pairs within the 5 A search radius, each counted once (ai <= parent): ~ N rho 4/3 pi r^3 / 2
    rho = cfg.n_atoms / abs(np.linalg.det(cfg.cell))
    expect = cfg.n_atoms * rho * 4.0 / 3.0 * np.pi * 5.0 ** 3 / 2
    assert 0.8 * expect < counts["n2"] < 1.2 * expect


def test_c3_translation_invariance(c3, native_lib):
    from chimes_calculator_gb300 import Calculator
    p, cfg = c3
    c = Calculator()
    c.load_params(p)
    a = c.evaluate(cfg.pos, cfg.types, cfg.cell)
    b = c.evaluate(cfg.pos + np.array([1.37, -2.11, 0.53]), cfg.types, cfg.cell)
    assert abs(a["energy"] - b["energy"]) <= 1e-9 * abs(a["energy"])
    assert np.abs(a["force"] - b["force"]).max() <= 1e-8
