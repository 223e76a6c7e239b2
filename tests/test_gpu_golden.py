"""GPU parity against the reference on every golden case: cluster lists
identical to the reference's (same members, same order), FP64 energies,
forces and stress within the stated tolerances, and the mixed-precision path
within its error budget."""

import numpy as np
import pytest

from conftest import (E_REL_TOL, F_ABS_TOL, MIXED_E_REL_TOL, MIXED_F_ABS_TOL, MIXED_S_ABS_TOL, S_ABS_TOL,
                      golden_names, list_digest, mixed_force_tol)

pytestmark = pytest.mark.gpu


def evaluate(g, precision=0, graph=False, tpc=None, factored=True):
    from chimes_calculator_gb300 import Calculator
    c = Calculator(precision=precision, graph=graph)
    c.set_contraction(factored)
    if tpc:
        c.set_tuning(*tpc)
    c.load_params(g.params)
    r = c.evaluate(g.cfg.pos, g.cfg.types, g.cfg.cell, small=g.small)
    return c, r


@pytest.mark.parametrize("factored", [1, 2, 3, 0], ids=["factored", "factored_nocache", "factored_noy", "per_coef"])
@pytest.mark.parametrize("name", golden_names())
def test_fp64_matches_reference(golden, native_lib, name, factored):
    g = golden[name]
    c, r = evaluate(g, factored=factored)
    assert abs(r["energy"] - g.energy) <= E_REL_TOL * max(1.0, abs(g.energy))
    assert g.force_error(r["force"]) <= F_ABS_TOL
    assert np.abs(r["stress"] - g.stress).max() <= S_ABS_TOL
    l2, l3, l4 = c.lists()
    for key, arr in (("l2", l2), ("l3", l3), ("l4", l4)):
        assert arr.shape[0] == g.lists[key]["n"], key
        assert list_digest(arr) == g.lists[key]["sha256"], key


@pytest.mark.parametrize("name", golden_names(large=False))
def test_lists_match_oracle(golden, native_lib, name):
    from oracle.oracle import Oracle
    g = golden[name]
    c, _ = evaluate(g)
    o = Oracle(g.params)
    o.calculate(g.cfg.pos, g.cfg.types, g.cfg.cell, small=g.small)
    for a, b in zip(c.lists(), o.lists()):
        assert np.array_equal(a, b)


@pytest.mark.parametrize("factored", [1, 2, 3, 0, 4],
                         ids=["factored", "factored_nocache", "factored_noy", "per_coef", "tensor_core"])
@pytest.mark.parametrize("name", golden_names())
def test_mixed_precision_error(golden, native_lib, name, factored):
    """The mixed form against the reference's own FP64 results (the values
    stored in the fixture), not against the GPU's FP64 path: energy 1e-6
    relative, forces 1e-5 absolute (5e-6 of the largest force for the fitted
    force fields, whose forces reach hundreds of kcal/mol/A), stress 1e-5."""
    g = golden[name]
    _, r32 = evaluate(g, precision=1, factored=factored)
    assert abs(r32["energy"] - g.energy) <= MIXED_E_REL_TOL * max(1.0, abs(g.energy))
    assert g.force_error(r32["force"]) <= mixed_force_tol(np.abs(g.force).max())
    assert np.abs(r32["stress"] - g.stress).max() <= MIXED_S_ABS_TOL


def test_tensor_core_form_runs(golden, native_lib):
    """The tensor-core 3-body and 4-body contractions are the ones that run
    when asked for in the mixed form (3-body orders 2-11; 4-body with 2-4
    powers per pair: c3_cut, c2_small and smallbox have 4, rc4_gt_rc3 3, c1 no
    4-body term), give the reference's results within the mixed budget, and
    leave the FP64 form on the CUDA cores."""
    for name, tc4 in (("c3_cut", 1), ("c2_small", 1), ("c1", 0), ("smallbox", 1), ("rc4_gt_rc3", 1),
                      ("ref_hn3", 1)):
        g = golden[name]
        c, r = evaluate(g, precision=1, factored=4)
        assert c.tuning()["tc3"] == 1, name
        assert c.tuning()["tc4"] == tc4, name
        assert abs(r["energy"] - g.energy) <= MIXED_E_REL_TOL * max(1.0, abs(g.energy)), name
        assert g.force_error(r["force"]) <= mixed_force_tol(np.abs(g.force).max()), name
        c64, r64 = evaluate(g, precision=0, factored=4)
        assert c64.tuning()["tc3"] == 0 and c64.tuning()["tc4"] == 0
        assert abs(r64["energy"] - g.energy) <= E_REL_TOL * max(1.0, abs(g.energy))


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "mixed"])
@pytest.mark.parametrize("factored", [1, 3, 0], ids=["factored", "factored_noy", "per_coef"])
@pytest.mark.parametrize("tpc", [(1, 1, 2), (2, 4, 4), (8, 16, 4), (32, 32, 2), (4, 2, 1), (1, 2, 4)])
def test_threads_per_cluster_variants(golden, native_lib, tpc, factored, precision):
    """Every launch shape of every contraction form (lanes per cluster, one-warp
    blocks per SM; one lane per cluster takes the one-stream passes) gives the
    reference's results, FP64 within the FP64 tolerances and mixed within its
    error budget."""
    g = golden["c2_small"]
    _, r = evaluate(g, precision=precision, tpc=tpc, factored=factored)
    et, ft = (E_REL_TOL, F_ABS_TOL) if precision == 0 else (MIXED_E_REL_TOL, MIXED_F_ABS_TOL)
    assert abs(r["energy"] - g.energy) <= et * max(1.0, abs(g.energy))
    assert np.abs(r["force"] - g.force).max() <= ft


def test_autotune_keeps_results(golden, native_lib):
    from chimes_calculator_gb300 import MIXED, Calculator
    g = golden["c2_small"]
    for prec in (0, MIXED):
        c = Calculator(precision=prec)
        c.load_params(g.params)
        packed = c.pack([(g.cfg.pos, g.cfg.types, g.cfg.cell)])
        t3, t4, bps = c.autotune(packed)
        assert t3 in (1, 2, 4, 8, 16, 32) and t4 in (1, 2, 4, 8, 16, 32) and bps in (1, 2, 4, 8)
        assert c.autotune() == (t3, t4, bps)          # cached for the same batch shape
        r = c.evaluate(g.cfg.pos, g.cfg.types, g.cfg.cell)
        tol = E_REL_TOL if prec == 0 else 1e-6
        assert abs(r["energy"] - g.energy) <= tol * max(1.0, abs(g.energy))


def test_graph_replay(golden, native_lib):
    from chimes_calculator_gb300 import Calculator
    g = golden["c2"]
    c = Calculator(graph=True)
    c.load_params(g.params)
    for _ in range(3):
        r = c.evaluate(g.cfg.pos, g.cfg.types, g.cfg.cell)
        assert abs(r["energy"] - g.energy) <= E_REL_TOL * abs(g.energy)
        assert np.abs(r["force"] - g.force).max() <= F_ABS_TOL


def test_tensor_core_4body_two_powers(tmp_path, native_lib):
    """4-body order 2 runs the tensor-core 4-body kernel at its smallest width
    (two powers per pair: rows and columns of 8, K = 8, N = 16) and gives the
    oracle's result within the mixed budget; the FP64 form matches it within
    the FP64 tolerances."""
    from chimes_calculator_gb300 import FP64, MIXED, Calculator, synth
    from oracle.oracle import Oracle
    spec = synth.ParamSpec(elements=["C", "N"], orders=(10, 4, 2), rin=0.9, rout=5.0, lam=(1.3, 1.6),
                           fcut=("TERSOFF", 0.5), s3max=4.0, s4max=3.2, seed=4343)
    p = synth.write_param_file(str(tmp_path / "p.txt"), spec)
    cfg = synth.random_config(160, np.diag([12.0, 12.0, 12.0]), ["C", "N"], 1.0, seed=4344)
    ref = Oracle(p).calculate(cfg.pos, cfg.types, cfg.cell)
    for prec, etol, ftol in ((MIXED, MIXED_E_REL_TOL, MIXED_F_ABS_TOL), (FP64, E_REL_TOL, F_ABS_TOL)):
        c = Calculator(precision=prec)
        c.set_contraction(4)
        c.load_params(p)
        r = c.evaluate(cfg.pos, cfg.types, cfg.cell)
        assert c.tuning()["tc4"] == (1 if prec == MIXED else 0)
        assert abs(r["energy"] - ref["energy"]) <= etol * max(1.0, abs(ref["energy"]))
        assert np.abs(r["force"] - ref["force"]).max() <= ftol
