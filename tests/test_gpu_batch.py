"""Batched evaluation: many configurations of different sizes, cells and
parameter sets in one set of launches give each configuration's own result,
and match the oracle on a sample of the mixed-size workload."""

import numpy as np
import pytest

from conftest import E_REL_TOL, F_ABS_TOL, MIXED_E_REL_TOL, MIXED_F_ABS_TOL, S_ABS_TOL

pytestmark = pytest.mark.gpu


def test_heterogeneous_batch_equals_golden(golden, native_lib):
    from chimes_calculator_gb300 import Calculator
    names = [n for n in sorted(golden) if n != "c2"]
    c = Calculator()
    slots = {n: c.load_params(golden[n].params) for n in names}
    configs = [(golden[n].cfg.pos, golden[n].cfg.types, golden[n].cfg.cell) for n in names]
    # string types are mapped per slot
    packed_types = []
    for n in names:
        packed_types.append(c.type_indices(golden[n].cfg.types, slots[n]))
    configs = [(cf[0], t, cf[2]) for cf, t in zip(configs, packed_types)]
    res = c.evaluate_batch(configs, slots=[slots[n] for n in names], small=[golden[n].small for n in names])
    for n, r in zip(names, res):
        g = golden[n]
        assert abs(r["energy"] - g.energy) <= E_REL_TOL * max(1.0, abs(g.energy)), n
        assert g.force_error(r["force"]) <= F_ABS_TOL, n
        assert np.abs(r["stress"] - g.stress).max() <= S_ABS_TOL, n


def test_mixed_size_batch_matches_oracle(tmp_path, native_lib):
    from chimes_calculator_gb300 import FP64, MIXED, Calculator, synth
    from oracle.oracle import Oracle
    spec = synth.ParamSpec(elements=["C", "N", "O"], orders=(12, 6, 3), rin=0.9, rout=5.0, lam=(1.3, 1.6),
                           fcut=("TERSOFF", 0.5), s3max=4.0, s4max=3.2, seed=4242)
    p = synth.write_param_file(str(tmp_path / "p.txt"), spec)
    cfgs = synth.configs_c4(n_configs=24, seed=77, n_max=96)
    o = Oracle(p)
    ref = [o.calculate(cf.pos, cf.types, cf.cell) for cf in cfgs]
    for prec, etol, ftol in ((FP64, E_REL_TOL, F_ABS_TOL), (MIXED, MIXED_E_REL_TOL, MIXED_F_ABS_TOL)):
        c = Calculator(precision=prec)
        c.load_params(p)
        res = c.evaluate_batch([(cf.pos, cf.types, cf.cell) for cf in cfgs])
        for cf, r, e in zip(cfgs, res, ref):
            assert abs(r["energy"] - e["energy"]) <= etol * max(1.0, abs(e["energy"]))
            assert np.abs(r["force"] - e["force"]).max() <= ftol


def test_batch_reuse_and_growth(golden, native_lib):
    """The workspace grows for a larger batch and shrinks back without stale state."""
    from chimes_calculator_gb300 import Calculator
    g1, g2 = golden["c2_small"], golden["c2"]
    c = Calculator(graph=True)
    c.load_params(g1.params)
    s2 = c.load_params(g2.params)
    for cfgs, slots in (([g1], [0]), ([g1, g2, g1], [0, s2, 0]), ([g1], [0])):
        res = c.evaluate_batch([(g.cfg.pos, c.type_indices(g.cfg.types, s), g.cfg.cell) for g, s in zip(cfgs, slots)],
                               slots=slots)
        for g, r in zip(cfgs, res):
            assert abs(r["energy"] - g.energy) <= E_REL_TOL * abs(g.energy)
            assert np.abs(r["force"] - g.force).max() <= F_ABS_TOL


def test_sparse_and_tiny_configurations(golden, native_lib):
    """Edge cases in one batch: a single atom (1-body only), two atoms beyond
    every cutoff, a pair without triplets, beside a normal configuration --
    each equals the oracle, alone and batched."""
    from chimes_calculator_gb300 import Calculator, synth
    from oracle.oracle import Oracle
    g = golden["c2_small"]
    o = Oracle(g.params)
    el = sorted(set(g.cfg.types))
    box = np.diag([13.0, 13.0, 13.0])
    cases = [
        synth.Config(types=[el[0]], pos=np.array([[1.0, 2.0, 3.0]]), cell=box),
        synth.Config(types=[el[0], el[-1]], pos=np.array([[1.0, 1.0, 1.0], [7.5, 7.5, 7.5]]), cell=box),
        synth.Config(types=[el[0], el[-1]], pos=np.array([[1.0, 1.0, 1.0], [3.5, 1.0, 1.0]]), cell=box),
        g.cfg,
    ]
    ref = [o.calculate(cf.pos, cf.types, cf.cell) for cf in cases]
    c = Calculator()
    c.load_params(g.params)
    batched = c.evaluate_batch([(cf.pos, cf.types, cf.cell) for cf in cases])
    alone = [c.evaluate(cf.pos, cf.types, cf.cell) for cf in cases]
    for cf, e, rb, ra in zip(cases, ref, batched, alone):
        for r in (rb, ra):
            assert abs(r["energy"] - e["energy"]) <= E_REL_TOL * max(1.0, abs(e["energy"]))
            assert np.abs(r["force"] - e["force"]).max() <= F_ABS_TOL
            assert np.abs(r["stress"] - e["stress"]).max() <= S_ABS_TOL


@pytest.mark.parametrize("factored", [1, 4], ids=["factored", "tensor_core"])
def test_batch_of_parameter_sets_with_different_orders(golden, native_lib, factored):
    """The serving workload's three parameter sets (3-body orders 8, 10, 8) in
    one mixed batch, with the 4096-configuration workload's extremes: each
    configuration within the mixed budget of the reference's values (the
    tensor-core form runs every set at the batch's largest order, the
    smaller sets' coefficient matrices padded with zeros)."""
    from chimes_calculator_gb300 import MIXED, Calculator
    from conftest import mixed_force_tol
    names = ["c5_set0", "c5_set1", "c5_set2", "c4_n8_rho012", "c4_n512_rho005"]
    c = Calculator(precision=MIXED)
    c.set_contraction(factored)
    slots = {}
    for n in names:
        if golden[n].params not in slots:
            slots[golden[n].params] = c.load_params(golden[n].params)
    sl = [slots[golden[n].params] for n in names]
    confs = [(golden[n].cfg.pos, c.type_indices(golden[n].cfg.types, s), golden[n].cfg.cell) for n, s in zip(names, sl)]
    res = c.evaluate_batch(confs, slots=sl)
    if factored == 4:
        assert c.tuning()["tc3"] == 1
    for n, r in zip(names, res):
        g = golden[n]
        assert abs(r["energy"] - g.energy) <= MIXED_E_REL_TOL * max(1.0, abs(g.energy)), n
        assert g.force_error(r["force"]) <= mixed_force_tol(np.abs(g.force).max()), n


@pytest.mark.parametrize("copies", [1, 3, 6, 10])
def test_enumeration_warps_per_atom(golden, native_lib, copies):
    """The cluster enumeration spreads one atom over 8, 4, 2 or 1 warps,
    fewer as the batch's atom count grows (on 152 SMs these batches of 1536,
    3584, 6656 and 10752 atoms take 8, 4, 2 and 1).  c2 repeated and ref_hn3,
    whose atoms have up to 251 list entries (beyond the bit-matrix form, so
    enumerated entry by entry), give the reference's result in every copy."""
    from chimes_calculator_gb300 import Calculator
    names = ["c2"] * copies + ["ref_hn3"]
    c = Calculator()
    slot = {n: c.load_params(golden[n].params) for n in set(names)}
    res = c.evaluate_batch([(golden[n].cfg.pos, c.type_indices(golden[n].cfg.types, slot[n]), golden[n].cfg.cell)
                            for n in names], slots=[slot[n] for n in names])
    for n, r in zip(names, res):
        g = golden[n]
        assert abs(r["energy"] - g.energy) <= E_REL_TOL * max(1.0, abs(g.energy)), n
        assert g.force_error(r["force"]) <= F_ABS_TOL, n
        assert np.abs(r["stress"] - g.stress).max() <= S_ABS_TOL, n
