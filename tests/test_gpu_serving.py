"""Continuous-batching server: every request's result is the same when it is
served in a mix of concurrent requests (several parameter sets, sizes,
overlapping batches on two workers) as when it is evaluated alone, within the
FP64 tolerances; admission under a tiny HBM budget still serves everything;
a failing request is isolated from the others in its batch."""

import numpy as np
import pytest

from conftest import E_REL_TOL, F_ABS_TOL, MIXED_E_REL_TOL, MIXED_F_ABS_TOL, S_ABS_TOL

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def workload(tmp_path_factory):
    from chimes_calculator_gb300 import synth
    from chimes_calculator_gb300.serving import serving_workload
    d = tmp_path_factory.mktemp("serve")
    specs, reqs = serving_workload(36, seed=99, n_min=16, n_max=400)
    paths = [synth.write_param_file(str(d / ("p%d.txt" % k)), s) for k, s in enumerate(specs)]
    return paths, reqs


def _solo(paths, reqs, precision):
    from chimes_calculator_gb300 import Calculator
    c = Calculator(precision=precision)
    for p in paths:
        c.load_params(p)
    out = [c.evaluate(cfg.pos, c.type_indices(cfg.types, slot), cfg.cell, slot=slot) for slot, cfg in reqs]
    return c, out


@pytest.mark.parametrize("precision", [0, 1])
def test_each_result_same_alone_and_in_the_mix(workload, native_lib, precision):
    from chimes_calculator_gb300.serving import Server
    paths, reqs = workload
    calc, solo = _solo(paths, reqs, precision)
    srv = Server(workers=2, precision=precision, max_batch_atoms=1500)
    try:
        for p in paths:
            srv.load_params(p)
        ids = [srv.submit(cfg.pos, calc.type_indices(cfg.types, slot), cfg.cell, slot=slot) for slot, cfg in reqs]
        got = [srv.take(i) for i in ids]
        st = srv.stats()
    finally:
        srv.close()
    assert st["completed"] == len(reqs) and st["batches"] < len(reqs)   # requests were batched
    etol = E_REL_TOL if precision == 0 else 1e-12
    for (slot, cfg), a, b in zip(reqs, solo, got):
        # same path alone and in the mix: agreement far below the FP64 / mixed error budgets
        assert abs(a["energy"] - b["energy"]) <= etol * max(1.0, abs(a["energy"]))
        assert np.abs(a["force"] - b["force"]).max() <= F_ABS_TOL
        assert np.abs(a["stress"] - b["stress"]).max() <= S_ABS_TOL
        assert b["latency"] > 0


def test_mixed_server_within_error_budget_of_fp64(workload, native_lib):
    from chimes_calculator_gb300.serving import Server
    paths, reqs = workload
    calc, solo64 = _solo(paths, reqs, 0)
    srv = Server(workers=2, precision=1)
    try:
        for p in paths:
            srv.load_params(p)
        ids = [srv.submit(cfg.pos, calc.type_indices(cfg.types, slot), cfg.cell, slot=slot) for slot, cfg in reqs]
        got = [srv.take(i) for i in ids]
    finally:
        srv.close()
    for a, b in zip(solo64, got):
        assert abs(a["energy"] - b["energy"]) <= MIXED_E_REL_TOL * max(1.0, abs(a["energy"]))
        assert np.abs(a["force"] - b["force"]).max() <= MIXED_F_ABS_TOL


def test_admission_under_tiny_budget_and_failure_isolation(workload, native_lib):
    from chimes_calculator_gb300 import ChimesError
    from chimes_calculator_gb300.serving import Server
    paths, reqs = workload
    calc, solo = _solo(paths, reqs[:8], 0)
    srv = Server(workers=2, hbm_budget_gb=1e-9, precision=0)
    try:
        for p in paths:
            srv.load_params(p)
        ids = []
        for k, (slot, cfg) in enumerate(reqs[:8]):
            ids.append(srv.submit(cfg.pos, calc.type_indices(cfg.types, slot), cfg.cell, slot=slot))
            if k == 3:   # a configuration whose cell is degenerate fails alone
                bad = srv.submit(cfg.pos, calc.type_indices(cfg.types, slot), np.diag([10.0, 10.0, 0.0]), slot=slot)
        got = [srv.take(i) for i in ids]
        with pytest.raises(ChimesError):
            srv.take(bad)
        st = srv.stats()
    finally:
        srv.close()
    for a, b in zip(solo, got):
        assert abs(a["energy"] - b["energy"]) <= E_REL_TOL * max(1.0, abs(a["energy"]))
    assert st["largest_batch"] == 1          # the budget admits one request at a time


def test_native_replay_driver(workload, native_lib):
    """ck_server_replay (the native client the serving measurement uses) serves
    every request of a Poisson trace, after autotuning on a sample (which may
    pick another contraction form than the default, and which every worker
    takes, the tensor-core preference included), with the energies of the
    requests evaluated alone within the mixed form's budget and positive
    latencies."""
    import ctypes

    from chimes_calculator_gb300.serving import Server, _dp, _ip
    paths, reqs = workload
    calc, solo = _solo(paths, reqs, 1)
    srv = Server(workers=3, precision=1, max_batch_atoms=2000)
    try:
        for p in paths:
            srv.load_params(p)
        srv.autotune([(cfg.pos, calc.type_indices(cfg.types, s), cfg.cell) for s, cfg in reqs[:6]],
                     [s for s, _ in reqs[:6]])
        tunings = srv.worker_tunings()   # every worker takes worker 0's choices, the contraction form included
        assert len(tunings) == 3 and tunings[1] == tunings[0] and tunings[2] == tunings[0]
        arrival = np.cumsum(np.random.default_rng(3).exponential(1e-4, size=len(reqs)))
        slots = np.array([s for s, _ in reqs], dtype=np.int32)
        natoms = np.array([c.n_atoms for _, c in reqs], dtype=np.int32)
        pos = np.ascontiguousarray(np.concatenate([c.pos for _, c in reqs]))
        types = np.ascontiguousarray(np.concatenate([calc.type_indices(c.types, s) for s, c in reqs]).astype(np.int32))
        cells = np.ascontiguousarray(np.stack([c.cell.reshape(9) for _, c in reqs]))
        lat, en = np.zeros(len(reqs)), np.zeros(len(reqs))
        wall = ctypes.c_double()
        rc = srv.lib.ck_server_replay(srv.h, len(reqs), _ip(slots), _ip(natoms), _dp(pos), _ip(types), _dp(cells),
                                      None, _dp(arrival), _dp(lat), _dp(en), ctypes.byref(wall))
        assert rc == 0, srv.lib.ck_last_error()
        st = srv.stats()
    finally:
        srv.close()
    assert st["completed"] == len(reqs)
    assert np.all(lat > 0) and wall.value > 0
    for a, e in zip(solo, en):
        assert abs(a["energy"] - e) <= MIXED_E_REL_TOL * max(1.0, abs(a["energy"]))
