"""The reference-facing interfaces on the GPU: the serial C ABI through the
reference-style ctypes wrapper (accumulate semantics, handles, replication),
the per-cluster C ABI and chimesFF batch entry, and error reporting."""

import ctypes
import os

import numpy as np
import pytest

from conftest import E_REL_TOL, F_ABS_TOL, S_ABS_TOL, golden_names

pytestmark = pytest.mark.gpu


def test_serial_wrapper_accumulates(golden, native_lib):
    import chimes_calculator_gb300.chimescalc_serial_py as w
    g = golden["triclinic"]
    w.chimes_wrapper = w.init_chimes_wrapper()
    w.chimes_wrapper.ck_set_error_mode(1)
    w.set_chimes(False)
    w.init_chimes(g.params, 0)
    n = g.cfg.n_atoms
    x, y, z = (list(g.cfg.pos[:, k]) for k in range(3))
    f0 = 0.5
    fx, fy, fz, st, e = w.calculate_chimes(n, x, y, z, g.cfg.types, list(g.cfg.cell[0]), list(g.cfg.cell[1]),
                                           list(g.cfg.cell[2]), 2.0, [f0] * n, [f0] * n, [f0] * n, [7.0] * 9)
    assert abs(e - (g.energy + 2.0)) <= E_REL_TOL * abs(g.energy) + 1e-12
    F = np.stack([np.array(fx[:]), np.array(fy[:]), np.array(fz[:])], axis=1)
    assert np.abs(F - (g.force + f0)).max() <= F_ABS_TOL
    assert np.abs(np.array(st[:]) - g.stress).max() <= S_ABS_TOL   # stress is overwritten


def test_repeated_calls_replay_and_autotune(golden, native_lib):
    """An MD-style loop through the serial C ABI: graph replay from the second
    call and an autotune on the third; every call returns the reference result."""
    lib = native_lib
    lib.ck_set_error_mode(1)
    g = golden["c2_small"]
    h = lib.chimes_open_instance()
    try:
        lib.set_chimes_serial_instance(h, 0)
        lib.init_chimes_serial_instance(h, g.params.encode(), 0)
        n = g.cfg.n_atoms
        arr = lambda v: (ctypes.c_double * len(v))(*v)
        x, y, z = (arr(g.cfg.pos[:, k]) for k in range(3))
        ty = (ctypes.c_char_p * n)(*[t.encode() for t in g.cfg.types])
        ca, cb, cc = (arr(g.cfg.cell[k]) for k in range(3))
        for call in range(5):
            fx, fy, fz, st = arr([0.0] * n), arr([0.0] * n), arr([0.0] * n), arr([0.0] * 9)
            e = ctypes.c_double(0.0)
            lib.calculate_chimes_instance(h, n, x, y, z, ty, ca, cb, cc, ctypes.byref(e), fx, fy, fz, st)
            assert lib.ck_last_error() == b"", lib.ck_last_error()
            assert abs(e.value - g.energy) <= E_REL_TOL * abs(g.energy), call
            F = np.stack([np.array(fx[:]), np.array(fy[:]), np.array(fz[:])], axis=1)
            assert np.abs(F - g.force).max() <= F_ABS_TOL, call
    finally:
        lib.chimes_close_instance(h)


def test_instances_and_replication(golden, native_lib):
    lib = native_lib
    lib.ck_set_error_mode(1)
    ga, gb = golden["replicate"], golden["smallbox"]
    ha, hb = lib.chimes_open_instance(), lib.chimes_open_instance()
    try:
        for h, g in ((ha, ga), (hb, gb)):
            lib.set_chimes_serial_instance(h, 1 if g.small else 0)
            lib.init_chimes_serial_instance(h, g.params.encode(), 0)
        for h, g in ((ha, ga), (hb, gb), (ha, ga)):
            n = g.cfg.n_atoms
            arr = lambda v: (ctypes.c_double * len(v))(*v)
            x, y, z = (arr(g.cfg.pos[:, k]) for k in range(3))
            types = (ctypes.c_char_p * n)(*[t.encode() for t in g.cfg.types])
            e = ctypes.c_double(0.0)
            fx, fy, fz = arr([0.0] * n), arr([0.0] * n), arr([0.0] * n)
            st = arr([0.0] * 9)
            lib.calculate_chimes_instance(h, n, x, y, z, types, arr(g.cfg.cell[0]), arr(g.cfg.cell[1]),
                                          arr(g.cfg.cell[2]), ctypes.byref(e), fx, fy, fz, st)
            assert lib.ck_last_error() == b""
            assert abs(e.value - g.energy) <= E_REL_TOL * max(1.0, abs(g.energy))
            F = np.stack([np.array(fx[:]), np.array(fy[:]), np.array(fz[:])], axis=1)
            assert np.abs(F - g.force).max() <= F_ABS_TOL
    finally:
        lib.chimes_close_instance(ha)
        lib.chimes_close_instance(hb)


def _clusters_from(g, nb, count, rng):
    """Clusters of nb atoms (distance/vector inputs) drawn from a golden configuration."""
    pos, cell = g.cfg.pos, g.cfg.cell
    inv = np.linalg.inv(cell)
    out = []
    pairs = [(i, j) for i in range(nb) for j in range(i + 1, nb)]
    reach = {2: 5.5, 3: 4.2, 4: 3.3}[nb]
    while len(out) < count:
        i0 = int(rng.integers(len(pos)))
        d = (pos - pos[i0]) @ inv
        d -= np.round(d)
        r = np.sqrt(((d @ cell) ** 2).sum(1))
        near = np.where((r > 0) & (r < reach))[0]
        if len(near) < nb - 1:
            continue
        ids = np.concatenate([[i0], rng.choice(near, size=nb - 1, replace=False)])
        p = [pos[i0] + d[k] @ cell for k in ids]
        dr = np.array([p[j] - p[i] for i, j in pairs])
        dx = np.sqrt((dr ** 2).sum(1))
        out.append((dx, dr, ids))
    return out


@pytest.mark.parametrize("nb", [2, 3, 4])
def test_cluster_batch_matches_oracle(golden, native_lib, nb):
    from chimes_calculator_gb300 import Calculator, _lib
    from oracle.oracle import Oracle
    g = golden["excluded"]
    rng = np.random.default_rng(nb)
    cl = _clusters_from(g, nb, 300, rng)
    o = Oracle(g.params)
    typ_all = o.type_indices(g.cfg.types)
    c = Calculator()
    c.load_params(g.params)
    npair = nb * (nb - 1) // 2
    dx = np.ascontiguousarray(np.array([a for a, _, _ in cl]).reshape(len(cl), npair))
    dr = np.ascontiguousarray(np.array([b for _, b, _ in cl]).reshape(len(cl), npair, 3))
    ty = np.ascontiguousarray(np.array([typ_all[ids] for _, _, ids in cl], dtype=np.int32))
    f = np.zeros((len(cl), nb, 3)); s = np.zeros((len(cl), 6)); e = np.zeros(len(cl)); fs = np.zeros((len(cl), npair))
    dp = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    rc = c.lib.ck_compute_cluster_batch(c.h, nb, len(cl), dp(dx), dp(dr), ty.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                                        dp(f), dp(s), dp(e), dp(fs))
    assert rc == 0, c.lib.ck_last_error()
    nonzero = 0
    for q in range(len(cl)):
        fo = np.zeros(3 * nb); so = np.zeros(6)
        fn = {2: o.compute_2b, 3: o.compute_3b, 4: o.compute_4b}[nb]
        eo = fn(dx[q][0] if nb == 2 else dx[q], dr[q].reshape(-1), ty[q], fo, so, 0.0)
        assert abs(e[q] - eo) <= 1e-10 * max(1.0, abs(eo))
        assert np.abs(f[q].reshape(-1) - fo).max() <= 1e-9
        assert np.abs(s[q] - so).max() <= 1e-9
        nonzero += eo != 0.0
    assert nonzero > 10


@pytest.mark.parametrize("nb", [3, 4])
def test_cluster_batch_lane_split_consistent(golden, native_lib, nb):
    """The per-cluster kernels split a cluster's coefficient list over 1-32
    lanes by batch size: 3000 clusters (several lanes each) and the same
    clusters inside a batch of about 90000 (one lane each) agree, the
    reference's force_scalar_in values included."""
    from chimes_calculator_gb300 import Calculator
    from oracle.oracle import Oracle
    g = golden["excluded"]
    cl = _clusters_from(g, nb, 3000, np.random.default_rng(40 + nb))
    typ_all = Oracle(g.params).type_indices(g.cfg.types)
    c = Calculator()
    c.load_params(g.params)
    npair = nb * (nb - 1) // 2
    dx = np.array([a for a, _, _ in cl]).reshape(len(cl), npair)
    dr = np.array([b for _, b, _ in cl]).reshape(len(cl), npair, 3)
    ty = np.array([typ_all[ids] for _, _, ids in cl], dtype=np.int32)
    small = c.clusters(nb, dx, dr, ty)
    rep = 90000 // len(cl) + 1
    big = c.clusters(nb, np.tile(dx, (rep, 1)), np.tile(dr, (rep, 1, 1)), np.tile(ty, (rep, 1)))
    for k in ("energy", "force", "stress", "fscal"):
        a, b = small[k], big[k][:len(cl)]
        assert np.abs(a - b).max() <= 1e-12 * max(1.0, np.abs(a).max()), k
    assert np.count_nonzero(small["energy"]) > 100


def test_per_cluster_c_interface(golden, native_lib):
    lib = native_lib
    lib.ck_set_error_mode(1)
    from oracle.oracle import Oracle
    g = golden["c2_small"]
    lib.set_chimes()
    lib.init_chimes(0)
    lib.chimes_read_params(g.params.encode())
    o = Oracle(g.params)
    assert lib.get_chimes_2b_order() == 12 and lib.get_chimes_4b_order() == 4
    assert lib.get_chimes_max_3b_cutoff() == pytest.approx(o.max_cutoffs[1], abs=0)
    rng = np.random.default_rng(3)
    cl = _clusters_from(g, 3, 40, rng)
    arr = lambda v: (ctypes.c_double * len(v))(*v)
    for dx, dr, ids in cl:
        names = [g.cfg.types[i] for i in ids]
        f = (ctypes.c_double * 9)(); st = arr([1.0] * 9); e = ctypes.c_double(5.0)
        dist = ctypes.cast(arr(dr.reshape(-1)), ctypes.POINTER(ctypes.c_double))
        lib.chimes_compute_3b_props(arr(dx), dist, (ctypes.c_char_p * 3)(*[n.encode() for n in names]), f, st,
                                    ctypes.byref(e))
        fo = np.zeros(9); so = np.zeros(6)
        eo = o.compute_3b(dx, dr.reshape(-1), o.type_indices(names), fo, so, 5.0)
        assert abs(e.value - eo) <= 1e-10 * max(1.0, abs(eo))
        assert np.abs(np.array(f[:]) - fo).max() <= 1e-9
        assert np.abs(np.array(st[:6]) - (1.0 + so)).max() <= 1e-9 and st[6] == 1.0


def test_error_reporting(golden, native_lib):
    from chimes_calculator_gb300 import Calculator, ChimesError
    g = golden["c1"]
    c = Calculator()
    with pytest.raises(ChimesError, match="parameter set not loaded"):
        c.evaluate(g.cfg.pos, [0] * g.cfg.n_atoms, g.cfg.cell)
    c.load_params(g.params)
    with pytest.raises(ChimesError, match="not in parameter set"):
        c.evaluate(g.cfg.pos, ["X"] * g.cfg.n_atoms, g.cfg.cell)
    # a 4 A box cannot hold a 5 A cutoff without replication ... but ghost layers make it legal;
    # what the reference rejects is a cell whose layered box is still too small: a zero-length axis
    with pytest.raises(ChimesError):
        c.evaluate(g.cfg.pos[:2], g.cfg.types[:2], np.diag([9.0, 9.0, 0.0]))
    r = c.evaluate(g.cfg.pos, g.cfg.types, g.cfg.cell)   # the handle stays usable
    assert abs(r["energy"] - g.energy) <= E_REL_TOL * abs(g.energy)


def test_badness_and_diagnostics(golden, native_lib):
    """The penalty fixture has pairs inside the penalty region and below the inner
    cutoff: the badness the GPU reports (get_badness, chimesFF.h:388-429) equals
    the oracle's, and penalty hits and below-rin pairs are counted."""
    from chimes_calculator_gb300 import Calculator
    from oracle.oracle import Oracle
    g = golden["penalty"]
    c = Calculator()
    c.load_params(g.params)
    r = c.evaluate(g.cfg.pos, g.cfg.types, g.cfg.cell)
    d = c.diagnostics()
    ref = Oracle(g.params).calculate(g.cfg.pos, g.cfg.types, g.cfg.cell)
    assert d["badness"] == ref["badness"] and d["badness"] > 0
    assert d["penalty_hits"] > 0
    assert abs(r["energy"] - g.energy) <= E_REL_TOL * max(1.0, abs(g.energy))


@pytest.mark.parametrize("name", ["c2", "ref_hn3", "triclinic"])
def test_parameter_cache_evaluates_like_text(golden, native_lib, tmp_path, name):
    """A set loaded from the binary parameter cache (ck_convert_params) gives the
    reference's results, as the text file does."""
    from chimes_calculator_gb300 import Calculator
    g = golden[name]
    native_lib.ck_set_error_mode(1)
    cache = str(tmp_path / "p.ckpc")
    assert native_lib.ck_convert_params(g.params.encode(), cache.encode()) == 0, native_lib.ck_last_error()
    c = Calculator()
    c.load_params(cache)
    r = c.evaluate(g.cfg.pos, g.cfg.types, g.cfg.cell, small=g.small)
    assert abs(r["energy"] - g.energy) <= E_REL_TOL * max(1.0, abs(g.energy))
    assert g.force_error(r["force"]) <= F_ABS_TOL
    assert np.abs(r["stress"] - g.stress).max() <= S_ABS_TOL
