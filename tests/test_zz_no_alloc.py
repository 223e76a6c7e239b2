"""ck_calculate_noalloc: the evaluation entry point for callers that cannot
call cudaMalloc while they compute forces (an MD code or framework that owns
all device memory through its own allocator, or a step loop where an
allocation could fail or stall).  It takes the caller's device buffers and
keeps every intermediate array in a static device array.

Checked here: its results equal those of the allocating entry point within the
FP64 tolerances of the other GPU tests, on two calls in a row and over a
sequence of different configurations (a large one, then smaller ones with
other parameter sets, a replicated small cell, and the large one again: the
static array keeps each call's contents, so a missing clear would show); the
outputs are overwritten; no device memory is taken by the calls; oversized
inputs, lists beyond the static maximum, bad type indices and non-finite
coordinates are rejected with a clear error.  This file is collected last so
that a run which stops at the first failure has already run every other
test."""

import ctypes

import numpy as np
import pytest

from conftest import E_REL_TOL, F_ABS_TOL, S_ABS_TOL

pytestmark = pytest.mark.gpu


class _Case:
    """One golden configuration on the device, with its allocating-path result."""

    def __init__(self, g):
        import torch
        from chimes_calculator_gb300 import Calculator
        self.g = g
        self.calc = Calculator()
        self.calc.load_params(g.params)
        self.ref = self.calc.evaluate(g.cfg.pos, g.cfg.types, g.cfg.cell, small=g.small)   # existing entry point
        dev = torch.device("cuda", 0)
        n = g.cfg.n_atoms
        self.n = n
        self.pos = torch.tensor(g.cfg.pos, dtype=torch.float64, device=dev).contiguous()
        self.types = torch.tensor(self.calc.type_indices(g.cfg.types), dtype=torch.int32, device=dev)
        self.energy = torch.empty(1, dtype=torch.float64, device=dev)
        self.force = torch.empty((n, 3), dtype=torch.float64, device=dev)
        self.stress = torch.empty(9, dtype=torch.float64, device=dev)
        self.cell = (ctypes.c_double * 9)(*g.cfg.cell.reshape(-1))

    def call(self, lib, stream, pos=None, types=None):
        import torch
        self.energy.fill_(-1.0)
        self.force.fill_(123.0)
        self.stress.fill_(5.0)
        torch.cuda.synchronize()
        pos = self.pos if pos is None else pos
        types = self.types if types is None else types
        return lib.ck_calculate_noalloc(self.calc.h, self.n, ctypes.c_void_p(pos.data_ptr()),
                                        ctypes.c_void_p(types.data_ptr()), self.cell, int(self.g.small),
                                        ctypes.c_void_p(self.energy.data_ptr()), ctypes.c_void_p(self.force.data_ptr()),
                                        ctypes.c_void_p(self.stress.data_ptr()), stream)

    def check(self, tag):
        e = float(self.energy.item())
        f = self.force.cpu().numpy()
        s = self.stress.cpu().numpy()
        ref, g = self.ref, self.g
        assert abs(e - ref["energy"]) <= E_REL_TOL * max(1.0, abs(ref["energy"])), tag
        assert np.abs(f - ref["force"]).max() <= F_ABS_TOL, tag
        assert np.abs(s - ref["stress"]).max() <= S_ABS_TOL, tag
        assert abs(e - g.energy) <= E_REL_TOL * max(1.0, abs(g.energy)), tag
        assert g.force_error(f) <= F_ABS_TOL, tag


def _stream():
    import torch
    return ctypes.c_void_p(torch.cuda.current_stream(torch.device("cuda", 0)).cuda_stream)


def test_noalloc_matches_allocating_entry_point(golden, native_lib):
    import torch
    lib = native_lib
    c = _Case(golden["c2"])
    stream = _stream()
    for call in range(2):
        # the first call on a device loads the module that holds the static
        # array; later calls take no device memory
        free_before = torch.cuda.mem_get_info(torch.device("cuda", 0))[0]
        rc = c.call(lib, stream)
        assert rc == 0, lib.ck_last_error()
        if call > 0:
            assert torch.cuda.mem_get_info(torch.device("cuda", 0))[0] >= free_before - (1 << 20)
        c.check("c2 call %d" % call)


def test_noalloc_sequence_of_configurations(golden, native_lib):
    """Larger, then smaller configurations with other parameter sets (multi-image
    clusters, a replicated cell with small = 1), then the larger one again: each
    call clears what the previous one left in the shared array."""
    lib = native_lib
    cases = [_Case(golden[n]) for n in ("c2", "smallbox", "replicate", "c2_small", "c2")]
    stream = _stream()
    for c in cases:
        rc = c.call(lib, stream)
        assert rc == 0, (c.g.name, lib.ck_last_error())
        c.check(c.g.name)


def test_noalloc_rejects_oversized_input(golden, native_lib):
    import torch
    from chimes_calculator_gb300 import Calculator

    lib = native_lib
    g = golden["c1"]
    calc = Calculator()
    calc.load_params(g.params)
    dev = torch.device("cuda", 0)
    n = 3000
    pos = torch.zeros((n, 3), dtype=torch.float64, device=dev)
    types = torch.zeros(n, dtype=torch.int32, device=dev)
    out = torch.zeros(3 * n + 10, dtype=torch.float64, device=dev)
    cell = (ctypes.c_double * 9)(40.0, 0, 0, 0, 40.0, 0, 0, 0, 40.0)
    rc = lib.ck_calculate_noalloc(calc.h, n, ctypes.c_void_p(pos.data_ptr()), ctypes.c_void_p(types.data_ptr()),
                                  cell, 0, ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(out.data_ptr() + 8),
                                  ctypes.c_void_p(out.data_ptr() + 8 * (3 * n + 1)), None)
    assert rc == -2
    assert b"2048" in lib.ck_last_error()


def test_noalloc_list_capacity_exceeded(golden, native_lib):
    """The CO2400K configuration passes the host-side size checks (128 atoms) but
    lists 91,794 quadruplets, more than the static array holds (65,536): the
    fill kernels stop at the capacity and the call reports it; a following
    call is unaffected."""
    lib = native_lib
    big = _Case(golden["ref_co2400k"])
    rc = big.call(lib, _stream())
    assert rc == -5
    assert b"quadruplets" in lib.ck_last_error()
    ok = _Case(golden["c2_small"])
    assert ok.call(lib, _stream()) == 0, lib.ck_last_error()
    ok.check("after capacity error")


def test_noalloc_rejects_bad_type_and_coordinate(golden, native_lib):
    """Inputs already on the device are checked there: a type index outside the
    parameter set and a non-finite coordinate give an input error instead of a
    table read out of bounds or silent garbage."""
    import torch
    lib = native_lib
    c = _Case(golden["c2_small"])
    bad_types = c.types.clone()
    bad_types[7] = 5
    rc = c.call(lib, _stream(), types=bad_types)
    assert rc == -2
    assert b"type index" in lib.ck_last_error()
    bad_pos = c.pos.clone()
    bad_pos[3, 1] = float("nan")
    rc = c.call(lib, _stream(), pos=bad_pos)
    assert rc == -2
    assert b"non-finite" in lib.ck_last_error()
    torch.cuda.synchronize()
    assert c.call(lib, _stream()) == 0, lib.ck_last_error()
    c.check("after input errors")
