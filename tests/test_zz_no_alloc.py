"""ck_calculate_noalloc: the evaluation entry point for callers that cannot
call cudaMalloc while they compute forces (an MD code or framework that owns
all device memory through its own allocator, or a step loop where an
allocation could fail or stall).  It takes the caller's device buffers and
keeps every intermediate array in a static device array.

Checked here: its results equal those of the allocating entry point
(ck_calculate_batch) within the FP64 tolerances of the other GPU tests, on two
calls in a row (the static array keeps the first call's contents, so the
second call proves that each call clears what it must); the outputs are
overwritten; no device memory is taken by the calls; oversized inputs are
rejected with a clear error.  This file is collected last so that a run which
stops at the first failure has already run every other test."""

import ctypes

import numpy as np
import pytest

from conftest import E_REL_TOL, F_ABS_TOL, S_ABS_TOL

pytestmark = pytest.mark.gpu


def test_noalloc_matches_allocating_entry_point(golden, native_lib):
    import torch
    from chimes_calculator_gb300 import Calculator

    lib = native_lib
    g = golden["c2"]
    calc = Calculator()
    calc.load_params(g.params)
    ref = calc.evaluate(g.cfg.pos, g.cfg.types, g.cfg.cell)        # existing entry point

    n = g.cfg.n_atoms
    dev = torch.device("cuda", 0)
    pos = torch.tensor(g.cfg.pos, dtype=torch.float64, device=dev).contiguous()
    types = torch.tensor(calc.type_indices(g.cfg.types), dtype=torch.int32, device=dev)
    energy = torch.empty(1, dtype=torch.float64, device=dev)
    force = torch.empty((n, 3), dtype=torch.float64, device=dev)
    stress = torch.empty(9, dtype=torch.float64, device=dev)
    cell = (ctypes.c_double * 9)(*g.cfg.cell.reshape(-1))
    stream = ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
    torch.cuda.synchronize()

    free_before = None
    for call in range(2):
        energy.fill_(-1.0)
        force.fill_(123.0)
        stress.fill_(5.0)
        torch.cuda.synchronize()
        if call == 1:
            free_before = torch.cuda.mem_get_info(dev)[0]
        rc = lib.ck_calculate_noalloc(calc.h, n, ctypes.c_void_p(pos.data_ptr()), ctypes.c_void_p(types.data_ptr()),
                                      cell, 0, ctypes.c_void_p(energy.data_ptr()), ctypes.c_void_p(force.data_ptr()),
                                      ctypes.c_void_p(stress.data_ptr()), stream)
        assert rc == 0, lib.ck_last_error()
        if call == 1:
            assert torch.cuda.mem_get_info(dev)[0] >= free_before - (1 << 20)
        e = float(energy.item())
        f = force.cpu().numpy()
        s = stress.cpu().numpy()
        assert abs(e - ref["energy"]) <= E_REL_TOL * abs(ref["energy"]), call
        assert np.abs(f - ref["force"]).max() <= F_ABS_TOL, call
        assert np.abs(s - ref["stress"]).max() <= S_ABS_TOL, call
        assert abs(e - g.energy) <= E_REL_TOL * abs(g.energy)


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
