"""The checked build and run-to-run spread.

The checked build (libchimescalc_bounds.so: the CUDA sources compiled with
-DCK_BOUNDS) checks every computed index of the cluster kernels against its
array -- ghost slots, caller atoms, type tuples, coefficient and factored-entry
ranges, Chebyshev powers, tensor-core images; the analogue of the
reference's DEBUG size checks (chimesFF/src/chimesFF.cpp:1984-1990,
2539-2544).  A failed check raises an error flag and skips the access, so a
bad index gives an error status, never a fault.  Here it runs the golden
cases in every contraction form (FP64 and mixed) in a child process and must
report no violation and the reference's results.

Forces, energies and virials are summed with FP64 atomics, so two identical
evaluations agree only to rounding; the spread is measured and bounded."""

import json
import os
import subprocess
import sys

import numpy as np
import pytest

from conftest import (E_REL_TOL, F_ABS_TOL, MIXED_E_REL_TOL, MIXED_S_ABS_TOL, REPO, S_ABS_TOL,
                      mixed_force_tol)

pytestmark = pytest.mark.gpu

CHILD = r'''
import json, sys
sys.path.insert(0, sys.argv[1]); sys.path.insert(0, sys.argv[1] + "/tests")
import numpy as np
from conftest import Golden
from chimes_calculator_gb300 import Calculator
out = []
for name in ("c2_small", "smallbox", "triclinic", "penalty", "c4_n8_rho012", "c5_set1", "ref_tio2_arbrot"):
    g = Golden(name)
    for prec, modes in ((0, (1, 3, 0)), (1, (1, 3, 0, 4))):
        for mode in modes:
            c = Calculator(precision=prec)
            c.set_contraction(mode)
            c.load_params(g.params)
            try:
                r = c.evaluate(g.cfg.pos, g.cfg.types, g.cfg.cell, small=g.small)
                out.append([name, prec, mode, "ok", abs(r["energy"] - g.energy) / max(1.0, abs(g.energy)),
                            g.force_error(r["force"]), float(np.abs(r["stress"] - g.stress).max()),
                            float(np.abs(g.force).max())])
            except Exception as e:
                out.append([name, prec, mode, str(e), 0, 0, 0, 0])
print(json.dumps(out))
'''


def test_checked_build_reports_no_violation(native_lib):
    from chimes_calculator_gb300.build import build
    lib = build(bounds=True)
    env = dict(os.environ, CHIMES_GB300_LIB=lib)
    p = subprocess.run([sys.executable, "-c", CHILD, REPO], capture_output=True, text=True, env=env, timeout=900)
    assert p.returncode == 0, p.stderr[-2000:]
    rows = json.loads(p.stdout.strip().splitlines()[-1])
    assert len(rows) == 7 * 7
    for name, prec, mode, st, de, df, ds, fmax in rows:
        assert st == "ok", (name, prec, mode, st)
        if prec == 0:
            et, ft, stol = E_REL_TOL, F_ABS_TOL, S_ABS_TOL
        else:
            et, ft, stol = MIXED_E_REL_TOL, mixed_force_tol(fmax), MIXED_S_ABS_TOL
        assert de <= et and df <= ft and ds <= stol, (name, prec, mode, de, df, ds)


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "mixed"])
def test_run_to_run_spread(golden, native_lib, precision):
    """Two identical evaluations of the 1024-atom configuration differ only by
    the order of the FP64 atomic sums: measured spread below 1e-13 relative in
    energy and 1e-12 in forces and stress (FP64 and mixed alike, since every
    accumulation is FP64)."""
    from chimes_calculator_gb300 import Calculator
    g = golden["c2"]
    c = Calculator(precision=precision)
    c.load_params(g.params)
    runs = [c.evaluate(g.cfg.pos, g.cfg.types, g.cfg.cell) for _ in range(4)]
    e = np.array([r["energy"] for r in runs])
    f = np.stack([r["force"] for r in runs])
    s = np.stack([r["stress"] for r in runs])
    assert (e.max() - e.min()) <= 1e-13 * abs(e[0])
    assert np.abs(f - f[0]).max() <= 1e-12
    assert np.abs(s - s[0]).max() <= 1e-12
