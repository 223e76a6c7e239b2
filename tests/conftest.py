"""Shared fixtures.  Tests marked ``gpu`` need a GB300 and the built native
library; the rest run on the CPU (oracle, host logic, ABI surface)."""

import json
import os
import sys

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if REPO not in sys.path:
    sys.path.insert(0, REPO)

GOLDEN = os.path.join(REPO, "tests", "golden")

# tolerances of the FP64 path against the reference (kcal/mol, kcal/mol/A, kcal/mol/A^3)
E_REL_TOL = 1e-10
F_ABS_TOL = 1e-9
S_ABS_TOL = 1e-9
# mixed FP32/FP64 path against the FP64 results
MIXED_E_REL_TOL = 1e-6
MIXED_F_ABS_TOL = 1e-5


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 GPU and the built native library")


def golden_names():
    return sorted(d for d in os.listdir(GOLDEN) if os.path.isfile(os.path.join(GOLDEN, d, "expected.json")))


class Golden:
    def __init__(self, name):
        d = os.path.join(GOLDEN, name)
        self.name = name
        self.params = os.path.join(d, "params.txt")
        self.xyz = os.path.join(d, "config.xyz")
        with open(os.path.join(d, "expected.json")) as f:
            e = json.load(f)
        self.small = e["small"]
        self.energy = float(e["energy"])
        self.stress = np.array([float(v) for v in e["stress"]])
        self.force = np.array([[float(v) for v in r] for r in e["force"]])
        self.lists = e["lists"]
        from chimes_calculator_gb300 import synth
        self.cfg = synth.read_xyz(self.xyz)


@pytest.fixture(scope="session")
def golden():
    return {n: Golden(n) for n in golden_names()}


@pytest.fixture(scope="session")
def native_lib():
    """Builds (if needed) and loads the native library."""
    from chimes_calculator_gb300 import _lib
    from chimes_calculator_gb300.build import build
    build()
    return _lib.load()


def list_digest(a):
    import hashlib
    return hashlib.sha256(np.ascontiguousarray(np.asarray(a, dtype="<i4")).tobytes()).hexdigest()
