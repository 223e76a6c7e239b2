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
MIXED_S_ABS_TOL = 1e-5
# fitted force fields (the reference's CHON, HN3, CO2400K, TiO2 files) reach forces of
# 20-520 kcal/mol/A; there the FP32 contraction's force error is stated relative to the
# largest force of the configuration (measured <= 2.2e-6 of it)
MIXED_F_REL_TOL = 5e-6


def mixed_force_tol(fmax):
    """Mixed-form force gate: 1e-5 absolute, or 5e-6 of the largest force when that is larger."""
    return max(MIXED_F_ABS_TOL, MIXED_F_REL_TOL * float(fmax))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 GPU and the built native library")


def golden_names(large=True):
    """Every fixture directory; ``large=False`` leaves out the full-size case
    (32768 atoms) for checks that run a CPU implementation on it."""
    names = sorted(d for d in os.listdir(GOLDEN) if os.path.isfile(os.path.join(GOLDEN, d, "expected.json")))
    if not large:
        names = [n for n in names if not json.load(open(os.path.join(GOLDEN, n, "expected.json"))).get("large")]
    return names


class Golden:
    """One fixture made by the compiled reference (tests/golden/make_golden.py).

    Parameters come from ``params.txt``, a gzipped ``params.txt.gz`` (the
    reference's own force fields) or another case (``params_from``); the
    configuration from ``config.xyz`` or, for the full-size case, regenerated
    from its seed and checked against the digest of the text the reference
    read (``config_from``).  ``force`` holds every atom's force, or every
    ``stride``-th atom's for the full-size case (``force_index``), with the
    total force and the sum of squares of all of them."""

    def __init__(self, name):
        d = os.path.join(GOLDEN, name)
        self.name = name
        with open(os.path.join(d, "expected.json")) as f:
            e = json.load(f)
        self.large = bool(e.get("large", False))
        self.params = self._params(d, e)
        self.small = e["small"]
        self.n_atoms = int(e["n_atoms"])
        self.energy = float(e["energy"])
        self.stress = np.array([float(v) for v in e["stress"]])
        self.force = np.array([[float(v) for v in r] for r in e["force"]])
        fi = e.get("force_index")
        self.force_index = None if fi is None else np.arange(fi["start"], self.n_atoms, fi["stride"])
        self.force_sum = None if "force_sum" not in e else np.array([float(v) for v in e["force_sum"]])
        self.force_sumsq = None if "force_sumsq" not in e else float(e["force_sumsq"])
        self.lists = e["lists"]
        self.xyz = self._config(d, e)
        from chimes_calculator_gb300 import synth
        self.cfg = synth.read_xyz(self.xyz)

    @staticmethod
    def _cache_dir(name):
        import tempfile
        d = os.path.join(tempfile.gettempdir(), "chimes_gb300_golden_%d" % os.getuid(), name)
        os.makedirs(d, exist_ok=True)
        return d

    def _params(self, d, e):
        if "params_from" in e:
            return os.path.join(GOLDEN, e["params_from"], "params.txt")
        p = os.path.join(d, "params.txt")
        if os.path.exists(p):
            return p
        import gzip
        with gzip.open(p + ".gz", "rb") as f:
            data = f.read()
        out = os.path.join(self._cache_dir(self.name), "params.txt")
        if not (os.path.exists(out) and open(out, "rb").read() == data):
            with open(out + ".tmp%d" % os.getpid(), "wb") as f:
                f.write(data)
            os.replace(out + ".tmp%d" % os.getpid(), out)
        return out

    def _config(self, d, e):
        if "config_from" not in e:
            return os.path.join(d, "config.xyz")
        import hashlib
        from chimes_calculator_gb300 import synth
        text = getattr(synth, e["config_from"])().xyz_text()
        if hashlib.sha256(text.encode()).hexdigest() != e["config_sha256"]:
            raise AssertionError("%s: regenerated configuration differs from the one the reference ran" % self.name)
        out = os.path.join(self._cache_dir(self.name), "config.xyz")
        if not (os.path.exists(out) and open(out).read() == text):
            with open(out + ".tmp%d" % os.getpid(), "w") as f:
                f.write(text)
            os.replace(out + ".tmp%d" % os.getpid(), out)
        return out

    def force_rows(self, F):
        """The rows of a full force array that the fixture stores."""
        F = np.asarray(F)
        return F if self.force_index is None else F[self.force_index]

    def force_error(self, F):
        """Max-abs force difference over the stored rows; for a sampled fixture
        also the total force and the sum of squares (relative) of all atoms."""
        F = np.asarray(F)
        err = float(np.abs(self.force_rows(F) - self.force).max())
        if self.force_sum is not None:
            err = max(err, float(np.abs(F.sum(axis=0) - self.force_sum).max()) / max(1, self.n_atoms) ** 0.5)
            err = max(err, abs(float((F * F).sum()) - self.force_sumsq) / max(1.0, self.force_sumsq))
        return err


class _Goldens(dict):
    """Fixtures loaded on first use (the full-size case regenerates its configuration)."""

    def __missing__(self, name):
        g = Golden(name)
        self[name] = g
        return g

    def __iter__(self):
        return iter(golden_names())

    def __len__(self):
        return len(golden_names())

    def values(self):
        return [self[n] for n in golden_names()]

    def items(self):
        return [(n, self[n]) for n in golden_names()]


@pytest.fixture(scope="session")
def golden():
    return _Goldens()


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
