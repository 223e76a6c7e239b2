"""ctypes wrapper of the oracle (test infrastructure only).

Loads ``oracle/_build/libchimes_oracle.so`` -- the C restatement of the
reference calculator in ``oracle/chimes_oracle.c`` -- and exposes a
``serial_chimes_interface``-like ``calculate`` plus the cluster lists of the
last call.  ``run_reference`` drives the unmodified reference build in
``oracle/_ref/ref_driver`` when it exists (only where the reference sources
were available to compile it).

Only tests, the smoke check and the bench's CPU-baseline leg import this.
"""

from __future__ import annotations

import ctypes
import os
import subprocess
from typing import Dict, Optional, Sequence

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_SO = os.path.join(HERE, "_build", "libchimes_oracle.so")
REF_DRIVER = os.path.join(HERE, "_ref", "ref_driver")


def _default_refroot() -> str:
    """The reference checkout: $CHIMES_REFERENCE_ROOT, else the Makefile's REFROOT default."""
    env = os.environ.get("CHIMES_REFERENCE_ROOT")
    if env:
        return env
    with open(os.path.join(HERE, "Makefile")) as f:
        for ln in f:
            if ln.startswith("REFROOT") and "?=" in ln:
                return ln.split("?=", 1)[1].strip()
    return ""


REFROOT = _default_refroot()

_lib = None


def build_port(force: bool = False) -> str:
    if force or not os.path.exists(PORT_SO) or \
            os.path.getmtime(PORT_SO) < os.path.getmtime(os.path.join(HERE, "chimes_oracle.c")):
        subprocess.run(["make", "-s", "-C", HERE, "port"], check=True)
    return PORT_SO


def build_reference() -> Optional[str]:
    """Compiles the reference's own sources into oracle/_ref when they exist here."""
    if not os.path.isdir(REFROOT):
        return REF_DRIVER if os.path.exists(REF_DRIVER) else None
    try:
        subprocess.run(["make", "-s", "-C", HERE, "ref", "REFROOT=" + REFROOT], check=True,
                       stdout=subprocess.DEVNULL)
    except subprocess.CalledProcessError:
        return None
    return REF_DRIVER


def _load():
    global _lib
    if _lib is None:
        lib = ctypes.CDLL(build_port())
        D, I, L, P = ctypes.c_double, ctypes.c_int, ctypes.c_long, ctypes.c_void_p
        dp, ip, lp = ctypes.POINTER(D), ctypes.POINTER(I), ctypes.POINTER(L)
        lib.ora_load.restype = P
        lib.ora_load.argtypes = [ctypes.c_char_p, ctypes.c_char_p, I]
        lib.ora_free.argtypes = [P]
        lib.ora_error.restype = ctypes.c_char_p
        lib.ora_error.argtypes = [P]
        lib.ora_info.argtypes = [P, ip, ip, dp]
        lib.ora_type_index.restype = I
        lib.ora_type_index.argtypes = [P, ctypes.c_char_p]
        lib.ora_badness.restype = I
        lib.ora_badness.argtypes = [P]
        lib.ora_calculate.restype = I
        lib.ora_calculate.argtypes = [P, I, dp, dp, dp, ip, dp, dp, dp, I, dp, dp, dp, dp, dp]
        lib.ora_list_sizes.argtypes = [P, lp, lp, lp]
        lib.ora_get_lists.argtypes = [P, ip, ip, ip]
        lib.ora_compute_1b.argtypes = [P, I, dp]
        lib.ora_compute_2b.argtypes = [P, D, dp, I, I, dp, dp, dp]
        lib.ora_compute_3b.argtypes = [P, dp, dp, ip, dp, dp, dp]
        lib.ora_compute_4b.argtypes = [P, dp, dp, ip, dp, dp, dp]
        llp = ctypes.POINTER(ctypes.c_longlong)
        lib.ora_lammps_compute.restype = I
        lib.ora_lammps_compute.argtypes = [P, I, dp, ip, llp, I, ip, ip, ip, D, I, dp, dp, dp, dp, dp]
        lib.ora_tab2.restype = D
        lib.ora_tab2.argtypes = [P, I, D, I]
        lib.ora_tab3.argtypes = [P, I, D, D, D, dp]
        lib.ora_compute_2b_tab.argtypes = [P, D, dp, I, I, dp, dp, dp, dp]
        lib.ora_compute_3b_tab.argtypes = [P, dp, dp, ip, dp, dp, dp, dp]
        lib.ora_tab_flags.restype = I
        lib.ora_tab_flags.argtypes = [P, ip, ip]
        lib.ora_lammps_fp.argtypes = [P, I]
        lib.ora_lammps_fp_sizes.argtypes = [P, lp]
        lib.ora_lammps_fp_records.argtypes = [P, I, dp, ip]
        lib.ora_fp_histogram.restype = I
        lib.ora_fp_histogram.argtypes = [P, I, L, dp, ip, L, dp, ip, I, I, llp, llp]
        lib.ora_lammps_sizes.argtypes = [P, lp, lp]
        lib.ora_lammps_lists.argtypes = [P, ip, ip]
        _lib = lib
    return _lib


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _ip(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int))


class Oracle:
    """One parameter set loaded into the C restatement."""

    def __init__(self, param_file: str):
        self.lib = _load()
        err = ctypes.create_string_buffer(512)
        self.h = self.lib.ora_load(param_file.encode(), err, 512)
        if not self.h:
            raise ValueError("oracle: " + err.value.decode())
        orders = (ctypes.c_int * 3)()
        nt = ctypes.c_int()
        cuts = (ctypes.c_double * 3)()
        self.lib.ora_info(self.h, orders, ctypes.byref(nt), cuts)
        self.orders = tuple(orders)
        self.ntypes = nt.value
        self.max_cutoffs = tuple(cuts)

    def type_indices(self, types: Sequence[str]) -> np.ndarray:
        cache: Dict[str, int] = {}
        out = np.empty(len(types), dtype=np.int32)
        for i, t in enumerate(types):
            if t not in cache:
                cache[t] = self.lib.ora_type_index(self.h, t.encode())
                if cache[t] < 0:
                    raise ValueError("oracle: atom type %s not in parameter file" % t)
            out[i] = cache[t]
        return out

    def calculate(self, pos, types, cell, small: bool = False, energy: float = 0.0,
                  force=None) -> Dict[str, object]:
        pos = np.ascontiguousarray(pos, dtype=np.float64)
        n = pos.shape[0]
        x, y, z = (np.ascontiguousarray(pos[:, k]) for k in range(3))
        cell = np.ascontiguousarray(cell, dtype=np.float64).reshape(3, 3)
        ca, cb, cc = (np.ascontiguousarray(cell[k]) for k in range(3))
        typ = self.type_indices(types)
        f = np.zeros((n, 3)) if force is None else np.array(force, dtype=np.float64)
        fx, fy, fz = (np.ascontiguousarray(f[:, k]) for k in range(3))
        e = ctypes.c_double(energy)
        st = np.zeros(9)
        rc = self.lib.ora_calculate(self.h, n, _dp(x), _dp(y), _dp(z), _ip(typ), _dp(ca), _dp(cb), _dp(cc),
                                    int(bool(small)), ctypes.byref(e), _dp(fx), _dp(fy), _dp(fz), _dp(st))
        if rc != 0:
            raise ValueError("oracle: " + self.lib.ora_error(self.h).decode())
        return {"energy": e.value, "force": np.stack([fx, fy, fz], axis=1), "stress": st,
                "badness": self.lib.ora_badness(self.h)}

    def lammps_compute(self, nl, skin: float, rebuild: bool = True):
        """pair_style chimesFF (etc/lmp/src/pair_chimes.cpp) on a LAMMPS-style
        neighbour list `nl` (synth.NeighborData): forces on local and ghost
        atoms, energy and virial (xx yy zz xy xz yz), all from zero."""
        x = np.ascontiguousarray(nl.x, dtype=np.float64)
        nall = x.shape[0]
        f = np.zeros((nall, 3))
        e = ctypes.c_double(0.0)
        vir = np.zeros(6)
        eatom, vatom = np.zeros(nall), np.zeros((nall, 6))
        tag = np.ascontiguousarray(nl.tag, dtype=np.int64)
        rc = self.lib.ora_lammps_compute(
            self.h, nall, _dp(x), _ip(np.ascontiguousarray(nl.type, dtype=np.int32)),
            tag.ctypes.data_as(ctypes.POINTER(ctypes.c_longlong)), len(nl.ilist),
            _ip(np.ascontiguousarray(nl.ilist, dtype=np.int32)), _ip(np.ascontiguousarray(nl.numneigh, dtype=np.int32)),
            _ip(np.ascontiguousarray(nl.neigh, dtype=np.int32)), float(skin), int(bool(rebuild)), _dp(f),
            ctypes.byref(e), _dp(vir), _dp(eatom), _dp(vatom))
        if rc != 0:
            raise ValueError("oracle: " + self.lib.ora_error(self.h).decode())
        return {"energy": e.value, "force": f, "virial": vir, "eatom": eatom, "vatom": vatom}

    def lammps_fingerprint(self, on: bool = True):
        """Record the FINGERPRINT build's cluster records on later lammps_compute calls."""
        self.lib.ora_lammps_fp(self.h, int(bool(on)))

    def lammps_fp_records(self, body: int):
        """(distances [n][P], types [n][body]) recorded by the last lammps_compute."""
        n = (ctypes.c_long * 3)()
        self.lib.ora_lammps_fp_sizes(self.h, n)
        P = body * (body - 1) // 2
        d = np.zeros((n[body - 2], P))
        t = np.zeros((n[body - 2], body), dtype=np.int32)
        self.lib.ora_lammps_fp_records(self.h, body, _dp(d), _ip(t))
        return d, t

    def fp_histogram(self, body: int, d1, t1, d2=None, t2=None, nbin: int = 100):
        """Cluster-distance histogram of multi_calc_histogram.cpp (one process):
        counts[nbin] and the sample count; d2/t2 None means the same set (pairs j > i)."""
        same = d2 is None
        d1 = np.ascontiguousarray(d1, dtype=np.float64)
        t1 = np.ascontiguousarray(t1, dtype=np.int32)
        d2 = d1 if same else np.ascontiguousarray(d2, dtype=np.float64)
        t2 = t1 if same else np.ascontiguousarray(t2, dtype=np.int32)
        counts = np.zeros(nbin, dtype=np.int64)
        ns = ctypes.c_longlong(0)
        llp = ctypes.POINTER(ctypes.c_longlong)
        rc = self.lib.ora_fp_histogram(self.h, body, len(t1), _dp(d1), _ip(t1), len(t2), _dp(d2), _ip(t2), int(same),
                                       nbin, counts.ctypes.data_as(llp), ctypes.byref(ns))
        if rc != 0:
            raise ValueError("oracle: " + self.lib.ora_error(self.h).decode())
        return counts, ns.value

    def lammps_lists(self):
        n3, n4 = ctypes.c_long(), ctypes.c_long()
        self.lib.ora_lammps_sizes(self.h, ctypes.byref(n3), ctypes.byref(n4))
        l3 = np.zeros((n3.value, 3), dtype=np.int32)
        l4 = np.zeros((n4.value, 4), dtype=np.int32)
        self.lib.ora_lammps_lists(self.h, _ip(l3), _ip(l4))
        return l3, l4

    def lists(self):
        n2, n3, n4 = ctypes.c_long(), ctypes.c_long(), ctypes.c_long()
        self.lib.ora_list_sizes(self.h, ctypes.byref(n2), ctypes.byref(n3), ctypes.byref(n4))
        l2 = np.zeros((n2.value, 2), dtype=np.int32)
        l3 = np.zeros((n3.value, 3), dtype=np.int32)
        l4 = np.zeros((n4.value, 4), dtype=np.int32)
        self.lib.ora_get_lists(self.h, _ip(l2), _ip(l3), _ip(l4))
        return l2, l3, l4

    # per-cluster entry points (chimesFF::compute_nB semantics: accumulate)
    def compute_2b(self, dx, dr, typ, force, stress, energy):
        dr = np.ascontiguousarray(dr, dtype=np.float64)
        e = ctypes.c_double(energy)
        self.lib.ora_compute_2b(self.h, float(dx), _dp(dr), int(typ[0]), int(typ[1]), _dp(force), _dp(stress),
                                ctypes.byref(e))
        return e.value

    def compute_3b(self, dx, dr, typ, force, stress, energy):
        dx = np.ascontiguousarray(dx, dtype=np.float64)
        dr = np.ascontiguousarray(dr, dtype=np.float64)
        t = np.ascontiguousarray(typ, dtype=np.int32)
        e = ctypes.c_double(energy)
        self.lib.ora_compute_3b(self.h, _dp(dx), _dp(dr), _ip(t), _dp(force), _dp(stress), ctypes.byref(e))
        return e.value

    # tabulated terms (TABULATION build of the reference)
    def tab_flags(self):
        """(tab2, tab3, error bits since the last call)."""
        t2, t3 = ctypes.c_int(), ctypes.c_int()
        e = self.lib.ora_tab_flags(self.h, ctypes.byref(t2), ctypes.byref(t3))
        return t2.value, t3.value, e

    def compute_2b_tab(self, dx, dr, typ):
        """compute_2B_tab from zero: (energy, force[6], stress[6], force_scalar_in)."""
        dr = np.ascontiguousarray(dr, dtype=np.float64)
        f, st, fs = np.zeros(6), np.zeros(6), np.zeros(1)
        e = ctypes.c_double(0.0)
        self.lib.ora_compute_2b_tab(self.h, float(dx), _dp(dr), int(typ[0]), int(typ[1]), _dp(f), _dp(st),
                                    ctypes.byref(e), _dp(fs))
        return e.value, f, st, fs[0]

    def compute_3b_tab(self, dx, dr, typ):
        """compute_3B_tab from zero: (energy, force[9], stress[6], force_scalar_in[3])."""
        dx = np.ascontiguousarray(dx, dtype=np.float64)
        dr = np.ascontiguousarray(dr, dtype=np.float64)
        t = np.ascontiguousarray(typ, dtype=np.int32)
        f, st, fs = np.zeros(9), np.zeros(6), np.zeros(3)
        e = ctypes.c_double(0.0)
        self.lib.ora_compute_3b_tab(self.h, _dp(dx), _dp(dr), _ip(t), _dp(f), _dp(st), ctypes.byref(e), _dp(fs))
        return e.value, f, st, fs

    def compute_4b(self, dx, dr, typ, force, stress, energy):
        dx = np.ascontiguousarray(dx, dtype=np.float64)
        dr = np.ascontiguousarray(dr, dtype=np.float64)
        t = np.ascontiguousarray(typ, dtype=np.int32)
        e = ctypes.c_double(energy)
        self.lib.ora_compute_4b(self.h, _dp(dx), _dp(dr), _ip(t), _dp(force), _dp(stress), ctypes.byref(e))
        return e.value


def build_reference_tab() -> Optional[str]:
    """Compiles the reference's chimesFF.cpp with -DTABULATION into oracle/_ref
    (tabulated 2B/3B terms) when the reference sources exist here."""
    drv = os.path.join(HERE, "_ref", "ref_tab_driver")
    if not os.path.isdir(REFROOT):
        return drv if os.path.exists(drv) else None
    try:
        subprocess.run(["make", "-s", "-C", HERE, "reftab", "REFROOT=" + REFROOT], check=True,
                       stdout=subprocess.DEVNULL)
    except subprocess.CalledProcessError:
        return None
    return drv


def run_reference_tab(param_file: str, queries: str, out_file: str) -> list:
    """Runs compute_2B_tab / compute_3B_tab of the reference on a query file
    (see oracle/ref_tab_driver.cpp); returns one float array per query."""
    drv = build_reference_tab()
    if drv is None or not os.path.exists(drv):
        raise FileNotFoundError("reference tabulation driver not available")
    # the reference joins the parameter file's directory and a table name with
    # no separator, so it is run from that directory on the bare file name
    subprocess.run([drv, os.path.basename(param_file), os.path.abspath(queries), os.path.abspath(out_file)],
                   check=True, capture_output=True, cwd=os.path.dirname(os.path.abspath(param_file)))
    with open(out_file) as f:
        return [np.array([float(v) for v in ln.split()]) for ln in f if ln.strip()]


def run_reference(param_file: str, xyz_file: str, small: bool, out_prefix: str, lists: bool = False,
                  time_reps: int = 0):
    """Runs the compiled reference driver; returns (result dict, lists or None, timing or None)."""
    drv = build_reference()
    if drv is None or not os.path.exists(drv):
        raise FileNotFoundError("reference driver not available")
    cmd = [drv, param_file, xyz_file, "1" if small else "0", out_prefix]
    if lists:
        cmd.append("--lists")
    if time_reps:
        cmd += ["--time", str(time_reps)]
    p = subprocess.run(cmd, check=True, capture_output=True, text=True)
    timing = None
    if time_reps:
        import json
        timing = json.loads(p.stdout.strip().splitlines()[-1])
    with open(out_prefix + ".res") as f:
        rows = f.read().split("\n")
    energy = float(rows[0])
    stress = np.array([float(v) for v in rows[1].split()])
    force = np.array([[float(v) for v in r.split()] for r in rows[2:] if r.strip()])
    lst = None
    if lists:
        with open(out_prefix + ".lists") as f:
            head = f.readline().split()
            n2, n3, n4 = int(head[2]), int(head[3]), int(head[4])
            flat = np.array(f.read().split(), dtype=np.int64)
        l2 = flat[:2 * n2].reshape(n2, 2)
        l3 = flat[2 * n2:2 * n2 + 3 * n3].reshape(n3, 3)
        l4 = flat[2 * n2 + 3 * n3:].reshape(n4, 4)
        lst = (l2, l3, l4)
    return {"energy": energy, "force": force, "stress": stress}, lst, timing
