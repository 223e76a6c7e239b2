"""Python API over the native library: load parameter sets once, evaluate one
configuration or a batch of configurations on the GPU.

    calc = Calculator()                       # one CUDA stream + workspace
    slot = calc.load_params("model.txt")
    res = calc.evaluate(pos, types, cell)     # energy, forces, stress (one config)
    res = calc.evaluate_batch(configs)        # many configs in one set of launches

Energies/forces/stress follow serial_chimes_interface::calculate
(serial_interface/src/serial_chimes_interface.cpp:960-1124) with zero initial
energy and forces: kcal/mol, kcal/mol/A and the 3x3 stress in kcal/mol/A^3.
"""

from __future__ import annotations

import ctypes
import itertools
from typing import Dict, List, Optional, Sequence

import numpy as np

from . import _lib

FP64 = 0
MIXED = 1


def _dp(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _ip(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int))


class ChimesError(RuntimeError):
    pass


class Calculator:
    def __init__(self, precision: int = FP64, graph: bool = False):
        self.lib = _lib.load()
        self.lib.ck_set_error_mode(1)
        self.h = self.lib.ck_open()
        self.slots: List[int] = []
        self._types: List[Dict[str, int]] = []
        self.set_precision(precision)
        self.use_graph(graph)

    def close(self):
        if self.h:
            self.lib.ck_close(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc):
        if rc is not None and rc < 0:
            raise ChimesError(self.lib.ck_last_error().decode())
        return rc

    def load_params(self, path: str) -> int:
        slot = self._check(self.lib.ck_load_params(self.h, path.encode()))
        self.slots.append(slot)
        self._types.append({})
        return slot

    def save_params_cache(self, path: str, slot: int = 0):
        """Writes the slot's parsed tables as a binary cache that load_params reads without parsing."""
        self._check(self.lib.ck_save_params_cache(self.h, slot, path.encode()))

    def info(self, slot: int = 0):
        orders = (ctypes.c_int * 3)()
        nt = ctypes.c_int()
        cuts = (ctypes.c_double * 3)()
        self._check(self.lib.ck_param_info(self.h, slot, orders, ctypes.byref(nt), cuts))
        return {"orders": tuple(orders), "ntypes": nt.value, "max_cutoffs": tuple(cuts)}

    def tuple_table(self, slot: int = 0):
        """{nbody: (valid[nt^nbody], ncoef[...], rout[..., 6])} of a parameter set."""
        nt = self.info(slot)["ntypes"]
        out = {}
        for nb in (3, 4):
            n = nt ** nb
            valid = np.zeros(n, dtype=np.int32)
            ncoef = np.zeros(n, dtype=np.int32)
            rout = np.zeros((n, 6))
            self._check(self.lib.ck_tuple_table(self.h, slot, nb, _ip(valid), _ip(ncoef), _dp(rout)))
            out[nb] = (valid, ncoef, rout)
        return out

    def tuple_factored(self, slot: int = 0):
        """{nbody: (nrow[nt^nbody], ncol[...], R)} of the factored coefficient lists."""
        nt = self.info(slot)["ntypes"]
        out = {}
        for nb in (3, 4):
            n = nt ** nb
            nrow = np.zeros(n, dtype=np.int32)
            ncol = np.zeros(n, dtype=np.int32)
            R = ctypes.c_int()
            self._check(self.lib.ck_tuple_factored(self.h, slot, nb, _ip(nrow), _ip(ncol), ctypes.byref(R)))
            out[nb] = (nrow, ncol, R.value)
        return out

    def tuning(self) -> dict:
        v = np.zeros(11, dtype=np.int32)
        self._check(self.lib.ck_get_tuning(self.h, _ip(v)))
        keys = ["tpc3", "tpc4", "blocks_per_sm", "fact3", "fact4", "ftpc3", "ftpc4", "fbps3", "fbps4", "noy3"]
        out = {k: int(x) for k, x in zip(keys, v)}
        out["tc3"] = int(v[10]) & 1      # tensor-core 3-body contraction in use
        out["tc4"] = (int(v[10]) >> 1) & 1
        return out

    def type_indices(self, types: Sequence[str], slot: int = 0) -> np.ndarray:
        cache = self._types[slot]
        for t in set(types).difference(cache):   # names not looked up before
            k = self.lib.ck_type_index(self.h, slot, str(t).encode())
            if k < 0:
                raise ChimesError("atom type %s is not in parameter set %d" % (t, slot))
            cache[t] = k
        return np.fromiter(map(cache.__getitem__, types), dtype=np.int32, count=len(types))

    def set_precision(self, precision: int):
        self._check(self.lib.ck_set_precision(self.h, int(precision)))

    def set_tuning(self, tpc3: int = 4, tpc4: int = 8, blocks_per_sm: int = 4):
        self._check(self.lib.ck_set_tuning(self.h, tpc3, tpc4, blocks_per_sm))

    def nl_compute(self, nl, skin: float, rebuild: bool = True, per_atom: bool = False):
        """LAMMPS pair-style evaluation on a neighbour list `nl` (fields x, type,
        tag, ilist, numneigh, neigh as synth.NeighborData): forces on local and
        ghost atoms, energy and virial (xx yy zz xy xz yz), all from zero, and
        with per_atom the per-atom energy and virial."""
        x = np.ascontiguousarray(nl.x, dtype=np.float64)
        nall = x.shape[0]
        f = np.zeros((nall, 3))
        e = ctypes.c_double(0.0)
        vir = np.zeros(6)
        eatom = np.zeros(nall) if per_atom else None
        vatom = np.zeros((nall, 6)) if per_atom else None
        tag = np.ascontiguousarray(nl.tag, dtype=np.int64)
        self._check(self.lib.ck_nl_compute(
            self.h, nall, _dp(x), _ip(np.ascontiguousarray(nl.type, dtype=np.int32)),
            tag.ctypes.data_as(ctypes.POINTER(ctypes.c_longlong)), len(nl.ilist),
            _ip(np.ascontiguousarray(nl.ilist, dtype=np.int32)), _ip(np.ascontiguousarray(nl.numneigh, dtype=np.int32)),
            _ip(np.ascontiguousarray(nl.neigh, dtype=np.int32)), float(skin), int(bool(rebuild)), _dp(f),
            ctypes.byref(e), _dp(vir), _dp(eatom) if per_atom else None, _dp(vatom) if per_atom else None))
        out = {"energy": e.value, "force": f, "virial": vir}
        if per_atom:
            out["eatom"], out["vatom"] = eatom, vatom
        return out

    def nl_lists(self):
        cnt = (ctypes.c_longlong * 2)()
        self._check(self.lib.ck_nl_lists(self.h, cnt, None, None))
        l3 = np.zeros((cnt[0], 3), dtype=np.int32)
        l4 = np.zeros((cnt[1], 4), dtype=np.int32)
        self._check(self.lib.ck_nl_lists(self.h, cnt, _ip(l3), _ip(l4)))
        return l3, l4

    def nl_fingerprint(self, nbody: int):
        """Fingerprint records of the last nl_compute (the pair style's
        FINGERPRINT output): distances [n][P] and type indices [n][nbody]."""
        n = ctypes.c_longlong(0)
        self._check(self.lib.ck_nl_fingerprint(self.h, nbody, ctypes.byref(n), None, None))
        P = nbody * (nbody - 1) // 2
        d = np.zeros((n.value, P))
        t = np.zeros((n.value, nbody), dtype=np.int32)
        self._check(self.lib.ck_nl_fingerprint(self.h, nbody, ctypes.byref(n), _dp(d), _ip(t)))
        return d, t

    def fp_histogram(self, nbody: int, d1, t1, d2=None, t2=None, nbin: int = 100):
        """Cluster-distance histogram of the reference's fingerprint tool on the
        GPU: (counts[nbin], number of counted pairs).  d2/t2 None compares the
        first set with itself (pairs j > i)."""
        P = nbody * (nbody - 1) // 2
        same = d2 is None
        d1 = np.ascontiguousarray(d1, dtype=np.float64).reshape(-1, P)
        t1 = np.ascontiguousarray(t1, dtype=np.int32).reshape(-1, nbody)
        if same:
            d2, t2 = d1, t1
        else:
            d2 = np.ascontiguousarray(d2, dtype=np.float64).reshape(-1, P)
            t2 = np.ascontiguousarray(t2, dtype=np.int32).reshape(-1, nbody)
        counts = np.zeros(nbin, dtype=np.int64)
        ns = ctypes.c_longlong(0)
        llp = ctypes.POINTER(ctypes.c_longlong)
        self._check(self.lib.ck_fp_histogram(self.h, nbody, len(t1), _dp(d1), _ip(t1), len(t2), _dp(d2), _ip(t2),
                                              int(same), nbin, counts.ctypes.data_as(llp), ctypes.byref(ns)))
        return counts, ns.value

    def tabulated(self):
        """(2-body tabulated, 3-body tabulated) for the current parameter set."""
        t = np.zeros(2, dtype=np.int32)
        self._check(self.lib.ck_tabulated(self.h, _ip(t)))
        return bool(t[0]), bool(t[1])

    def clusters(self, nbody: int, dx, dr, typ, tab: bool = False):
        """Per-cluster evaluation of n clusters (compute_nB, or compute_2B_tab /
        compute_3B_tab with tab=True): dx[n][P], dr[n][P][3], typ[n][nbody] ->
        dict of per-cluster energy[n], force[n][nbody][3], stress[n][6] and the
        reference's force scalars fscal[n][P]."""
        P = nbody * (nbody - 1) // 2
        dx = np.ascontiguousarray(dx, dtype=np.float64).reshape(-1, P)
        n = dx.shape[0]
        dr = np.ascontiguousarray(dr, dtype=np.float64).reshape(n, P, 3)
        typ = np.ascontiguousarray(typ, dtype=np.int32).reshape(n, nbody)
        force, stress = np.zeros((n, nbody, 3)), np.zeros((n, 6))
        energy, fscal = np.zeros(n), np.zeros((n, P))
        fn = self.lib.ck_compute_cluster_batch_tab if tab else self.lib.ck_compute_cluster_batch
        self._check(fn(self.h, nbody, n, _dp(dx), _dp(dr), _ip(typ), _dp(force), _dp(stress), _dp(energy),
                       _dp(fscal)))
        return {"energy": energy, "force": force, "stress": stress, "fscal": fscal}

    def set_contraction(self, factored=True):
        """3-/4-body contraction kernels: True/1 factored (default), False/0
        per-coefficient, 2 factored without the per-entry pair-table cache,
        3 factored with the 3-body column products formed per coefficient,
        4 factored with the 3-body and 4-body contractions on the tensor cores
        (mixed form; tuning()["tc3"] and ["tc4"] report which run)."""
        self._check(self.lib.ck_set_contraction(self.h, int(factored)))

    def autotune(self, packed=None):
        """Picks threads per cluster and resident blocks for the staged batch
        (stages `packed` first when given); returns (tpc3, tpc4, blocks_per_sm)."""
        if packed is not None:
            self.stage(packed)
        out = (ctypes.c_int * 3)()
        self._check(self.lib.ck_autotune(self.h, out))
        return tuple(out)

    def use_graph(self, on: bool):
        self._check(self.lib.ck_use_graph(self.h, 1 if on else 0))

    # -- packing -------------------------------------------------------------
    def pack(self, configs, slots=None, small=None):
        """configs: sequence of (pos[N,3], types (names or indices), cell[3,3])."""
        n = len(configs)
        slots = [0] * n if slots is None else list(slots)
        natoms = np.array([len(c[0]) for c in configs], dtype=np.int32)
        pos = np.ascontiguousarray(np.concatenate([np.asarray(c[0], dtype=np.float64).reshape(-1, 3)
                                                   for c in configs]))
        if len(set(slots)) == 1 and all(len(c[1]) and isinstance(c[1][0], str) for c in configs):
            # names throughout, one parameter set: one mapping over the whole batch
            types = self.type_indices(list(itertools.chain.from_iterable(c[1] for c in configs)), slots[0])
        else:
            tys = []
            for c, s in zip(configs, slots):
                t = c[1]
                if len(t) and isinstance(t[0], str):
                    tys.append(self.type_indices(t, s))
                else:
                    tys.append(np.asarray(t, dtype=np.int32))
            types = np.ascontiguousarray(np.concatenate(tys).astype(np.int32))
        cells = np.ascontiguousarray(np.stack([np.asarray(c[2], dtype=np.float64).reshape(3, 3) for c in configs]))
        sm = np.zeros(n, dtype=np.int32) if small is None else np.asarray(small, dtype=np.int32).reshape(n)
        ps = np.asarray(slots, dtype=np.int32)
        return natoms, pos, types, cells, sm, ps

    def evaluate_batch(self, configs, slots=None, small=None):
        """Energy, forces and stress of every configuration in one launch
        sequence; per configuration a dict whose force and stress are views into
        arrays allocated for this call."""
        natoms, pos, types, cells, sm, ps = self.pack(configs, slots, small)
        n = len(configs)
        energy = np.zeros(n)
        force = np.zeros((int(natoms.sum()), 3))
        stress = np.zeros((n, 9))
        self._check(self.lib.ck_calculate_batch(self.h, n, _ip(natoms), _dp(pos), _ip(types), _dp(cells), _ip(sm),
                                                _ip(ps), _dp(energy), _dp(force), _dp(stress)))
        # per configuration: views into the batch's freshly allocated arrays
        ends = np.cumsum(natoms).tolist()
        starts = [0] + ends[:-1]
        return [{"energy": energy[s], "force": force[a:b], "stress": stress[s]}
                for s, (a, b) in enumerate(zip(starts, ends))]

    def evaluate(self, pos, types, cell, slot: int = 0, small: bool = False):
        return self.evaluate_batch([(pos, types, cell)], slots=[slot], small=[int(small)])[0]

    # -- split form (device timing) ------------------------------------------
    def stage(self, packed):
        natoms, pos, types, cells, sm, ps = packed
        self._staged_n = (len(natoms), int(natoms.sum()))
        self._check(self.lib.ck_stage_batch(self.h, len(natoms), _ip(natoms), _dp(pos), _ip(types), _dp(cells),
                                            _ip(sm), _ip(ps)))

    def launch(self):
        self._check(self.lib.ck_launch(self.h))

    def collect(self):
        ns, na = self._staged_n
        energy = np.zeros(ns)
        force = np.zeros((na, 3))
        stress = np.zeros((ns, 9))
        self._check(self.lib.ck_collect(self.h, _dp(energy), _dp(force), _dp(stress)))
        return energy, force, stress

    def stream_ptr(self) -> int:
        return self.lib.ck_stream(self.h) or 0

    def counts(self):
        out = (ctypes.c_longlong * 5)()
        self._check(self.lib.ck_last_counts(self.h, out))
        return {"n2": out[0], "n3": out[1], "n4": out[2], "n_ghost": out[3], "n_atoms": out[4]}

    def diagnostics(self):
        out = (ctypes.c_int * 3)()
        self._check(self.lib.ck_last_diagnostics(self.h, out))
        return {"badness": out[0], "penalty_hits": out[1], "below_rin": out[2]}

    def lists(self):
        """Cluster lists of the last evaluation in system-local ghost numbering
        (the reference's indices): l2 (n2,2) [atom, ghost], l3 (n3,3), l4 (n4,4)."""
        c = self.counts()
        l2 = np.zeros((c["n2"], 2), dtype=np.int32)
        l3 = np.zeros((c["n3"], 3), dtype=np.int32)
        l4 = np.zeros((c["n4"], 4), dtype=np.int32)
        self._check(self.lib.ck_export_lists(self.h, _ip(l2), _ip(l3), _ip(l4)))
        return l2, l3, l4
