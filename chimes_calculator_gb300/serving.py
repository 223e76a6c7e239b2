"""Continuous-batching serving of single-point energy/force/stress requests.

``Server`` wraps the library's request server (ck_server_* in
include/chimes_gb300.h): worker threads, each with its own CUDA stream and
device-resident parameter sets, batch the waiting requests under an atom limit
and an HBM budget and overlap their batches on the GPU.  ``poisson_run``
offers requests at Poisson-distributed arrival times and reports per-request
latency percentiles and throughput; ``serial_run`` is the plain per-request
path (one evaluation at a time through ``Calculator``) for comparison.
"""

from __future__ import annotations

import ctypes
import math
import threading
import time
from typing import Dict, List, Optional, Sequence, Tuple

import numpy as np

from . import _lib
from .api import FP64, Calculator, ChimesError


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _ip(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int))


class Server:
    def __init__(self, workers: int = 2, hbm_budget_gb: float = 150.0, max_batch_atoms: int = 1 << 16,
                 precision: int = FP64):
        self.lib = _lib.load()
        self.lib.ck_set_error_mode(1)
        self.h = self.lib.ck_server_open(workers, hbm_budget_gb, max_batch_atoms, precision)
        self.workers = workers
        if not self.h:
            raise ChimesError(self.lib.ck_last_error().decode())
        self._natoms: Dict[int, int] = {}
        self._lock = threading.Lock()

    def close(self):
        if self.h:
            self.lib.ck_server_close(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def load_params(self, path: str) -> int:
        slot = self.lib.ck_server_load_params(self.h, path.encode())
        if slot < 0:
            raise ChimesError(self.lib.ck_last_error().decode())
        return slot

    def submit(self, pos, types, cell, slot: int = 0, small: bool = False) -> int:
        pos = np.ascontiguousarray(pos, dtype=np.float64)
        types = np.ascontiguousarray(types, dtype=np.int32)
        cell = np.ascontiguousarray(cell, dtype=np.float64).reshape(9)
        rid = self.lib.ck_server_submit(self.h, slot, pos.shape[0], _dp(pos), _ip(types), _dp(cell), int(small))
        if rid < 0:
            raise ChimesError(self.lib.ck_last_error().decode())
        with self._lock:
            self._natoms[rid] = pos.shape[0]
        return rid

    def take(self, rid: int, wait: bool = True, timeout: float = 120.0) -> Optional[dict]:
        with self._lock:
            n = self._natoms[rid]
        e = ctypes.c_double()
        lat = ctypes.c_double()
        force = np.zeros((n, 3))
        stress = np.zeros(9)
        st = self.lib.ck_server_take(self.h, rid, int(wait), timeout, ctypes.byref(e), _dp(force), _dp(stress),
                                     ctypes.byref(lat))
        if st == 0:
            return None
        with self._lock:
            self._natoms.pop(rid, None)
        if st < 0:
            raise ChimesError(self.lib.ck_last_error().decode())
        return {"energy": e.value, "force": force, "stress": stress, "latency": lat.value}

    def autotune(self, configs: Sequence[Tuple[object, object, object]], slots: Sequence[int]) -> Tuple[int, int, int]:
        """Tunes every worker on a representative batch of (pos, type indices,
        cell) with their parameter slots; returns (lanes per 3-body cluster,
        lanes per 4-body cluster, blocks per SM)."""
        natoms = np.array([np.asarray(c[0]).shape[0] for c in configs], dtype=np.int32)
        pos = np.ascontiguousarray(np.concatenate([np.asarray(c[0], dtype=np.float64).reshape(-1, 3)
                                                   for c in configs]))
        types = np.ascontiguousarray(np.concatenate([np.asarray(c[1], dtype=np.int32) for c in configs]))
        cells = np.ascontiguousarray(np.stack([np.asarray(c[2], dtype=np.float64).reshape(9) for c in configs]))
        ps = np.ascontiguousarray(np.asarray(slots, dtype=np.int32))
        chosen = np.zeros(3, dtype=np.int32)
        rc = self.lib.ck_server_autotune(self.h, len(configs), _ip(natoms), _dp(pos), _ip(types), _dp(cells), None,
                                         _ip(ps), _ip(chosen))
        if rc != 0:
            raise ChimesError(self.lib.ck_last_error().decode())
        return tuple(int(v) for v in chosen)

    def worker_tunings(self) -> list:
        """Each worker's launch preferences (11 values, ck_get_tuning's order
        with the contraction-form entries as preferences)."""
        out = []
        for w in range(self.workers):
            buf = (ctypes.c_int * 11)()
            if self.lib.ck_server_worker_tuning(self.h, w, buf) != 0:
                raise ChimesError(self.lib.ck_last_error().decode())
            out.append(tuple(buf))
        return out

    def stats(self) -> dict:
        out = (ctypes.c_longlong * 6)()
        self.lib.ck_server_stats(self.h, out)
        return {"submitted": out[0], "completed": out[1], "batches": out[2], "largest_batch": out[3],
                "bytes_in_flight": out[4], "peak_bytes_in_flight": out[5]}


def serving_workload(n_requests: int, seed: int = 1105, n_min: int = 16, n_max: int = 4096, processes: int = 0):
    """Requests of the serving workload: each draws one of three parameter
    sets (12/8/4 with one element, 12/10/4 with two, 12/8/4 with three); atom
    counts log-uniform in [n_min, n_max]; density U(0.05, 0.12) per A^3.
    ``processes`` > 1 generates the configurations in a spawned pool."""
    from . import synth
    rng = np.random.default_rng(seed)
    specs = synth.specs_c5()
    slots, jobs = [], []
    for q in range(n_requests):
        slot = int(rng.integers(len(specs)))
        n = int(round(math.exp(rng.uniform(math.log(n_min), math.log(n_max)))))
        rho = rng.uniform(0.05, 0.12)
        L = (n / rho) ** (1.0 / 3.0)
        slots.append(slot)
        jobs.append((n, L, list(specs[slot].elements), int(rng.integers(1 << 31))))
    cfgs = synth.generate_configs(jobs, processes)
    return specs, list(zip(slots, cfgs))


def poisson_run(server: Server, requests: Sequence[Tuple[int, object]], type_idx, rate_hz: float,
                seed: int = 7) -> dict:
    """Submits requests at Poisson arrival times (mean rate rate_hz) from one
    thread while another collects them; returns latency percentiles and
    throughput.  type_idx(slot, cfg) -> int32 type indices."""
    rng = np.random.default_rng(seed)
    gaps = rng.exponential(1.0 / rate_hz, size=len(requests))
    ids: List[int] = [0] * len(requests)
    ready = [threading.Event() for _ in requests]
    prepared = [(slot, cfg.pos, type_idx(slot, cfg), cfg.cell) for slot, cfg in requests]

    def submitter():
        t_next = time.perf_counter()
        for q, (slot, pos, ty, cell) in enumerate(prepared):
            t_next += gaps[q]
            while True:
                dt = t_next - time.perf_counter()
                if dt <= 0:
                    break
                time.sleep(min(dt, 0.002))
            ids[q] = server.submit(pos, ty, cell, slot=slot)
            ready[q].set()

    t0 = time.perf_counter()
    th = threading.Thread(target=submitter)
    th.start()
    lat = []
    atoms = 0
    for q in range(len(requests)):
        ready[q].wait()
        r = server.take(ids[q], wait=True)
        lat.append(r["latency"])
        atoms += requests[q][1].n_atoms
    wall = time.perf_counter() - t0
    th.join()
    lat = np.array(lat)
    return {"offered_rate_hz": rate_hz, "requests": len(requests), "wall_s": wall,
            "throughput_atoms_per_s": atoms / wall, "throughput_req_per_s": len(requests) / wall,
            "p50_ms": 1e3 * float(np.percentile(lat, 50)), "p99_ms": 1e3 * float(np.percentile(lat, 99)),
            "mean_ms": 1e3 * float(lat.mean()), "stats": server.stats()}


def replay_run(server: Server, requests: Sequence[Tuple[int, object]], type_idx, rate_hz: float,
               seed: int = 7) -> dict:
    """Poisson arrivals (mean rate rate_hz) offered by the server's native
    replay driver (ck_server_replay): the same measurement as poisson_run
    without the Python client's per-request cost."""
    rng = np.random.default_rng(seed)
    arrival = np.cumsum(rng.exponential(1.0 / rate_hz, size=len(requests)))
    slots = np.array([s for s, _ in requests], dtype=np.int32)
    natoms = np.array([c.n_atoms for _, c in requests], dtype=np.int32)
    pos = np.ascontiguousarray(np.concatenate([np.asarray(c.pos, dtype=np.float64) for _, c in requests]))
    types = np.ascontiguousarray(np.concatenate([np.asarray(type_idx(s, c), dtype=np.int32) for s, c in requests]))
    cells = np.ascontiguousarray(np.stack([np.asarray(c.cell, dtype=np.float64).reshape(9) for _, c in requests]))
    lat = np.zeros(len(requests))
    wall = ctypes.c_double()
    rc = server.lib.ck_server_replay(server.h, len(requests), _ip(slots), _ip(natoms), _dp(pos), _ip(types),
                                     _dp(cells), None, _dp(arrival), _dp(lat), None, ctypes.byref(wall))
    if rc != 0:
        raise ChimesError(server.lib.ck_last_error().decode())
    atoms = int(natoms.sum())
    return {"offered_rate_hz": rate_hz, "requests": len(requests), "wall_s": wall.value,
            "throughput_atoms_per_s": atoms / wall.value, "throughput_req_per_s": len(requests) / wall.value,
            "p50_ms": 1e3 * float(np.percentile(lat, 50)), "p99_ms": 1e3 * float(np.percentile(lat, 99)),
            "mean_ms": 1e3 * float(lat.mean()), "client": "native replay (ck_server_replay)",
            "stats": server.stats()}


def serial_run(calc: Calculator, requests: Sequence[Tuple[int, object]], type_idx) -> dict:
    """The plain per-request GPU path: one evaluation at a time through the
    C ABI (ck_calculate_batch with one configuration, host arrays in and
    out).  Each request's arguments are marshalled before the timing, so the
    times hold the library call alone."""
    prepared = []
    for slot, cfg in requests:
        n = cfg.n_atoms
        prepared.append((np.array([n], dtype=np.int32), np.ascontiguousarray(cfg.pos, dtype=np.float64),
                         np.ascontiguousarray(type_idx(slot, cfg), dtype=np.int32),
                         np.ascontiguousarray(np.asarray(cfg.cell, dtype=np.float64).reshape(9)),
                         np.zeros(1, dtype=np.int32), np.array([slot], dtype=np.int32), np.zeros(1),
                         np.zeros((n, 3)), np.zeros(9)))
    args = [tuple(_ip(a) if a.dtype == np.int32 else _dp(a) for a in pr) for pr in prepared]
    lib, h = calc.lib, calc.h
    lat = np.zeros(len(requests))
    t0 = time.perf_counter()
    for q, a in enumerate(args):
        t = time.perf_counter()
        rc = lib.ck_calculate_batch(h, 1, *a)
        lat[q] = time.perf_counter() - t
        if rc != 0:
            raise ChimesError(lib.ck_last_error().decode())
    wall = time.perf_counter() - t0
    atoms = sum(c.n_atoms for _, c in requests)
    return {"requests": len(requests), "wall_s": wall, "throughput_atoms_per_s": atoms / wall,
            "throughput_req_per_s": len(requests) / wall, "p50_ms": 1e3 * float(np.percentile(lat, 50)),
            "p99_ms": 1e3 * float(np.percentile(lat, 99)), "api": "ck_calculate_batch, one configuration per call"}
