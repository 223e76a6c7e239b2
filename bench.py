"""Benchmark of the GB300 ChIMES force path.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Workload (per GPU): one periodic configuration of 1024 atoms of 2 elements in
a 22 A cubic box, ChIMES 2B order 12 / 3B order 8 (outer 4.0 A) / 4B order 4
(outer 3.2 A), Tersoff cutoff, seeded synthetic positions and coefficients --
the plain FP64 single-configuration workload.  A step is one full evaluation
(ghost images, cluster lists, Chebyshev stage, contraction, energy/force/virial
reduction and the copy of the results to pinned host memory).

value : atom-evaluations/s with the inputs resident in HBM, CUDA events on
        the library's stream around each step, L2 flushed (256 MB write)
        before every step;
e2e   : the same metric through the reference-facing C ABI
        (calculate_chimes_instance) with host arrays, timed on the host.
targets (default, one GPU): the batched mixed-size workload in FP64 and
        mixed against the plain FP64 path one configuration per call, the
        serving loop (p50/p99 latency at three offered rates) against the
        plain path one request at a time, and the mixed form's error against
        the reference's FP64 results in the committed fixtures; about a
        minute (--no-targets skips it).
Under torchrun each rank runs an independent replica (weak scaling; the path
has no exchange step, so there is no collective on the data path).

--impl reference times the CPU implementation of the same path (the
reference build when it can run here, else the oracle's C restatement of it)
on all host cores.
"""

from __future__ import annotations

import argparse
import ctypes
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

import numpy as np  # noqa: E402

N_ATOMS = 1024
METRIC = "atom-evals/s (E+F+virial), plain FP64 single configuration"
UNIT = "atom-evals/s"
WORKLOAD = ("C2: 1024 atoms, 2 elements (50/50), cubic 22.0 A, ChIMES 12/8/4, Tersoff fcut, "
            "3B outer 4.0 A, 4B outer 3.2 A, plain FP64, one configuration per launch")


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def make_workload(tmpdir):
    from chimes_calculator_gb300 import synth
    params = synth.write_param_file(os.path.join(tmpdir, "c2.params"), synth.spec_c2())
    cfg = synth.config_c2()
    return params, cfg


# ----------------------------------------------------------------------------
# clocks during the timed region
# ----------------------------------------------------------------------------
class ClockSampler:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.QUERY,
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"], "samples": 0}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        rows = []
        for ln in open(self.path).read().splitlines():
            w = [x.strip() for x in ln.split(",")]
            if len(w) >= 9:
                rows.append(w)
        os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            for k, nm in enumerate(names):
                if r[5 + k].lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(rows)}


# ----------------------------------------------------------------------------
# algorithmic work of one evaluation (flop model of the force kernels)
# ----------------------------------------------------------------------------
# DRAM bytes (read + write) per launch of the force kernels on this workload,
# from one ncu capture each (profiles/k_forcef_c2_fp64.md, k_forcen_c2_fp64.md)
PROFILED_TRAFFIC = {
    "k_forcef<3,double,1>": 4272384,
    "k_forcef<3,double,1,true>": 4273408,
    "k_forcef<4,double,4>": 2047488,
    "k_forcen<3,double,4>": 872704,
    "k_forcen<4,double,8>": 599552,
}


def ghost_position_fn(calc, cfg):
    """Position of a system-local ghost index of the last evaluation (image 0 =
    the wrapped atoms, then the periodic layers in the library's order)."""
    info = calc.info(0)
    cell = np.asarray(cfg.cell, dtype=np.float64)
    f = cfg.pos @ np.linalg.inv(cell)
    f -= np.floor(f)
    n = cfg.n_atoms
    L = np.linalg.norm(cell, axis=1).min()
    nl = int(math.ceil(2 * info["max_cutoffs"][0] / L + 1))
    side = 2 * nl + 1

    def ghost_pos(g):
        img = g // n
        a = g % n
        full = img - 1
        center = (nl * side + nl) * side + nl
        full = np.where(full >= center, full + 1, full)
        sh = np.stack([full // (side * side) - nl, (full // side) % side - nl, full % side - nl], axis=-1)
        sh = np.where((img == 0)[..., None], 0, sh)
        return (f[a] + sh) @ cell
    return ghost_pos


def algorithmic_flops(calc, cfg, params_path):
    """Per-launch algorithmic FLOPs of the 3B and 4B force kernels:
        flops(cluster) = P*(6*o + 15) + n_c*(5*P + 1) + P*21
    over the clusters that pass the per-type outer cutoffs (exp/sin/cos count
    as one flop).  Cluster geometry is rebuilt here from the exported lists."""
    info = calc.info(0)
    o2, o3, o4 = info["orders"]
    l2, l3, l4 = calc.lists()
    n = cfg.n_atoms
    ghost_pos = ghost_position_fn(calc, cfg)
    tup = calc.tuple_table(0)
    fac = calc.tuple_factored(0)
    out = {}
    for nb, lst, order in ((3, l3, o3), (4, l4, o4)):
        if lst.shape[0] == 0 or order == 0:
            out[nb] = (0, 0.0, 0.0, 0.0)
            continue
        P = nb * (nb - 1) // 2
        pairs = [(i, j) for i in range(nb) for j in range(i + 1, nb)]
        pos = ghost_pos(lst)
        r = np.stack([np.linalg.norm(pos[:, b] - pos[:, a], axis=1) for a, b in pairs], axis=1)
        t = np.asarray(cfg_types_idx(calc, cfg))[lst % n]
        u = np.zeros(lst.shape[0], dtype=np.int64)
        nt = info["ntypes"]
        for k in range(nb):
            u = u * nt + t[:, k]
        valid, ncoef, rout = tup[nb]
        ok = valid[u].astype(bool) & np.all(r < rout[u][:, :P], axis=1)
        nc = ncoef[u][ok].astype(np.float64)
        flops = ok.sum() * (P * (6 * order + 15) + P * 21) + (nc * (5 * P + 1)).sum()
        # operations the factored kernel performs instead of n_c*(5P+1): two
        # multiply-adds per coefficient per pass, the row/column products and
        # the gradient terms of the nested per-record sums (two multiply-adds
        # per record, plus three or four per run of equal leading powers; runs
        # counted as whole, i.e. one lane per cluster)
        nrow, ncol, R = fac[nb]
        K = 1 if nb == 3 else 3
        C = P - K
        Rf = float(max(R, 1))
        per_row = 4 if K == 1 else 4 + 6 / Rf + 8 / Rf ** 2
        per_col = 4 + 4 / Rf if C == 2 else 4 + 6 / Rf + 6 / Rf ** 2
        ex = ok.sum() * (P * (6 * order + 15) + P * 21 + R ** C * (C - 1) + R ** K * (K - 1)) \
            + (4.0 * nc).sum() + (per_row * nrow[u][ok].astype(np.float64)).sum() \
            + (per_col * ncol[u][ok].astype(np.float64)).sum()
        # without the Y table (3-body): one more multiply per row entry, no table
        ex_noy = ex + nc.sum() - ok.sum() * (R ** C * (C - 1)) if nb == 3 else ex
        out[nb] = (int(ok.sum()), float(flops), float(ex), float(ex_noy))
    return out


_type_cache = {}


def cfg_types_idx(calc, cfg):
    key = id(cfg)
    if key not in _type_cache:
        _type_cache[key] = calc.type_indices(cfg.types, 0)
    return _type_cache[key]


# ----------------------------------------------------------------------------
# our arm
# ----------------------------------------------------------------------------
def run_ours(args):
    import torch
    from chimes_calculator_gb300 import FP64, Calculator, _lib

    world, rank, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    else:
        torch.cuda.set_device(0)
    dev = torch.device("cuda", torch.cuda.current_device())

    tmp = tempfile.mkdtemp(prefix="ckbench")
    params, cfg = make_workload(tmp)
    calc = Calculator(precision=args.precision, graph=True)
    calc.load_params(params)
    packed = calc.pack([(cfg.pos, cfg.types, cfg.cell)])
    if args.contraction == "auto":
        calc.stage(packed)
        calc.autotune()
    else:   # a fixed launch shape (profiler runs): no autotuning
        calc.set_contraction({"factored": 1, "nocache": 2, "noy": 3, "percoef": 0, "tensor": 4}[args.contraction])
        if args.tuning:
            calc.set_tuning(*[int(v) for v in args.tuning.split(",")])
        calc.stage(packed)
    stream = torch.cuda.ExternalStream(calc.stream_ptr(), device=dev)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)

    def one_step():
        calc.launch()

    # warm-up (also sizes the capacities and captures the graph)
    for _ in range(max(3, args.warmup)):
        one_step()
        e, fo, so = calc.collect()
    # correctness of the timed configuration against the committed reference output
    check = None
    gpath = os.path.join(REPO, "tests", "golden", "c2", "expected.json")
    if os.path.exists(gpath):
        g = json.load(open(gpath))
        ge = float(g["energy"])
        gf = np.array([[float(v) for v in r] for r in g["force"]])
        check = {"dE_rel": abs(e[0] - ge) / abs(ge), "dF_max": float(np.abs(fo - gf).max()),
                 "reference_energy": ge}

    lib = _lib.load()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    clocks = ClockSampler(local)
    stage_ms = (ctypes.c_double * 4)()
    nlaunch = ctypes.c_longlong()
    kpl = ctypes.c_int()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    clocks.start()
    t0 = time.perf_counter()
    for k in range(args.steps):
        with torch.cuda.stream(stream):
            flush.fill_(float(k))          # evict L2 (256 MB > 129 MB) before every step
            starts[k].record(stream)
        one_step()
        ends[k].record(stream)
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    clk = clocks.stop()
    step_ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    calc.collect()
    # the stage split, from three more launches after the timed region with the
    # library's stage events (which run the stages one after another instead of
    # the timed steps' two concurrent branches)
    lib.ck_set_profiling(calc.h, 1)
    for k in range(3):
        with torch.cuda.stream(stream):
            flush.fill_(float(k))
        one_step()
        lib.ck_read_stage_times(calc.h, stage_ms, ctypes.byref(nlaunch), ctypes.byref(kpl))
    calc.collect()
    lib.ck_set_profiling(calc.h, 0)
    from chimes_calculator_gb300.replicas import job_time_and_throughput
    total_ms, value = job_time_and_throughput(sum(step_ms), N_ATOMS, args.steps)
    if world > 1:
        torch.distributed.barrier()
    ms_per_step = total_ms / args.steps

    # roofline of the dominant kernel (from the in-library stage events)
    stage = [stage_ms[k] / max(1, nlaunch.value) for k in range(4)]
    names = ["list build", "force 1B+2B", "force 3B", "force 4B"]
    counts = calc.counts()
    work = algorithmic_flops(calc, cfg, params)
    # FP64 FMA probe, repeated for half a second with the SM clock sampled
    # beside it (the roofline denominator and the clock it was measured at)
    peak64 = ctypes.c_double()
    probe_clk = ClockSampler(local)
    probe_clk.start()
    probes, t_probe = [], time.perf_counter()
    while len(probes) < 200 and (time.perf_counter() - t_probe < 0.5 or len(probes) < 3):
        lib.ck_fma_peak(0, ctypes.byref(peak64))
        probes.append(peak64.value)
    peak64.value = statistics.median(probes)
    probe_s = time.perf_counter() - t_probe
    probe_clocks = probe_clk.stop()
    # the dominant single kernel: the list build is ~15 short kernels, each
    # force stage is one kernel, so the longest force stage is the top kernel
    dom = 1 + int(np.argmax(stage[1:]))
    roof = None
    tun = calc.tuning()
    if dom in (2, 3):
        nb = 3 if dom == 2 else 4
        fact = tun["fact%d" % nb]
        tpc = tun[("ftpc%d" if fact else "tpc%d") % nb]
        noy = fact and nb == 3 and tun.get("noy3", 0)
        kname = ("k_forcef<%d,double,%d>" if fact else "k_forcen<%d,double,%d>") % (nb, tpc)
        if noy:
            kname = kname[:-1] + ",true>"
            work[nb] = (work[nb][0], work[nb][1], work[nb][3])
        # DRAM traffic of the kernel's ncu capture on this workload; a launch
        # shape without its own capture (lanes per cluster) reads the same
        # pair tables, coefficient lists and cluster lists as the captured
        # shape of the same contraction form (4.27 MB for the 3-body table and
        # no-table forms alike)
        traffic, traffic_src = PROFILED_TRAFFIC.get(kname), None
        if traffic is not None:
            traffic_src = "ncu dram__bytes_read.sum + dram__bytes_write.sum of this kernel on this workload (profiles/)"
        else:
            same = [v for k, v in PROFILED_TRAFFIC.items() if k.startswith("k_forcef<%d,double," % nb)] if fact else []
            if same:
                traffic = same[0]
                traffic_src = ("ncu capture of the same factored %d-body kernel at another launch shape on this "
                               "workload (profiles/)" % nb)
        achieved = work[nb][1] / (stage[dom] * 1e-3) / 1e12
        executed = (work[nb][2] if fact else work[nb][1]) / (stage[dom] * 1e-3) / 1e12
        roof = {"bound": "fp64", "kernel": kname, "achieved": achieved,
                "peak": peak64.value, "unit": "TFLOP/s", "frac": achieved / peak64.value,
                "traffic": traffic,
                "traffic_source": traffic_src,
                "peak_source": "measured in-run FP64 FMA probe (ck_fma_peak, median of %d runs over %.2f s); "
                "MEASURED_PEAKS.json has no CUDA-core FP64 figure" % (len(probes), probe_s),
                "peak_clocks": probe_clocks,
                "flops_per_launch": work[nb][1], "clusters_evaluated": work[nb][0],
                "executed_flops_per_launch": work[nb][2] if fact else work[nb][1],
                "executed_tflops": executed, "executed_frac": executed / peak64.value,
                "kernel_ms": stage[dom], "share_of_step": stage[dom] / sum(stage)}
    else:
        roof = {"bound": "fp64", "kernel": names[dom], "achieved": None, "peak": peak64.value,
                "unit": "TFLOP/s", "frac": None, "traffic": None}

    # end to end through the reference-facing C ABI with host buffers
    e2e = None
    if not args.profile_run:
        lib.ck_set_error_mode(1)
        h = lib.chimes_open_instance()
        lib.set_chimes_serial_instance(h, 0)
        lib.init_chimes_serial_instance(h, params.encode(), 0)
        n = cfg.n_atoms
        arr = lambda v: (ctypes.c_double * len(v))(*v)
        x, y, z = (arr(cfg.pos[:, k]) for k in range(3))
        ty = (ctypes.c_char_p * n)(*[t.encode() for t in cfg.types])
        ca, cb, cc = (arr(cfg.cell[k]) for k in range(3))
        fx, fy, fz, st = arr([0.0] * n), arr([0.0] * n), arr([0.0] * n), arr([0.0] * 9)
        en = ctypes.c_double(0.0)
        for _ in range(3):
            lib.calculate_chimes_instance(h, n, x, y, z, ty, ca, cb, cc, ctypes.byref(en), fx, fy, fz, st)
        reps = max(20, min(200, args.steps))
        ts = []
        for _ in range(reps):
            en.value = 0.0
            a = time.perf_counter()
            lib.calculate_chimes_instance(h, n, x, y, z, ty, ca, cb, cc, ctypes.byref(en), fx, fy, fz, st)
            ts.append(time.perf_counter() - a)
        err = lib.ck_last_error().decode()
        lib.chimes_close_instance(h)
        sec = sum(ts) / len(ts)
        e2e = {"value": world * n / sec, "unit": UNIT, "h2d_bytes_per_step": n * 24 + n * 4 + 1024,
               "d2h_bytes_per_step": n * 24 + 8 * 8 + 8 * 4 + 3 * 8, "ms_per_call": sec * 1e3,
               "p50_ms": 1e3 * statistics.median(ts), "p99_ms": 1e3 * float(np.percentile(ts, 99)),
               "api": "calculate_chimes_instance", "error": err or None}

    # CPU baseline: the oracle's C restatement of the reference path on one host core
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        cpu = cpu_baseline(params, cfg, seconds=args.cpu_seconds)

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
            "config": {"workload": WORKLOAD, "atoms": N_ATOMS, "pairs": counts["n2"], "triplets": counts["n3"],
                       "quadruplets": counts["n4"], "ghost_atoms": counts["n_ghost"],
                       "l2_flush": "256 MB write before every timed step", "graph": True,
                       "timed_form": "one CUDA graph per step with two concurrent branches (1B+2B beside the "
                                     "cluster enumeration, the 4-body stage beside the 3-body one); stage_ms from "
                                     "three later launches that run the stages one after another",
                       "autotuned": tun,
                       "parallelism": "replicas" if world > 1 else "single GPU"},
            "e2e": e2e,
            "roofline": roof,
            "stage_ms": dict(zip(names, stage)),
            "gpu_launches": kpl.value * args.steps,
            "kernels_per_step": kpl.value,
            "clocks": clk,
            "wall_s_timed_region": wall,
            "cpu_baseline": cpu,
            "check": check,
        }
        if world == 1 and not args.no_targets and not args.profile_run:
            line["targets"] = targets(args)
        if args.extras:
            line["extras"] = extras(args)
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()


def extras(args):
    """Other paths on the same GPU, for context (not the headline): the mixed
    path on the same configuration, and batched FP64 / mixed evaluation of the
    mixed-size workload (configurations of 8-512 atoms)."""
    from chimes_calculator_gb300 import FP64, MIXED, Calculator, synth
    out = {}
    tmp = tempfile.mkdtemp(prefix="ckx")
    params, cfg = make_workload(tmp)
    for prec, name in ((MIXED, "c2_mixed"),):
        c = Calculator(precision=prec, graph=True)
        c.load_params(params)
        c.stage(c.pack([(cfg.pos, cfg.types, cfg.cell)]))
        c.autotune()
        out[name] = time_steps(c, N_ATOMS, 50)
        out[name]["autotuned"] = c.tuning()
    # one large configuration (32768 atoms, 70 x 70 x 72 A, ChIMES 12/10/4),
    # FP64 and mixed, with the mixed result's error against FP64
    p3 = synth.write_param_file(os.path.join(tmp, "c3.params"), synth.spec_c3())
    cfg3 = synth.config_c3()
    res = {}
    for prec, name in ((FP64, "c3_fp64"), (MIXED, "c3_mixed")):
        c = Calculator(precision=prec, graph=True)
        c.load_params(p3)
        c.stage(c.pack([(cfg3.pos, cfg3.types, cfg3.cell)]))
        c.autotune()
        r = time_steps(c, cfg3.n_atoms, 10)
        r["autotuned"] = c.tuning()
        res[name] = c.evaluate(cfg3.pos, cfg3.types, cfg3.cell)
        out[name] = r
    r64, r32 = res["c3_fp64"], res["c3_mixed"]
    out["c3_mixed"]["error_vs_fp64"] = {
        "energy_rel": abs(r32["energy"] - r64["energy"]) / abs(r64["energy"]),
        "force_max_abs": float(np.abs(r32["force"] - r64["force"]).max()),
        "stress_max_abs": float(np.abs(r32["stress"] - r64["stress"]).max())}
    out["pair_style_c2"] = pair_style(params, cfg)
    # the same with the 2- and 3-body terms tabulated (the reference's
    # TABULATION option: spline / tricubic look-up instead of the Chebyshev sums)
    ptab = synth.write_tabulated_param_file(os.path.join(tmp, "c2tab.params"), synth.spec_c2(), step3=0.1)
    out["pair_style_c2_tabulated"] = pair_style(ptab, cfg, cpu_calls=1)
    out["fingerprint_c2"] = fingerprint(params, cfg)
    return out


def gen_processes():
    return max(1, min(8, os.cpu_count() or 1))


def targets(args):
    """The comparisons the path is built for, on bounded samples of their
    workloads (seeded synthetic configurations):
      batched : the 4096-configuration mixed-size workload (8-512 atoms,
                0.05-0.12 atoms/A^3, 1-3 elements, ChIMES 12/10/4) in one
                autotuned launch sequence (CUDA graph), FP64 and mixed; device
                throughput with the inputs resident and end to end through
                ck_calculate_batch with host arrays;
      plain   : the plain FP64 path on the same configurations, one per call
                through the C ABI with host arrays, as a caller without
                batching runs it;
      serving : single-point requests of 16-4096 atoms over three parameter
                sets, Poisson arrivals; the plain FP64 path one request at a
                time, then the continuous-batching server (mixed; FP64 at
                saturation) at offered rates of 1x and 4x the plain path's
                request rate and at saturation, with p50/p99 latency;
      error   : the mixed form against the reference's FP64 results stored in
                the fixtures (the full 32768-atom 12/10/4 configuration, the
                batched workload's extremes, the serving sets and the
                reference's own force fields)."""
    from chimes_calculator_gb300 import FP64, MIXED, Calculator, synth
    out = {}
    tmp = tempfile.mkdtemp(prefix="ckns")
    t_all = time.perf_counter()
    # -- batched vs plain on the mixed-size workload --------------------------
    p4 = synth.write_param_file(os.path.join(tmp, "c4.params"), synth.spec_c4())
    cfgs = synth.configs_c4(n_configs=args.batch_configs, processes=gen_processes())
    atoms = sum(c.n_atoms for c in cfgs)
    batched = {"workload": "%d configurations, 8-512 atoms log-uniform, 0.05-0.12 atoms/A^3, 1-3 elements, "
                           "ChIMES 12/10/4 (3 elements)" % len(cfgs), "atoms": atoms}
    confs = [(x.pos, x.types, x.cell) for x in cfgs]
    for prec, name in ((FP64, "fp64"), (MIXED, "mixed")):
        c = Calculator(precision=prec, graph=True)
        c.load_params(p4)
        c.stage(c.pack(confs))
        c.autotune()
        r = time_steps(c, atoms, 3)
        r["autotuned"] = c.tuning()
        c.evaluate_batch(confs)
        ts = []
        for _ in range(2):
            t0 = time.perf_counter()
            c.evaluate_batch(confs)
            ts.append(time.perf_counter() - t0)
        r["e2e"] = {"value": atoms / min(ts), "unit": UNIT, "api": "ck_calculate_batch (host arrays)",
                    "h2d_bytes": atoms * 28 + len(cfgs) * 100, "d2h_bytes": atoms * 24 + len(cfgs) * 80}
        batched[name] = r
        c.close()
    c = Calculator(precision=FP64, graph=True)
    c.load_params(p4)
    sample = cfgs[: min(len(cfgs), args.plain_configs)]
    for x in sample[:8]:
        c.evaluate(x.pos, x.types, x.cell)
    t0 = time.perf_counter()
    for x in sample:
        c.evaluate(x.pos, x.types, x.cell)
    wall = time.perf_counter() - t0
    sa = sum(x.n_atoms for x in sample)
    c.close()
    plain = {"value": sa / wall, "unit": UNIT, "configs": len(sample), "atoms": sa,
             "ms_per_config": 1e3 * wall / len(sample), "api": "ck_calculate_batch with one configuration per call"}
    batched["plain_fp64_per_config"] = plain
    batched["ratio_mixed_over_plain_fp64"] = batched["mixed"]["value"] / plain["value"]
    batched["ratio_mixed_e2e_over_plain_fp64"] = batched["mixed"]["e2e"]["value"] / plain["value"]
    batched["ratio_fp64_over_plain_fp64"] = batched["fp64"]["value"] / plain["value"]
    out["batched"] = batched
    # -- serving --------------------------------------------------------------
    out["serving"] = serving(args)
    # -- error of the mixed form against the reference ------------------------
    out["error_vs_reference"] = mixed_error_vs_fixtures()
    out["wall_s"] = time.perf_counter() - t_all
    return out


def _golden(name):
    """(params path, Config, small, expected dict, force row index or None) of a committed fixture."""
    import gzip
    import hashlib
    from chimes_calculator_gb300 import synth
    d = os.path.join(REPO, "tests", "golden", name)
    e = json.load(open(os.path.join(d, "expected.json")))
    if "params_from" in e:
        params = os.path.join(REPO, "tests", "golden", e["params_from"], "params.txt")
    elif os.path.exists(os.path.join(d, "params.txt")):
        params = os.path.join(d, "params.txt")
    else:
        params = os.path.join(tempfile.mkdtemp(prefix="ckg"), "params.txt")
        with gzip.open(os.path.join(d, "params.txt.gz"), "rb") as f, open(params, "wb") as g:
            g.write(f.read())
    if "config_from" in e:
        cfg = getattr(synth, e["config_from"])()
        if hashlib.sha256(cfg.xyz_text().encode()).hexdigest() != e["config_sha256"]:
            raise RuntimeError("%s: regenerated configuration differs from the reference's" % name)
        cfg = synth.read_xyz(cfg.write_xyz(os.path.join(tempfile.mkdtemp(prefix="ckg"), "c.xyz")))
    else:
        cfg = synth.read_xyz(os.path.join(d, "config.xyz"))
    idx = None
    if "force_index" in e:
        idx = np.arange(e["force_index"]["start"], cfg.n_atoms, e["force_index"]["stride"])
    return params, cfg, e["small"], e, idx


def mixed_error_vs_fixtures():
    """Mixed form vs the reference's FP64 values in the committed fixtures:
    relative energy, max-abs force (over the stored rows) and stress."""
    from chimes_calculator_gb300 import MIXED, Calculator
    groups = {"full_size_32768_atoms_12_10_4": ["c3_full"],
              "batched_workload_extremes_12_10_4": ["c4_n8_rho005", "c4_n8_rho012", "c4_n512_rho005",
                                                    "c4_n512_rho012"],
              "serving_parameter_sets": ["c5_set0", "c5_set1", "c5_set2"],
              "reference_force_fields": ["ref_hn3", "ref_co2400k", "ref_tio2_arbrot", "ref_chon"]}
    out = {}
    for gname, names in groups.items():
        er = {"energy_rel": 0.0, "force_max_abs": 0.0, "force_max_rel_to_largest": 0.0, "stress_max_abs": 0.0,
              "cases": names}
        for n in names:
            params, cfg, small, e, idx = _golden(n)
            c = Calculator(precision=MIXED)
            c.load_params(params)
            r = c.evaluate(cfg.pos, cfg.types, cfg.cell, small=small)
            c.close()
            ref_f = np.array([[float(v) for v in row] for row in e["force"]])
            got_f = r["force"] if idx is None else r["force"][idx]
            ref_e = float(e["energy"])
            fe = float(np.abs(got_f - ref_f).max())
            er["energy_rel"] = max(er["energy_rel"], abs(r["energy"] - ref_e) / max(1.0, abs(ref_e)))
            er["force_max_abs"] = max(er["force_max_abs"], fe)
            er["force_max_rel_to_largest"] = max(er["force_max_rel_to_largest"],
                                                 fe / max(1.0, float(np.abs(ref_f).max())))
            er["stress_max_abs"] = max(er["stress_max_abs"], float(np.abs(
                r["stress"] - np.array([float(v) for v in e["stress"]])).max()))
        out[gname] = er
    return out


def pair_style(params, cfg, skin=1.0, calls=30, cpu_calls=0):
    """The LAMMPS pair-style path (ck_nl_compute) on the C2 configuration as
    a rank sees it: 1024 local atoms plus ghosts, full neighbour lists within
    cutoff + skin; clusters built once, then evaluated per call with the host
    positions copied in and forces copied out (as between re-neighbourings).
    cpu_calls > 0 also times the oracle's single-core restatement of the
    same pair-style call (lists reused) for scale."""
    from chimes_calculator_gb300 import Calculator, synth
    c = Calculator()
    c.load_params(params)
    info = c.info(0)
    nl = synth.lammps_neighbors(cfg, c.type_indices(cfg.types, 0), max(info["max_cutoffs"]) + skin, seed=11)
    c.nl_compute(nl, skin, rebuild=True)
    t0 = time.perf_counter()
    c.nl_compute(nl, skin, rebuild=True)
    build = time.perf_counter() - t0
    for _ in range(3):
        c.nl_compute(nl, skin, rebuild=False)
    t0 = time.perf_counter()
    for _ in range(calls):
        c.nl_compute(nl, skin, rebuild=False)
    sec = (time.perf_counter() - t0) / calls
    l3, l4 = c.nl_lists()
    out = {"value": nl.nlocal / sec, "unit": UNIT, "ms_per_call": 1e3 * sec, "ms_rebuild_call": 1e3 * build,
           "local_atoms": nl.nlocal, "ghost_atoms": int(len(nl.x) - nl.nlocal), "list_entries": int(len(nl.neigh)),
           "listed_triplets": int(len(l3)), "listed_quadruplets": int(len(l4)), "skin": skin,
           "tabulated": list(c.tabulated())}
    if cpu_calls > 0:
        from oracle.oracle import Oracle
        o = Oracle(params)
        o.lammps_compute(nl, skin, rebuild=True)
        t0 = time.perf_counter()
        for _ in range(cpu_calls):
            o.lammps_compute(nl, skin, rebuild=False)
        out["cpu_oracle_1core_ms_per_call"] = 1e3 * (time.perf_counter() - t0) / cpu_calls
    return out


def fingerprint(params, cfg, skin=1.0, cpu_records=3000):
    """The FINGERPRINT pipeline on the C2 configuration: the pair style's
    cluster records of one step (GPU) and the self-histograms of the
    reference's histogram tool per body order (GPU all-pairs kernel), with
    the oracle's single-core histogram timed on the first `cpu_records`
    records of each order for scale."""
    from chimes_calculator_gb300 import Calculator, synth
    from oracle.oracle import Oracle
    c = Calculator()
    c.load_params(params)
    nl = synth.lammps_neighbors(cfg, c.type_indices(cfg.types, 0), max(c.info(0)["max_cutoffs"]) + skin, seed=11)
    c.nl_compute(nl, skin, rebuild=True)
    o = Oracle(params)
    out = {}
    for nb in (2, 3, 4):
        t0 = time.perf_counter()
        d, t = c.nl_fingerprint(nb)
        rec_s = time.perf_counter() - t0
        c.fp_histogram(nb, d[:64], t[:64])                 # warm-up (module load, allocations)
        t0 = time.perf_counter()
        counts, ns = c.fp_histogram(nb, d, t)
        gpu_s = time.perf_counter() - t0
        m = min(cpu_records, len(t))
        t0 = time.perf_counter()
        _, cns = o.fp_histogram(nb, d[:m], t[:m])
        cpu_s = time.perf_counter() - t0
        out["%db" % nb] = {"records": int(len(t)), "pairs": int(ns), "records_ms": 1e3 * rec_s,
                           "histogram_ms": 1e3 * gpu_s, "pairs_per_s": ns / gpu_s,
                           "cpu_oracle_1core_pairs_per_s": cns / cpu_s if cpu_s > 0 else None,
                           "cpu_sample_records": m}
    return out


def profile_pairstyle(args, skin=1.0):
    """Profiler run of the pair-style path on the C2 configuration."""
    from chimes_calculator_gb300 import Calculator, synth
    tmp = tempfile.mkdtemp(prefix="ckp")
    params, cfg = make_workload(tmp)
    if args.profile_pairstyle == "tabulated":
        params = synth.write_tabulated_param_file(os.path.join(tmp, "c2tab.params"), synth.spec_c2(), step3=0.1)
    c = Calculator()
    c.load_params(params)
    nl = synth.lammps_neighbors(cfg, c.type_indices(cfg.types, 0), max(c.info(0)["max_cutoffs"]) + skin, seed=11)
    c.nl_compute(nl, skin, rebuild=True)
    if args.profile_pairstyle == "fingerprint":
        d, t = c.nl_fingerprint(3)
        counts, ns = c.fp_histogram(3, d, t)
        print(json.dumps({"records": int(len(t)), "pairs": int(ns)}))
        return
    t0 = time.perf_counter()
    for _ in range(5):
        c.nl_compute(nl, skin, rebuild=False)
    print(json.dumps({"mode": args.profile_pairstyle, "ms_per_call": 1e3 * (time.perf_counter() - t0) / 5}))


def profile_direct(args, reps=5):
    """The per-cluster entry points (chimesFF::compute_2B/3B/4B through
    ck_compute_cluster_batch) on every cluster the C2 configuration lists:
    distances, displacements (second atom minus first) and type indices built
    on the host from the exported lists, one batched call per body order,
    timed on the host with the copies in and out."""
    from chimes_calculator_gb300 import Calculator
    tmp = tempfile.mkdtemp(prefix="ckd")
    params, cfg = make_workload(tmp)
    c = Calculator()
    c.load_params(params)
    c.evaluate(cfg.pos, cfg.types, cfg.cell)
    lists = c.lists()
    gp = ghost_position_fn(c, cfg)
    ti = c.type_indices(cfg.types)
    out = {}
    for nb, lst in zip((2, 3, 4), lists):
        pos = gp(lst)
        dr = np.stack([pos[:, b] - pos[:, a] for a in range(nb) for b in range(a + 1, nb)], axis=1)
        dx = np.linalg.norm(dr, axis=2)
        typ = ti[lst % cfg.n_atoms]
        c.clusters(nb, dx, dr, typ)
        t0 = time.perf_counter()
        for _ in range(reps):
            c.clusters(nb, dx, dr, typ)
        dt = (time.perf_counter() - t0) / reps
        out["%db" % nb] = {"clusters": int(len(lst)), "ms_per_call": 1e3 * dt, "clusters_per_s": len(lst) / dt}
    print(json.dumps(out))


def serving(args):
    """Continuous batching of single-point requests (three parameter sets,
    16-4096 atoms log-uniform): the plain FP64 path one request at a time,
    then the server (tuned once on a sample of the requests) with Poisson
    arrivals at 1x and 4x the plain path's request rate and at saturation;
    p50/p99 latency and throughput per rate."""
    from chimes_calculator_gb300 import Calculator, synth
    from chimes_calculator_gb300.serving import Server, replay_run, serial_run, serving_workload
    tmp = tempfile.mkdtemp(prefix="cks")
    specs, reqs = serving_workload(args.serve_requests, processes=gen_processes())
    paths = [synth.write_param_file(os.path.join(tmp, "p%d.txt" % k), sp) for k, sp in enumerate(specs)]
    calc = Calculator(graph=False)
    for p in paths:
        calc.load_params(p)
    tidx = lambda slot, cfg: calc.type_indices(cfg.types, slot)
    serial_run(calc, reqs[:50], tidx)                      # warm-up
    base = serial_run(calc, reqs, tidx)
    out = {"workload": "%d requests, 16-4096 atoms log-uniform, 0.05-0.12 atoms/A^3, parameter sets 12/8/4 "
                       "(1 element), 12/10/4 (2), 12/8/4 (3)" % len(reqs),
           "requests": len(reqs), "atoms": int(sum(c.n_atoms for _, c in reqs)),
           "workers": args.serve_workers, "max_batch_atoms": args.serve_batch_atoms,
           "plain_fp64_per_request": base}
    for prec, name, mults in ((1, "mixed", (1.0, 4.0, 1e3)), (0, "fp64", (1e3,))):
        srv = Server(workers=args.serve_workers, precision=prec, max_batch_atoms=args.serve_batch_atoms)
        for p in paths:
            srv.load_params(p)
        sample, na = [], 0
        for slot, cf in reqs:
            if na + cf.n_atoms > args.serve_batch_atoms:
                break
            sample.append((slot, cf))
            na += cf.n_atoms
        tuned = srv.autotune([(cf.pos, tidx(sl, cf), cf.cell) for sl, cf in sample], [sl for sl, _ in sample])
        # warm-up: every request once, back to back, so the workspaces and
        # list capacities reach their steady-state sizes before the timed sweeps
        replay_run(srv, reqs, tidx, rate_hz=1e6)
        runs = []
        for mult in mults:
            r = replay_run(srv, reqs, tidx, rate_hz=mult * base["throughput_req_per_s"])
            r["offered_over_plain"] = mult if mult < 1e3 else "saturation"
            runs.append(r)
        srv.close()
        out["server_" + name] = {"autotuned": tuned, "runs": runs}
    sat = out["server_mixed"]["runs"][-1]["throughput_atoms_per_s"]
    out["ratio_server_mixed_over_plain_fp64"] = sat / base["throughput_atoms_per_s"]
    out["ratio_server_fp64_over_plain_fp64"] = (out["server_fp64"]["runs"][-1]["throughput_atoms_per_s"] /
                                                base["throughput_atoms_per_s"])
    return out


def profile_batched(args):
    """The batched workload alone, for a profiler's launch list."""
    import torch
    from chimes_calculator_gb300 import Calculator, synth
    torch.cuda.set_device(0)
    tmp = tempfile.mkdtemp(prefix="ckp")
    p4 = synth.write_param_file(os.path.join(tmp, "c4.params"), synth.spec_c4())
    cfgs = synth.configs_c4(n_configs=args.batch_configs)
    atoms = sum(c.n_atoms for c in cfgs)
    c = Calculator(precision=args.precision, graph=True)
    c.load_params(p4)
    c.stage(c.pack([(x.pos, x.types, x.cell) for x in cfgs]))
    if args.contraction == "auto":
        c.autotune()
    else:   # one contraction form at a fixed launch shape, no autotuning
        c.set_contraction({"factored": 1, "nocache": 2, "noy": 3, "percoef": 0, "tensor": 4}[args.contraction])
        if args.tuning:
            c.set_tuning(*[int(v) for v in args.tuning.split(",")])
        c.stage(c.pack([(x.pos, x.types, x.cell) for x in cfgs]))
    r = time_steps(c, atoms, 2)
    r["autotuned"] = c.tuning()
    r["configs"] = len(cfgs)
    print(json.dumps(r))


def time_steps(c, atoms, steps):
    import torch
    from chimes_calculator_gb300 import _lib
    lib = _lib.load()
    stream = torch.cuda.ExternalStream(c.stream_ptr())
    for _ in range(3):
        c.launch()
        c.collect()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    for a, b in ev:
        a.record(stream)
        c.launch()
        b.record(stream)
    torch.cuda.synchronize()
    c.collect()
    ms = sum(a.elapsed_time(b) for a, b in ev) / steps
    # stage split from one more launch with the in-library stage events
    lib.ck_set_profiling(c.h, 1)
    stage_ms = (ctypes.c_double * 4)()
    nl, kpl = ctypes.c_longlong(), ctypes.c_int()
    c.launch()
    lib.ck_read_stage_times(c.h, stage_ms, ctypes.byref(nl), ctypes.byref(kpl))
    c.collect()
    lib.ck_set_profiling(c.h, 0)
    names = ["list build", "force 1B+2B", "force 3B", "force 4B"]
    return {"value": atoms / (ms * 1e-3), "unit": UNIT, "ms_per_step": ms, "counts": c.counts(),
            "stage_ms": {k: stage_ms[i] / max(1, nl.value) for i, k in enumerate(names)}}


# ----------------------------------------------------------------------------
# CPU paths (the oracle is the checker and the CPU baseline only)
# ----------------------------------------------------------------------------
def _cpu_worker(job):
    params, xyz, reps = job
    sys.path.insert(0, REPO)
    from chimes_calculator_gb300 import synth
    from oracle.oracle import Oracle
    cfg = synth.read_xyz(xyz)
    o = Oracle(params)
    o.calculate(cfg.pos, cfg.types, cfg.cell)     # load + first call
    ts = []
    for _ in range(reps):
        a = time.perf_counter()
        o.calculate(cfg.pos, cfg.types, cfg.cell)
        ts.append(time.perf_counter() - a)
    return ts


def cpu_kind():
    ref = os.path.join(REPO, "oracle", "_ref", "ref_driver")
    if os.path.exists(ref) and os.access(ref, os.X_OK):
        try:
            subprocess.run([ref], capture_output=True, timeout=10)
            return "reference", ref
        except Exception:
            pass
    return "port", None


def cpu_baseline(params, cfg, seconds=10.0):
    from oracle.oracle import build_port
    build_port()
    tmp = tempfile.mkdtemp(prefix="ckcpu")
    xyz = cfg.write_xyz(os.path.join(tmp, "c2.xyz"))
    kind, ref = cpu_kind()
    if kind == "reference":
        from oracle.oracle import run_reference
        t0 = time.perf_counter()
        _, _, tm = run_reference(params, xyz, False, os.path.join(tmp, "r"), time_reps=3)
        sec = tm["best_s"]
        reps = 3
    else:
        t0 = time.perf_counter()
        ts = _cpu_worker((params, xyz, 1))
        reps = max(2, min(50, int(seconds / max(ts[0], 1e-3))))
        ts = _cpu_worker((params, xyz, reps))
        sec = statistics.median(ts)
    import platform
    return {"value": N_ATOMS / sec, "unit": UNIT, "cores": 1, "kind": kind,
            "sample": "%d evaluations of the full 1024-atom workload on one core (median %.3f s each); %s" % (
                reps, sec, platform.processor() or platform.machine()),
            "wall_s": time.perf_counter() - t0}


def run_reference_arm(args):
    world, rank, local = dist_env()
    if rank != 0:
        return
    import multiprocessing as mp
    tmp = tempfile.mkdtemp(prefix="ckref")
    params, cfg = make_workload(tmp)
    xyz = cfg.write_xyz(os.path.join(tmp, "c2.xyz"))
    kind, _ = cpu_kind()
    cores = os.cpu_count() or 1
    ctx = mp.get_context("spawn")
    from oracle.oracle import build_port
    build_port()
    # bounded sample: every core evaluates the workload once per step; the number
    # of timed steps is capped so the run ends within a few minutes
    with ctx.Pool(cores) as pool:
        t = time.perf_counter()
        pool.map(_cpu_worker, [(params, xyz, 1)] * cores)
        one = (time.perf_counter() - t) / 2.0
        steps = max(1, min(args.steps, int(120.0 / max(one, 1e-3))))
        warm = min(max(3, args.warmup), 10)   # at least 3 warm-up steps, bounded like the timed ones
        for _ in range(warm):
            pool.map(_cpu_worker, [(params, xyz, 1)] * cores)
        t0 = time.perf_counter()
        per = pool.map(_cpu_worker, [(params, xyz, steps)] * cores)
        wall = time.perf_counter() - t0
    evals = cores * steps
    sec_per_eval = statistics.median([x for ts in per for x in ts])
    value = cores * N_ATOMS / sec_per_eval
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": steps, "warmup": warm, "ms_per_step": 1e3 * sec_per_eval, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
            "config": {"workload": WORKLOAD, "atoms": N_ATOMS, "parallelism": "%d independent processes" % cores},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": kind,
                             "sample": "%d evaluations (%d per core) of the 1024-atom workload, %s; wall %.1f s" % (
                                 evals, steps, "oracle C restatement of the reference path (the reference "
                                 "sources are not on this machine)" if kind == "port" else "reference build",
                                 wall)},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=300)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--extras", action="store_true",
                    help="also time the mixed form on C2, the 32768-atom configuration, the pair-style path "
                         "and the fingerprint pipeline")
    ap.add_argument("--no-targets", action="store_true",
                    help="skip the batched / plain / serving / error block of the default line")
    ap.add_argument("--serve-requests", type=int, default=6000)
    ap.add_argument("--serve-workers", type=int, default=4)
    ap.add_argument("--serve-batch-atoms", type=int, default=16384)
    ap.add_argument("--batch-configs", type=int, default=4096)
    ap.add_argument("--plain-configs", type=int, default=1024,
                    help="configurations of the mixed-size workload timed one per call (plain FP64)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--precision", type=int, default=0, help="0 FP64 (headline), 1 mixed")
    ap.add_argument("--profile-run", action="store_true",
                    help="minimal run for a profiler: 3 warm-up + 2 steps, no e2e / CPU legs")
    ap.add_argument("--profile-batched", action="store_true",
                    help="profiler run of the batched workload (--batch-configs configurations, "
                         "--precision): autotune, 3 warm-up + 2 launches")
    ap.add_argument("--contraction", default="auto", choices=["auto", "factored", "nocache", "noy", "percoef", "tensor"],
                    help="autotune (auto) or one fixed 3-/4-body contraction form (profiler runs)")
    ap.add_argument("--tuning", default="",
                    help="with a fixed --contraction: tpc3,tpc4,blocks_per_sm (ck_set_tuning)")
    ap.add_argument("--profile-pairstyle", default="", choices=["", "chebyshev", "tabulated", "fingerprint"],
                    help="profiler run of the pair-style path on C2 (Chebyshev or tabulated terms: one list "
                         "build + 5 calls), or of the 3-body fingerprint histogram of its records")
    ap.add_argument("--profile-direct", action="store_true",
                    help="the per-cluster entry points (compute_2B/3B/4B, ck_compute_cluster_batch) on every "
                         "listed cluster of C2, one batched call per body order")
    args = ap.parse_args()
    if args.profile_direct:
        profile_direct(args)
        return
    if args.profile_batched:
        profile_batched(args)
        return
    if args.profile_pairstyle:
        profile_pairstyle(args)
        return
    if args.profile_run:
        args.steps, args.warmup, args.no_cpu, args.extras = 2, 3, True, False
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference_arm(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
