"""Cluster fingerprints: the files and the histogram workflow of the
reference's FINGERPRINT build, on the GPU entry points.

The reference's pair style, built with FINGERPRINT and run as
``pair_style chimesFF fingerprint <every>``, writes the clusters it evaluates
every ``<every>`` steps to ``<step>.<rank>.<n>b_clusters.txt``
(etc/lmp/src/pair_chimes.cpp:236-256, 525-536, 656-662, 736-742, 818-824);
``chimesFF/src/FP/post_process.sh`` concatenates each frame's files by rank
into ``<frame>.all-<n>b-clusters.txt``; ``multi_calc_histogram.cpp`` turns each
frame into self-histograms of cluster distances, ``<f>-<f>.<n>b_clu-s.hist``.

Here ``record_step`` writes a step's files from ``Calculator.nl_fingerprint``
(the records of the last ``nl_compute``), ``combine_frames`` does what
post_process.sh does, and ``histogram_frames`` does what the histogram tool
does, with the all-pairs loop on the GPU (``Calculator.fp_histogram``).  Files
use the reference's number format (C++ stream default: 6 significant digits),
so the histograms are computed from the same rounded distances.
"""

from __future__ import annotations

import math
import os
import re
from typing import Dict, List, Tuple

import numpy as np

NBIN = 100   # bins per histogram in the reference's tool


def fmt(v: float) -> str:
    """A double as a default-formatted C++ stream writes it (%g, 6 digits)."""
    return "%g" % v


def write_clusters(path: str, dist: np.ndarray, types: np.ndarray) -> None:
    """writeClusterDataComp (pair_chimes.cpp:236-256): per record its
    distances then its type indices, space-separated."""
    dist = np.asarray(dist, dtype=np.float64)
    types = np.asarray(types)
    with open(path, "w") as f:
        for d, t in zip(dist.reshape(len(types), -1), types):
            f.write(" ".join([fmt(v) for v in d] + [fmt(float(v)) for v in t]) + "\n")


def read_clusters(path: str, nbody: int) -> Tuple[np.ndarray, np.ndarray]:
    """read_flat_clusters' parse (multi_calc_histogram.cpp:26-60): P distances
    and nbody type indices per line."""
    P = nbody * (nbody - 1) // 2
    d, t = [], []
    with open(path) as f:
        for line in f:
            items = line.split()
            if not items:
                continue
            if len(items) != P + nbody:
                raise ValueError("%s: read %d items, expected %d (wrong cluster file?)" % (path, len(items), P + nbody))
            d.append([float(v) for v in items[:P]])
            t.append([int(v) for v in items[P:]])
    return np.array(d, dtype=np.float64).reshape(-1, P), np.array(t, dtype=np.int32).reshape(-1, nbody)


def record_step(calc, step: int, rank: int = 0, directory: str = ".") -> Dict[int, int]:
    """Writes the three cluster files of one step from the last nl_compute of
    `calc` (empty for a body order the parameter set does not have); returns
    the record count per body order."""
    orders = calc.info(calc.slots[0] if calc.slots else 0)["orders"]
    counts = {}
    for nb in (2, 3, 4):
        if nb == 2 or orders[nb - 2] > 0:
            d, t = calc.nl_fingerprint(nb)
        else:
            d, t = np.zeros((0, nb * (nb - 1) // 2)), np.zeros((0, nb), dtype=np.int32)
        write_clusters(os.path.join(directory, "%d.%d.%db_clusters.txt" % (step, rank, nb)), d, t)
        counts[nb] = len(t)
    return counts


def combine_frames(directory: str = ".") -> List[str]:
    """post_process.sh: per body order and frame, the ranks' files
    concatenated in rank order into <frame>.all-<n>b-clusters.txt; the
    per-rank files are removed."""
    made = []
    for nb in (2, 3, 4):
        pat = re.compile(r"^(\d+)\.(\d+)\.%db_clusters\.txt$" % nb)
        frames: Dict[str, List[Tuple[int, str]]] = {}
        for name in os.listdir(directory):
            m = pat.match(name)
            if m:
                frames.setdefault(m.group(1), []).append((int(m.group(2)), name))
        for frame, files in frames.items():
            out = os.path.join(directory, "%s.all-%db-clusters.txt" % (frame, nb))
            with open(out, "w") as fo:
                for _, name in sorted(files):
                    with open(os.path.join(directory, name)) as fi:
                        fo.write(fi.read())
            for _, name in files:
                os.remove(os.path.join(directory, name))
            made.append(out)
    return made


def max_distance(nbody: int) -> float:
    """Histogram range of the reference's tool (the transformed distances lie
    in [-1, 1] inside the cutoffs; 1.0 added for its composition term)."""
    return {2: 3.0, 3: math.sqrt(12.0) + 1.0, 4: math.sqrt(24.0) + 1.0}[nbody]


def write_hist(path: str, nbody: int, counts: np.ndarray, nsamples: int) -> None:
    """The histogram file: bin centre and counts / nsamples per line."""
    nbin = len(counts)
    binw = max_distance(nbody) / nbin
    with open(path, "w") as f:
        for i, c in enumerate(counts):
            v = float(c) / nsamples if nsamples else float("nan")
            f.write("%s %s\n" % (fmt(i * binw + 0.5 * binw), fmt(v)))


def histogram_frames(calc, directory: str = ".", nbin: int = NBIN) -> Dict[str, Dict[int, Tuple[np.ndarray, int]]]:
    """multi_calc_histogram.cpp's main: every frame with a
    <frame>.all-2b-clusters.txt, in numeric order, gets its 2-, 3- and 4-body
    self-histograms written to <frame>-<frame>.<n>b_clu-s.hist.  `calc` holds
    the parameter set the records were made with."""
    frames = []
    for name in os.listdir(directory):
        m = re.match(r"^(\d+)\.all-2b-clusters\.txt$", name)
        if m:
            frames.append(m.group(1))
    frames.sort(key=int)
    out = {}
    for fr in frames:
        res = {}
        for nb in (2, 3, 4):
            d, t = read_clusters(os.path.join(directory, "%s.all-%db-clusters.txt" % (fr, nb)), nb)
            counts, ns = calc.fp_histogram(nb, d, t, nbin=nbin) if len(t) else (np.zeros(nbin, np.int64), 0)
            write_hist(os.path.join(directory, "%s-%s.%db_clu-s.hist" % (fr, fr, nb)), nb, counts, ns)
            res[nb] = (counts, ns)
        out[fr] = res
    return out
