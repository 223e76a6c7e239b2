"""Cluster fingerprints (the reference's FINGERPRINT build and its histogram
tool), host side: the oracle's restatement reproduces the reference's own
expected histograms of its fingerprint example (read from the reference tree
at test time, when present); the oracle's histogram against an independent
numpy restatement; the file formats and the frame workflow of
chimes_calculator_gb300.fingerprint."""

import math
import os

import numpy as np
import pytest

from chimes_calculator_gb300 import fingerprint as fp
from chimes_calculator_gb300 import synth
from oracle.oracle import REFROOT

EX = os.path.join(REFROOT, "etc", "lmp", "tests", "example-fingerprint")


def read_lammps_data(path):
    """Atoms section of a LAMMPS data file (atomic style), by atom id."""
    lines = open(path).read().split("\n")
    start = [i for i, ln in enumerate(lines) if ln.strip().startswith("Atoms")][0]
    box = {}
    for ln in lines[:start]:
        t = ln.split()
        if len(t) >= 4 and t[2] in ("xlo", "ylo", "zlo"):
            box[t[2][0]] = float(t[1]) - float(t[0])
    atoms = []
    for ln in lines[start + 1:]:
        t = ln.split()
        if len(t) == 5:
            atoms.append((int(t[0]), int(t[1]), float(t[2]), float(t[3]), float(t[4])))
    atoms.sort()
    pos = np.array([[a[2], a[3], a[4]] for a in atoms])
    return pos, [a[1] for a in atoms], np.diag([box["x"], box["y"], box["z"]])


@pytest.mark.skipif(not os.path.isdir(EX), reason="reference tree not present")
def test_oracle_reproduces_reference_fingerprint_example(tmp_path):
    """The reference's LAMMPS fingerprint example (96-atom water, step 0,
    neighbour skin 1.0): the pair style's records -> the cluster files (6
    significant digits) -> the histogram tool's self-histograms, against its
    expected 0-0.{2,3,4}b_clu-s.hist at the printed precision."""
    from oracle.oracle import Oracle
    pos, ltype, cell = read_lammps_data(os.path.join(EX, "data.in"))
    o = Oracle(os.path.join(EX, "params.txt"))
    names = ["O", "H"]   # LAMMPS types 1, 2 (masses 15.999, 1.00784) in the parameter file's order
    cfg = synth.Config([names[t - 1] for t in ltype], pos, cell)
    ti = o.type_indices(cfg.types)
    nl = synth.lammps_neighbors(cfg, ti, o.max_cutoffs[0] + 1.0)
    o.lammps_fingerprint(True)
    o.lammps_compute(nl, 1.0, rebuild=True)
    for nb in (2, 3, 4):
        d, t = o.lammps_fp_records(nb)
        f = tmp_path / ("0.0.%db_clusters.txt" % nb)
        fp.write_clusters(str(f), d, t)
        d6, t6 = fp.read_clusters(str(f), nb)
        counts, ns = o.fp_histogram(nb, d6, t6)
        out = tmp_path / ("0-0.%db_clu-s.hist" % nb)
        fp.write_hist(str(out), nb, counts, ns)
        got = np.loadtxt(out)
        want = np.loadtxt(os.path.join(EX, "expected_output", "0-0.%db_clu-s.hist" % nb))
        assert got.shape == want.shape == (100, 2)
        assert np.abs(got - want).max() <= 1e-12, nb   # identical at the printed 6 digits
        assert ns > 5000


def test_oracle_histogram_against_numpy(tmp_path):
    """An independent restatement of the histogram (numpy: transform, sort,
    all pairs j > i, floor(dist / binw)) on seeded 2-body and 3-body records
    gives the oracle's counts."""
    from oracle.oracle import Oracle
    spec = synth.ParamSpec(elements=["C", "N"], orders=(8, 4, 0), rin=0.9, rout=(4.5, 5.2), lam=(1.3, 1.6),
                           fcut=("CUBIC",), s3max={0: [4.0, 4.0, 4.0], 1: [4.2, 3.8, 3.8], 2: [3.6, 3.9, 3.9],
                                                   3: [4.0, 4.0, 4.0]}, seed=4001)
    p = synth.write_param_file(str(tmp_path / "p.txt"), spec)
    o = Oracle(p)
    rng = np.random.default_rng(4002)
    # parameter tables the transform needs, read back from the file the way the reference builds them
    text = open(p).read().split("\n")
    rin, rout, lam = {}, {}, {}
    i0 = [k for k, ln in enumerate(text) if ln.startswith("# PAIRIDX #")][0]
    for ln in text[i0 + 1:i0 + 4]:
        t = ln.split()
        rin[int(t[0])], rout[int(t[0])], lam[int(t[0])] = float(t[3]), float(t[4]), float(t[7])
    pmap = {(0, 0): 0, (0, 1): 1, (1, 0): 1, (1, 1): 2}

    def tr(rc_in, rc_out, la, r):
        x_min, x_max = math.exp(-1 * rc_in / la), math.exp(-1 * rc_out / la)
        return (math.exp(-1 * r / la) - 0.5 * (x_max + x_min)) / (-(0.5 * (x_max - x_min)))

    # 2-body
    n = 400
    t2 = rng.integers(0, 2, size=(n, 2)).astype(np.int32)
    d2 = rng.uniform(0.95, 4.4, size=(n, 1))
    e = np.array([[tr(rin[pmap[tuple(t)]], rout[pmap[tuple(t)]], lam[pmap[tuple(t)]], r[0])] for r, t in zip(d2, t2)])
    counts, ns = o.fp_histogram(2, d2, t2)
    binw = 3.0 / 100
    iu = np.triu_indices(n, 1)
    dist = np.abs(e[:, None, 0] - e[None, :, 0])[iu]
    ref = np.bincount(np.floor(dist / binw).astype(int), minlength=100)
    assert ns == n * (n - 1) // 2 and np.array_equal(counts, ref)
    # 3-body, same-type clusters of type C C C (cutoffs of triplet type 0, all pairs C-C)
    n = 300
    t3 = np.zeros((n, 3), dtype=np.int32)
    d3 = rng.uniform(0.95, 3.95, size=(n, 3))
    e = np.sort(np.array([[tr(rin[0], 4.0, lam[0], r) for r in row] for row in d3]), axis=1)
    counts, ns = o.fp_histogram(3, d3, t3)
    binw = (math.sqrt(12.0) + 1.0) / 100
    dist = np.sqrt(((e[:, None, :] - e[None, :, :]) ** 2).sum(-1))[np.triu_indices(n, 1)]
    ref = np.bincount(np.floor(dist / binw).astype(int), minlength=100)
    assert ns == n * (n - 1) // 2 and np.array_equal(counts, ref)
    # two different sets: all n1 * n2 pairs
    c2, ns2 = o.fp_histogram(3, d3[:100], t3[:100], d3[100:], t3[100:])
    assert ns2 == 100 * 200 and c2.sum() == ns2
    # the tool's one-process rule: a first set of one record counts nothing
    c1, ns1 = o.fp_histogram(3, d3[:1], t3[:1], d3[1:], t3[1:])
    assert ns1 == 0 and not c1.any()


def test_file_formats_and_frame_workflow(tmp_path):
    d = np.array([[1.23456789], [2.0], [0.000123456789]])
    t = np.array([[0, 1], [1, 1], [0, 0]], dtype=np.int32)
    f = tmp_path / "x.txt"
    fp.write_clusters(str(f), d, t)
    assert f.read_text().split("\n")[:3] == ["1.23457 0 1", "2 1 1", "0.000123457 0 0"]
    d2, t2 = fp.read_clusters(str(f), 2)
    assert np.array_equal(t2, t) and np.allclose(d2, d, rtol=1e-5)
    with pytest.raises(ValueError):
        fp.read_clusters(str(f), 3)
    # per-rank files of two frames combine in rank order and are removed
    for step in (0, 2):
        for rank in (1, 0):
            for nb in (2, 3, 4):
                P = nb * (nb - 1) // 2
                fp.write_clusters(str(tmp_path / ("%d.%d.%db_clusters.txt" % (step, rank, nb))),
                                  np.full((1, P), 1.0 + rank), np.full((1, nb), rank))
    made = fp.combine_frames(str(tmp_path))
    assert len(made) == 6
    rows = (tmp_path / "2.all-3b-clusters.txt").read_text().split("\n")
    assert rows[0].startswith("1 1 1 0") and rows[1].startswith("2 2 2 1")
    assert not any(n.endswith("_clusters.txt") for n in os.listdir(tmp_path))
    h = tmp_path / "h.hist"
    fp.write_hist(str(h), 2, np.arange(100), 4950)
    first = h.read_text().split("\n")[1]
    assert first == "%g %g" % (1.5 * 0.03, 1 / 4950)
