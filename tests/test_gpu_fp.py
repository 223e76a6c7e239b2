"""Cluster fingerprints on the GPU (the reference's FINGERPRINT build and its
histogram tool): the pair-style records (ck_nl_fingerprint) equal the
oracle's restatement of pair_chimes.cpp's, in order; the all-pairs
histogram (ck_fp_histogram) gives the oracle's counts; the frame workflow
(record -> combine -> histogram files) end to end; a large histogram keeps
its pair count."""

import os

import numpy as np
import pytest

from chimes_calculator_gb300 import fingerprint as fp
from chimes_calculator_gb300 import synth

pytestmark = pytest.mark.gpu

SKIN = 1.0


@pytest.fixture(scope="module")
def system(tmp_path_factory):
    from oracle.oracle import Oracle
    d = tmp_path_factory.mktemp("fp")
    spec = synth.ParamSpec(elements=["C", "N"], orders=(10, 6, 4), rin=0.9, rout=4.6, lam=(1.3, 1.6),
                           fcut=("TERSOFF", 0.5), s3max=3.8, s4max=3.0, excluded3=(2,), seed=5001)
    p = synth.write_param_file(str(d / "p.txt"), spec)
    o = Oracle(p)
    cfg = synth.random_config(160, np.diag([11.5, 11.5, 11.5]), ["C", "N"], 1.0, seed=5002)
    ti = o.type_indices(cfg.types)
    nl = synth.lammps_neighbors(cfg, ti, max(o.max_cutoffs) + SKIN, seed=5003)
    o.lammps_fingerprint(True)
    o.lammps_compute(nl, SKIN, rebuild=True)
    return p, o, nl


def _calc(p, nl):
    from chimes_calculator_gb300 import Calculator
    c = Calculator()
    c.load_params(p)
    c.nl_compute(nl, SKIN, rebuild=True)
    return c


@pytest.mark.parametrize("nb", [2, 3, 4])
def test_records_match_oracle(native_lib, system, nb):
    p, o, nl = system
    c = _calc(p, nl)
    d, t = c.nl_fingerprint(nb)
    od, ot = o.lammps_fp_records(nb)
    assert len(t) == len(ot) > 50
    assert np.array_equal(t, ot)
    assert np.array_equal(d, od)   # same FP64 distances, same order


@pytest.mark.parametrize("nb", [2, 3, 4])
def test_histogram_matches_oracle(native_lib, system, nb):
    p, o, nl = system
    c = _calc(p, nl)
    d, t = c.nl_fingerprint(nb)
    counts, ns = c.fp_histogram(nb, d, t)
    oc, ons = o.fp_histogram(nb, d, t)
    assert ns == ons == len(t) * (len(t) - 1) // 2
    assert np.array_equal(counts, oc)
    # two sets, and a bin count other than the tool's 100
    h = len(t) // 3
    counts, ns = c.fp_histogram(nb, d[:h], t[:h], d[h:], t[h:], nbin=37)
    oc, ons = o.fp_histogram(nb, d[:h], t[:h], d[h:], t[h:], nbin=37)
    assert ns == ons == h * (len(t) - h) and np.array_equal(counts, oc)


def test_frame_workflow(native_lib, system, tmp_path):
    """record_step -> combine_frames -> histogram_frames writes the tool's
    files; the histograms equal the oracle's on the same (6-digit) files."""
    p, o, nl = system
    c = _calc(p, nl)
    fp.record_step(c, 0, rank=0, directory=str(tmp_path))
    moved = synth.NeighborData(**{**nl.__dict__, "x": nl.x + np.random.default_rng(1).uniform(-0.1, 0.1, nl.x.shape)})
    c.nl_compute(moved, SKIN, rebuild=False)
    fp.record_step(c, 2, rank=0, directory=str(tmp_path))
    fp.combine_frames(str(tmp_path))
    res = fp.histogram_frames(c, str(tmp_path))
    assert sorted(res) == ["0", "2"]
    for fr in ("0", "2"):
        for nb in (2, 3, 4):
            assert os.path.exists(tmp_path / ("%s-%s.%db_clu-s.hist" % (fr, fr, nb)))
            d, t = fp.read_clusters(str(tmp_path / ("%s.all-%db-clusters.txt" % (fr, nb))), nb)
            oc, ons = o.fp_histogram(nb, d, t)
            counts, ns = res[fr][nb]
            assert ns == ons and np.array_equal(counts, oc)


def test_large_histogram_pair_count(native_lib, tmp_path):
    """C2-size 3-body records (1024 atoms): every pair j > i is counted once."""
    from chimes_calculator_gb300 import Calculator
    p = synth.write_param_file(str(tmp_path / "c2.txt"), synth.spec_c2())
    cfg = synth.config_c2()
    c = Calculator()
    c.load_params(p)
    nl = synth.lammps_neighbors(cfg, c.type_indices(cfg.types), max(c.info(0)["max_cutoffs"]) + SKIN, seed=7)
    c.nl_compute(nl, SKIN, rebuild=True)
    d, t = c.nl_fingerprint(3)
    n = len(t)
    assert n > 20000
    counts, ns = c.fp_histogram(3, d, t)
    assert ns == n * (n - 1) // 2 == counts.sum()


def test_errors(native_lib, system):
    from chimes_calculator_gb300 import ChimesError
    p, o, nl = system
    c = _calc(p, nl)
    d, t = c.nl_fingerprint(3)
    bad = t.copy()
    bad[0] = [0, 1, 1]   # triplet type 2 (C N N) is excluded in this set
    with pytest.raises(ChimesError, match="excluded"):
        c.fp_histogram(3, d, bad)
    with pytest.raises(ChimesError, match="nbin"):
        c.fp_histogram(3, d, t, nbin=5000)
    counts, ns = c.fp_histogram(3, d[:1], t[:1], d, t)   # one record in the first set: nothing counted
    assert ns == 0 and not counts.any()
