"""Parameter-file parsing in the product (host only, no GPU): the formats the
reference reads, and the errors it reports (the reference prints and calls
exit(0); the library returns a status in error mode 1)."""

import ctypes
import os

import pytest

from chimes_calculator_gb300 import synth
from oracle.oracle import REFROOT

REFFF = os.path.join(REFROOT, "serial_interface", "tests", "force_fields")


def check(lib, path):
    orders = (ctypes.c_int * 3)()
    nt = ctypes.c_int()
    cuts = (ctypes.c_double * 3)()
    rc = lib.ck_check_params(str(path).encode(), orders, ctypes.byref(nt), cuts)
    return rc, tuple(orders), nt.value, tuple(cuts), lib.ck_last_error().decode()


@pytest.fixture
def lib(native_lib):
    native_lib.ck_set_error_mode(1)
    return native_lib


def test_golden_parameter_files_parse(lib, golden):
    from oracle.oracle import Oracle
    for g in golden.values():
        rc, orders, nt, cuts, _ = check(lib, g.params)
        assert rc == 0, g.name
        o = Oracle(g.params)
        assert orders == o.orders and nt == o.ntypes
        assert cuts == pytest.approx(o.max_cutoffs, abs=0)


@pytest.mark.skipif(not os.path.isdir(REFFF), reason="reference tree not present")
def test_reference_parameter_files_parse(lib):
    from oracle.oracle import Oracle
    n = 0
    for f in sorted(os.listdir(REFFF)):
        rc, orders, nt, cuts, err = check(lib, os.path.join(REFFF, f))
        try:
            o = Oracle(os.path.join(REFFF, f))
        except ValueError:
            continue
        assert rc == 0, (f, err)
        assert orders == o.orders and cuts == pytest.approx(o.max_cutoffs, abs=0), f
        n += 1
    assert n >= 10


def _write(tmp_path, text, name="p.txt"):
    p = tmp_path / name
    p.write_text(text)
    return p


def base_text():
    return synth.build_param_text(synth.ParamSpec(elements=["C", "N"], orders=(8, 4, 3), s3max=3.5, s4max=3.0,
                                                  seed=7))


@pytest.mark.parametrize("mutate,msg", [
    (lambda t: t.replace("PAIRTYP: CHEBYSHEV", "PAIRTYP: POLYNOMIAL"), "PAIRTYP"),
    (lambda t: t.replace("FCUT TYPE: TERSOFF", "FCUT TYPE: GAUSSIAN"), "unknown FCUT TYPE"),
    (lambda t: t.replace("MORSE", "INVRSE"), "MORSE"),
    (lambda t: t.split("PAIRMAPS:")[0] + "ENDFILE\n", "PAIRMAPS"),
    (lambda t: t.replace("ENDFILE\n", ""), "ENDFILE"),
    (lambda t: t.replace("\n0 ", "\n15 ", 1), "power"),
])
def test_parser_errors(lib, tmp_path, mutate, msg):
    p = _write(tmp_path, mutate(base_text()))
    rc, _, _, _, err = check(lib, p)
    assert rc == -1
    assert msg.lower() in err.lower()


def test_missing_file(lib, tmp_path):
    rc, _, _, _, err = check(lib, tmp_path / "absent.txt")
    assert rc == -1 and "cannot open" in err


def test_seven_column_pair_lines(lib, tmp_path):
    """Version-2 pair lines without S_DELTA (chimesFF.cpp:517-537) parse the same."""
    t = base_text()
    lines = t.splitlines()
    out = []
    in_pairs = False
    for ln in lines:
        if "# PAIRIDX #" in ln:
            in_pairs = True
            out.append(ln)
            continue
        if in_pairs and ln.strip() and ln.split()[0].isdigit() and len(ln.split()) == 8:
            w = ln.split()
            del w[5]
            out.append("\t".join(w))
            continue
        if in_pairs and not ln.strip():
            in_pairs = False
        out.append(ln)
    p7 = _write(tmp_path, "\n".join(out) + "\n", "p7.txt")
    p8 = _write(tmp_path, t, "p8.txt")
    a = check(lib, p7)
    b = check(lib, p8)
    assert a[0] == 0 and a[1:4] == b[1:4]


@pytest.fixture(scope="module")
def factored_check(tmp_path_factory):
    """tests/factored_check.cpp built against the product's parameter packer."""
    import subprocess
    here = os.path.dirname(os.path.abspath(__file__))
    csrc = os.path.join(os.path.dirname(here), "chimes_calculator_gb300", "csrc")
    exe = str(tmp_path_factory.mktemp("fc") / "factored_check")
    subprocess.run(["g++", "-O1", "-std=c++17", "-ffp-contract=off", "-I" + csrc,
                    os.path.join(here, "factored_check.cpp"), os.path.join(csrc, "ck_params.cpp"), "-o", exe],
                   check=True)
    return exe


def test_factored_tables_reproduce_the_coefficient_sums(factored_check, golden, tmp_path):
    """Per tuple of every parameter file: the factored lists and the tensor-core
    images (3-body and 4-body) give the per-coefficient sums."""
    import subprocess
    paths = [g.params for g in golden.values()]
    for k, spec in enumerate([synth.spec_c3(), synth.spec_c4()] + list(synth.specs_c5())):
        paths.append(synth.write_param_file(str(tmp_path / ("s%d.txt" % k)), spec))
    if os.path.isdir(REFFF):
        paths += [os.path.join(REFFF, f) for f in sorted(os.listdir(REFFF)) if f.endswith(".txt")]
    for p in paths:
        out = subprocess.run([factored_check, str(p)], capture_output=True, text=True)
        assert out.returncode == 0 and out.stdout.startswith("ok"), (p, out.stdout)


def test_parameter_cache_round_trip(lib, factored_check, golden, tmp_path):
    """A binary cache parses to the same tables (same device image) as its text file."""
    import subprocess
    paths = [g.params for g in golden.values()]
    if os.path.isdir(REFFF):
        paths += [os.path.join(REFFF, f) for f in sorted(os.listdir(REFFF)) if f.endswith(".txt")]
    for k, p in enumerate(paths):
        cache = str(tmp_path / ("c%d.ckpc" % k))
        assert lib.ck_convert_params(str(p).encode(), cache.encode()) == 0, lib.ck_last_error()
        a, b = check(lib, p), check(lib, cache)
        assert a[:4] == b[:4] and a[0] == 0
        out = subprocess.run([factored_check, str(p), cache], capture_output=True, text=True)
        assert out.returncode == 0 and out.stdout.startswith("ok"), (p, out.stdout)


def test_parameter_cache_rejects_corruption(lib, golden, tmp_path):
    g = golden["c2"]
    cache = tmp_path / "c2.ckpc"
    assert lib.ck_convert_params(str(g.params).encode(), str(cache).encode()) == 0
    data = cache.read_bytes()
    for cut in (6, len(data) // 2, len(data) - 3):
        bad = tmp_path / ("cut%d.ckpc" % cut)
        bad.write_bytes(data[:cut])
        rc, *_, msg = check(lib, bad)
        assert rc == -1 and "cache" in msg
