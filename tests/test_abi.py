"""The C-ABI library loads without a GPU and exports every entry point that
include/*.h declares; the C++ drop-in headers compile and link against it."""

import ctypes
import glob
import os
import re
import subprocess

import pytest

from conftest import REPO

INCLUDE = os.path.join(REPO, "include")


def declared_c_functions():
    names = set()
    for h in glob.glob(os.path.join(INCLUDE, "*.h")):
        src = open(h).read()
        if "extern \"C\"" not in src:
            continue
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b([a-z_][a-z0-9_]*)\s*\(", src, flags=re.M):
            names.add(m.group(1))
    names.discard("defined")
    return sorted(names)


def test_headers_declare_the_reference_symbols():
    names = declared_c_functions()
    for ref in ["calculate_chimes", "calculate_chimes_instance", "set_chimes_serial", "init_chimes_serial",
                "chimes_open_instance", "chimes_close_instance", "set_chimes_serial_instance",
                "init_chimes_serial_instance", "chimes_compute_2b_props", "chimes_compute_3b_props",
                "chimes_compute_4b_props", "chimes_read_params", "set_chimes", "init_chimes"]:
        assert ref in names


def test_library_exports_every_declared_symbol(native_lib):
    missing = [n for n in declared_c_functions() if not hasattr(native_lib, n)]
    assert not missing, missing


def test_python_signature_table_covers_headers():
    from chimes_calculator_gb300 import _lib
    missing = [n for n in declared_c_functions() if n not in _lib.SIGNATURES]
    assert not missing, missing


def test_error_mode_returns_status_without_gpu(native_lib):
    native_lib.ck_set_error_mode(1)
    rc = native_lib.ck_check_params(b"/nonexistent/params.txt", None, None, None)
    assert rc == -1
    assert b"cannot open parameter file" in native_lib.ck_last_error()


def test_cpp_dropin_headers_link(native_lib, tmp_path):
    """Code written against the reference's C++ classes compiles and links."""
    src = tmp_path / "main.cpp"
    src.write_text(r'''
#include <string>
#include <vector>
#include "serial_chimes_interface.h"
#include "chimescalc_serial_C.h"
#include "chimescalc_C.h"
#include "chimes_gb300.h"
int main(int argc, char** argv) {
    if (argc < 3) return 0;   // link check only: running needs a GPU
    serial_chimes_interface chimes(false);
    chimes.init_chimesFF(argv[1], 0);
    std::vector<double> x(1), y(1), z(1), a{10,0,0}, b{0,10,0}, c{0,0,10}, stress(9);
    std::vector<std::string> types{"C"};
    std::vector<std::vector<double>> force(1, std::vector<double>(3));
    double e = 0;
    chimes.calculate(x, y, z, a, b, c, types, e, force, stress);
    chimesFF ff;
    chimes2BTmp t2(12);
    std::vector<double> dr{1, 0, 0}, f(6), s(6);
    ff.compute_2B(1.0, dr, {0, 0}, f, s, e, t2);
    return 0;
}
''')
    exe = tmp_path / "a.out"
    lib_dir = os.path.dirname(native_lib._name)
    subprocess.run(["g++", "-std=c++11", "-I", INCLUDE, str(src), "-o", str(exe), "-L", lib_dir, "-lchimescalc",
                    "-Wl,-rpath," + lib_dir], check=True)
    subprocess.run([str(exe)], check=True)
