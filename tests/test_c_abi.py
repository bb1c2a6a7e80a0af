"""The C ABI from C: tests/c/abi_host.c (C99, -Wall -Werror) includes
include/gbfv.h, links the in-tree libgbfv.so and runs the entry points that
need no device.  Checks that the header is plain C and the exports are
usable without Python; tests/c/abi_cxx_a.cc and abi_cxx_b.cc do the same
from two C++17 units of one program."""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def test_c99_consumer_compiles_links_and_runs(built, tmp_path):
    libdir = os.path.join(ROOT, "opm-models_gb300", "_build")
    exe = str(tmp_path / "abi_host")
    cc = subprocess.run(["gcc", "-std=c99", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"),
                         os.path.join(HERE, "c", "abi_host.c"), "-L", libdir, "-lgbfv", "-Wl,-rpath," + libdir,
                         "-o", exe], capture_output=True, text=True)
    assert cc.returncode == 0, cc.stderr
    run = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert run.returncode == 0 and run.stdout.startswith("abi ok"), (run.returncode, run.stdout, run.stderr)


def test_two_cxx_translation_units_link_and_run(built, tmp_path):
    """The header from C++ in two units of one program (the reference's
    multi-compile-unit check, tests/lens_immiscible_ecfv_ad_cu1.cc, _cu2.cc,
    _main.cc): compiles with -Wall -Werror, links, and rejects an
    inconsistent problem without a device."""
    libdir = os.path.join(ROOT, "opm-models_gb300", "_build")
    exe = str(tmp_path / "abi_cxx")
    cc = subprocess.run(["g++", "-std=c++17", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"),
                         os.path.join(HERE, "c", "abi_cxx_a.cc"), os.path.join(HERE, "c", "abi_cxx_b.cc"),
                         "-L", libdir, "-lgbfv", "-Wl,-rpath," + libdir, "-o", exe], capture_output=True, text=True)
    assert cc.returncode == 0, cc.stderr
    run = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert run.returncode == 0 and run.stdout.startswith("abi c++ ok"), (run.returncode, run.stdout, run.stderr)
    assert "conn_ptr" in run.stdout
