"""The C ABI from C: tests/c/abi_host.c (C99, -Wall -Werror) includes
include/gbfv.h, links the in-tree libgbfv.so and runs the entry points that
need no device.  Checks that the header is plain C and the exports are
usable without Python."""
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
