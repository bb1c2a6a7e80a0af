"""Host sanitizers on the CPU restatement: the oracle built with
AddressSanitizer and UndefinedBehaviorSanitizer (the Makefile's `sanitize`
target, serial) runs a lens and a black-oil time integration, both local
linearizers and the stand-alone linear solver in a child process that
preloads the sanitizer runtimes; the library's restart-file unit, built on
the host with both sanitizers, parses some 40 000 mutated files (every
prefix, byte edits, cut and repeated chunks, NaN / huge / fractional numbers
in every field) handed over in buffers of exactly their length.  Any report
fails the test."""
import os
import subprocess
import sys

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)

SCRIPT = r"""
import sys
sys.path[:0] = [%(pkg)r, %(orc)r, %(root)r]
import numpy as np
import oracle as O
from gbfv import capi, problems
for lin in (capi.LIN_AD, capi.LIN_FD):
    o = O.Oracle(problems.lens(nx=12, ny=8), capi.default_params(linear_tolerance=1e-6, local_linearizer=lin))
    assert o.time_integration(3, 250.0)[0] == 0
    o = O.Oracle(problems.blackoil(6, 5, 3), capi.default_params(linear_tolerance=1e-6, newton_tolerance=1e-6,
                                                                local_linearizer=lin))
    assert o.time_integration(2, 86400.0, fixed_dt=True)[0] == 0
o.linearize(86400.0, 0)
rp, col, blk = o.jacobian()
st, x, it = O.bcrs_solve(rp, col, blk, o.residual(), capi.default_params(linear_tolerance=1e-8))
assert st == 0
print("sanitized run ok")
"""


def _runtime(name):
    out = subprocess.run(["g++", "-print-file-name=" + name], capture_output=True, text=True)
    path = out.stdout.strip()
    return path if out.returncode == 0 and os.path.isabs(path) and os.path.exists(path) else None


def test_oracle_under_address_and_undefined_behaviour_sanitizers():
    asan, ubsan = _runtime("libasan.so"), _runtime("libubsan.so")
    if not asan or not ubsan:
        pytest.skip("no sanitizer runtimes for this compiler")
    mk = subprocess.run(["make", "-C", os.path.join(ROOT, "oracle"), "sanitize"], capture_output=True, text=True)
    assert mk.returncode == 0, mk.stdout + mk.stderr
    env = dict(os.environ)
    env.update(LD_PRELOAD=asan + ":" + ubsan, ASAN_OPTIONS="detect_leaks=0:abort_on_error=1",
               UBSAN_OPTIONS="print_stacktrace=1:halt_on_error=1",
               GBFV_ORACLE_LIB=os.path.join(ROOT, "oracle", "_build", "liboracle_san.so"))
    code = SCRIPT % dict(pkg=os.path.join(ROOT, "opm-models_gb300"), orc=os.path.join(ROOT, "oracle"), root=ROOT)
    r = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True, timeout=600)
    report = r.stdout + r.stderr
    assert r.returncode == 0 and "sanitized run ok" in r.stdout, report[-4000:]
    assert "AddressSanitizer" not in report and "runtime error" not in report, report[-4000:]


def test_restart_parser_mutation_sweep_under_sanitizers(tmp_path):
    if not _runtime("libasan.so") or not _runtime("libubsan.so"):
        pytest.skip("no sanitizer runtimes for this compiler")
    exe = str(tmp_path / "restart_fuzz")
    cc = subprocess.run(["g++", "-std=c++17", "-O1", "-g", "-fsanitize=address,undefined",
                         "-fno-sanitize-recover=undefined", "-fno-omit-frame-pointer",
                         "-I" + os.path.join(ROOT, "include"),
                         "-x", "c++", os.path.join(ROOT, "opm-models_gb300", "csrc", "restart.cu"),
                         "-x", "none", os.path.join(HERE, "c", "restart_fuzz.cc"), "-o", exe, "-lpthread"],
                        capture_output=True, text=True)
    assert cc.returncode == 0, cc.stderr[-4000:]
    env = dict(os.environ, ASAN_OPTIONS="detect_leaks=1:abort_on_error=1",
               UBSAN_OPTIONS="print_stacktrace=1:halt_on_error=1")
    r = subprocess.run([exe], env=env, capture_output=True, text=True, timeout=300)
    report = r.stdout + r.stderr
    assert r.returncode == 0 and "unexpected 0" in r.stdout, report[-4000:]
    assert "AddressSanitizer" not in report and "runtime error" not in report, report[-4000:]
