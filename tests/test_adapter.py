"""The reference-side adapter (include/gbfv_opm.hh) compiled and run.

tests/c/adapter_lens.cc instantiates the adapter's linearizer, backend,
Newton method and boundary recorder in the lens problem's type tag, on a test
shim of the reference's types (tests/c/opm_shim.hh: property lookup, ECFV
stencil, NewtonMethod::apply and its hooks, the model's solution history,
FvBaseProblem::timeIntegration and the Simulator time loop, restated).

CPU: the program compiles against the shim, and the gbfv_problem the adapter
builds from the problem's callbacks (gbfvDescribe) equals the lens
description the parity tests use (problems.lens), array by array.
GPU: 30 lens time steps through the reference's loops and the adapter give
exactly gbfv_time_integration's dt sequence, Newton counts and final bits;
with a NaN injected into the host solution before one time step, the first
attempt fails, the model resets to the old time level, the retry with dt/2
succeeds, and the run equals the device path with the same failure; the
Jacobian and residual are never copied to the host, and the host solution is
written once per converged step."""
import os
import struct
import subprocess

import numpy as np
import pytest

from gbfv import Context, capi, problems

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "c", "adapter_lens.cc")
LIBDIR = os.path.join(ROOT, "opm-models_gb300", "_build")


def _build(tmp_path):
    exe = str(tmp_path / "adapter_lens")
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-Wextra", "-Werror", "-ffp-contract=off",
           "-I" + os.path.join(ROOT, "include"), "-I" + os.path.join(ROOT, "tests", "c", "shim_include"),
           "-o", exe, SRC, "-L" + LIBDIR, "-lgbfv",
           "-Wl,-rpath," + LIBDIR]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def _records(path, kinds):
    out = []
    with open(path, "rb") as f:
        for k in kinds:
            (n,) = struct.unpack("<q", f.read(8))
            dt = {"d": np.float64, "i": np.int32, "q": np.int64}[k]
            out.append(np.frombuffer(f.read(n * np.dtype(dt).itemsize), dt).copy())
    return out


def test_adapter_describes_the_lens_as_the_parity_tests_do(built, tmp_path):
    exe = _build(tmp_path)
    out = str(tmp_path / "desc.bin")
    r = subprocess.run([exe, "describe", out], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    kinds = "dddd" "i" "d" "iii" "ddd" "i" "ddd" "i" "d" "d"
    (center, volume, poro, perm, mat, matp, cptr, cnbr, cdir, cnorm, ccent, carea, bptr, bnorm, bcent, barea,
     btype, bval, scal) = _records(out, kinds)
    p = problems.lens(48, 32)
    assert np.array_equal(center, p.center)
    assert np.array_equal(volume, p.volume)
    assert np.array_equal(poro, p.porosity)
    # the reference's DimMatrix is 2 x 2 in 2D: the third diagonal entry is unused
    # (the Python builder repeats K there, the adapter leaves 0)
    assert np.array_equal(perm.reshape(-1, 3)[:, :2], p.perm.reshape(-1, 3)[:, :2])
    assert np.array_equal(mat, p.material)
    assert np.array_equal(matp, p.material_params)
    assert np.array_equal(cptr, p.conn_ptr) and np.array_equal(cnbr, p.conn_nbr) and np.array_equal(cdir, p.conn_dir)
    assert np.array_equal(cnorm, p.conn_normal) and np.array_equal(ccent, p.conn_center)
    assert np.array_equal(carea, p.conn_area)
    assert np.array_equal(bptr, p.bface_ptr) and np.array_equal(bnorm, p.bface_normal)
    assert np.array_equal(bcent, p.bface_center) and np.array_equal(barea, p.bface_area)
    assert np.array_equal(btype, p.bface_type) and np.array_equal(bval, p.bface_value)
    assert np.array_equal(scal, np.array(list(p.gravity) + list(p.rho) + list(p.mu) + [p.temperature]))


def _device_path(steps, nan_step):
    """The same run on the device path: gbfv_time_integration, and at the
    failing step the failed attempt and the dt/2 retry issued through the C
    ABI as the time loop does."""
    prob = problems.lens(48, 32)
    prm = capi.default_params(linear_tolerance=1e-6)
    ctx = Context(prob, prm)
    if nan_step < 0:
        st, sdt, sn, _, _ = ctx.time_integration(steps, 250.0)
        assert st == 0
        x, _ = ctx.solution()
        ctx.close()
        return sdt, sn, x, 0
    dts, its = [], []
    st, sdt, sn, _, _ = ctx.time_integration(nan_step, 250.0)
    assert st == 0
    dts += list(sdt)
    its += list(sn)
    dt = ctx.lib.gbfv_suggest_time_step(ctx.h, float(sdt[-1]), int(sn[-1])) if nan_step > 0 else 250.0
    x, m = ctx.solution()
    bad = x.copy()
    bad[(prob.num_cells // 2) * 2] = np.nan
    ctx.set_solution(bad, m)
    st, rep = ctx.newton_apply(dt)
    assert st != 0 and not rep.converged
    ctx.set_solution(x, m)  # updateFailed: solution(0) = solution(1)
    dt /= 2.0
    st, rep = ctx.newton_apply(dt)
    assert st == 0
    dts.append(dt)
    its.append(rep.iterations)
    dt = ctx.lib.gbfv_suggest_time_step(ctx.h, dt, rep.iterations)
    st, sdt, sn, _, _ = ctx.time_integration(steps - nan_step - 1, dt)
    assert st == 0
    dts += list(sdt)
    its += list(sn)
    x, _ = ctx.solution()
    ctx.close()
    return np.array(dts), np.array(its), x, 1


@pytest.mark.gpu
@pytest.mark.parametrize("nan_step", [-1, 7])
def test_lens_through_the_adapter_equals_the_device_path(built, tmp_path, nan_step):
    exe = _build(tmp_path)
    out = str(tmp_path / "run.bin")
    steps = 30
    r = subprocess.run([exe, "run", str(steps), str(nan_step), out], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    dts, its, x, counts = _records(out, "didq")
    failures, linearizations, res_syncs, jac_syncs, host_syncs, lin_total = counts.tolist()
    ref_dt, ref_its, ref_x, ref_failures = _device_path(steps, nan_step)
    assert failures == ref_failures
    assert np.array_equal(dts, ref_dt), (dts, ref_dt)
    assert np.array_equal(its, ref_its), (its, ref_its)
    assert np.array_equal(x, ref_x)
    assert jac_syncs == 0 and res_syncs == 0
    assert host_syncs == steps
    assert linearizations >= int(its.sum()) and lin_total > 0


def test_tpfa_adapter_compiles_and_refuses_on_the_host(built, tmp_path):
    """GbfvTpfaLinearizer (the TPFA type tag's Linearizer) is instantiated
    in full against the shim; on the host it refuses a non-black-oil model
    and a pressure or sequential-transport linearization type, keeps the
    implicit one, and has empty flows / flores / velocity records and
    constraints, as TpfaLinearizer without FLOWS, FLORES or DISPERC."""
    exe = _build(tmp_path)
    r = subprocess.run([exe, "tpfa"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "tpfa refused 2 kept 1 empty 1" in r.stdout
