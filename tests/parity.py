"""Parity metrics shared by the GPU tests.

Residuals are sums of terms that cancel (fluxes against storage); a
difference is judged against the size of the summed terms (the oracle's
per-row sum of |terms| / V), which is what "1e-12 relative" means for a
floating-point sum.  Jacobian entries are judged per (row equation, primary
variable) against the largest magnitude of that entry across the row's
blocks, since primary variables carry very different units.
"""
import numpy as np

RTOL_LIN = 1e-12


def residual_mismatch(r_gpu, r_ref, scale):
    s = np.maximum(scale, np.finfo(float).tiny)
    return float(np.max(np.abs(r_gpu - r_ref) / s)) if len(s) else 0.0


def jacobian_mismatch(rp, col, blk_gpu, blk_ref):
    """max over entries of |a-b| / (max |b| of that (eq, pv) in the row)."""
    n = len(rp) - 1
    worst = 0.0
    for i in range(n):
        sl = slice(rp[i], rp[i + 1])
        ref = blk_ref[sl]
        scale = np.max(np.abs(ref), axis=0)  # b x b over the row's blocks
        scale = np.maximum(scale, np.finfo(float).tiny)
        d = np.abs(blk_gpu[sl] - ref) / scale
        worst = max(worst, float(d.max()))
    return worst


def jacobian_mismatch_fast(rp, col, blk_gpu, blk_ref):
    n = len(rp) - 1
    rows = np.repeat(np.arange(n), np.diff(rp))
    b = blk_ref.shape[1]
    absref = np.abs(blk_ref).reshape(len(rows), b * b)
    scale = np.zeros((n, b * b))
    np.maximum.at(scale, rows, absref)
    scale = np.maximum(scale[rows], np.finfo(float).tiny)
    d = np.abs(blk_gpu - blk_ref).reshape(len(rows), b * b) / scale
    return float(d.max()) if len(d) else 0.0


def rel_state_diff(a, b, bs):
    """max relative difference per primary variable column (pressure-like
    columns relative to their magnitude, saturation-like absolute)."""
    a = a.reshape(-1, bs)
    b = b.reshape(-1, bs)
    out = []
    for k in range(bs):
        scale = max(np.max(np.abs(b[:, k])), 1.0)
        out.append(float(np.max(np.abs(a[:, k] - b[:, k])) / scale))
    return max(out)
