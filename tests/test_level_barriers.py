"""The push sweeps' level-barrier placement (host code of the library,
gbfv_selftest_level_barriers) checked by an independent model of what the
kernel guarantees.  A block finishes its levels in order (a block barrier
per level); a row starts after its block finished the previous level and
after the rows it depends on were computed (their values arrive by push);
a cluster barrier after a level makes every block know that every block
finished it.  A row of level l pushes into its consumers' dependency buffer
(l+1) mod D, which the consumer last read at level l+1-D: the push is safe
only if the producer then knows the consumer block finished that level.
Every push of every level is checked on structured 2D and 3D patterns, for
several cluster sizes, both ownership modes and both sweep directions."""
import ctypes as ct

import numpy as np
import pytest

from gbfv import capi


def _pattern(shape):
    """rows in level order (level = i+j(+k), then natural order), slots
    [lower (dim), self, upper (dim)] as level-order indices"""
    dim = len(shape)
    nat = np.arange(int(np.prod(shape))).reshape(shape[::-1]).T  # nat[i, j(, k)], x fastest
    idx = np.array(np.unravel_index(np.arange(nat.size), shape, order="F")).T  # natural -> (i, j, k)
    lev = idx.sum(axis=1)
    order = np.lexsort((np.arange(nat.size), lev))
    pos = np.empty_like(order)
    pos[order] = np.arange(nat.size)
    n = nat.size
    col = -np.ones((2 * dim + 1, n), np.int32)
    for r, I in enumerate(order):
        c = idx[I]
        col[dim, r] = r
        for a in range(dim):
            lo = c.copy()
            lo[a] -= 1
            hi = c.copy()
            hi[a] += 1
            if lo[a] >= 0:
                col[dim - 1 - a, r] = pos[np.ravel_multi_index(lo, shape, order="F")]
            if hi[a] < shape[a]:
                col[dim + 1 + a, r] = pos[np.ravel_multi_index(hi, shape, order="F")]
    nl = int(lev.max()) + 1
    lev_ptr = np.zeros(nl + 1, np.int32)
    np.add.at(lev_ptr, lev + 1, 1)
    return dim, np.cumsum(lev_ptr).astype(np.int32), col, n


def _owner(t, width, C, mode):
    if mode == 0:
        return (t >> 5) % C
    chunk = (((width + C - 1) // C) + 31) & ~31
    return t // chunk


def _check(dim, lev_ptr, col, n, C, mode, D, forward, barrier):
    nl = len(lev_ptr) - 1
    lev = np.repeat(np.arange(nl), np.diff(lev_ptr))
    own = np.array([_owner(p - lev_ptr[lev[p]], lev_ptr[lev[p] + 1] - lev_ptr[lev[p]], C, mode) for p in range(n)])
    fin = -np.ones((C, C), int)          # fin[X]: what block X knows finished, after its last level
    clock = -np.ones((n, C), int)        # what a row's block knows when the row starts
    deps = range(dim) if forward else [2 * dim - q for q in range(dim)]
    cons = [dim + 1 + q for q in range(dim)] if forward else list(range(dim))
    for step in range(nl):
        l = step if forward else nl - 1 - step
        new = fin.copy()
        for p in range(lev_ptr[l], lev_ptr[l + 1]):
            X = own[p]
            c = fin[X].copy()
            for s in deps:
                j = col[s, p]
                if j >= 0:
                    c = np.maximum(c, clock[j])
            for s in cons:
                u = col[s, p]
                if u >= 0:
                    assert c[own[u]] >= step + 1 - D, ("unsafe push", forward, l, p, own[u])
            clock[p] = c
            new[X] = np.maximum(new[X], c)
        for X in range(C):
            new[X, X] = step
        if barrier[l]:
            new[:, :] = np.maximum(new, step)
        fin = new


@pytest.mark.parametrize("shape", [(12, 9), (40, 3), (9, 7, 4), (6, 6, 6), (20, 5, 3)])
@pytest.mark.parametrize("C", [2, 4, 8, 16])
@pytest.mark.parametrize("mode", [0, 1])
def test_every_push_is_covered(shape, C, mode):
    f = capi.load().gbfv_selftest_level_barriers
    f.restype = ct.c_int
    dim, lev_ptr, col, n = _pattern(shape)
    nl = len(lev_ptr) - 1
    colf = np.ascontiguousarray(col.ravel(), np.int32)
    for forward in (1, 0):
        bar = np.zeros(nl, np.int8)
        st = f(n, dim, lev_ptr.ctypes.data_as(ct.c_void_p), nl, colf.ctypes.data_as(ct.c_void_p), C, mode, 4,
               forward, bar.ctypes.data_as(ct.c_void_p))
        assert st == 0
        _check(dim, lev_ptr, col, n, C, mode, 4, forward == 1, bar)
        if bar.any():
            # the barriers are needed: up to the first one the knowledge is the
            # same with and without, so without any the model finds an unsafe push
            with pytest.raises(AssertionError):
                _check(dim, lev_ptr, col, n, C, mode, 4, forward == 1, np.zeros(nl, np.int8))


def test_wide_levels_need_barriers():
    """On a pattern whose levels span several blocks the placement is not
    empty (so the check above exercises the model's strict side)."""
    f = capi.load().gbfv_selftest_level_barriers
    f.restype = ct.c_int
    dim, lev_ptr, col, n = _pattern((40, 30, 4))
    nl = len(lev_ptr) - 1
    bar = np.zeros(nl, np.int8)
    colf = np.ascontiguousarray(col.ravel(), np.int32)
    assert f(n, dim, lev_ptr.ctypes.data_as(ct.c_void_p), nl, colf.ctypes.data_as(ct.c_void_p), 16, 0, 4, 1,
             bar.ctypes.data_as(ct.c_void_p)) == 0
    assert 0 < bar.sum() < nl
    _check(dim, lev_ptr, col, n, 16, 0, 4, True, bar)
