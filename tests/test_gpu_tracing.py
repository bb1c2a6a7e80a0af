"""Per-solve records (GBFV_SOLVE_LOG): with the variable set when a context
is created, every linear solve appends one JSON line -- iterations,
refinements, the residual reduction it reached (for the mixed form the FP64
true residual's), device time and algorithmic bytes of its solver launches
-- and the lines add up to the context's kernel statistics."""
import json

import pytest

from gbfv import Context, capi, problems

pytestmark = pytest.mark.gpu


def test_solve_log_lines(built, tmp_path, monkeypatch):
    path = tmp_path / "solves.jsonl"
    monkeypatch.setenv("GBFV_SOLVE_LOG", str(path))
    prm = capi.default_params(linear_tolerance=1e-6, newton_tolerance=1e-6, precision=capi.PREC_MIXED,
                              inner_tolerance=1e-6)
    ctx = Context(problems.blackoil(16, 12, 5), prm)
    ctx.reset_kernel_stats()
    st, _, nits, lits, _ = ctx.time_integration(2, 86400.0, fixed_dt=True)
    assert st == 0
    ks = ctx.kernel_stats()
    ctx.close()
    recs = [json.loads(line) for line in path.read_text().splitlines()]
    # one solve per Newton iteration that did not stop at its error check
    assert 0 < len(recs) <= int(nits.sum())
    assert all(r["status"] == 0 and r["precision"] == "mixed" and r["cells"] == 16 * 12 * 5 for r in recs)
    assert sum(r["iterations"] for r in recs) == int(lits.sum())
    assert abs(sum(r["solve_ms"] for r in recs) - ks["solve_ms"]) <= 1e-6 * max(1.0, ks["solve_ms"])
    assert abs(sum(r["bytes"] for r in recs) - ks["solve_bytes"]) <= 1e-6 * ks["solve_bytes"]
    # every mixed solve met the tolerance on its FP64 true residual: the
    # relative reduction 1e-6 or the absolute bar (Newton tolerance / 100)
    assert all(r["residual_reduction"] <= 1e-6 * (1 + 1e-9) or r["residual"] <= 1e-8 * (1 + 1e-9) for r in recs), \
        [(r["residual_reduction"], r["residual"]) for r in recs]
