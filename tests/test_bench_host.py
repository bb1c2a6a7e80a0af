"""Host logic of bench.py that needs no GPU: the solve kernel a solver
configuration names, and the DRAM-traffic figure taken from the ncu
capture of that same kernel only."""
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

import bench  # noqa: E402


def test_kernel_names_follow_the_solver_configuration():
    tagged = bench.solver_kernel_name({"mode": "gilu+tagged", "blocks": 152})
    assert tagged.startswith("kGiluBicgstab<float,3,tagged>") and "152 blocks" in tagged
    level = bench.solver_kernel_name({"mode": "gilu", "blocks": 8})
    assert level.startswith("kGiluBicgstab<float,3,level>")
    hybrid = bench.solver_kernel_name({"mode": "hybrid-256", "blocks": 112})
    assert hybrid.startswith("kBicgstab<float,3>") and "hybrid-256" in hybrid


def test_traffic_comes_from_a_capture_of_the_same_kernel():
    kst = {"solve_bytes": 2.0e11, "solve_launches": 2}
    tagged = bench.solver_kernel_name({"mode": "gilu+tagged", "blocks": 152})
    cluster = bench.solver_kernel_name({"mode": "cluster", "blocks": 16})
    t, kind = bench.solver_traffic("blackoil-100x100x100", kst, tagged)
    assert t is not None and kind and abs(t / 1.0e11 - 1.108) < 0.01
    assert bench.solver_traffic("blackoil-100x100x100", kst, cluster) == (None, None)
    t2, _ = bench.solver_traffic("blackoil-100x100x20", kst, cluster)
    assert t2 is not None and abs(t2 / 1.0e11 - 0.354) < 0.01
    assert bench.solver_traffic("no-such-workload", kst, tagged) == (None, None)
