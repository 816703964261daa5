"""bench.py helpers that run without a GPU: the CPU baseline legs (the
reference's own parallelism, one thread, and the port over every core) and
the velocity-error measure used for the 16-bit batch and serving results."""
import os
import sys
import types

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def test_cpu_baseline_reports_one_core_and_all_cores():
    import bench

    a = types.SimpleNamespace(storage="f32", size=24, nu=0.0192, lid=0.05, cpu_seconds=0.3)
    cpu = bench.cpu_baseline(a)
    assert cpu["cores"] == 1 and cpu["value"] > 0 and cpu["unit"] == "MLUPS"
    assert cpu["kind"] in ("reference", "port")
    assert cpu["nproc"] == os.cpu_count()
    allc = cpu["all_cores"]
    assert allc["kind"] == "port" and allc["cores"] >= 1 and allc["value"] > 0
    assert "1 core used" in cpu["sample"]


def test_velocity_error_is_relative_l2_over_all_fields():
    import bench

    ref = [np.ones((3, 2, 2, 2)), 2 * np.ones((3, 1, 1, 1))]
    got = [r.copy() for r in ref]
    assert bench.velocity_error(got, ref) == (0.0, 0.0)
    got[1][0, 0, 0, 0] += 0.5
    l2, worst = bench.velocity_error(got, ref)
    den = 3 * 8 * 1.0 + 3 * 4.0
    assert abs(l2 - np.sqrt(0.25 / den)) < 1e-15 and worst == 0.5
