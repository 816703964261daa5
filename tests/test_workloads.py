"""The seeded workload generators of the batching and serving benchmarks (CPU)."""
import numpy as np

from cavityflow_cuda_gb300.workloads import (MT19937_64, NU_MIN, SERVE_EDGES, batch_workload, lattice_tau,
                                             serving_workload)


def test_mt19937_64_known_answers():
    """Same stream as C++ std::mt19937_64: the 10000th output of the default
    seed is the standard's known answer, and the first outputs of seed 0."""
    g = MT19937_64()
    x = 0
    for _ in range(10000):
        x = g.next()
    assert x == 9981545732273789042
    h = MT19937_64(0)
    assert [h.next() for _ in range(3)] == [2947667278772165694, 18301848765998365067, 729919693006235833]


def test_batch_workload_shape():
    b = batch_workload()
    assert len(b) == 512
    assert all(16 <= s <= 96 for c in b for s in c.size)
    assert all(0.02 <= c.lid <= 0.1 for c in b) and all(10 <= c.reynolds <= 2000 for c in b)
    assert all(c.nu >= NU_MIN for c in b)
    assert all(lattice_tau(c.nu, "f32")[0] >= np.float32(0.51) for c in b)
    assert batch_workload()[17].size == b[17].size            # deterministic
    assert sum(c.cells for c in b) == 92330913


def test_serving_workload_shape():
    s = serving_workload(count=2000)
    arr = np.array([c.arrival for c in s])
    assert np.all(np.diff(arr) > 0)
    assert abs(len(s) / arr[-1] - 200) < 20                   # Poisson at 200 req/s
    assert set(c.size[0] for c in s) <= set(SERVE_EDGES)
    assert all(500 <= c.steps <= 20000 for c in s) and all(c.nu >= NU_MIN for c in s)
