"""The request server (lbm_server_*): continuous batching under a memory
budget.  Each result is the same alone and in the mix, bit for bit."""
import numpy as np
import pytest

from cavityflow_cuda_gb300.workloads import lattice_tau

pytestmark = pytest.mark.gpu

REQS = [((12, 9, 7), 0.032, 0.05, 30), ((5, 6, 4), 0.05, 0.08, 7), ((33, 17, 9), 0.0192, 0.06, 101),
        ((8, 8, 8), 0.1, 0.03, 0), ((21, 13, 40), 0.02, 0.1, 64), ((3, 3, 3), 0.04, 0.05, 1),
        ((17, 29, 11), 0.012, 0.07, 45), ((40, 7, 6), 0.03, 0.02, 200)]


def _solo(size, nu, lid, steps, storage):
    from cavityflow_cuda_gb300 import CLbmSolverGB300

    _, inv_tau = lattice_tau(nu, storage)
    T = np.float64 if storage == "f64" else np.float32
    with CLbmSolverGB300(size, inv_tau, float(T(lid)), storage=storage) as s:
        s.run(steps)
        return s.getDensities(), s.getVelocities()


@pytest.mark.parametrize("storage", ["f32", "f16s", "f64", "f16sr"])
def test_served_results_match_solo_runs(gpu, storage):
    from cavityflow_cuda_gb300 import LbmServer

    T = np.float64 if storage == "f64" else np.float32
    results, ids = {}, {}
    with LbmServer(budget_bytes=2 << 30, storage=storage, max_round_steps=16, target_round_ms=0) as srv:
        pending = list(range(len(REQS)))
        while pending or srv.stats()["active"] or srv.stats()["queued"]:
            for _ in range(3):  # requests keep arriving between rounds
                if pending:
                    i = pending.pop(0)
                    size, nu, lid, steps = REQS[i]
                    ids[srv.submit(size, lattice_tau(nu, storage)[1], float(T(lid)), steps)] = i
            srv.round()
            for c in srv.poll():
                assert c["status"] == 0
                results[ids[c["id"]]] = srv.take_result(c["id"])
        assert srv.stats()["completed"] == len(REQS)
    for i, (size, nu, lid, steps) in enumerate(REQS):
        rho, u = _solo(size, nu, lid, steps, storage)
        assert np.array_equal(results[i][0], rho) and np.array_equal(results[i][1], u), (storage, i)


def test_budget_admission_and_rejection(gpu):
    from cavityflow_cuda_gb300 import LbmError, LbmServer

    # room for one 48^3 FP32 cavity at a time (~11 MB of populations)
    with LbmServer(budget_bytes=18 << 20, storage="f32", max_round_steps=8, target_round_ms=0) as srv:
        inv = lattice_tau(0.03, "f32")[1]
        for _ in range(4):
            srv.submit((48, 48, 48), inv, 0.05, 20)
        with pytest.raises(LbmError) as ei:
            srv.submit((160, 160, 160), inv, 0.05, 10)
        assert ei.value.status == 8  # LBM_ERR_BUDGET
        max_active, done = 0, []
        while len(done) < 4:
            srv.round()
            st = srv.stats()
            max_active = max(max_active, st["active"])
            assert st["bytes_in_use"] <= st["budget_bytes"]
            done += srv.poll()
        assert max_active == 1
        assert srv.stats()["peak_bytes"] <= 18 << 20
        for c in done:
            srv.take_result(c["id"], copy=False)


def test_late_short_request_overtakes_long_one(gpu):
    """Continuous batching: a request that arrives while a long one runs is
    admitted at the next round and finishes first."""
    from cavityflow_cuda_gb300 import LbmServer

    with LbmServer(budget_bytes=1 << 30, storage="f32", max_round_steps=32, target_round_ms=0) as srv:
        inv = lattice_tau(0.03, "f32")[1]
        a = srv.submit((40, 40, 40), inv, 0.05, 600)
        srv.round()
        b = srv.submit((24, 24, 24), inv, 0.05, 40)
        fin = {}
        while len(fin) < 2:
            srv.round()
            for c in srv.poll():
                fin[c["id"]] = c
        assert fin[b]["finish_time"] < fin[a]["finish_time"]
        assert fin[b]["admit_time"] < fin[a]["finish_time"]


def test_results_beyond_one_staging_buffer(gpu):
    """Six 256^3 FP32 requests that finish in the same round: their results
    (1.6 GB) exceed one 1 GiB host staging buffer, so the last two are
    written after the first four are copied out; all match solo runs."""
    from cavityflow_cuda_gb300 import LbmServer

    size, steps, nu = (256, 256, 256), 4, 0.02
    lids = [0.01 * (i + 1) for i in range(6)]
    inv = lattice_tau(nu, "f32")[1]
    out = {}
    with LbmServer(budget_bytes=12 << 30, storage="f32", max_round_steps=16, target_round_ms=0) as srv:
        ids = {srv.submit(size, inv, float(np.float32(lid)), steps): i for i, lid in enumerate(lids)}
        while len(out) < len(lids):
            srv.round()
            for c in srv.poll():
                assert c["status"] == 0
                out[ids[c["id"]]] = srv.take_result(c["id"])
        assert srv.stats()["rounds"] == 1
    for i in (0, 3, 4, 5):
        rho, u = _solo(size, nu, lids[i], steps, "f32")
        assert np.array_equal(out[i][0], rho) and np.array_equal(out[i][1], u), i
