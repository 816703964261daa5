"""Batches of box cavities (lbm_batch_*): each domain's result is the same
alone and in the mix, bit for bit, whatever its neighbours are."""
import numpy as np
import pytest

from cavityflow_cuda_gb300.workloads import batch_workload

pytestmark = pytest.mark.gpu


def _mix(storage, seed=3, count=11):
    cav = batch_workload(count=count, seed=seed, edge=(1, 40))
    return [c.solver_args(storage) for c in cav]


@pytest.mark.parametrize("storage", ["f32", "f64", "f16s", "bf16s", "f16sr"])
def test_batch_domains_match_single_solvers(gpu, storage):
    from cavityflow_cuda_gb300 import CLbmSolverGB300, LbmBatch

    doms = _mix(storage)
    steps = 149  # graphs of 64 steps plus single steps, ending after an alpha step
    with LbmBatch(doms, storage=storage) as b:
        b.run(steps)
        assert b.info()["step_counter"] == steps
        got = [b.domain(i).get_all() for i in range(len(doms))]
    for i, (size, inv_tau, lid) in enumerate(doms):
        with CLbmSolverGB300(size, inv_tau, lid, storage=storage) as s:
            s.run(steps)
            want = s.get_all()
        assert np.array_equal(got[i].view(np.uint8), want.view(np.uint8)), (storage, i, size)


@pytest.mark.parametrize("storage", ["f32", "f16sr", "bf16s"])
@pytest.mark.parametrize("variant", range(24))
def test_batch_every_variant(gpu, storage, variant):
    """Every register variant whose vectors fit the batch's packed rows (8
    bytes) gives each domain the bits it gets alone; wider ones are refused."""
    from cavityflow_cuda_gb300 import CLbmSolverGB300, LbmBatch, LbmError

    doms = _mix(storage, seed=variant + 10, count=6)
    with LbmBatch(doms, storage=storage) as b:
        try:
            b.set_fast_variant(variant)
        except LbmError as e:
            assert e.status == 5 and variant in (0, 1, 2, 10, 11, 12, 15, 16, 18, 19, 20, 21), variant
            return
        b.run(21)
        got = [b.domain(i).get_all() for i in range(len(doms))]
    for i, (size, inv_tau, lid) in enumerate(doms):
        with CLbmSolverGB300(size, inv_tau, lid, storage=storage) as s:
            s.run(21)
            assert np.array_equal(got[i].view(np.uint8), s.get_all().view(np.uint8)), (variant, i)


def test_batch_views_getters_and_guards(gpu):
    from cavityflow_cuda_gb300 import CLbmSolverGB300, LbmBatch, LbmError

    doms = _mix("f32", seed=5, count=4)
    with LbmBatch(doms, storage="f32") as b:
        b.run(10)
        v = b.domain(2)
        size, inv_tau, lid = doms[2]
        with CLbmSolverGB300(size, inv_tau, lid, storage="f32") as s:
            s.run(10)
            assert np.array_equal(v.getVelocities(), s.getVelocities())
            assert np.allclose(v.reduce(), s.reduce(), rtol=1e-12)
        best, ms = b.autotune(pairs=2)
        assert 0 <= best < 24 and b.info()["step_counter"] == 10
        v.simulationStepAlpha()          # a domain leaves the batch's time level
        with pytest.raises(LbmError):
            b.run(2)
        assert b._lib.lbm_destroy(v._h) == 1   # a batch domain is freed with its batch


@pytest.mark.parametrize("storage", ["f32", "f16sr", "f64"])
def test_batch_packed_rows(gpu, storage):
    """Batch domains pack their rows (x = 1 on an 8-byte boundary, rows sized
    for 8-byte vectors, 8-byte row pitch) while a single solver keeps the
    default 32-byte layout; the results are the same bit for bit."""
    from cavityflow_cuda_gb300 import CLbmSolverGB300, LbmBatch
    from cavityflow_cuda_gb300.workloads import lattice_tau

    T = np.float64 if storage == "f64" else np.float32
    sizes = [(12, 9, 7), (20, 11, 5), (30, 6, 9), (7, 13, 10), (40, 5, 6), (3, 4, 5)]
    doms = [(size, lattice_tau(0.02 + 0.01 * i, storage)[1], float(T(0.05 + 0.01 * i)))
            for i, size in enumerate(sizes)]
    elem = {"f32": 4, "f16sr": 2, "f64": 8}[storage]
    with LbmBatch(doms, storage=storage) as b:
        b.run(33)
        views = [b.domain(i) for i in range(len(doms))]
        assert all(v.info()["x1_column"] * elem == 8 for v in views)
        assert all(v.info()["row_pitch"] * elem % 8 == 0 for v in views)
        got = [v.get_all() for v in views]
    for i, (size, inv_tau, lid) in enumerate(doms):
        with CLbmSolverGB300(size, inv_tau, lid, storage=storage) as s:
            assert s.info()["x1_column"] * elem == 32
            s.run(33)
            assert np.array_equal(got[i].view(np.uint8), s.get_all().view(np.uint8)), (storage, size)
