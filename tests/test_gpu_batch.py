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


@pytest.mark.parametrize("variant", range(18))
def test_batch_every_variant(gpu, variant):
    from cavityflow_cuda_gb300 import CLbmSolverGB300, LbmBatch

    doms = _mix("f32", seed=variant + 10, count=6)
    with LbmBatch(doms, storage="f32") as b:
        b.set_fast_variant(variant)
        b.run(21)
        got = [b.domain(i).get_all() for i in range(len(doms))]
    for i, (size, inv_tau, lid) in enumerate(doms):
        with CLbmSolverGB300(size, inv_tau, lid, storage="f32") as s:
            s.run(21)
            assert np.array_equal(got[i], s.get_all()), (variant, i)


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
        assert 0 <= best < 18 and b.info()["step_counter"] == 10
        v.simulationStepAlpha()          # a domain leaves the batch's time level
        with pytest.raises(LbmError):
            b.run(2)
        assert b._lib.lbm_destroy(v._h) == 1   # a batch domain is freed with its batch
