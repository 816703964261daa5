"""FP16 / BF16 shifted-population storage (f - w stored in 16 bits, collision
in FP32 registers): bit-identical to the oracle's restatement of the same
arithmetic, for every launch variant, plus the macroscopic getters and the
FP64 reduction; and its velocity error against an FP64 run of this solver."""
import numpy as np
import pytest

from oracle import oracle as orc

pytestmark = pytest.mark.gpu

KIND = {"f16s": 0, "bf16s": 1, "f16sr": 2}


def shifted_solver(n, storage, inv_tau, lid, **kw):
    from cavityflow_cuda_gb300 import CLbmSolverGB300

    return CLbmSolverGB300(n, inv_tau, lid, storage=storage, **kw)


@pytest.mark.parametrize("storage", ["f16s", "bf16s", "f16sr"])
@pytest.mark.parametrize("variant", range(30))
def test_shifted_storage_matches_oracle(gpu, oracle, storage, variant):
    _, itau = orc.tau_of(0.0192, np.float32)
    lid = np.float32(0.08)
    from cavityflow_cuda_gb300 import LbmError

    ran = 0
    for n, steps in (((45, 9, 5), 13), ((300, 4, 3), 8), ((6, 7, 8), 11)):
        dd, _ = oracle.run_cavity_s(*n, KIND[storage], itau, lid, steps)
        want = oracle.unshift(dd, KIND[storage])
        try:
            s = shifted_solver(n, storage, itau, lid, fast_variant=variant)
        except LbmError as e:  # a bulk-copy variant whose buffers exceed shared memory
            assert e.status == 5
            continue
        with s:
            s.run(steps)
            got = s.get_all()
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), (storage, variant, n)
        ran += 1
    assert ran >= 2


def test_stochastic_storage_graph_replays_match_oracle(gpu, oracle):
    """F16SR keys each step's rounding by the step number: a run long enough
    to replay captured graphs (which rewrite their first step before each
    replay) equals the oracle, and so do the same steps taken one by one."""
    _, itau = orc.tau_of(0.0192, np.float32)
    lid = np.float32(0.08)
    n, steps = (20, 14, 11), 150
    dd, _ = oracle.run_cavity_s(*n, 2, itau, lid, steps)
    want = oracle.unshift(dd, 2)
    with shifted_solver(n, "f16sr", itau, lid) as s:
        s.run(steps)
        assert np.array_equal(s.get_all().view(np.uint32), want.view(np.uint32))
    with shifted_solver(n, "f16sr", itau, lid) as s:
        for i in range(steps):
            (s.simulationStepBeta if i & 1 else s.simulationStepAlpha)()
        assert np.array_equal(s.get_all().view(np.uint32), want.view(np.uint32))


@pytest.mark.parametrize("storage", ["f16s", "bf16s", "f16sr"])
def test_shifted_macros_and_reduce_match_oracle(gpu, oracle, storage):
    _, itau = orc.tau_of(0.032, np.float32)
    lid = np.float32(0.06)
    n = (14, 10, 9)
    for steps in (9, 10):
        dd, flags = oracle.run_cavity_s(*n, KIND[storage], itau, lid, steps)
        rho, jx, jy, jz = oracle.macros_s(dd, flags, bool(steps & 1), lid, KIND[storage])
        want_red = oracle.reduce_s(dd, flags, bool(steps & 1), KIND[storage])
        with shifted_solver(n, storage, itau, lid) as s:
            s.run(steps)
            full = ((0, 0, 0), (n[0] + 2, n[1] + 2, n[2] + 2))
            u = s.getVelocities(*full)
            r = s.getDensities(*full)
            red = s.reduce()
        assert np.array_equal(r, rho) and np.array_equal(u[0], jx) and np.array_equal(u[1], jy)
        assert np.array_equal(u[2], jz)
        assert np.allclose(red, want_red, rtol=1e-12, atol=1e-9)


@pytest.mark.parametrize("storage", ["f16s", "bf16s", "f16sr"])
def test_shifted_population_roundtrip(gpu, storage):
    """set -> get of populations converts f <-> f - w exactly where 16 bits hold it."""
    rng = np.random.default_rng(5)
    n = (10, 9, 8)
    with shifted_solver(n, storage, 1.7, 0.05) as s:
        base = s.get_all()
        w = base[:, 0, 0, 0]
        src = (w[:, None, None, None] + 0.001 * rng.standard_normal((19, 3, 4, 5))).astype(np.float32)
        s.setDensityDistributions(src, (2, 2, 2), (5, 4, 3))
        got = s.getDensityDistributions((2, 2, 2), (5, 4, 3))
        tol = 1e-5 if storage == "bf16s" else 1e-6
        assert np.abs(got - src).max() < tol


def test_fp16_velocity_error_against_fp64(gpu):
    """L2 velocity error of FP16/BF16 storage against an FP64 run of this
    solver on a 48^3 cavity after 1000 steps (the full-size measurement is
    bench.py's precision report)."""
    from cavityflow_cuda_gb300 import CLbmSolverGB300

    n, steps = (48, 48, 48), 1000
    _, itau64 = orc.tau_of(0.0512, np.float64)
    with CLbmSolverGB300(n, itau64, 0.1, storage="f64") as s:
        s.run(steps)
        u64 = s.getVelocities().astype(np.float64)
    errs = {}
    for storage in ("f32", "f16s", "bf16s", "f16sr"):
        _, itau = orc.tau_of(0.0512, np.float32)
        with CLbmSolverGB300(n, itau, np.float32(0.1), storage=storage) as s:
            s.run(steps)
            u = s.getVelocities().astype(np.float64)
        errs[storage] = np.sqrt(((u - u64) ** 2).sum() / (u64 ** 2).sum())
    assert errs["f32"] < 1e-4, errs   # unshifted FP32 loses digits in f - w itself
    assert errs["f16s"] < 1e-3, errs
    assert errs["f16sr"] < errs["f16s"], errs  # stochastic rounding removes the bias of rounding to nearest
    print("L2 velocity error vs FP64:", errs)


@pytest.mark.parametrize("storage", ["f16s", "bf16s", "f16sr"])
def test_shifted_flag_array_path_matches_oracle(gpu, oracle, storage):
    """16-bit storage through the flag-array kernels: an interior obstacle,
    the lid, whole-domain and cuboid steps (each keyed by the solver's step
    count for stochastic rounding), bit for bit against the oracle."""
    _, itau = orc.tau_of(0.0192, np.float32)
    lid = np.float32(0.08)
    n = (14, 12, 10)
    kind = KIND[storage]
    dd, flags = oracle.init_s(*n)
    oracle.set_lid(flags)
    flags[4:7, 5:8, 3:9] = orc.OBSTACLE
    halo = (n[0] + 2, n[1] + 2, n[2] + 2)
    seq = [(None, None)] * 4 + [((1, 1, 1), (7, 12, 10)), ((8, 1, 1), (7, 12, 10)),
                                ((0, 0, 0), halo), ((2, 3, 4), (9, 8, 5))] + [(None, None)] * 3
    with shifted_solver(n, storage, itau, lid, driven_cavity=False) as s:
        s.setFlags(flags, (0, 0, 0), halo)
        assert s.info()["fast_path"] == 0
        for i, (o, sz) in enumerate(seq):
            step = s.simulationStepBeta if i & 1 else s.simulationStepAlpha
            step(o, sz) if o is not None else step()
            oracle.step_s(dd, flags, i, itau, lid, kind, origin=o, size=sz)
        got = s.get_all()
    want = oracle.unshift(dd, kind)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), storage
