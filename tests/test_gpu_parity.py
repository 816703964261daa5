"""Parity of the CUDA path (through the C ABI) with the reference's kernels.

FP64 and FP32 populations must be bit-identical to the reference's own CPU
kernels: the golden fixtures and digests were produced by them
(tests/golden/make_golden.py), and the C oracle reproduces them bit for bit
(tests/test_oracle.py).  Velocity tolerance of the reference contract:
max |du| <= 1e-6 (FP32) and <= 1e-12 (FP64) after 1000 steps; bit-identity
is stronger and is what these tests require.
"""
import hashlib
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN
from oracle import oracle as orc

pytestmark = pytest.mark.gpu

DIGESTS = json.load(open(os.path.join(GOLDEN, "digests.json")))


def solver(size, dtype, inv_tau, lid_u, **kw):
    from cavityflow_cuda_gb300 import CLbmSolverGB300

    return CLbmSolverGB300(size, inv_tau, lid_u, storage="f64" if dtype == np.float64 else "f32", **kw)


def same_bits(a, b):
    return a.shape == b.shape and np.array_equal(np.ascontiguousarray(a).view(np.uint8),
                                                  np.ascontiguousarray(b).view(np.uint8))


SMALL = ["cube8_f64", "box10x7x5_f64", "cube8_f32", "box13x6x9_f32", "gravity12x9x6_f32", "gravity9x9x9_f64",
         "walls10_f64"]


@pytest.mark.parametrize("name", SMALL)
def test_fixture_parity(gpu, name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    dtype = z["init_dd"].dtype.type
    n = (int(z["nx"]), int(z["ny"]), int(z["nz"]))
    with solver(n, dtype, z["inv_tau"], z["lid_u"], gravity=tuple(z["gravity"]), driven_cavity=bool(z["lid"])) as s:
        assert same_bits(s.get_all(), z["init_dd"])
        assert np.array_equal(s.flags_all(), z["flags"])
        done = 0
        for k in z["steps"]:
            s.run(int(k) - done)
            done = int(k)
            assert same_bits(s.get_all(), z[f"dd_{k}"]), f"{name} after {k} steps"


@pytest.mark.parametrize("tag", ["f64", "f32"])
def test_cuboid_steps_with_interior_obstacle(gpu, tag):
    z = np.load(os.path.join(GOLDEN, f"cuboid_obstacle_{tag}.npz"))
    dtype = z["dd_final"].dtype.type
    n = (int(z["nx"]), int(z["ny"]), int(z["nz"]))
    with solver(n, dtype, z["inv_tau"], z["lid_u"], driven_cavity=False) as s:
        s.setFlags(z["flags"], (0, 0, 0), (n[0] + 2, n[1] + 2, n[2] + 2))
        assert s.info()["fast_path"] == 0
        for kind, o, sz in zip(z["seq_kind"], z["seq_origin"], z["seq_size"]):
            (s.simulationStepBeta if kind else s.simulationStepAlpha)(tuple(o), tuple(sz))
        assert same_bits(s.get_all(), z["dd_final"])


@pytest.mark.parametrize("name", sorted(DIGESTS))
def test_digest_parity(gpu, name):
    """Includes the 64^3 FP64, 1000-step lid-driven cavity (Re = 100)."""
    d = DIGESTS[name]
    dtype = np.dtype(d["dtype"]).type
    with solver((d["nx"], d["ny"], d["nz"]), dtype, dtype(d["inv_tau"]), dtype(d["lid_u"])) as s:
        assert s.info()["fast_path"] == 1
        s.run(d["steps"])
        dd = s.get_all()
    assert hashlib.sha256(dd.tobytes()).hexdigest() == d["sha256"]


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("n,steps", [((33, 17, 9), 23), ((300, 5, 4), 8), ((7, 31, 12), 15), ((1, 1, 1), 6),
                                     ((130, 3, 2), 5)])
def test_odd_shapes_match_oracle(gpu, oracle, dtype, n, steps):
    """Rows that do not fill a vector, warps spanning two rows, single-cell domains."""
    _, itau = orc.tau_of(0.0192, dtype)
    lid = dtype(0.08)
    want, _ = oracle.run_cavity(*n, dtype, itau, lid, steps)
    with solver(n, dtype, itau, lid) as s:
        for i in range(steps):
            (s.simulationStepBeta if i & 1 else s.simulationStepAlpha)()
        assert same_bits(s.get_all(), want)


@pytest.mark.parametrize("variant", [3, 8, 13, 15])
@pytest.mark.parametrize("n", [(3, 2, 70000), (70000, 2, 3), (2, 70000, 3)])
def test_extreme_aspect_ratios_match_oracle(gpu, oracle, variant, n):
    """More planes than one launch's grid holds (the step kernels launch the
    planes in chunks of 65535), and rows or columns of 70000 cells."""
    _, itau = orc.tau_of(0.0192, np.float32)
    lid = np.float32(0.08)
    steps = 5
    want, _ = oracle.run_cavity(*n, np.float32, itau, lid, steps)
    with solver(n, np.float32, itau, lid, fast_variant=variant) as s:
        s.run(steps)
        assert same_bits(s.get_all(), want), (variant, n)


@pytest.mark.parametrize("variant", range(30))
@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_every_launch_variant_matches_oracle(gpu, oracle, variant, dtype):
    """Each launch variant: register-blocked vector kernels (0-23; 8-12 with
    the block-wide beta exchange, whose blocks here straddle rows (37 cells)
    and split them (300 cells); 13-23 with direct shifted windows, 18-23
    packing 16-bit storage and running the direct beta otherwise) and the
    row-pipelined bulk-copy kernels (24-29)."""
    _, itau = orc.tau_of(0.032, dtype)
    lid = dtype(0.07)
    from cavityflow_cuda_gb300 import LbmError

    ran = 0
    for n, steps in (((37, 9, 5), 13), ((300, 4, 3), 6), ((5, 6, 7), 9)):
        want, _ = oracle.run_cavity(*n, dtype, itau, lid, steps)
        try:
            s = solver(n, dtype, itau, lid, fast_variant=variant)
        except LbmError as e:  # a bulk-copy variant whose buffers exceed shared memory
            assert e.status == 5
            continue
        with s:
            assert s.info()["fast_variant"] == variant
            s.run(steps)
            assert same_bits(s.get_all(), want), (variant, n)
            ran += 1
    assert ran >= 2


def test_autotune_keeps_state(gpu):
    _, itau = orc.tau_of(0.0192, np.float32)
    with solver((48, 40, 32), np.float32, itau, np.float32(0.05)) as a, \
            solver((48, 40, 32), np.float32, itau, np.float32(0.05)) as b:
        a.run(7)
        b.run(7)
        best, ms = a.autotune(pairs=2)
        assert 0 <= best < len(ms) and all(m > 0 for m in ms)
        assert a.info()["fast_variant"] == best and a.info()["step_counter"] == 7
        a.run(10)
        b.run(10)
        assert same_bits(a.get_all(), b.get_all())


def test_run_graph_matches_single_steps(gpu):
    _, itau = orc.tau_of(0.032, np.float32)
    with solver((40, 24, 16), np.float32, itau, np.float32(0.05)) as a, \
            solver((40, 24, 16), np.float32, itau, np.float32(0.05)) as b:
        a.simulationStepAlpha()
        a.run(150)                # odd start, then graphs of 64 steps, then the rest
        for i in range(151):
            (b.simulationStepBeta if i & 1 else b.simulationStepAlpha)()
        assert a.info()["step_counter"] == b.info()["step_counter"] == 151
        assert same_bits(a.get_all(), b.get_all())


def test_macros_match_oracle(gpu, oracle):
    for dtype in (np.float32, np.float64):
        _, itau = orc.tau_of(0.032, dtype)
        lid = dtype(0.06)
        n = (13, 11, 7)
        for steps in (9, 10):
            dd, flags = oracle.run_cavity(*n, dtype, itau, lid, steps)
            rho, jx, jy, jz = oracle.macros(dd, flags, last_was_alpha=bool(steps & 1), lid_u=lid)
            with solver(n, dtype, itau, lid) as s:
                s.run(steps)
                full = ((0, 0, 0), (n[0] + 2, n[1] + 2, n[2] + 2))
                u = s.getVelocities(*full)
                r = s.getDensities(*full)
                assert same_bits(r, rho) and same_bits(u[0], jx) and same_bits(u[1], jy) and same_bits(u[2], jz)
                # cuboid and default (interior) selections
                assert same_bits(s.getDensities(), rho[1:-1, 1:-1, 1:-1])
                assert same_bits(s.getVelocities((2, 3, 1), (4, 2, 3))[1], jy[1:4, 3:5, 2:6])


def test_set_velocities_and_densities_until_next_step(gpu):
    with solver((6, 5, 4), np.float32, 1.7, 0.05) as s:
        s.run(3)
        v = np.full((3, 2, 2, 2), 0.25, np.float32)
        s.setVelocities(v, (1, 1, 1), (2, 2, 2))
        assert (s.getVelocities((1, 1, 1), (2, 2, 2)) == 0.25).all()
        s.setDensities(np.full((2, 2, 2), 3.0, np.float32), (1, 1, 1), (2, 2, 2))
        assert (s.getDensities((1, 1, 1), (2, 2, 2)) == 3.0).all()
        s.simulationStepBeta()
        assert (s.getVelocities((1, 1, 1), (2, 2, 2)) != 0.25).all()


def test_population_copies_cuboid_and_direction(gpu):
    rng = np.random.default_rng(3)
    with solver((9, 8, 7), np.float64, 1.6, 0.05) as s:
        base = s.get_all()
        o, sz = (2, 1, 3), (5, 4, 2)
        src = rng.random((19, sz[2], sz[1], sz[0]))
        from cavityflow_cuda_gb300 import TOP

        s.setDensityDistributions(src, o, sz, direction=TOP)
        got = s.get_all()
        want = base.copy()
        cy = [0, 0, 1, -1, 1, -1, -1, 1, 0, 0, 0, 0, 1, -1, 1, -1, 0, 0, 0]
        for k in range(19):
            if -cy[k] > 0:  # TOP: norm (0,-1,0) . e_k > 0 (src/CLbmSolverGPU.cu:625-645)
                want[k, o[2]:o[2] + sz[2], o[1]:o[1] + sz[1], o[0]:o[0] + sz[0]] = src[k]
        assert np.array_equal(got, want)
        s.setDensityDistributions(src, o, sz)
        assert np.array_equal(s.getDensityDistributions(o, sz), src)


def test_flags_roundtrip_switches_paths(gpu):
    from cavityflow_cuda_gb300 import FLUID, OBSTACLE

    with solver((16, 12, 10), np.float32, 1.7, 0.05) as s:
        assert s.info()["fast_path"] == 1
        s.setFlags(np.full((2, 2, 2), OBSTACLE, np.int32), (5, 5, 5), (2, 2, 2))
        assert s.info()["fast_path"] == 0
        assert (s.getFlags((5, 5, 5), (2, 2, 2)) == OBSTACLE).all()
        s.setFlags(np.full((2, 2, 2), FLUID, np.int32), (5, 5, 5), (2, 2, 2))
        assert s.info()["fast_path"] == 1


def test_reduce_matches_oracle_and_conserves_mass(gpu, oracle):
    for dtype in (np.float64, np.float32):
        _, itau = orc.tau_of(0.05, dtype)
        n = (20, 18, 16)
        rng = np.random.default_rng(1)
        dd0, flags = oracle.init(*n, dtype)
        dd0 = (dd0 * (1 + 0.01 * rng.standard_normal(dd0.shape))).astype(dtype)
        with solver(n, dtype, itau, dtype(0.0), driven_cavity=False) as s:
            s.set_all(dd0)
            m0 = s.reduce()
            assert np.allclose(m0, oracle.reduce(dd0, flags, False), rtol=1e-12, atol=1e-12)
            s.run(1001)
            m1 = s.reduce()
            dd = dd0.copy()
            for i in range(1001):
                oracle.step(dd, flags, i, itau, dtype(0.0))
            assert np.allclose(m1, oracle.reduce(dd, flags, True), rtol=1e-12, atol=1e-12)
            # FP64: the conservation criterion; FP32: collision round-off from a 1%-noise start
            tol = 1e-10 if dtype == np.float64 else 1e-4
            assert abs(m1[0] - m0[0]) <= tol * m0[0]


def test_errors_are_status_codes(gpu):
    from cavityflow_cuda_gb300 import LbmError

    with solver((8, 8, 8), np.float32, 1.7, 0.05) as s:
        with pytest.raises(LbmError) as ei:
            s.simulationStepAlpha((0, 0, 0), (11, 1, 1))
        assert ei.value.status == 2
        with pytest.raises(LbmError) as ei:
            s.setFlags(np.full((1, 1, 1), 3, np.int32), (1, 1, 1), (1, 1, 1))
        assert ei.value.status == 1
        with pytest.raises(LbmError):
            s.getDensityDistributions((9, 0, 0), (2, 1, 1))


def test_user_stream(gpu):
    import torch

    _, itau = orc.tau_of(0.032, np.float32)
    st = torch.cuda.Stream()
    with solver((24, 20, 16), np.float32, itau, np.float32(0.05)) as a, \
            solver((24, 20, 16), np.float32, itau, np.float32(0.05)) as b:
        a.run(200, stream=st)
        st.synchronize()
        b.run(200)
        assert same_bits(a.get_all(), b.get_all())


def test_full_size_384_fp32_steps_match_oracle(gpu, oracle):
    """The 384^3 FP32 benchmark domain: the first alpha/beta pair and one
    more alpha, bit-identical to the oracle."""
    dtype = np.float32
    _, itau = orc.tau_of(0.0192, dtype)
    lid = dtype(0.05)
    n = (384, 384, 384)
    with solver(n, dtype, itau, lid) as s:
        s.run(3)
        got = s.get_all()
    want, _ = oracle.run_cavity(*n, dtype, itau, lid, 3)
    assert same_bits(got, want)


@pytest.mark.parametrize("variant", [3, 8, 11, 12])
def test_fp64_fused_multiply_add_close_to_oracle(gpu, oracle, variant):
    """The opt-in FP64 kernels with fused multiply-adds: not bit-identical to
    the reference CPU kernels any more, but within rounding of them, and the
    same whatever the register variant (single steps and graph replays)."""
    _, itau = orc.tau_of(0.032, np.float64)
    lid = 0.07
    n, steps = (37, 20, 30), 70
    want, _ = oracle.run_cavity(*n, np.float64, itau, lid, steps)
    with solver(n, np.float64, itau, lid, fast_variant=variant, fused_multiply_add=True) as s:
        s.run(steps)
        got = s.get_all()
    with solver(n, np.float64, itau, lid, fast_variant=3, fused_multiply_add=True) as s:
        for i in range(steps):
            (s.simulationStepBeta if i & 1 else s.simulationStepAlpha)()
        one_by_one = s.get_all()
    assert same_bits(got, one_by_one)
    assert np.abs(got - want).max() <= 1e-13
    assert not same_bits(got, want)  # the multiply-adds really are fused


@pytest.mark.parametrize("variant", [13, 8, 15, 25])
def test_fp32_fused_multiply_add_close_to_oracle(gpu, oracle, variant):
    """The opt-in FP32 kernels with fused multiply-adds (the reference's CUDA
    build's arithmetic): within FP32 rounding of the unfused oracle, and the
    same whatever the register variant (variant 25 is a bulk-copy variant,
    which stays unfused)."""
    _, itau = orc.tau_of(0.032, np.float32)
    lid = np.float32(0.07)
    n, steps = (37, 20, 30), 70
    want, _ = oracle.run_cavity(*n, np.float32, itau, lid, steps)
    with solver(n, np.float32, itau, lid, fast_variant=variant, fused_multiply_add=True) as s:
        assert s.info()["fused_multiply_add"] == 1
        s.run(steps)
        got = s.get_all()
    if variant >= 24:
        assert same_bits(got, want)
        return
    with solver(n, np.float32, itau, lid, fast_variant=13, fused_multiply_add=True) as s:
        s.run(steps)
        other = s.get_all()
    assert same_bits(got, other)
    assert np.abs(got - want).max() <= 2e-6
    assert not same_bits(got, want)
