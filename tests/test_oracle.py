"""The CPU oracle pinned against the reference's own kernels (CPU only).

Golden fixtures in tests/golden were produced by running the reference's CPU
kernels (src/cpukernels/CLbm{Init,Alpha,Beta}CPU.cpp) built from its sources;
see tests/golden/make_golden.py.  The oracle must reproduce them bit for bit.
"""
import hashlib
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN
from oracle import oracle as orc


def _load(name):
    return np.load(os.path.join(GOLDEN, name + ".npz"))


SMALL = ["cube8_f64", "box10x7x5_f64", "cube8_f32", "box13x6x9_f32", "gravity12x9x6_f32", "gravity9x9x9_f64",
         "walls10_f64"]


@pytest.mark.parametrize("name", SMALL)
def test_oracle_matches_reference_fixtures(oracle, name):
    z = _load(name)
    dtype = z["init_dd"].dtype
    nx, ny, nz = int(z["nx"]), int(z["ny"]), int(z["nz"])
    dd, flags = oracle.init(nx, ny, nz, dtype)
    assert np.array_equal(dd, z["init_dd"])
    if bool(z["lid"]):
        oracle.set_lid(flags)
    assert np.array_equal(flags, z["flags"])
    itau, lid_u, g = dtype.type(z["inv_tau"]), dtype.type(z["lid_u"]), tuple(dtype.type(v) for v in z["gravity"])
    done = 0
    for n in z["steps"]:
        while done < n:
            oracle.step(dd, flags, done, itau, lid_u, g)
            done += 1
        assert np.array_equal(dd.view(np.uint8), z[f"dd_{n}"].view(np.uint8)), f"{name} after {n} steps"


@pytest.mark.parametrize("tag", ["f64", "f32"])
def test_oracle_cuboid_steps_and_obstacles(oracle, tag):
    z = _load(f"cuboid_obstacle_{tag}")
    dtype = z["dd_final"].dtype
    nx, ny, nz = int(z["nx"]), int(z["ny"]), int(z["nz"])
    dd, _ = oracle.init(nx, ny, nz, dtype)
    flags = z["flags"].copy()
    itau, lid_u = dtype.type(z["inv_tau"]), dtype.type(z["lid_u"])
    for kind, o, s in zip(z["seq_kind"], z["seq_origin"], z["seq_size"]):
        if kind:
            oracle.beta(dd, flags, itau, lid_u, origin=o, size=s)
        else:
            oracle.alpha(dd, flags, itau, lid_u, origin=o, size=s)
    assert np.array_equal(dd.view(np.uint8), z["dd_final"].view(np.uint8))


DIGESTS = json.load(open(os.path.join(GOLDEN, "digests.json")))


@pytest.mark.parametrize("name", sorted(DIGESTS))
def test_oracle_matches_reference_digests(oracle, name):
    d = DIGESTS[name]
    dtype = np.dtype(d["dtype"]).type
    dd, _ = oracle.run_cavity(d["nx"], d["ny"], d["nz"], dtype, dtype(d["inv_tau"]), dtype(d["lid_u"]), d["steps"])
    assert hashlib.sha256(dd.tobytes()).hexdigest() == d["sha256"]


def test_oracle_matches_live_reference(oracle, reference):
    """Random-ish cases against the reference kernels run now (skipped off this host)."""
    rng = np.random.default_rng(7)
    for dtype in (np.float64, np.float32):
        for _ in range(3):
            nx, ny, nz = (int(v) for v in rng.integers(3, 14, size=3))
            nu = float(rng.uniform(0.005, 0.2))
            U = dtype(rng.uniform(0.0, 0.1))
            _, itau = orc.tau_of(nu, dtype)
            steps = int(rng.integers(1, 30))
            a, _ = oracle.run_cavity(nx, ny, nz, dtype, itau, U, steps)
            b, _ = reference.run_cavity(nx, ny, nz, dtype, itau, U, steps)
            assert np.array_equal(a.view(np.uint8), b.view(np.uint8)), (dtype, nx, ny, nz, steps)


def test_initial_state_is_rest_equilibrium(oracle):
    dd, flags = oracle.init(5, 4, 3, np.float64)
    w = np.array([1 / 18] * 4 + [1 / 36] * 12 + [1 / 18] * 2 + [1 / 3])
    assert np.array_equal(dd[:, 0, 0, 0], w)
    assert (flags[1:-1, 1:-1, 1:-1] == orc.FLUID).all()
    assert (flags[0] == orc.OBSTACLE).all() and (flags[:, :, -1] == orc.OBSTACLE).all()


def test_walls_only_conserve_mass(oracle):
    """Bounce-back on all six walls conserves the live mass to round-off
    (populations that enter a wall cell's slot wait there one step)."""
    _, itau = orc.tau_of(0.05, np.float64)
    dd, flags = oracle.init(12, 10, 9, np.float64)
    # a non-uniform start so that the walls do work
    rng = np.random.default_rng(0)
    dd *= 1 + 0.01 * rng.standard_normal(dd.shape)
    m0 = oracle.reduce(dd, flags, last_was_alpha=False)[0]
    for i in range(50):
        oracle.step(dd, flags, i, itau, 0.0)
        m = oracle.reduce(dd, flags, last_was_alpha=bool(i % 2 == 0))[0]
        assert abs(m - m0) <= 1e-13 * m0


def test_lid_changes_mass(oracle):
    _, itau = orc.tau_of(0.032, np.float64)
    dd, flags = oracle.init(10, 10, 10, np.float64)
    oracle.set_lid(flags)
    m0 = oracle.reduce(dd, flags, last_was_alpha=False)[0]
    for i in range(40):
        oracle.step(dd, flags, i, itau, 0.1)
    assert abs(oracle.reduce(dd, flags, last_was_alpha=True)[0] - m0) > 1e-9 * m0


def test_moving_wall_conserves_mass_and_drives_the_flow(oracle):
    """The opt-in moving top wall: every cell under it gets -U/6 on population
    5 and +U/6 on population 6, so FP64 mass stays at its initial value to
    rounding while the lid drives a flow in +x under it, and the x momentum
    the wall puts in grows the total."""
    _, itau = orc.tau_of(0.032, np.float64)
    n = (12, 10, 9)
    dd, flags = oracle.init(*n, np.float64)
    m0 = oracle.reduce(dd, flags, last_was_alpha=False)[0]
    for i in range(200):
        oracle.step(dd, flags, i, itau, 0.08, wall=True)
    out = oracle.reduce(dd, flags, last_was_alpha=False)
    assert abs(out[0] - m0) <= 1e-13 * m0
    assert out[1] > 0.01
    rho, jx, _, _ = oracle.macros(dd, flags, last_was_alpha=False, lid_u=0.08)
    assert (jx[1:-1, n[1], 1:-1] > 0.01).all()  # the row under the wall moves with it
    assert (flags[1:-1, 1:-1, 1:-1] == orc.FLUID).all()  # no injection cells


@pytest.mark.parametrize("kind", [0, 2])
def test_moving_wall_16bit_tracks_fp32(oracle, kind):
    """The same wall on shifted 16-bit storage stays within the storage's
    rounding of the FP32 run."""
    _, itau = orc.tau_of(0.032, np.float32)
    n, steps = (10, 9, 8), 60
    ref, flags = oracle.run_cavity(*n, np.float32, itau, np.float32(0.08), steps, lid="wall")
    dd, _ = oracle.run_cavity_s(*n, kind, itau, 0.08, steps, lid="wall")
    got = oracle.unshift(dd, kind)
    inner = (slice(None), slice(1, -1), slice(1, -1), slice(1, -1))
    assert np.abs(got[inner] - ref[inner]).max() < 2e-4


def test_macros_of_lid_and_walls(oracle):
    _, itau = orc.tau_of(0.032, np.float64)
    dd, flags = oracle.run_cavity(6, 5, 4, np.float64, itau, 0.07, 9)
    rho, jx, jy, jz = oracle.macros(dd, flags, last_was_alpha=True, lid_u=0.07)
    assert (rho[:, 5, 1:-1][1:-1] == 1.0).all() and (jx[1:-1, 5, 1:-1] == 0.07).all()
    assert (rho[0] == 0).all() and (jx[:, 0] == 0).all()
    # interior fluid: sums of post-collision populations
    assert np.all(np.abs(rho[1:-1, 1:-2, 1:-1] - 1.0) < 0.05)


def test_16bit_conversions_round_to_nearest_even(oracle):
    """The oracle's FP16/BF16 conversions are IEEE round-to-nearest-even
    (checked against numpy's float16 and torch's bfloat16)."""
    import torch

    rng = np.random.default_rng(0)
    x = np.concatenate([rng.standard_normal(3000).astype(np.float32) * s for s in (1e-7, 1e-5, 1e-2, 1, 3e4)] +
                       [np.array([0, -0.0, 65504, 65519.99, 5.96e-8, 2.98e-8, 2.99e-8, np.inf], np.float32)])
    with np.errstate(over="ignore"):
        assert np.array_equal(oracle.to_half(x, 0), x.astype(np.float16).view(np.uint16))
    assert np.array_equal(oracle.to_half(x, 1),
                          torch.from_numpy(x).to(torch.bfloat16).view(torch.int16).numpy().view(np.uint16))


@pytest.mark.parametrize("kind", [0, 1, 2])
def test_shifted_storage_tracks_fp32(oracle, kind):
    """FP16/BF16 deviation storage follows the FP32 run closely on a small cavity."""
    _, itau = orc.tau_of(0.032, np.float32)
    n, steps = (12, 10, 8), 60
    ref, flags = oracle.run_cavity(*n, np.float32, itau, np.float32(0.05), steps)
    dd, _ = oracle.run_cavity_s(*n, kind, itau, np.float32(0.05), steps)
    assert (dd[:, 0, 0, 0] == 0).all()
    _, ux, uy, uz = oracle.macros(ref, flags, False, np.float32(0.05))
    _, sx, sy, sz = oracle.macros_s(dd, flags, False, np.float32(0.05), kind)
    err = np.sqrt(((sx - ux) ** 2 + (sy - uy) ** 2 + (sz - uz) ** 2).sum() / (ux ** 2 + uy ** 2 + uz ** 2).sum())
    assert err < (2e-2 if kind == 1 else 2e-3), err


def _lowbias32(cell, step):
    """The stochastic-rounding key hash (C. Wellons' lowbias32 of cell ^ step * golden), in Python."""
    m = 0xFFFFFFFF
    x = (cell ^ (step * 0x9E3779B9)) & m
    x ^= x >> 16
    x = (x * 0x7FEB352D) & m
    x ^= x >> 15
    x = (x * 0x846CA68B) & m
    x ^= x >> 16
    return x


def test_stochastic_rounding_keys_and_truncation(oracle):
    """The oracle's key hash matches an independent statement of it, and its
    round-toward-zero half conversion returns the largest-magnitude half not
    above the value."""
    import ctypes as C

    lib = oracle.lib
    lib.orc_sr_hash.argtypes = [C.c_uint32, C.c_uint32]
    lib.orc_sr_hash.restype = C.c_uint32
    for cell, step in ((0, 0), (1, 0), (0, 1), (123456, 789), (2 ** 31 + 5, 2 ** 32 - 1)):
        assert lib.orc_sr_hash(cell, step) == _lowbias32(cell, step)
    lib.orc_float_to_half_rz.argtypes = [C.c_float]
    lib.orc_float_to_half_rz.restype = C.c_uint16
    rng = np.random.default_rng(1)
    x = np.concatenate([rng.standard_normal(2000).astype(np.float32) * s for s in (1e-7, 1e-5, 1e-2, 1, 3e4)] +
                       [np.array([0, -0.0, 65504, 65519.99, 70000, 5.96e-8, 2.98e-8], np.float32)])
    got = np.array([lib.orc_float_to_half_rz(float(v)) for v in x], dtype=np.uint16).view(np.float16)
    with np.errstate(over="ignore"):
        near = x.astype(np.float16)
    want = near.copy()
    too_big = np.abs(near.astype(np.float64)) > np.abs(x.astype(np.float64))
    mag = want.view(np.uint16) & 0x7FFF
    want.view(np.uint16)[too_big] = (want.view(np.uint16)[too_big] & 0x8000) | (mag[too_big] - 1)
    assert np.array_equal(got.view(np.uint16), want.view(np.uint16))


def test_stochastic_rounding_is_unbiased(oracle):
    """Kind 2's stores average to the exact value: one value between two
    halves, stored under 20000 keys (cells) of one step, rounds to its two
    neighbours with a mean within 2 % of a unit of the exact value."""
    import ctypes as C

    scaled = np.float32(np.float32(1.2345e-3) * 4096)
    lo = np.float16(scaled)
    lib = oracle.lib
    lib.orc_float_to_half_rz.argtypes = [C.c_float]
    lib.orc_float_to_half_rz.restype = C.c_uint16
    bits = np.frombuffer(np.float32(scaled).tobytes(), np.uint32)[0]
    d = np.array([(_lowbias32(c, 7) * 0x2545F491 & 0xFFFFFFFF) >> 19 for c in range(20000)], dtype=np.uint64)
    stored = np.array([lib.orc_float_to_half_rz(float(np.frombuffer(np.uint32(bits + int(x)).tobytes(), np.float32)[0]))
                       for x in d], dtype=np.uint16).view(np.float16).astype(np.float64)
    ulp = float(np.spacing(lo))
    assert set(np.unique(stored)) <= {float(np.float16(scaled)), float(np.float16(scaled)) - ulp,
                                      float(np.float16(scaled)) + ulp}
    assert abs(stored.mean() - float(scaled)) < 0.02 * ulp
