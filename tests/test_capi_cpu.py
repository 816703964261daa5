"""The C ABI library without a GPU: it loads, exports every declared entry
point, derives lattice parameters exactly as the reference does, and reports
errors as status codes."""
import ctypes as C
import glob
import json
import os
import xml.etree.ElementTree as ET

import numpy as np
import pytest

from conftest import GOLDEN

PARAMS = json.load(open(os.path.join(GOLDEN, "params.json")))


def test_library_exports_every_declared_symbol(lib):
    from cavityflow_cuda_gb300 import declared_functions

    names = declared_functions()
    assert len(names) >= 25
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def _physical(path):
    r = ET.parse(path).getroot()
    ph, gr, sim = r.find("physics"), r.find("grid"), r.find("simulation")

    def v3(node, tag, conv=float):
        e = node.find(tag)
        return tuple(conv(e.find(a).text) for a in "xyz")

    return dict(velocity=v3(ph, "velocity"), acceleration=v3(ph, "acceleration"),
                viscosity=float(ph.find("viscosity").text), max_velocity=float(ph.find("max-velocity").text),
                max_acceleration=float(ph.find("max-acceleration").text),
                domain_size=v3(gr, "domain-size", int), domain_length=v3(gr, "domian-length"),
                timestep=float(sim.find("timestep").text))


@pytest.mark.parametrize("name", sorted(PARAMS))
@pytest.mark.parametrize("tag", ["f64", "f32"])
def test_derive_lattice_matches_reference(lib, name, tag):
    from cavityflow_cuda_gb300 import LbmError, derive_lattice

    want = PARAMS[name][tag]
    ph = _physical(os.path.join(GOLDEN, "configs", name + ".xml"))
    storage = "f64" if tag == "f64" else "f32"
    if want.get("error"):
        with pytest.raises(LbmError) as ei:
            derive_lattice(**ph, storage=storage)
        assert ei.value.status == 6  # LBM_ERR_CONFIG, where the reference exit()s
        return
    got = derive_lattice(**ph, storage=storage)
    assert got["timestep"] == want["timestep"]
    assert got["tau"] == want["tau"]
    assert got["inv_tau"] == want["tau_inv"]
    assert got["velocity"] == (want["ux"], want["uy"], want["uz"])
    assert got["acceleration"] == (want["gx"], want["gy"], want["gz"])
    assert got["viscosity"] == want["nu"]


def test_status_strings_and_errors_without_device(lib):
    import torch

    from cavityflow_cuda_gb300 import CLbmSolverGB300, LbmError
    from cavityflow_cuda_gb300 import solver as solver_mod

    assert lib.lbm_status_string(0) == b"ok"
    assert b"bounds" in lib.lbm_status_string(2)
    with pytest.raises(LbmError) as ei:
        CLbmSolverGB300((8, 8, 8), 1.6, 0.05, storage="f32", boundary=(1, 1, 1, 1, 1, 3))
    assert ei.value.status == 1  # invalid boundary flag, checked before any CUDA call
    with pytest.raises(LbmError) as ei:
        CLbmSolverGB300((8, 8, 8), 1.6, 0.05, storage="f16sr", fused_multiply_add=True)
    assert ei.value.status == 1  # fused multiply-adds are an FP64 and FP32 option
    with pytest.raises(LbmError) as ei:
        CLbmSolverGB300((8, 8, 8), 1.6, 0.05, storage="f32", lid="wall", boundary=(1, 1, 1, 2, 1, 1))
    assert ei.value.status == 1  # a moving top wall needs an obstacle top face
    p = solver_mod._Params()
    p.size[:] = [8, 8, 8]
    p.boundary[:] = [1] * 6
    p.inv_tau, p.lid_mode = 1.6, 2
    h = C.c_void_p()
    assert lib.lbm_create(C.byref(p), C.byref(h)) == 1 and not h.value  # unknown lid mode
    if not torch.cuda.is_available():
        with pytest.raises(LbmError) as ei:
            CLbmSolverGB300((8, 8, 8), 1.6, 0.05)
        assert ei.value.status == 10  # LBM_ERR_NO_DEVICE
    # a NULL handle is rejected, not dereferenced
    assert lib.lbm_step_alpha(None, None) == 1
    assert lib.lbm_get_info(None, None) == 1


def test_header_cites_reference_for_each_replaced_entry_point():
    text = open(os.path.join(os.path.dirname(GOLDEN), "..", "include", "lbm_gb300.h")).read()
    for sym in ["lbm_create", "lbm_step_alpha", "lbm_step_beta", "lbm_get_density_distributions",
                "lbm_set_density_distributions", "lbm_get_flags", "lbm_get_velocities", "lbm_derive_lattice",
                "lbm_set_driven_cavity", "lbm_run"]:
        i = text.index(sym + "(")
        block = text[max(0, i - 700):i]
        assert "src/" in block, sym


def test_cli_usage_and_argument_errors(lib, tmp_path):
    """The lbm_gb300 command parses its arguments and reads the configuration
    before it touches a GPU; errors exit 1 as the reference's exit(EXIT_FAILURE)."""
    import subprocess

    from cavityflow_cuda_gb300 import build

    cli = build.CLI
    assert os.access(cli, os.X_OK)
    r = subprocess.run([cli, "--help"], capture_output=True, text=True)
    assert r.returncode == 0 and "usage: lbm_gb300" in r.stderr
    cfg = os.path.join(GOLDEN, "configs", "cavity64_re100.xml")
    for args in ([], [cfg, cfg], [cfg, "--storage", "f8"], [cfg, "--bogus"], [cfg, "--checkpoint-every", "5"],
                 [str(tmp_path / "absent.xml")], [os.path.join(GOLDEN, "configs", "infeasible.xml")]):
        r = subprocess.run([cli, *args], capture_output=True, text=True)
        assert r.returncode == 1 and r.stderr.startswith("usage") or "lbm_gb300:" in r.stderr, (args, r.stderr)
        assert r.returncode == 1, args
    import torch

    if not torch.cuda.is_available():
        r = subprocess.run([cli, cfg], capture_output=True, text=True)
        assert r.returncode == 1 and "no CUDA device" in r.stderr


def test_launch_variant_menu_size(lib):
    """24 register variants (0-23) and 6 bulk-copy variants (24-29); the GPU
    parity tests enumerate exactly these."""
    assert lib.lbm_fast_variant_count() == 30
    assert lib.lbm_register_variant_count() == 24


def test_batch_and_server_arguments_checked_before_the_device(lib):
    """Batches and servers reject bad arguments before any CUDA call, with
    LBM_ERR_INVALID_ARGUMENT (1); valid ones reach the device check."""
    import math

    import torch

    from cavityflow_cuda_gb300 import LbmBatch, LbmError, LbmServer

    good = [((8, 8, 8), 1.6, 0.05), ((5, 6, 7), 1.2, 0.02)]
    big = ((1 << 19, 1 << 19, 1), 1.6, 0.05)  # 0.8 * 2^40 cells with its halo: accepted alone
    for bad in ([((8, 0, 8), 1.6, 0.05)], [((8, 8, 8), 0.0, 0.05)], [((8, 8, 8), math.inf, 0.05)],
                [((8, 8, 8), 1.6, math.nan)], [((8, 8, (1 << 20) + 1), 1.6, 0.05)],
                [((1 << 20, 1 << 20, 1 << 20), 1.6, 0.05)], [big, big]):  # a domain, or the pool, above 2^40 cells
        with pytest.raises(LbmError) as ei:
            LbmBatch(good + bad, storage="f32")
        assert ei.value.status == 1, bad
    for kw in (dict(budget_bytes=1 << 19), dict(budget_bytes=1 << 30, max_round_steps=1)):
        with pytest.raises(LbmError) as ei:
            LbmServer(storage="f32", **kw)
        assert ei.value.status == 1, kw
    if not torch.cuda.is_available():
        for ok in (good, good + [big]):
            with pytest.raises(LbmError) as ei:
                LbmBatch(ok, storage="f16sr")
            assert ei.value.status == 10
        with pytest.raises(LbmError) as ei:
            LbmServer(budget_bytes=1 << 30, storage="f16s")
        assert ei.value.status == 10


@pytest.mark.parametrize("kw,status", [
    (dict(size=(0, 8, 8)), 1),
    (dict(size=(8, 8, (1 << 20) + 1)), 1),
    (dict(size=(1 << 20, 1 << 20, 1 << 20)), 1),  # more than 2^40 cells: byte counts would overflow
    (dict(size=(1 << 19, 1 << 19, 2)), 1),        # (2^19 + 2)^2 * 4 > 2^40 cells
    (dict(boundary=(1, 1, 1, 1, 16, 1)), 1),
    (dict(inv_tau=0.0), 1),
    (dict(inv_tau=float("nan")), 1),
    (dict(inv_tau=float("inf")), 1),
    (dict(lid_velocity=float("nan")), 1),
    (dict(storage="f16s", gravity=(0.0, -1e-5, 0.0)), 5),   # gravity: F64 and F32 only
    (dict(storage="bf16s", fused_multiply_add=True), 1),    # fused multiply-adds: F64 and F32 only
    (dict(lid="wall", boundary=(1, 1, 1, 8, 1, 1)), 1),     # moving wall: the top face must be an obstacle
])
def test_create_argument_checks_before_the_device(lib, kw, status):
    """lbm_create rejects bad parameters with a status code (the reference
    asserts or exits) before any CUDA call, so these hold without a GPU."""
    from cavityflow_cuda_gb300 import CLbmSolverGB300, LbmError

    args = dict(size=(8, 8, 8), inv_tau=1.6, lid_velocity=0.05, storage="f32")
    args.update(kw)
    with pytest.raises(LbmError) as ei:
        CLbmSolverGB300(args.pop("size"), args.pop("inv_tau"), args.pop("lid_velocity"), **args)
    assert ei.value.status == status, kw
