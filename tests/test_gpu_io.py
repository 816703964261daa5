"""Checkpoint/resume, VTK output and the lbm_gb300 command on the GPU.

* A run resumed from a checkpoint is bit-identical to the uninterrupted run
  (populations, step counter and A-A parity are restored).
* VTK files carry the reference's records (src/libvis/CLbmVisualizationVTK.cpp
  :69-205): the binary form holds exactly the getters' values, which are
  bit-identical to the oracle's macroscopic fields; the ASCII form holds them
  to the 6 significant digits the reference's stream output prints.
* The command runs a configuration end to end as the reference's program
  does (src/CController.cpp:1354-1510): VTK at step 0 and every `rate` steps,
  the benchmark file's five lines, and results equal to the oracle's.
"""
import os
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN
from oracle import oracle as orc

pytestmark = pytest.mark.gpu

PKG = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "cavityflow_cuda_gb300")
CLI = os.path.join(PKG, "lbm_gb300")


def same_bits(a, b):
    return a.shape == b.shape and np.array_equal(np.ascontiguousarray(a).view(np.uint8),
                                                  np.ascontiguousarray(b).view(np.uint8))


def full(s):
    return (0, 0, 0), tuple(n + 2 for n in s.size)


def read_vtk(path):
    """A legacy structured-grid VTK file with this writer's records."""
    raw = open(path, "rb").read()
    pos = 0

    def line():
        nonlocal pos
        end = raw.index(b"\n", pos)
        out = raw[pos:end].decode()
        pos = end + 1
        return out

    out = {"version": line(), "title": line(), "mode": line(), "dataset": line()}
    dims = tuple(int(v) for v in line().split()[1:])
    _, npts, ptype = line().split()
    npts = int(npts)
    binary = out["mode"] == "BINARY"

    def block(count, typ):
        nonlocal pos
        if binary:
            dt = {"float": ">f4", "double": ">f8", "INT": ">i4"}[typ]
            a = np.frombuffer(raw, dtype=dt, count=count, offset=pos)
            pos += a.nbytes + 1  # the newline after the block
            return a.astype(dt[1:] if typ != "INT" else "i4")
        vals = []
        while len(vals) < count:
            vals.extend(line().split())
        return np.array(vals, dtype=np.int32 if typ == "INT" else np.float64)

    out["dims"] = dims
    out["points"] = block(3 * npts, ptype).reshape(npts, 3)
    cells = int(line().split()[1])
    assert line() == "SCALARS flags INT 1" and line() == "LOOKUP_TABLE default"
    out["flags"] = block(cells, "INT")
    hdr = line().split()
    assert hdr[:2] == ["SCALARS", "densities"] and line() == "LOOKUP_TABLE default"
    out["densities"] = block(cells, hdr[2])
    hdr = line().split()
    assert hdr[:2] == ["VECTORS", "velocities"]
    out["velocities"] = block(3 * cells, hdr[2]).reshape(cells, 3)
    out["type"] = hdr[2]
    return out


@pytest.mark.parametrize("storage,fma", [("f64", False), ("f32", False), ("f16s", False), ("bf16s", False),
                                         ("f16sr", False), ("f64", True)])
def test_checkpoint_resume_is_bit_identical(gpu, tmp_path, storage, fma):
    """Also for FP64 with fused multiply-adds: the checkpoint records the
    arithmetic, and a solver created from it resumes with the same."""
    from cavityflow_cuda_gb300 import CLbmSolverGB300

    size = (17, 12, 9)
    ck = str(tmp_path / "run.ckpt")
    with CLbmSolverGB300(size, 1.6, 0.07, storage=storage, fused_multiply_add=fma) as a:
        a.run(37)                       # odd: the populations sit in the alpha convention
        a.save_checkpoint(ck)
        a.run(40)
        want = a.getDensityDistributions(*full(a))
        want_info = a.info()
    with CLbmSolverGB300.from_checkpoint(ck) as b:
        assert b.storage == storage and b.size == size
        assert b.info()["fused_multiply_add"] == int(fma)
        assert b.info()["step_counter"] == 37 and b.info()["last_step_was_alpha"] == 1
        b.run(40)
        assert same_bits(b.getDensityDistributions(*full(b)), want)
        assert b.info()["step_counter"] == want_info["step_counter"]
    # restoring into an existing solver of the same shape
    with CLbmSolverGB300(size, 1.6, 0.07, storage=storage, fused_multiply_add=fma) as c:
        c.run(5)
        c.load_checkpoint(ck)
        c.run(40)
        assert same_bits(c.getDensityDistributions(*full(c)), want)


def test_checkpoint_errors(gpu, tmp_path):
    from cavityflow_cuda_gb300 import CLbmSolverGB300, LbmError

    ck = str(tmp_path / "a.ckpt")
    with CLbmSolverGB300((8, 8, 8), 1.6, 0.05, storage="f32") as a:
        a.run(4)
        a.save_checkpoint(ck)
    with CLbmSolverGB300((8, 8, 9), 1.6, 0.05, storage="f32") as other:
        with pytest.raises(LbmError) as ei:
            other.load_checkpoint(ck)
        assert ei.value.status == 1
    with CLbmSolverGB300((8, 8, 8), 1.6, 0.05, storage="f64") as other:
        with pytest.raises(LbmError):
            other.load_checkpoint(ck)
    data = open(ck, "rb").read()
    cut = tmp_path / "cut.ckpt"
    cut.write_bytes(data[:len(data) // 2])
    with pytest.raises(LbmError) as ei:
        CLbmSolverGB300.from_checkpoint(str(cut))
    assert ei.value.status == 7
    bad = tmp_path / "bad.ckpt"
    bad.write_bytes(b"X" + data[1:])
    with pytest.raises(LbmError) as ei:
        CLbmSolverGB300.from_checkpoint(str(bad))
    assert ei.value.status == 7
    with pytest.raises(LbmError) as ei:
        CLbmSolverGB300.from_checkpoint(str(tmp_path / "absent.ckpt"))
    assert ei.value.status == 7


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_vtk_matches_oracle_fields(gpu, oracle, tmp_path, dtype):
    from cavityflow_cuda_gb300 import CLbmSolverGB300

    n = (11, 7, 5)
    _, itau = orc.tau_of(0.032, dtype)
    lid = dtype(0.06)
    steps = 21
    dd, flags = oracle.run_cavity(*n, dtype, itau, lid, steps)
    rho, jx, jy, jz = (a[1:-1, 1:-1, 1:-1].reshape(-1) for a in
                       oracle.macros(dd, flags, last_was_alpha=bool(steps & 1), lid_u=lid))
    length = (2.2, 1.4, 1.0)
    with CLbmSolverGB300(n, itau, lid, storage="f64" if dtype == np.float64 else "f32") as s:
        s.run(steps)
        s.write_vtk(str(tmp_path / "b.vtk"), length=length, binary=True)
        s.write_vtk(str(tmp_path / "a.vtk"), length=length)
    b = read_vtk(str(tmp_path / "b.vtk"))
    a = read_vtk(str(tmp_path / "a.vtk"))
    tname = "double" if dtype == np.float64 else "float"
    for v in (a, b):
        assert v["version"] == "# vtk DataFile Version 3.0"
        assert v["dataset"] == "DATASET STRUCTURED_GRID" and v["dims"] == (12, 8, 6) and v["type"] == tname
        assert (v["flags"] == flags[1:-1, 1:-1, 1:-1].reshape(-1)).all()
    assert same_bits(b["densities"], rho)
    assert same_bits(b["velocities"][:, 0].copy(), jx) and same_bits(b["velocities"][:, 2].copy(), jz)
    assert same_bits(b["velocities"][:, 1].copy(), jy)
    # ASCII: 6 significant digits, as the reference's default stream precision
    np.testing.assert_allclose(a["densities"], rho, rtol=1e-5, atol=1e-30)
    np.testing.assert_allclose(a["velocities"], b["velocities"], rtol=1e-5, atol=1e-11)
    # corner points (i * length / n), x fastest
    T = dtype
    i, j, k = 3, 5, 2
    p = b["points"][(k * 8 + j) * 12 + i]
    want = [T(i) * T(length[0]) / T(n[0]), T(j) * T(length[1]) / T(n[1]), T(k) * T(length[2]) / T(n[2])]
    assert [float(x) for x in p] == [float(x) for x in want]


CONFIG = """<?xml version="1.0" encoding="ISO-8859-1"?>
<lbm-configuration>
  <physics>
    <velocity><x>0.05</x><y>0</y><z>0</z></velocity>
    <acceleration><x>0</x><y>0</y><z>0</z></acceleration>
    <viscosity>0.032</viscosity>
    <max-velocity>0.1</max-velocity>
    <max-acceleration>0.1</max-acceleration>
  </physics>
  <grid>
    <domain-size><x>{n}</x><y>{n}</y><z>{n}</z></domain-size>
    <domian-length><x>{n}</x><y>{n}</y><z>{n}</z></domian-length>
    <subdomain-num><x>1</x><y>1</y><z>1</z></subdomain-num>
    <cpu-subdomain-ratio>0.0</cpu-subdomain-ratio>
  </grid>
  <simulation>
    <loops>{loops}</loops>
    <timestep>1</timestep>
    <benchmark><do>1</do><output-dir>{d}/bench</output-dir></benchmark>
    <logging><do>{log}</do><output-dir>{d}/log</output-dir></logging>
    <validation><do>0</do><output-dir>{d}/valid</output-dir></validation>
    <visualization><do>1</do><rate>{rate}</rate><output-dir>{d}/vis</output-dir></visualization>
  </simulation>
  <cpu>
    <block-configuration>
      <alpha-block-configuration><x>32</x><y>32</y><z>32</z></alpha-block-configuration>
      <beta-block-configuration><x>32</x><y>32</y><z>32</z></beta-block-configuration>
    </block-configuration>
  </cpu>
  <gpu>
    <grid-configuration>
      <init-grid-configuration><x>32</x><y>16</y><z>1</z></init-grid-configuration>
      <alpha-grid-configuration><x>32</x><y>8</y><z>1</z></alpha-grid-configuration>
      <beta-grid-configuration><x>32</x><y>8</y><z>1</z></beta-grid-configuration>
    </grid-configuration>
  </gpu>
</lbm-configuration>
"""


def write_config(tmp_path, name, n, loops, rate, log=0):
    d = tmp_path / name
    for sub in ("bench", "log", "valid", "vis"):
        (d / sub).mkdir(parents=True, exist_ok=True)
    p = d / "config.xml"
    p.write_text(CONFIG.format(n=n, loops=loops, rate=rate, d=str(d), log=log))
    return str(p), d


def run_cli(*args):
    r = subprocess.run([CLI, *args], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    return r


@pytest.mark.parametrize("storage,dtype", [("f64", np.float64), ("f32", np.float32)])
def test_cli_runs_the_configuration(gpu, oracle, tmp_path, storage, dtype):
    from cavityflow_cuda_gb300 import configuration_lattice

    n, loops, rate = 20, 60, 20
    cfg, d = write_config(tmp_path, "run", n, loops, rate, log=1)
    run_cli(cfg, "--storage", storage, "--vtk-binary")
    vis = sorted(os.listdir(d / "vis"))
    assert vis == sorted(f"visualization_0_{i}.vtk" for i in (0, 20, 40, 60))
    bench = open(d / "bench" / "benchmark_0.txt").read().splitlines()
    assert [l.split(":")[0] for l in bench] == ["loops", "time", "iterations", "lattice updates", "bandwidth"]
    assert bench[0].split()[-1] == str(loops)
    assert bench[3].endswith("GLUPS") and bench[4].endswith("GBytes/s")
    log = open(d / "log" / "log_0.txt").read()
    assert "Do iteration 0:" in log and f"Iteration {loops - 1} successful." in log
    lat = configuration_lattice(cfg, storage)
    dd, flags = oracle.run_cavity(n, n, n, dtype, dtype(lat["inv_tau"]), dtype(lat["velocity"][0]), loops)
    rho, jx, jy, jz = (a[1:-1, 1:-1, 1:-1].reshape(-1) for a in
                       oracle.macros(dd, flags, last_was_alpha=False, lid_u=dtype(lat["velocity"][0])))
    v = read_vtk(str(d / "vis" / f"visualization_0_{loops}.vtk"))
    assert same_bits(v["densities"], rho) and same_bits(v["velocities"][:, 0].copy(), jx)
    assert same_bits(v["velocities"][:, 1].copy(), jy) and same_bits(v["velocities"][:, 2].copy(), jz)
    # step 0: the initial state (rho = 1, u = 0; the lid row reports its injected (1, U, 0, 0))
    dd0, flags0 = oracle.run_cavity(n, n, n, dtype, dtype(lat["inv_tau"]), dtype(lat["velocity"][0]), 0)
    rho0, jx0 = (a[1:-1, 1:-1, 1:-1].reshape(-1) for a in
                 oracle.macros(dd0, flags0, last_was_alpha=False, lid_u=dtype(lat["velocity"][0]))[:2])
    v0 = read_vtk(str(d / "vis" / "visualization_0_0.vtk"))
    assert same_bits(v0["densities"], rho0) and same_bits(v0["velocities"][:, 0].copy(), jx0)
    # (the 19 weights sum to 1 within one rounding)
    assert np.allclose(v0["densities"], 1, rtol=0, atol=4e-7) and (v0["velocities"][:, 1:] == 0).all()


def test_cli_checkpoint_resume_matches_uninterrupted(gpu, tmp_path):
    n, rate = 16, 50
    full_cfg, dfull = write_config(tmp_path, "full", n, 100, rate)
    run_cli(full_cfg, "--storage", "f32", "--vtk-binary")
    first_cfg, dfirst = write_config(tmp_path, "first", n, 57, rate)
    ck = str(tmp_path / "ck.bin")
    run_cli(first_cfg, "--storage", "f32", "--vtk-binary", "--checkpoint", ck, "--checkpoint-every", "19")
    # the last checkpoint is at step 57 - 57 % 19 = 57
    second_cfg, dsecond = write_config(tmp_path, "second", n, 100, rate)
    run_cli(second_cfg, "--storage", "f32", "--vtk-binary", "--resume", ck)
    assert sorted(os.listdir(dsecond / "vis")) == ["visualization_0_100.vtk"]
    a = open(dfull / "vis" / "visualization_0_100.vtk", "rb").read()
    b = open(dsecond / "vis" / "visualization_0_100.vtk", "rb").read()
    assert a == b


def test_cli_rejects_bad_arguments(gpu, tmp_path):
    cfg, _ = write_config(tmp_path, "bad", 8, 2, 1)
    for args in ([], [cfg, cfg], [cfg, "--storage", "f8"], [cfg, "--checkpoint-every", "3"],
                 [str(tmp_path / "absent.xml")]):
        r = subprocess.run([CLI, *args], capture_output=True, text=True, timeout=120)
        assert r.returncode == 1, args
