"""The C++ drop-in (include/CLbmSolverGB300.hpp) built the way a maintainer of
the reference would use it: compiled with the reference's own headers and its
CConfiguration, CDomain and CLbmSolver sources (src/CLbmSolver.hpp:30-89,
src/CLbmSolverGPU.cuh:25-95, compiled where they lie in the checkout named by
LBM_REFERENCE_DIR) and linked against liblbm_gb300.so.  Without a GPU the
adapter's constructor must report the missing device and exit with
LBM_ERR_NO_DEVICE, as the reference's GPU solver exits through
GPU_ERROR_CHECK; with one, its alpha/beta steps must equal the Python
binding's bit for bit.  Skipped where no reference checkout exists."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN, ROOT
from oracle import oracle as orc

HERE = os.path.join(ROOT, "tests", "dropin")


@pytest.fixture(scope="module")
def dropin(lib, tmp_path_factory):
    src = orc.reference_src()
    if src is None:
        pytest.skip("reference checkout not present (LBM_REFERENCE_DIR)")
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    out = {}
    build = tmp_path_factory.mktemp("dropin")
    pkg = os.path.join(ROOT, "cavityflow_cuda_gb300")
    ref_sources = [os.path.join(src, f) for f in ("CLbmSolver.cpp", "CConfiguration.cpp", "CDomain.cpp",
                                                  "libmath/CMath.cpp", "libmath/CVector3.cpp")]
    ref_sources.append(os.path.join(src, "..", "external", "tinyxml2", "tinyxml2.cpp"))
    for tag, real in (("f32", "float"), ("f64", "double")):
        exe = str(build / f"dropin_{tag}")
        cmd = [cxx, "-O1", "-w", f"-DDROPIN_REAL={real}", f"-I{src}", f"-I{os.path.join(ROOT, 'include')}",
               "-I/usr/local/cuda/include", os.path.join(HERE, "dropin_main.cpp"), *ref_sources, "-o", exe,
               f"-L{pkg}", "-llbm_gb300", "-L/usr/local/cuda/lib64", "-lcudart", f"-Wl,-rpath,{pkg}"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        assert r.returncode == 0, r.stderr[-3000:]
        out[tag] = exe
    return out


@pytest.mark.parametrize("tag", ["f32", "f64"])
def test_dropin_builds_against_reference_and_runs(dropin, tag, tmp_path):
    import torch

    xml = os.path.join(GOLDEN, "configs", "cavity64_re100.xml")
    small = tmp_path / "cavity.xml"
    text = open(xml).read()
    for tag_ in ("domain-size", "domian-length"):  # the reference's cells must be cubes (CConfiguration.cpp:185)
        text = text.replace(f"<x>64</x><y>64</y><z>64</z></{tag_}>", f"<x>20</x><y>14</y><z>11</z></{tag_}>")
    small.write_text(text)
    res = tmp_path / "dd.bin"
    r = subprocess.run([dropin[tag], str(small), "24", str(res)], capture_output=True, text=True, timeout=300)
    if not torch.cuda.is_available():
        assert r.returncode == 10, (r.returncode, r.stdout, r.stderr)
        assert "no CUDA device" in r.stderr
        return
    assert r.returncode == 0, r.stderr
    from cavityflow_cuda_gb300 import CLbmSolverGB300, configuration_lattice

    lat = configuration_lattice(str(small), storage=tag)
    dtype = np.float64 if tag == "f64" else np.float32
    got = np.fromfile(res, dtype=dtype).reshape(19, 11, 14, 20)
    with CLbmSolverGB300((20, 14, 11), lat["inv_tau"], lat["velocity"][0], storage=tag) as s:
        s.run(24)
        want = s.getDensityDistributions()
    assert np.array_equal(got.view(np.uint8), want.view(np.uint8))
