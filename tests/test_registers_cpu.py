"""Register budgets of the default kernels, checked on the CPU from ptxas's
resource report (-Xptxas -v) of the per-storage translation units.

The step kernels stream at the HBM roofline only while their populations
stay in registers: a spill adds local-memory traffic to every cell, and a
kernel that needs more registers than its shape allows runs fewer warps.
These are the shapes the library launches by default (single domain: FP32
variant 13, the 16-bit storages variant 20; batches: FP32 variant 17, the
16-bit storages variant 22).  Two of the limits guard measured regressions:
bfloat16 widened by a shift took the 8-cell alpha from 168 to 239 registers,
and the batch kernel's packed beta spills at 102 registers (so its default
has 128)."""
import os
import re
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "..", "cavityflow_cuda_gb300", "csrc")

# (translation unit, demangled kernel name, most registers or None, most spilled bytes)
BUDGETS = [
    ("fast_f32.cu", "lbm::alpha_fast<lbm::F32, 2, 64, 8>", None, 0),
    ("fast_f32.cu", "lbm::beta_fast_direct<lbm::F32, 2, 64, 8>", None, 0),
    # the batch alpha holds its domain's layout in registers and spills a little (48 bytes,
    # cached in L1; a variant without the spill measured no faster)
    ("fast_f32.cu", "lbm::batch_step<lbm::F32, 2, 256, 2, true, 2>", None, 48),
    ("fast_f32.cu", "lbm::batch_step<lbm::F32, 2, 256, 2, false, 2>", None, 0),
    ("fast_f16sr.cu", "lbm::alpha_fast<lbm::F16SR, 8, 64, 4>", 168, 0),
    ("fast_f16sr.cu", "lbm::beta_fast_pk<lbm::F16SR, 4, 64, 10, true>", 96, 16),
    ("fast_f16sr.cu", "lbm::batch_step<lbm::F16SR, 4, 64, 8, true, 4>", None, 0),
    ("fast_f16sr.cu", "lbm::batch_step<lbm::F16SR, 4, 64, 8, false, 4>", None, 8),
    ("fast_bf16s.cu", "lbm::alpha_fast<lbm::BF16S, 8, 64, 4>", 168, 0),
    ("fast_bf16s.cu", "lbm::beta_fast_pk<lbm::BF16S, 4, 64, 10, true>", 96, 16),
    ("fast_bf16s.cu", "lbm::batch_step<lbm::BF16S, 4, 64, 8, true, 4>", None, 0),
]


def ptxas_report(unit: str, out_dir: str) -> dict:
    """{mangled kernel name: (registers, spill store bytes)} for one translation unit."""
    cmd = ["nvcc", "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17", "-fmad=false", "-Xptxas",
           "-v", "-c", os.path.join(CSRC, unit), "-o", os.path.join(out_dir, unit + ".o")]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stderr[-2000:]
    report, name = {}, None
    for line in (r.stdout + r.stderr).splitlines():
        m = re.search(r"Compiling entry function '(\S+)'", line)
        if m:
            name = m.group(1)
            report[name] = [None, None]
            continue
        if name is None:
            continue
        m = re.search(r"(\d+) bytes spill stores", line)
        if m:
            report[name][1] = int(m.group(1))
        m = re.search(r"Used (\d+) registers", line)
        if m:
            report[name][0] = int(m.group(1))
    return report


@pytest.mark.skipif(shutil.which("nvcc") is None or shutil.which("c++filt") is None,
                    reason="nvcc and c++filt are needed")
def test_default_kernels_fit_their_register_budgets(tmp_path):
    units = sorted({u for u, *_ in BUDGETS})
    with ThreadPoolExecutor(len(units)) as pool:
        reports = dict(zip(units, pool.map(lambda u: ptxas_report(u, str(tmp_path)), units)))
    for unit, prefix, max_regs, max_spill in BUDGETS:
        mangled = list(reports[unit])
        names = subprocess.run(["c++filt"], input="\n".join(mangled), capture_output=True, text=True,
                               check=True).stdout.splitlines()
        hits = [reports[unit][m] for m, n in zip(mangled, names) if n.split("(")[0] == "void " + prefix]
        assert len(hits) == 1, (unit, prefix, len(hits))
        regs, spill = hits[0]
        assert spill is not None and spill <= max_spill, (prefix, regs, spill)
        if max_regs is not None:
            assert regs <= max_regs, (prefix, regs, spill)
