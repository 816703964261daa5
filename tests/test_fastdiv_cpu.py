"""FastDiv (csrc/lbm_core.cuh), the multiply-and-shift division by a
run-time constant (Granlund and Montgomery, "Division by invariant integers
using multiplication", 1994) that the batch kernel and the plane-indexed
grids use for their thread indices: checked on the CPU against exact
division for every divisor up to 2^17 and selected larger ones."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CORE = os.path.join(HERE, "..", "cavityflow_cuda_gb300", "csrc", "lbm_core.cuh")

PROGRAM = r"""
#include <cstdio>
#include <cstdint>
#include "%s"
static int check(uint32_t d, uint32_t n)
{
    const lbm::FastDiv f = lbm::FastDiv::make(d);
    if (f.div(n) != n / d) { printf("d=%%u n=%%u got %%u\n", d, n, f.div(n)); return 1; }
    return 0;
}
int main()
{
    int bad = 0;
    uint64_t x = 0x9E3779B97F4A7C15ull;  // xorshift64 numerators
    auto next = [&]() { x ^= x << 13; x ^= x >> 7; x ^= x << 17; return (uint32_t)(x >> 16); };
    for (uint64_t d = 1; d <= (1u << 17) && bad < 20; ++d) {
        const uint32_t dd = (uint32_t)d;
        const uint32_t edge[] = {0u, 1u, dd - 1, dd, dd + 1, 2 * dd - 1, 2 * dd, 0xFFFFFFFFu, 0xFFFFFFFEu,
                                 0xFFFFFFFFu / dd * dd, 0xFFFFFFFFu / dd * dd - 1, 0x80000000u, 0x7FFFFFFFu};
        for (uint32_t n : edge) bad += check(dd, n);
        for (int i = 0; i < 64; ++i) bad += check(dd, next());
    }
    const uint32_t big[] = {(1u << 20) + 1, 3000017u, (1u << 24) - 3, 0x7FFFFFFFu, 0x80000000u, 0x80000001u,
                            0xFFFFFFFEu, 0xFFFFFFFFu};
    for (uint32_t d : big) {
        for (int i = 0; i < 100000; ++i) bad += check(d, next());
        bad += check(d, 0xFFFFFFFFu) + check(d, d - 1) + check(d, d);
    }
    printf("checked\n");
    return bad != 0;
}
"""


@pytest.mark.skipif(shutil.which("nvcc") is None, reason="nvcc not found")
def test_fastdiv_matches_exact_division(tmp_path):
    src = tmp_path / "fastdiv.cu"
    src.write_text(PROGRAM % os.path.abspath(CORE).replace("\\", "/"))
    exe = tmp_path / "fastdiv"
    subprocess.run(["nvcc", "-std=c++17", "-O2", "-o", str(exe), str(src)], check=True, capture_output=True,
                   timeout=300)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and r.stdout.strip().endswith("checked"), r.stdout[-2000:]
