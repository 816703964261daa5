"""The padded population layout (make_grid in csrc/lbm_core.cuh), checked on
the CPU for every row layout (the default 32-byte one, a 16-byte one and the
packed 8-byte one of batches and servers) and every storage width: the
invariants the vectorised kernels' memory accesses rely on."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CORE = os.path.join(HERE, "..", "cavityflow_cuda_gb300", "csrc", "lbm_core.cuh")

PROGRAM = r"""
#include <cstdio>
#include "%s"
// Prints one line per violated invariant; nothing when all hold.
int main()
{
    int bad = 0;
    const int widths[3] = {2, 4, 8};
    const int aligns[3] = {8, 16, 32};
    for (int eb : widths)
        for (int al : aligns)
            for (int nx = 1; nx <= 300; ++nx)
                for (int ny = 1; ny <= 3; ++ny) {
                    const int nz = 2;
                    const lbm::Grid g = lbm::make_grid(nx, ny, nz, eb, al);
                    const long long x1 = (long long)(g.xoff + 1) * eb;  // byte column of x = 1
                    const long long last = g.xoff + (long long)g.G * g.V;  // last column of the last vector
                    if (g.xoff < 0) { printf("xoff<0 eb=%%d al=%%d nx=%%d\n", eb, al, nx); ++bad; }
                    if (x1 %% al != 0) { printf("x1 eb=%%d al=%%d nx=%%d\n", eb, al, nx); ++bad; }
                    if ((g.P * eb) %% al != 0) { printf("pitch eb=%%d al=%%d nx=%%d\n", eb, al, nx); ++bad; }
                    // the last vector, and a window shifted one cell right of it, stay in the row
                    if (last + 1 > g.P - 1) { printf("room eb=%%d al=%%d nx=%%d\n", eb, al, nx); ++bad; }
                    // rows sized for vectors as wide as x = 1's alignment (16 bytes at most)
                    if ((long long)g.G * g.V < nx || g.V * eb != (al < 16 ? al : 16)) { printf("groups eb=%%d nx=%%d\n", eb, nx); ++bad; }
                    // a variant's vectors fit exactly when they are no wider than that
                    for (int vb = 2; vb <= 16; vb *= 2)
                        if (vb >= eb && lbm::vector_fits(g, eb, vb) != (vb <= (al < 16 ? al : 16))) { printf("fits eb=%%d al=%%d vb=%%d\n", eb, al, vb); ++bad; }
                    if (g.PY != g.P * (ny + 2)) { printf("plane eb=%%d nx=%%d\n", eb, nx); ++bad; }
                    if ((g.S * eb) %% 256 != 0 || g.S < g.PY * (nz + 2)) { printf("slot eb=%%d al=%%d nx=%%d\n", eb, al, nx); ++bad; }
                    if (lbm::default_layout(g, eb) != (al == 32)) { printf("default eb=%%d al=%%d\n", eb, al); ++bad; }
                    // interior cells map to distinct columns inside the row
                    if (g.idx(nx + 1, 0, 0) - g.idx(0, 0, 0) != nx + 1 || g.idx(0, 1, 0) - g.idx(0, 0, 0) != g.P) {
                        printf("idx eb=%%d nx=%%d\n", eb, nx); ++bad;
                    }
                }
    printf("checked\n");
    return bad != 0;
}
"""


@pytest.mark.skipif(shutil.which("nvcc") is None, reason="nvcc not found")
def test_layout_invariants(tmp_path):
    src = tmp_path / "layout.cu"
    src.write_text(PROGRAM % os.path.abspath(CORE).replace("\\", "/"))
    exe = tmp_path / "layout"
    subprocess.run(["nvcc", "-std=c++17", "-o", str(exe), str(src)], check=True, capture_output=True, timeout=300)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0 and r.stdout.strip().endswith("checked"), r.stdout[-2000:]
