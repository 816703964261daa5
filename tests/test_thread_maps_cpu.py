"""The kernels' thread-to-cell maps in csrc/lbm_fast.cuh, checked on the
CPU: the batch kernel's (set_batch_shape, cells_of_vblock) and the single
domain's plane grid (cells_of_plane).  For boxes of many shapes, every
cells-per-thread and block size of the launch menu and both kernels, each
group of cells of each row is visited by exactly one active thread, and only
threads past the last group are inactive."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
FAST = os.path.join(HERE, "..", "cavityflow_cuda_gb300", "csrc", "lbm_fast.cuh")

PROGRAM = r"""
#include <cstdio>
#include <vector>
#include "%s"
int main()
{
    int bad = 0;
    const int sizes[][3] = {{1, 1, 1}, {3, 4, 5}, {16, 16, 16}, {17, 9, 3}, {33, 1, 7}, {1, 40, 2}, {96, 17, 11},
                            {5, 96, 9}, {130, 3, 4}, {64, 64, 8}, {7, 7, 90}};
    const int cpts[] = {1, 2, 4, 8};
    const int blocks[] = {64, 128, 256};
    for (const auto& n : sizes)
        for (int eb : {2, 4, 8})
            for (int cpt : cpts)
                for (int block : blocks)
                    for (int kind = 0; kind < 2; ++kind) {
                        lbm::BatchDomain d{};
                        d.g = lbm::make_grid(n[0], n[1], n[2], eb, lbm::kPackedX1Align);
                        const long long vbs = lbm::set_batch_shape(d, kind, cpt, block);
                        const long long G = (n[0] + cpt - 1) / cpt;
                        const long long groups = G * n[1] * n[2];
                        if (vbs != (groups + block - 1) / block) { printf("blocks %%d %%d %%d\n", n[0], cpt, block); ++bad; }
                        std::vector<int> seen((size_t)groups, 0);
                        for (long long t = 0; t < vbs * block; ++t) {
                            const lbm::Cells c = lbm::cells_of_vblock(d, kind, (uint32_t)t);
                            if (!c.active) {
                                if (t < groups) { printf("inactive t=%%lld size %%dx%%dx%%d cpt %%d\n", t, n[0], n[1], n[2], cpt); ++bad; }
                                continue;
                            }
                            if (t >= groups || c.gi < 0 || c.gi >= G || c.y < 1 || c.y > n[1] || c.z < 1 || c.z > n[2]) {
                                printf("range t=%%lld\n", t); ++bad; continue;
                            }
                            ++seen[(size_t)(((long long)(c.z - 1) * n[1] + (c.y - 1)) * G + c.gi)];
                        }
                        for (long long i = 0; i < groups; ++i)
                            if (seen[(size_t)i] != 1) { printf("group %%lld seen %%d\n", i, seen[(size_t)i]); ++bad; break; }
                        if (bad > 20) { printf("checked\n"); return 1; }
                    }
    printf("checked\n");
    return bad != 0;
}
"""


@pytest.mark.skipif(shutil.which("nvcc") is None, reason="nvcc not found")
def test_batch_thread_map_covers_every_group_once(tmp_path):
    src = tmp_path / "batchmap.cu"
    src.write_text(PROGRAM % os.path.abspath(FAST).replace("\\", "/"))
    exe = tmp_path / "batchmap"
    subprocess.run(["nvcc", "-std=c++17", "-O2", "-gencode", "arch=compute_103a,code=sm_103a", "-o", str(exe),
                    str(src)], check=True, capture_output=True, timeout=600)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and r.stdout.strip().endswith("checked"), r.stdout[-2000:]


PLANE_PROGRAM = r"""
#include <cstdio>
#include <vector>
#include "%s"
// The single-domain kernels' grid: x over the G * ny groups of a plane in
// blocks of `block` threads (ceil(G * ny / block) blocks, as the launcher
// computes them), y over planes.
int main()
{
    int bad = 0;
    const int sizes[][2] = {{1, 1}, {3, 4}, {17, 9}, {384, 384}, {130, 3}, {1, 300}, {512, 7}, {97, 61}};
    for (const auto& n : sizes)
        for (int eb : {2, 4, 8})
            for (int cpt : {1, 2, 4, 8})
                for (int block : {64, 128, 256}) {
                    const lbm::Grid g = lbm::make_grid(n[0], n[1], 3, eb);
                    const int G = (g.nx + cpt - 1) / cpt;
                    const lbm::FastDiv divG = lbm::FastDiv::make((uint32_t)G);
                    const long long per_plane = (long long)G * g.ny;
                    const long long bx = (per_plane + block - 1) / block;
                    std::vector<int> seen((size_t)per_plane, 0);
                    for (long long i = 0; i < bx * block; ++i) {
                        const lbm::Cells c = lbm::cells_of_plane(g, G, divG, (uint32_t)i, 2);
                        if (!c.active) {
                            if (i < per_plane) { printf("inactive %%lld\n", i); ++bad; }
                            continue;
                        }
                        if (c.gi < 0 || c.gi >= G || c.y < 1 || c.y > g.ny || c.z != 2) { printf("range %%lld\n", i); ++bad; continue; }
                        ++seen[(size_t)((c.y - 1) * (long long)G + c.gi)];
                    }
                    for (long long i = 0; i < per_plane; ++i)
                        if (seen[(size_t)i] != 1) { printf("group %%lld seen %%d\n", i, seen[(size_t)i]); ++bad; break; }
                }
    printf("checked\n");
    return bad != 0;
}
"""


@pytest.mark.skipif(shutil.which("nvcc") is None, reason="nvcc not found")
def test_plane_thread_map_covers_every_group_once(tmp_path):
    src = tmp_path / "planemap.cu"
    src.write_text(PLANE_PROGRAM % os.path.abspath(FAST).replace("\\", "/"))
    exe = tmp_path / "planemap"
    subprocess.run(["nvcc", "-std=c++17", "-O2", "-gencode", "arch=compute_103a,code=sm_103a", "-o", str(exe),
                    str(src)], check=True, capture_output=True, timeout=600)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and r.stdout.strip().endswith("checked"), r.stdout[-2000:]
