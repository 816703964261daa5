"""bench.py's multi-rank path on CPU (gloo, world size 2): replicas report
the slowest rank's time and the units of all ranks; the reference arm runs
on rank 0 only."""
import os
import subprocess
import sys
import textwrap

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

WORKER = textwrap.dedent("""
    import json, os, sys
    sys.path.insert(0, {root!r})
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo")
    rank, world = dist.get_rank(), dist.get_world_size()
    ms, ups = bench.combine_ranks(100.0 * (rank + 1), 1000.0, world, device="cpu")
    # one file per rank: the launcher may interleave the ranks' stdout
    with open(os.path.join({out!r}, f"rank{{rank}}.json"), "w") as fh:
        fh.write(json.dumps({{"rank": rank, "ms": ms, "ups": ups}}))
    dist.destroy_process_group()
""")


def _torchrun(script, nproc=2, extra_env=None):
    env = dict(os.environ, **(extra_env or {}))
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", f"--nproc-per-node={nproc}",
           "--master-addr", "127.0.0.1", "--master-port", "29533", script]
    return subprocess.run(cmd, capture_output=True, text=True, timeout=240, env=env, cwd=ROOT)


def test_replicas_take_the_slowest_rank(tmp_path):
    import json

    script = tmp_path / "worker.py"
    script.write_text(WORKER.format(root=ROOT, out=str(tmp_path)))
    r = _torchrun(str(script))
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [json.loads(open(tmp_path / f"rank{i}.json").read()) for i in range(2)]
    assert len(lines) == 2
    for d in lines:
        assert d["ms"] == 200.0                      # max over ranks
        assert abs(d["ups"] - 2 * 1000.0 / 0.2) < 1e-9  # units of both ranks / slowest time


def test_reference_arm_runs_on_rank0_only(tmp_path):
    """Under torchrun only rank 0 prints the reference line."""
    script = tmp_path / "ref.py"
    script.write_text(textwrap.dedent(f"""
        import sys
        sys.path.insert(0, {ROOT!r})
        sys.argv = ["bench.py", "--impl", "reference", "--size", "16", "--steps", "4", "--warmup", "3"]
        import bench
        bench.main()
    """))
    r = _torchrun(str(script))
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1 and '"impl": "reference"' in lines[0]
