"""The multi-process control path of bench.py (replicas, barrier, max over ranks) with two gloo
ranks on the CPU: every rank reports its own time and rank 0 sees the maximum."""
import os
import re
import socket
import subprocess
import sys
import textwrap
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent


def free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_gloo_ranks_max_over_ranks(tmp_path):
    script = tmp_path / "ranks.py"
    script.write_text(textwrap.dedent(f"""
        import sys
        sys.path.insert(0, {str(ROOT)!r})
        import bench
        d = bench.Dist()
        d.barrier()
        t = d.max(1.5 + d.rank)          # rank r "took" 1.5 + r seconds
        d.barrier()
        print(f"rank={{d.rank}} world={{d.world}} max={{t}}", flush=True)
        d.close()
    """))
    env = dict(os.environ, ATX_BENCH_BACKEND="gloo", MASTER_ADDR="127.0.0.1")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node=2",
           "--master-addr", "127.0.0.1", "--master-port", str(free_port()), str(script)]
    out = subprocess.run(cmd, env=env, capture_output=True, text=True, timeout=240)
    assert out.returncode == 0, out.stderr[-2000:]
    # the ranks share one stdout, so their lines may interleave
    got = sorted(re.findall(r"rank=\d+ world=\d+ max=[0-9.]+", out.stdout))
    assert got == ["rank=0 world=2 max=2.5", "rank=1 world=2 max=2.5"]
