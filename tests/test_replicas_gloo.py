"""bench.py's multi-process path on the host: torchrun with two ranks on gloo (no GPU).

Replicas only (the path shards into independent instances; nothing is exchanged but the
barrier and the max of the ranks' times).  Checks that the rank helpers agree across
processes and that the reference arm prints exactly one JSON line, from rank 0, with
n_gpus = 2, while the other rank exits 0 without work.
"""

import json
import os
import socket
import subprocess
import sys
import textwrap
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def torchrun(args, tmp_path, timeout=300):
    env = dict(os.environ, CUDA_VISIBLE_DEVICES="", OMP_NUM_THREADS="2")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes", "1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(free_port())] + args
    return subprocess.run(cmd, capture_output=True, text=True, timeout=timeout, cwd=ROOT, env=env)


def test_rank_helpers_agree_on_gloo(tmp_path):
    script = tmp_path / "ranks.py"
    script.write_text(textwrap.dedent(f"""
        import sys
        sys.path.insert(0, {str(ROOT)!r})
        import bench
        rank, ws = bench.dist_init()
        bench.barrier(ws)
        m = bench.allreduce_max(float(rank + 1), ws)
        with open({str(tmp_path)!r} + f"/rank{{rank}}.txt", "w") as f:  # stdout of the ranks interleaves
            f.write(f"rank {{rank}} of {{ws}} max {{m}}")
        import torch.distributed as dist
        dist.destroy_process_group()
    """))
    r = torchrun([str(script)], tmp_path)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [(tmp_path / f"rank{k}.txt").read_text() for k in range(2)]
    assert lines == ["rank 0 of 2 max 2.0", "rank 1 of 2 max 2.0"]


def test_reference_arm_prints_once_from_rank0(tmp_path):
    pytest.importorskip("numpy")
    r = torchrun(["bench.py", "--impl", "reference", "--steps", "1", "--warmup", "0"], tmp_path)
    assert r.returncode == 0, r.stderr[-2000:]
    js = [json.loads(l) for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(js) == 1
    line = js[0]
    assert line["impl"] == "reference" and line["n_gpus"] == 2 and line["value"] > 0
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["cpu_baseline"]["kind"] == "port"
