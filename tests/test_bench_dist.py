"""The multi-process path of bench.py on CPU (gloo, world size 2): replicas
aggregate whole-job throughput as the sum of the ranks' work over the
slowest rank's time, and the reference arm runs on rank 0 only."""
import json
import os
import re
import socket
import subprocess
import sys

import pytest

from conftest import ROOT

HELPER = r'''
import sys
sys.path.insert(0, %r)
import bench
d = bench.Dist()
s = d.sum(d.rank + 1.0)
m = d.max(float(d.rank) * 10.0)
d.barrier()
print("RANK%%d %%g %%g" %% (d.rank, s, m), flush=True)
'''


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _torchrun(args, timeout=300):
    pytest.importorskip("torch")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node=2",
           "--master-addr=127.0.0.1", "--master-port=%d" % _free_port()] + args
    return subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=timeout,
                          env=dict(os.environ, OMP_NUM_THREADS="1"))


def test_dist_sum_and_max(tmp_path):
    script = tmp_path / "agg.py"
    script.write_text(HELPER % ROOT)
    r = _torchrun([str(script)])
    assert r.returncode == 0, r.stderr[-2000:]
    # the ranks share one stdout, so their lines may interleave
    lines = sorted(re.findall(r"RANK\d \S+ \S+?(?=RANK|\s|$)", r.stdout))
    assert lines == ["RANK0 3 10", "RANK1 3 10"]


def test_reference_arm_rank0_only():
    import build_ref_path  # noqa: F401  (skips when the reference sources are absent)
    r = _torchrun(["bench.py", "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "0"], timeout=900)
    assert r.returncode == 0, r.stderr[-2000:]
    out = [json.loads(l) for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(out) == 1 and out[0]["impl"] == "reference"
    assert out[0]["e2e"]["h2d_bytes_per_step"] == 0 and out[0]["cpu_baseline"]["kind"] == "reference"
