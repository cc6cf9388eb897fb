"""The N > 1 bench path: the engine does not shard (one independent replica
per GPU, no collective on the data path); the only cross-rank step is the
max over ranks of the timed region, tested here with gloo on CPU."""
import os
import subprocess
import sys

import pytest

from conftest import ROOT

SCRIPT = r'''
import os, sys
sys.path.insert(0, {root!r})
import torch.distributed as dist
dist.init_process_group("gloo")
import bench
r = dist.get_rank()
v = bench.max_over_ranks(10.0 + 5.0 * r)
assert v == 15.0, v
print("rank", r, "ok", flush=True)
dist.destroy_process_group()
'''


def test_max_over_ranks_gloo(tmp_path):
    script = tmp_path / "mx.py"
    script.write_text(SCRIPT.format(root=ROOT))
    env = dict(os.environ, MASTER_ADDR="127.0.0.1")
    r = subprocess.run([sys.executable, "-m", "torch.distributed.run", "--nnodes=1",
                        "--nproc-per-node=2", "--master-addr=127.0.0.1", "--master-port=29533",
                        str(script)], capture_output=True, text=True, env=env, timeout=240)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.count("ok") == 2


def test_reference_arm_nonzero_rank_prints_nothing():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                        "--steps", "1", "--warmup", "3"], capture_output=True, text=True,
                       env=env, timeout=120)
    assert r.returncode == 0
    assert r.stdout.strip() == ""


def test_single_process_max_is_identity():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(3.5) == 3.5
