"""Multi-process host logic of bench.py on CPU (gloo, world size 2): every rank
runs its own replica, the timing is the maximum over ranks, and only rank 0
reports."""
import os
import socket
import subprocess
import sys

import pytest

from conftest import ROOT

WORKER = r"""
import os, sys, json
import torch
import torch.distributed as dist
dist.init_process_group("gloo")
rank, world = dist.get_rank(), dist.get_world_size()
# a replica's local step time (ms); the job's time is the max over ranks
local = torch.tensor([10.0 + 5.0 * rank])
dist.barrier()
dist.all_reduce(local, op=dist.ReduceOp.MAX)
ms = float(local.item())
slices = 512
value = world * slices / (ms / 1e3)
if rank == 0:
    print(json.dumps({"ms": ms, "value": value, "world": world}))
dist.destroy_process_group()
"""


def free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def test_replicas_max_over_ranks(tmp_path):
    script = tmp_path / "w.py"
    script.write_text(WORKER)
    port = free_port()
    procs = []
    for r in range(2):
        env = dict(os.environ, RANK=str(r), WORLD_SIZE="2", LOCAL_RANK=str(r),
                   MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
        procs.append(subprocess.Popen([sys.executable, str(script)], env=env,
                                      stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True))
    outs = [p.communicate(timeout=120) for p in procs]
    assert all(p.returncode == 0 for p in procs), [o[1][-500:] for o in outs]
    import json

    res = json.loads(outs[0][0].strip().splitlines()[-1])
    assert res["ms"] == 15.0 and res["world"] == 2
    assert res["value"] == pytest.approx(2 * 512 / 0.015)
    assert outs[1][0].strip() == ""


def test_reference_arm_other_ranks_exit_quietly():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                        "--steps", "1", "--warmup", "0"], env=env, capture_output=True, text=True,
                       timeout=120)
    assert r.returncode == 0 and r.stdout.strip() == ""
