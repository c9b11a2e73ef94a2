"""Multi-process host logic of bench.py on CPU (gloo, world size 2): every rank
runs its own replica through bench.py's own timing helper (barrier on both
sides, maximum over ranks), the job's value counts every rank's slices, and
only rank 0 reports."""
import os
import socket
import subprocess
import sys

import pytest

from conftest import ROOT

WORKER = r"""
import json, os, sys, time
sys.path.insert(0, %r)
import torch.distributed as dist
import bench
dist.init_process_group("gloo")
rank, world = dist.get_rank(), dist.get_world_size()
# a replica's step: rank r takes (r + 1) * 20 ms; the job's time is the slowest rank's
ms, outs = bench.timed_steps(lambda: time.sleep(0.02 * (rank + 1)) or rank, 3, world, None)
value = bench.job_value(world, ms)
if rank == 0:
    print(json.dumps({"ms": ms, "value": value, "world": world, "outs": outs}))
dist.destroy_process_group()
""" % ROOT


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
    assert res["world"] == 2 and res["outs"] == [0, 0, 0]
    assert 40.0 <= res["ms"] < 60.0  # rank 1's 40 ms per step, not rank 0's 20
    assert res["value"] == pytest.approx(2 * 512 / (res["ms"] / 1e3))
    assert outs[1][0].strip() == ""


def test_reference_arm_other_ranks_exit_quietly():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                        "--steps", "1", "--warmup", "0"], env=env, capture_output=True, text=True,
                       timeout=120)
    assert r.returncode == 0 and r.stdout.strip() == ""


def test_reference_arm_json_contract():
    """`bench.py --impl reference` (the reference's algorithm, plain CGLS, on
    this host's cores through the oracle's C restatement) prints one JSON line
    with the benchmark's metric, the reference marker, a cpu_baseline that
    names its cores and sample, and an e2e object with no host-device bytes.
    A sample of 2 of the 1200 angles keeps this to seconds."""
    import json

    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                          "--steps", "1", "--warmup", "0", "--ref-angle-step", "600"],
                         capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [ln for ln in out.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    import bench

    assert d["metric"] == bench.METRIC and d["impl"] == "reference"
    assert d["unit"] == "slices/s" and d["higher_is_better"] is True and d["value"] > 0
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == d["value"]
    assert "2 of the 1200 angles" in cb["sample"] and cb["host"]["nproc"] >= 1
    assert d["e2e"] == {"value": d["value"], "unit": "slices/s", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}
