"""The N>1 path of bench.py on CPU: world_size-2 gloo ranks (replicas only).

Frames are independent, so N GPUs run N replicas with no data-path collective;
the only cross-rank traffic is the barrier and the max-over-ranks reduction of
the timed region.  These tests run that logic with two gloo ranks on the host
and check the reference arm's rank rule (rank 0 alone prints; the rest exit 0).
"""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


WORKER = r"""
import os, sys, json
sys.path.insert(0, os.environ["ROOT"])
import torch.distributed as dist
import bench
dist.init_process_group("gloo")
rank = dist.get_rank()
t = bench.max_over_ranks(dist, 1.0 + rank)      # rank r took 1 + r seconds
dist.barrier()
print(json.dumps({"rank": rank, "t": t, "info": bench.dist_info()}), flush=True)
dist.destroy_process_group()
"""


def _run_two(code: str, extra_env=None):
    env = dict(os.environ, ROOT=ROOT, MASTER_ADDR="127.0.0.1", MASTER_PORT=str(_free_port()), WORLD_SIZE="2")
    env.update(extra_env or {})
    procs = []
    for r in range(2):
        e = dict(env, RANK=str(r), LOCAL_RANK=str(r))
        procs.append(subprocess.Popen([sys.executable, "-c", code], env=e, stdout=subprocess.PIPE,
                                      stderr=subprocess.PIPE, text=True))
    outs = [p.communicate(timeout=120) for p in procs]
    return [(p.returncode, o, e) for p, (o, e) in zip(procs, outs)]


def test_max_over_ranks_with_two_gloo_ranks():
    pytest.importorskip("torch")
    res = _run_two(WORKER)
    lines = []
    for rc, out, err in res:
        assert rc == 0, err
        lines.append(json.loads(out.strip().splitlines()[-1]))
    assert sorted(l["rank"] for l in lines) == [0, 1]
    assert all(l["t"] == 2.0 for l in lines)          # both see the slowest rank
    assert all(l["info"][1] == 2 for l in lines)


def test_reference_arm_rank_rule():
    # under torchrun the reference arm runs on rank 0 only; rank 1 exits 0 without output
    pytest.importorskip("torch")
    code = ("import os, sys; sys.path.insert(0, os.environ['ROOT']); import bench;"
            "sys.argv=['bench.py','--impl','reference','--gpus','2','--steps','1','--warmup','0',"
            "'--workload','car_640x480_fp32'];"
            "import oracle.oracle as O;"
            "rank=int(os.environ['RANK']);"
            "sys.exit(bench.main() if rank == 1 else 0)")
    res = _run_two(code)
    assert res[1][0] == 0 and res[1][1].strip() == ""
