"""CPU: the multi-rank path of the bench (replicas, one process per GPU) with two gloo
ranks on the host. Each rank reports its own timed region; every rank gets the maximum
over ranks, and the whole-job rate is the frequency points of all ranks over the slowest
rank's time (a multi-GPU launch runs the same code with NCCL, one rank per GPU)."""
import json
import os
import socket
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent

SCRIPT = r"""
import json, os, sys
sys.path.insert(0, sys.argv[1])
import torch.distributed as dist
import bench
dist.init_process_group("gloo")
r = dist.get_rank()
out = bench.whole_job_rates(dist.get_world_size(), 5, 1.0 + r, 2.0 + 0.5 * r)
bench.barrier(dist.get_world_size())
print(json.dumps(out))
dist.destroy_process_group()
"""


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_gloo_ranks_report_the_whole_job_rate():
    port = str(_free_port())
    procs = []
    for r in range(2):
        env = dict(os.environ, RANK=str(r), WORLD_SIZE="2", LOCAL_RANK=str(r),
                   MASTER_ADDR="127.0.0.1", MASTER_PORT=port)
        procs.append(subprocess.Popen([sys.executable, "-c", SCRIPT, str(ROOT)], env=env,
                                      stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True))
    outs = []
    for p in procs:
        o, e = p.communicate(timeout=300)
        assert p.returncode == 0, e[-2000:]
        outs.append(json.loads(o.strip().splitlines()[-1]))
    for value, e2e, gpu_max, wall_max in outs:
        assert (gpu_max, wall_max) == (2.0, 2.5)         # the slowest rank's times
        assert value == 2 * 5 / 2.0 and e2e == 2 * 5 / 2.5


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, str(ROOT))
    import bench
    assert bench.whole_job_rates(1, 4, 2.0, 4.0) == (2.0, 1.0, 2.0, 4.0)
