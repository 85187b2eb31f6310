"""The bench's N > 1 path on the CPU: one process per GPU, host-side reductions over gloo
(world size 2, 127.0.0.1). The colonies of the ranks are independent replicas, so the data path
has no collective; what crosses ranks is the timing: the barrier before the timed region, the
maximum of the ranks' device times and the sum of their particle-steps. The reference arm runs
on rank 0 alone; the other ranks join the group and exit 0 without work or output."""
import json
import os
import socket
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def launch(code: str, world: int, port: int, args=None):
    procs = []
    for r in range(world):
        env = dict(os.environ, RANK=str(r), LOCAL_RANK=str(r), WORLD_SIZE=str(world), MASTER_ADDR="127.0.0.1",
                   MASTER_PORT=str(port))
        cmd = [sys.executable, "-c", code] if args is None else [sys.executable] + args[r]
        procs.append(subprocess.Popen(cmd, cwd=ROOT, env=env, stdout=subprocess.PIPE, stderr=subprocess.PIPE,
                                      text=True))
    outs = [p.communicate(timeout=120) for p in procs]
    return [(p.returncode, o, e) for p, (o, e) in zip(procs, outs)]


RANK_CODE = """
import json, os, sys
sys.path.insert(0, os.getcwd())
import bench
rank, world, dist = bench.dist_init(2)
bench.barrier(dist)
dev_s = [0.25, 0.5][rank]             # device seconds of this rank's timed region
psteps = [2.0e9, 2.2e9][rank]         # particle-steps this rank processed
t_max = bench.allreduce_max(dist, dev_s)
ps_all = bench.allreduce_sum(dist, psteps)
print(json.dumps(dict(rank=rank, world=world, t_max=t_max, ps_all=ps_all, value=ps_all / t_max)))
dist.destroy_process_group()
"""


def test_rank_reductions_over_gloo():
    res = launch(RANK_CODE, 2, free_port())
    for rc, out, err in res:
        assert rc == 0, err
    lines = [json.loads(o.strip().splitlines()[-1]) for _, o, _ in res]
    assert sorted(x["rank"] for x in lines) == [0, 1]
    for x in lines:
        assert x["world"] == 2 and x["t_max"] == 0.5 and x["ps_all"] == 4.2e9
        assert x["value"] == 4.2e9 / 0.5  # whole-job throughput: all ranks' work over the slowest rank


JOIN_CODE = """
import os, sys
sys.path.insert(0, os.getcwd())
import bench
rank, world, dist = bench.dist_init(2)
dist.destroy_process_group()
"""


def test_reference_arm_runs_on_rank_zero_only():
    """Rank 1 of a two-rank reference run joins the group and exits 0 with no output (rank 0
    is played by a process that only joins: the real one times the CPU restatement)."""
    port = free_port()
    res = launch(None, 2, port, args=[["-c", JOIN_CODE],
                                      ["bench.py", "--impl", "reference", "--gpus", "2", "--steps", "1",
                                       "--warmup", "3"]])
    for rc, out, err in res:
        assert rc == 0, err
    assert res[1][1].strip() == ""
