"""The bench's multi-GPU path (independent replicas, one rank per GPU) on the
CPU: two gloo ranks reduce the slowest rank's time and the summed units the
way bench.py does, and the reference arm runs on rank 0 only."""
import os
import socket
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

RANK_SCRIPT = r"""
import sys
sys.path.insert(0, sys.argv[1])
import bench
rank, world, dist = bench.dist_init(2)
t = bench.barrier_max(dist, 10.0 + rank)          # per-rank device time
u = bench.barrier_sum(dist, 1000.0 * (rank + 1))  # per-rank units
print(f"RESULT {rank} {world} {t} {u} {dist.get_backend()}")
dist.destroy_process_group()
"""


def free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def launch(code_args, world=2):
    port = free_port()
    procs = []
    for r in range(world):
        env = dict(os.environ, RANK=str(r), WORLD_SIZE=str(world), LOCAL_RANK=str(r), MASTER_ADDR="127.0.0.1",
                   MASTER_PORT=str(port), CUDA_VISIBLE_DEVICES="")
        procs.append(subprocess.Popen([sys.executable] + code_args, env=env, cwd=ROOT, stdout=subprocess.PIPE,
                                      stderr=subprocess.PIPE, text=True))
    out = []
    for p in procs:
        o, e = p.communicate(timeout=300)
        assert p.returncode == 0, e
        out.append(o)
    return out


def test_two_rank_reductions():
    out = launch(["-c", RANK_SCRIPT, ROOT])
    for r, o in enumerate(out):
        line = [ln for ln in o.splitlines() if ln.startswith("RESULT")][0].split()
        assert int(line[1]) == r and int(line[2]) == 2
        assert float(line[3]) == 11.0          # the slowest rank's time
        assert float(line[4]) == 3000.0        # all ranks' units
        assert line[5] == "gloo"


def test_reference_arm_runs_on_rank_zero_only():
    out = launch(["bench.py", "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "3",
                  "--config", "pkj3x3", "--window-ms", "0.5"])
    assert '"impl": "reference"' in out[0]
    assert out[1].strip() == ""
    import json
    line = json.loads(out[0].strip().splitlines()[-1])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
              "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert k in line, k
    assert line["n_gpus"] == 2 and line["steps"] == 1 and line["warmup"] == 3 and line["value"] > 0
    assert line["config"]["workload"] and line["cpu_baseline"]["kind"] == "port"
    assert line["config"]["window_ms"] == [0.0, 0.5]
    assert line["e2e"]["value"] == line["value"] and line["e2e"]["h2d_bytes_per_step"] == 0
