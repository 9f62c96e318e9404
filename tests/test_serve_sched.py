"""The request server's host bookkeeping (slot arena, admission order,
latency percentiles), compiled from its header and checked on the CPU."""
import os
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "cerebellum-neuron-model-simulation-using-rkc_gb300", "csrc")
SRC = os.path.join(ROOT, "tests", "native", "serve_sched_check.cpp")


def test_serve_scheduler(tmp_path):
    exe = str(tmp_path / "serve_sched_check")
    subprocess.run([os.environ.get("CXX", "g++"), "-O1", "-std=c++17", "-Wall", "-Werror", f"-I{CSRC}", SRC,
                    "-o", exe], check=True)
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 0 and r.stdout.strip().endswith("OK"), r.stdout + r.stderr
