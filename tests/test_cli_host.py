"""gbrkc_main's solver-name handling, which runs before any device call, on
the CPU: names are matched on their first letters as main.cu:60-102 does; an
unknown name is main.cu's "Error!!" message and exit status 0; BE or CN is
refused (exit 1) for a type with cells, and opens <type>_*_by_BE/CN.csv."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "cerebellum-neuron-model-simulation-using-rkc_gb300")
CLI = os.path.join(PKG, "gbrkc_main")


@pytest.fixture(scope="module")
def cli():
    if not os.path.exists(CLI):
        import build as B
        B.build()
    return CLI


def run(cli, tmp_path, *args):
    return subprocess.run([cli, *args, "1"], cwd=tmp_path, capture_output=True, text=True, timeout=120)


def test_unknown_solver_name(cli, tmp_path):
    r = run(cli, tmp_path, "RKC", "0", "0", "XX", "0", "0", "RKC", "0", "0", "RKC", "0", "0")
    assert r.returncode == 0
    assert "Error!! -> set solver name in argv [ 4 ]" in r.stdout
    # main.cu:40-55's echo comes first
    assert r.stdout.startswith("argc = 14\nargv[0] = ")
    assert "argv[4] = XX\n" in r.stdout and "GO  solver -> XX\n" in r.stdout


def test_be_cn_refused_for_a_type_with_cells(cli, tmp_path):
    r = run(cli, tmp_path, "CN", "0", "0", "RKC", "0", "0", "BE", "2", "1", "RKC", "0", "0")
    assert r.returncode == 1
    assert "pkj: solver BE is not provided (only RKC)" in r.stdout
    # the names before it opened their files under the reference's names
    assert (tmp_path / "gr_v_by_CN.csv").exists() and (tmp_path / "go_v_by_RKC.csv").exists()
