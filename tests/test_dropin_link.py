"""The reference's own main.cu compiles against include/gbrkc_compat.h and
links against libgbrkc.so with no change but its include block, and the
linked program, run on the GPU, writes the reference's IO raster.

Runs only where the reference's sources are found (they are read, never
copied into the repository): main.cu is compiled from a scratch copy whose
directory holds one-line stand-ins for the reference's headers, each
including gbrkc_compat.h; the stand-in param.h also sets main.cu's
compile-time TS (param.h:7)."""
import os
import shutil
import subprocess

import pytest

import morph as M
import refsrc
from test_oracle_golden import load_gold

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "cerebellum-neuron-model-simulation-using-rkc_gb300")
REF = refsrc.reference_dir() or ""
HEADERS = ["param.h", "go.cuh", "go_solve.cuh", "go_ion.cuh", "gr.cuh", "gr_solve.cuh", "gr_ion.cuh", "pkj.cuh",
           "pkj_solve.cuh", "pkj_ion.cuh", "io.cuh", "io_solve.cuh", "io_ion.cuh", "solve_bem.cuh",
           "solve_rkc.cuh", "syn.cuh", "gap.cuh", "output.cuh"]


needs_ref = pytest.mark.skipif(not os.path.exists(os.path.join(REF, "main.cu")), reason="reference sources not found")
needs_nvcc = pytest.mark.skipif(shutil.which("nvcc") is None, reason="no nvcc")


def link_main(tmp_path, ts_ms):
    """Compile the reference's main.cu with TS = ts_ms against libgbrkc.so;
    returns the program's path."""
    lib = os.path.join(PKG, "libgbrkc.so")
    if not os.path.exists(lib):
        import build as B
        B.build()
    shutil.copy(os.path.join(REF, "main.cu"), tmp_path / "main.cu")
    for h in HEADERS:
        body = '#include "gbrkc_compat.h"\n'
        if h == "param.h":
            body += f"#define TS ( {ts_ms} )\n"
        (tmp_path / h).write_text(body)
    cmd = ["nvcc", "-O2", "-gencode", "arch=compute_103a,code=sm_103a", f"-I{os.path.join(ROOT, 'include')}",
           str(tmp_path / "main.cu"), f"-L{PKG}", "-lgbrkc", f"-Xlinker=-rpath,{PKG}", "-o", str(tmp_path / "main")]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert (tmp_path / "main").exists()
    return str(tmp_path / "main")


@needs_ref
@needs_nvcc
def test_reference_main_links_against_gbrkc(tmp_path):
    link_main(tmp_path, 1500)


@pytest.mark.gpu
@needs_ref
@needs_nvcc
def test_reference_main_runs_io_raster(tmp_path):
    """The reference's io run, `./main RKC 0 0 RKC 0 0 RKC 0 0 RKC 8 8` to
    809 ms, through libgbrkc.so: every one of the 64 cells spikes once, each
    within one output interval of the reference's own io_raster_by_RKC.csv
    and at least 62 of 64 at the identical time (the reference's raster is
    sampled on the 0.125 ms output grid, io.cu:271-283)."""
    prog = link_main(tmp_path, 809)
    (tmp_path / "IO.txt").write_text(M.write_rows(M.io_rows(), M.IO))
    env = dict(os.environ, GBRKC_MODEL_DIR=str(tmp_path))
    r = subprocess.run([prog, "RKC", "0", "0", "RKC", "0", "0", "RKC", "0", "0", "RKC", "8", "8"], cwd=tmp_path,
                       env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    assert "isnan" not in r.stdout
    mine = {}
    for line in open(tmp_path / "io_raster_by_RKC.csv"):
        t, c = line.strip().split(",")
        assert int(c) not in mine, f"cell {c} spiked twice"
        mine[int(c)] = float(t)
    gold = {c: t for t, c in load_gold()}
    assert sorted(mine) == list(range(64))
    assert all(abs(mine[c] - gold[c]) <= 0.125 for c in range(64))
    assert sum(mine[c] == gold[c] for c in range(64)) >= 62
    rows = open(tmp_path / "io_v_by_RKC.csv").read().splitlines()
    assert len(rows) == 809 * 8
