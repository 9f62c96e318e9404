"""The reference's own main.cu compiles against include/gbrkc_compat.h and
links against libgbrkc.so with no change but its include block.

Runs only where the reference checkout is mounted (it is read, never
copied into the repository): main.cu is compiled from a scratch copy whose
directory holds one-line stand-ins for the reference's headers, each
including gbrkc_compat.h.  Compile and link only; nothing is run."""
import os
import shutil
import subprocess

import pytest

import refsrc

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "cerebellum-neuron-model-simulation-using-rkc_gb300")
REF = refsrc.reference_dir() or ""
HEADERS = ["param.h", "go.cuh", "go_solve.cuh", "go_ion.cuh", "gr.cuh", "gr_solve.cuh", "gr_ion.cuh", "pkj.cuh",
           "pkj_solve.cuh", "pkj_ion.cuh", "io.cuh", "io_solve.cuh", "io_ion.cuh", "solve_bem.cuh",
           "solve_rkc.cuh", "syn.cuh", "gap.cuh", "output.cuh"]


@pytest.mark.skipif(not os.path.exists(os.path.join(REF, "main.cu")), reason="reference checkout not mounted")
@pytest.mark.skipif(shutil.which("nvcc") is None, reason="no nvcc")
def test_reference_main_links_against_gbrkc(tmp_path):
    lib = os.path.join(PKG, "libgbrkc.so")
    if not os.path.exists(lib):
        import build as B
        B.build()
    shutil.copy(os.path.join(REF, "main.cu"), tmp_path / "main.cu")
    for h in HEADERS:
        body = '#include "gbrkc_compat.h"\n'
        if h == "param.h":
            body += "#define TS ( 1500 )\n"
        (tmp_path / h).write_text(body)
    cmd = ["nvcc", "-O2", "-gencode", "arch=compute_103a,code=sm_103a", f"-I{os.path.join(ROOT, 'include')}",
           str(tmp_path / "main.cu"), f"-L{PKG}", "-lgbrkc", "-o", str(tmp_path / "main")]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert (tmp_path / "main").exists()
