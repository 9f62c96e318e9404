"""Generate tests/golden/ref_rkc/*.npz from the reference's own CUDA RKC path.

Runs oracle/_ref/ref_cuda/ref_rkc_run -- the reference simulator's
X_initialize / X_solve_update_v / X_output_file code compiled from its
sources for sm_103a by oracle/ref_cuda/Makefile -- on a GPU, for each case
below: seeded synthetic cells written in the reference's file formats, a
constant current at the compartment the reference stimulates, every
compartment's v_new recorded at every 0.125 ms interval.  The initial
jitter is the reference's own (srand(0), rand() in main.cu's type order).
tests/test_oracle_ref_rkc.py integrates the same cells with the oracle and
compares, so the pin travels without the reference sources.

Usage (on a machine with the GPU and the reference build):
    python tests/golden/make_ref_rkc_vectors.py [case ...]
"""
from __future__ import annotations

import json
import os
import subprocess
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, os.path.join(ROOT, "cerebellum-neuron-model-simulation-using-rkc_gb300"))
import morph as M  # noqa: E402

RUN = os.path.join(ROOT, "oracle", "_ref", "ref_cuda", "ref_rkc_run")
OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "ref_rkc")
FILES = {M.GR: "Gr.txt", M.GO: "Go_131.txt", M.PKJ: "Pkj.txt", M.IO: "IO.txt"}
NAMES = {M.GR: "gr", M.GO: "go", M.PKJ: "pkj", M.IO: "io"}

# case -> type, nx, ny, rows generator spec, constant current, intervals
CASES = {
    "pkj_1x1": dict(type=M.PKJ, nx=1, ny=1, rows=("pkj", 13, True), amp=0.5e-3, n_iv=16),
    "pkj_2x1_gj": dict(type=M.PKJ, nx=2, ny=1, rows=("pkj", 8, True), amp=0.4e-3, n_iv=16),
    "go_1x1": dict(type=M.GO, nx=1, ny=1, rows=("go", 2003), amp=0.3e-3, n_iv=16),
    "go_2x2_gj": dict(type=M.GO, nx=2, ny=2, rows=("go", 2001), amp=0.3e-3, n_iv=16),
    "gr_1x1": dict(type=M.GR, nx=1, ny=1, rows=("gr", 11), amp=0.01e-3, n_iv=8),
    "io_4x4": dict(type=M.IO, nx=4, ny=4, rows=("io",), amp=5.5, n_iv=16),
    # an untapered synthetic Purkinje tree at the current of a mixed-batch
    # cell: with this jitter it spikes at 2 ms and recovers
    "pkj_1x1_untapered": dict(type=M.PKJ, nx=1, ny=1, rows=("pkj", 7, False), amp=0.44846444072807815e-3, n_iv=40),
    # untapered trees on which the oracle (reference arithmetic, this jitter)
    # goes non-finite after 1.75 ms: the reference build's own run of them
    "pkj_1x1_untapered_s3": dict(type=M.PKJ, nx=1, ny=1, rows=("pkj", 3, False), amp=0.6e-3, n_iv=24),
    "pkj_1x1_untapered_s10": dict(type=M.PKJ, nx=1, ny=1, rows=("pkj", 10, False), amp=0.6e-3, n_iv=24),
    # a seeded Golgi tree of the mixed batch on which the oracle goes
    # non-finite after 3.25 ms: the reference build's own run of it
    "go_1x1_s200095": dict(type=M.GO, nx=1, ny=1, rows=("go", 200095), amp=0.6e-3, n_iv=40),
}


def rows_for(spec):
    kind = spec[0]
    if kind == "pkj":
        return M.pkj_synthetic(spec[1], taper=spec[2])
    if kind == "go":
        return M.go_synthetic(spec[1])
    if kind == "gr":
        return M.gr_synthetic(spec[1])
    return M.io_rows()


def run_case(name: str, c: dict) -> dict:
    t = c["type"]
    rows = rows_for(c["rows"])
    dims = [0] * 8
    dims[2 * t], dims[2 * t + 1] = c["nx"], c["ny"]
    ts = c["n_iv"] * 0.125
    with tempfile.TemporaryDirectory() as d:
        with open(os.path.join(d, FILES[t]), "w") as f:
            f.write(M.write_rows(rows, t))
        with open(os.path.join(d, "Pkj_GJ.csv"), "w") as f:
            for a, b in M.PKJ_GJ_PAIRS:
                f.write(f"{int(a)},{int(b)}\n")
        stim = f"const:{NAMES[t]}={c['amp']!r}"
        cmd = [RUN] + [str(x) for x in dims] + [repr(ts), stim, d, str(c["n_iv"])]
        r = subprocess.run(cmd, cwd=d, capture_output=True, text=True, timeout=1200)
        info = json.loads(r.stdout.strip().splitlines()[-1])
        nc = info["nc"][NAMES[t]]
        v0 = np.fromfile(os.path.join(d, f"{NAMES[t]}_v0.bin"), dtype=np.float64)
        vnew = np.fromfile(os.path.join(d, f"{NAMES[t]}_vnew.bin"), dtype=np.float64).reshape(-1, nc)
        raster = open(os.path.join(d, f"{NAMES[t]}_raster_by_RKC.csv")).read()
    meta = dict(case=name, type=t, nx=c["nx"], ny=c["ny"], rows=list(c["rows"]), amp=c["amp"], n_iv=c["n_iv"],
                stim=stim, returncode=r.returncode, run=info, raster=raster,
                command="ref_rkc_run " + " ".join(cmd[1:-2] + ["OUTDIR", cmd[-1]]))
    np.savez_compressed(os.path.join(OUT, f"{name}.npz"), v0=v0, vnew=vnew, meta=json.dumps(meta))
    return meta


def main() -> None:
    if not os.path.exists(RUN):
        sys.exit("oracle/_ref/ref_cuda/ref_rkc_run missing: build it with __graft_entry__.build()")
    os.makedirs(OUT, exist_ok=True)
    for name in (sys.argv[1:] or CASES):
        m = run_case(name, CASES[name])
        print(name, "rc", m["returncode"], "intervals", m["run"]["intervals"], "nan_type", m["run"]["nan_type"],
              "wall_s", m["run"]["wall_s"], flush=True)


if __name__ == "__main__":
    main()
