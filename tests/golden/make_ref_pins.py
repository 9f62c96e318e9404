"""Generate tests/golden/ref_pins.json from the reference's own code.

Runs oracle/_ref/ref_harness (the reference's *_ion.cu kernels and its
initialize_host_* / set_host_*_solve setup, compiled for the host from the
reference sources by oracle/ref_harness/Makefile) on seeded synthetic cells
written in the reference file formats, and records a SHA-256 per output array.
tests/test_oracle_pins.py recomputes the same arrays with the oracle and
compares hashes, so the pin travels without the reference sources.

Usage:  python tests/golden/make_ref_pins.py   (needs oracle/_ref/ref_harness)
"""
from __future__ import annotations

import hashlib
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, os.path.join(ROOT, "cerebellum-neuron-model-simulation-using-rkc_gb300"))
import morph as M  # noqa: E402

HARNESS = os.path.join(ROOT, "oracle", "_ref", "ref_harness")
FILES = {M.GR: "Gr.txt", M.GO: "Go_131.txt", M.PKJ: "Pkj.txt", M.IO: "IO.txt"}
NCOND = {M.GR: 10, M.GO: 13, M.PKJ: 11, M.IO: 8}
NION = {M.GR: 20, M.GO: 24, M.PKJ: 18, M.IO: 10}

# The pinned cases: type -> (rows generator, nx, ny, rand seed, ion steps, DT)
CASES = {
    M.GR: (lambda: M.gr_synthetic(11), 1, 2, 7, 6, 2.0 ** -9),
    M.GO: (lambda: M.go_synthetic(12), 2, 2, 8, 6, 2.0 ** -6),
    M.PKJ: (lambda: M.pkj_synthetic(13), 2, 2, 9, 6, 2.0 ** -6),
    M.IO: (lambda: M.io_rows(), 2, 2, 10, 6, 2.0 ** -6),
}


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def vnew_sweep(nc: int, k: int) -> np.ndarray:
    """The deterministic probe voltages the harness applies at update k."""
    x = np.arange(nc, dtype=np.float64) * 0.6180339887498949 + float(k) * 0.2718281828459045
    return -90.0 + 130.0 * (x - np.floor(x))


def write_inputs(d: str, t: int, rows: np.ndarray) -> None:
    with open(os.path.join(d, FILES[t]), "w") as f:
        f.write(M.write_rows(rows, t))
    if t == M.PKJ:
        with open(os.path.join(d, "Pkj_GJ.csv"), "w") as f:
            for a, b in M.PKJ_GJ_PAIRS:
                f.write(f"{int(a)},{int(b)}\n")


def setup_names(t: int):
    names = ["cm", "area", "compart"] + [f"cond{k}" for k in range(NCOND[t])]
    if t == M.PKJ:
        names.append("shell")
    return names


def state_names(t: int, tag: str):
    names = [f"{tag}_v", f"{tag}_ca"] + [f"{tag}_ion{k}" for k in range(NION[t])]
    if t in (M.GO, M.PKJ):
        names.append(f"{tag}_rev")
    if t == M.GO:
        names += [f"{tag}_ca2", f"{tag}_caold"]
    return names


def run_harness(t: int):
    gen, nx, ny, seed, nsteps, dt = CASES[t]
    rows = gen()
    out = {}
    with tempfile.TemporaryDirectory() as d:
        write_inputs(d, t, rows)
        sd = os.path.join(d, "setup")
        od = os.path.join(d, "ion")
        os.makedirs(sd)
        os.makedirs(od)
        subprocess.run([HARNESS, "setup", str(t), str(nx), str(ny), sd], cwd=d, check=True,
                       stdout=subprocess.DEVNULL)
        subprocess.run([HARNESS, "ion", str(t), str(nx), str(ny), str(seed), str(nsteps),
                        repr(dt), od], cwd=d, check=True, stdout=subprocess.DEVNULL)
        for nm in setup_names(t):
            out["setup:" + nm] = np.fromfile(os.path.join(sd, nm + ".bin"), dtype=np.float64)
        out["setup:row"] = np.fromfile(os.path.join(sd, "row.bin"), dtype=np.int32)
        out["setup:col"] = np.fromfile(os.path.join(sd, "col.bin"), dtype=np.int32)
        out["setup:val"] = np.fromfile(os.path.join(sd, "val.bin"), dtype=np.float64)
        for tag in ("init", "final"):
            for nm in state_names(t, tag):
                out["ion:" + nm] = np.fromfile(os.path.join(od, nm + ".bin"), dtype=np.float64)
    return out


def main() -> None:
    if not os.path.exists(HARNESS):
        sys.exit("oracle/_ref/ref_harness missing: run `make -C oracle/ref_harness` first")
    pins = {}
    for t, (gen, nx, ny, seed, nsteps, dt) in CASES.items():
        arrays = run_harness(t)
        pins[M.TYPE_NAMES[t]] = {
            "nx": nx, "ny": ny, "seed": seed, "nsteps": nsteps, "dt": dt,
            "sha256": {k: sha(v) for k, v in arrays.items()},
            "sample": {k: float(v[len(v) // 2]) for k, v in arrays.items() if v.dtype == np.float64},
        }
        print(M.TYPE_NAMES[t], len(arrays), "arrays")
    with open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "ref_pins.json"), "w") as f:
        json.dump(pins, f, indent=1, sort_keys=True)


if __name__ == "__main__":
    main()
