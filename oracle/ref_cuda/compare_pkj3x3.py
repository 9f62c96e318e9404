"""The Purkinje 3x3 plain-FP64 workload run by the reference's own CUDA build
(its RKC solver, and its Crank-Nicolson solver as the comparator) and by
gbrkc (plain FP64 and mixed precision) on the same GPU, with identical
inputs: one seeded tapered tree written as Pkj.txt, the reference's own
initial jitter (srand(0)), a constant 0.5 nA at every soma, x-neighbour
gap junctions, the same simulated window.

Reference-baseline infrastructure (needs oracle/_ref/ref_cuda/ref_rkc_run,
built from the reference's sources by this directory's Makefile); not part
of the product.  Prints one JSON line per run: wall time, spikes (the
reference's raster rule at the soma), compartment-updates where known
(gbrkc counts them; the reference's RKC runs the same algorithm, so its
time is also expressed per gbrkc's FP64 update count), and the largest soma
voltage difference against the reference's RKC CSV at a few times.

    python oracle/ref_cuda/compare_pkj3x3.py [TS_MS]
"""
from __future__ import annotations

import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "cerebellum-neuron-model-simulation-using-rkc_gb300"))
import configs  # noqa: E402
import morph as M  # noqa: E402

RUN = os.path.join(ROOT, "oracle", "_ref", "ref_cuda", "ref_rkc_run")


def reference(ts, solver):
    sp = configs.pkj_grid(3, 3)[0]
    with tempfile.TemporaryDirectory() as d:
        open(os.path.join(d, "Pkj.txt"), "w").write(M.write_rows(sp.rows, M.PKJ))
        with open(os.path.join(d, "Pkj_GJ.csv"), "w") as f:
            for a, b in M.PKJ_GJ_PAIRS:
                f.write(f"{int(a)},{int(b)}\n")
        solvers = "RKC" if solver == "RKC" else f"RKC,RKC,{solver},RKC"
        cmd = [RUN, "0", "0", "0", "0", "3", "3", "0", "0", repr(ts), "const:pkj=0.0005", d, "0", solvers]
        r = subprocess.run(cmd, cwd=d, capture_output=True, text=True, timeout=3000)
        info = json.loads(r.stdout.strip().splitlines()[-1])
        soma = np.loadtxt(os.path.join(d, f"pkj_v_by_{solver}.csv"), delimiter=",", usecols=range(10), ndmin=2)
        raster = [ln for ln in open(os.path.join(d, f"pkj_raster_by_{solver}.csv")).read().splitlines() if ln]
        v0 = np.fromfile(os.path.join(d, "pkj_v0.bin"))
    return info, soma[:, 1:], len(raster), v0


def gbrkc(ts, prec, steps=10):
    import gbrkc as G
    sp = configs.pkj_grid(3, 3)[0]
    n_all = int(round(ts / 0.125))
    e = G.Engine(prec)
    sid = configs.add_to(e, [sp])[0]
    e.build()
    v0 = e.read(sid, G.F_V)
    e.advance(0.0, 1)                                    # load the kernels, then start again at t = 0
    e.reset_systems(sid, 1, sp.jitter, stim=(np.full(9, 1599, np.int32), np.full(9, 0.5e-3), np.zeros(9),
                                            np.full(9, 1e9)))
    e.advance(0.0, 0)
    e.record_soma(n_all)
    n_iv = n_all // steps
    u0 = e.compartment_updates(-1)
    w0 = time.perf_counter()
    for k in range(steps):
        e.advance(k * n_iv * 0.125, n_iv)
    wall = time.perf_counter() - w0
    units = e.compartment_updates(-1) - u0
    soma = e.read_soma(sid, n_all)
    prev = np.vstack([np.full((1, 9), 100.0), soma[:-1]])
    spikes = int(((soma > -10.0) & (prev <= -10.0)).sum())
    e.close()
    return wall, units, soma, spikes, v0


def main():
    ts = float(sys.argv[1]) if len(sys.argv) > 1 else 200.0
    import gbrkc as G
    ref = {s: reference(ts, s) for s in ("RKC", "CN")}
    rkc_soma = ref["RKC"][1]
    units64 = None
    for name, prec in (("gbrkc_fp64", G.FP64), ("gbrkc_mixed", G.MIXED)):
        wall, units, soma, spikes, v0 = gbrkc(ts, prec)
        if prec == G.FP64:
            units64 = units
        n = min(len(soma), len(rkc_soma))
        err = np.abs(soma[:n] - rkc_soma[:n])
        print(json.dumps({"run": name, "wall_s": wall, "compartment_updates": units, "cu_per_s": units / wall,
                          "spikes": spikes, "v0_equal_reference": bool(np.array_equal(v0, ref["RKC"][3])),
                          "soma_max_abs_diff_vs_reference_rkc_mv": {f"{c:g}ms": float(err[:int(c / 0.125)].max())
                                                                   for c in (1, 5, 20, 50, ts)},
                          "speedup_vs_reference_rkc": ref["RKC"][0]["wall_s"] / wall}))
    for s in ("RKC", "CN"):
        info, soma, nsp, _ = ref[s]
        out = {"run": f"reference_{s.lower()}", "wall_s": info["wall_s"], "spikes": nsp, "ts_ms": info["ts_ms"],
               "nan": info["nan_type"] >= 0}
        if s == "RKC":
            out["cu_per_s_at_gbrkc_fp64_count"] = units64 / info["wall_s"]
        else:
            n = min(len(soma), len(rkc_soma))
            out["soma_max_abs_diff_vs_reference_rkc_mv"] = {f"{c:g}ms": float(np.abs(soma[:n] - rkc_soma[:n])
                                                                              [:int(c / 0.125)].max())
                                                            for c in (1, 5, 20, 50, ts)}
        print(json.dumps(out))


if __name__ == "__main__":
    main()
