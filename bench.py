"""Benchmark: compartment-updates/s of the RKC hot path on one GB300.

Default workload (the mixed-type batch): 4096 reduced granule
cells, 1024 Golgi cells, 256 Purkinje cells and one 16x16 inferior-olive
gap-junction network, FP32 gating with FP64 voltage, advanced together.
A step advances every system by --step-ms of simulated time (default 5 ms =
40 output intervals) in one persistent launch: every CTA takes a cell-type
role and pulls systems from that role's work queue.

Unit: one compartment-update = one RKC right-hand-side (stage) evaluation of
one compartment: sum over step attempts of (m + 1) x compartments, accepted
and rejected steps counted, power iterations excluded.

  python bench.py [--gpus N --steps K --warmup W] [--precision fp64|mixed]
                  [--config mixed|pkj3x3] [--impl reference]

Multi-GPU: independent replicas of the workload (each rank its own), no
collective on the data path; value = units of all ranks / max rank time.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "cerebellum-neuron-model-simulation-using-rkc_gb300")
ORACLE = os.path.join(ROOT, "oracle")
for p in (PKG, ORACLE):
    if p not in sys.path:
        sys.path.insert(0, p)

import numpy as np  # noqa: E402

H_MAX = 0.125
ALG_BYTES = {"mixed": 56, "fp64": 68}   # algorithmic bytes per compartment-update
# the simulated window each workload's timed steps cover from t = 0: the
# workloads' own durations (the sweep's systems run 100-1000 ms each; its
# default window is their first 50 ms, when every system is still running;
# the network's 1000 ms take minutes of host-timed launches, its default
# window is its first 20 ms)
WINDOW_MS = {"mixed": 500.0, "screened": 500.0, "pkj3x3": 200.0, "sweep": 50.0, "network": 20.0}


# Arm CPU part numbers (/proc/cpuinfo "CPU part", implementer 0x41)
_ARM_PARTS = {"0xd40": "Neoverse-V1", "0xd49": "Neoverse-N2", "0xd4f": "Neoverse-V2", "0xd84": "Neoverse-V3",
              "0xd0c": "Neoverse-N1"}


def cpu_model():
    """The host CPU's model name (for the CPU baseline's record)."""
    import platform
    try:
        with open("/proc/cpuinfo", errors="replace") as f:
            for line in f:
                k, _, v = line.partition(":")
                k, v = k.strip(), v.strip()
                if k in ("model name", "Model") and v:
                    return v
                if k == "CPU part" and v:
                    return f"{_ARM_PARTS.get(v.lower(), 'Arm part ' + v)} ({platform.machine()})"
    except Exception:
        pass
    return platform.machine()


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def fp64_peak_tflops(torch, n=4096, reps=5):
    """Measured FP64 throughput of this GPU: a cuBLAS DGEMM (torch.matmul in
    float64, n^3), best of reps, CUDA events -- the FP64 counterpart of the
    measured bf16 peak, for the FP64-pipe fraction of the kernels."""
    a = torch.randn(n, n, dtype=torch.float64, device="cuda")
    b = torch.randn(n, n, dtype=torch.float64, device="cuda")
    torch.matmul(a, b)
    torch.cuda.synchronize()
    best = 1e30
    for _ in range(reps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a, b)
        e1.record()
        e1.synchronize()
        best = min(best, e0.elapsed_time(e1))
    del a, b
    return 2.0 * n ** 3 / (best * 1e-3) / 1e12


# ---------------------------------------------------------------- clocks
class ClockSampler:
    def __init__(self, gpu_index=0):
        self.idx = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.idx), f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 7:
                continue
            try:
                sm.append(float(f[0]))
                mx.append(float(f[1]))
            except ValueError:
                continue
            for nm, v in zip(names, f[3:7]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ------------------------------------------------------------ workloads
STATED_DESC = ("mixed-type batch: 4096 GrC x4 + 1024 GoC x131 + 256 PC x1600 + IO 16x16 net x3, "
               "step currents U[0,0.6] nA (olive: 0.6 nA over its dendrite, U[0,60] uA/cm^2) switched on at "
               "U[0,20] ms, a distinct seeded tree per GoC and per PC, g_gap U[0.5,1.5] x nominal; one stated "
               "deviation: PC dendrite diameters tapered by depth (main x5.5, smooth x3) -- untapered trees go "
               "non-finite within ms in the reference's own frozen-current scheme")


def workload(name, scale=1.0):
    import configs
    if name == "mixed":
        if scale < 1.0:
            specs = configs.scaled_stated_batch(scale)
            return specs, f"{STATED_DESC}; populations scaled x{scale:g} (small profiling case)"
        return configs.stated_mixed_batch(), STATED_DESC
    if name == "screened" and scale < 1.0:
        specs = configs.scaled_mixed_batch(scale)
        c = configs.type_counts(specs)
        return specs, (f"mixed-type batch scaled x{scale:g}: {c['gr'][0]} GrC x4 + {c['go'][0]} GoC x131 + "
                       f"{c['pkj'][0]} PC x1600 + IO 16x16 net x3 (small profiling case)")
    if name == "screened":
        return configs.mixed_batch(), ("mixed-type batch, screened: 4096 GrC x4 + 1024 GoC x131 (6 tree variants) + "
                                       "256 PC x1600 (5 tapered trees) + IO 16x16 net x3; currents U[0,0.05] nA GrC, "
                                       "U[0,0.4] nA GoC/PC, U[0,6] uA/cm^2 IO")
    if name == "sweep":
        n = max(1, int(32768 * scale))
        return configs.sweep_batch(n_gr=n, n_go=n), (
            f"parameter sweep: {n} GrC x4 + {n} GoC x131 (one seeded tree) independent systems, every channel "
            "density x U[0.8,1.2] per instance, step current U[0,0.4] nA from t = 0, durations U[100,1000] ms as "
            "per-system interval budgets, no gap junctions" + ("" if scale == 1.0 else
                                                               f" (populations scaled x{scale:g}: small case)"))
    if name == "pkj3x3":
        return configs.pkj_grid(3, 3), ("Purkinje 3x3 grid, one RKC system of 14400 compartments (one seeded tapered "
                                        "tree), x-neighbour gap junctions, constant 0.5 nA at every soma, the "
                                        "reference's own initial jitter (srand(0)), plain FP64")
    raise SystemExit(f"unknown config {name}")


# ------------------------------------------------------------ network
def run_network(args, G, configs, torch, precision, rank, world, dist):
    """The network workload: 2048 GrC, 512 GoC, 512 PC as independent systems
    coupled by 780 404 chemical synapses with delays (configs.network_batch).
    Network mode advances every system one interval per launch, then updates
    every synapse.  Warm-up steps run on a first engine; a fresh engine is
    then timed over [0, window] (an engine with synapses cannot refill its
    systems), on the host wall clock around the synchronous advances
    (launches included).  The same window then runs in plain FP64 -- the
    throughput ratio -- and in FP64 with every initial jitter moved by
    1e-14, the floor for the mixed precision's voltage and spike-time
    differences."""
    specs, groups = configs.network_batch()
    window = args.window_ms
    n_iv = int(round(window / args.steps / H_MAX))
    if n_iv < 1 or abs(n_iv * args.steps * H_MAX - window) > 1e-9:
        raise SystemExit(f"--window-ms {window} is not {args.steps} steps of whole 0.125 ms intervals")
    step_ms = n_iv * H_MAX
    n_all = int(round(window / H_MAX))

    def build(prec, sp=specs):
        e = G.Engine(prec)
        configs.add_network(e, sp, groups)
        e.build()
        return e

    eng = build(G.MIXED if precision == "mixed" else G.FP64)
    for k in range(args.warmup):
        eng.advance(k * step_ms, n_iv, tolerate_retire=True)
    eng.close()
    t0 = time.perf_counter()
    eng = build(G.MIXED if precision == "mixed" else G.FP64)
    setup_s = time.perf_counter() - t0
    for ty, w in RASTER_W.items():
        eng.record_width(ty, w)
    eng.record_soma(n_all)
    clocks = ClockSampler(int(os.environ.get("LOCAL_RANK", "0")))
    clocks.start()
    torch.cuda.synchronize()
    w0 = time.perf_counter()
    for k in range(args.steps):
        eng.advance(k * step_ms, n_iv, tolerate_retire=True)
    torch.cuda.synchronize()
    wall = barrier_max(dist, time.perf_counter() - w0)
    clk = clocks.stop()
    units = barrier_sum(dist, eng.compartment_updates(-1))
    nsyn = sum(len(g["post_system"]) for g in groups)
    n_spk = eng.read_synapses(G.SYNF_S0, nsyn)
    ids = list(range(len(specs)))
    stopped = stopped_systems(G, eng, specs, ids)
    res = {"run": (np.concatenate([eng.vnew(i) for i in ids]), raster_traces(eng, n_all), stopped)}
    eng.close()
    peak, peak_kind = peaks()
    bpu = ALG_BYTES[precision]
    achieved = bpu * units / wall / 1e9
    vs_fp64 = None
    if rank == 0 and precision == "mixed" and not args.no_fp64_compare:
        import copy
        pert = []
        for sp in specs:
            q = copy.copy(sp)
            q.jitter = np.asarray(sp.jitter, dtype=np.float64) + 1e-14
            pert.append(q)
        walls = {}
        for name, sp in (("fp64", specs), ("fp64_perturbed", pert)):
            e = build(G.FP64, sp)
            for ty, w in RASTER_W.items():
                e.record_width(ty, w)
            e.record_soma(n_all)
            w1 = time.perf_counter()
            e.advance(0.0, n_all, tolerate_retire=True)
            walls[name] = (time.perf_counter() - w1, e.compartment_updates(-1))
            res[name] = (np.concatenate([e.vnew(i) for i in ids]), raster_traces(e, n_all),
                         stopped_systems(G, e, sp, ids))
            e.close()
        sp_of = {}
        for name in ("run", "fp64", "fp64_perturbed"):
            tr = res[name][1]
            sp_of[name] = sum((spike_times(tr[ty], ty=ty) for ty in sorted(tr)), [])
        fp64_v = walls["fp64"][1] / walls["fp64"][0]
        # per system, over the systems that stopped in none of the three runs
        # (a stopped system keeps the state it diverged with)
        out_of = {x["index"] for name in ("run", "fp64", "fp64_perturbed") for x in res[name][2]}
        bounds = np.cumsum([0] + [sp.nc for sp in specs])
        keep = [k for k in ids if k not in out_of]

        def max_err(a, b, ty=None):
            e = [float(np.max(np.abs(a[bounds[k]:bounds[k + 1]] - b[bounds[k]:bounds[k + 1]])))
                 for k in keep if ty is None or specs[k].cell_type == ty]
            return max(e, default=0.0)

        by_type = {TYPE_NAMES[ty]: {"mixed": max_err(res["run"][0], res["fp64"][0], ty),
                                    "floor": max_err(res["fp64_perturbed"][0], res["fp64"][0], ty)}
                   for ty in sorted({sp.cell_type for sp in specs})}
        vs_fp64 = {"fp64_value": fp64_v, "mixed_value": units / wall, "ratio": (units / wall) / fp64_v,
                   "window_ms": [0.0, window], "unit": "compartment-updates/s (host wall clock, same window)",
                   "accuracy": {"max_abs_err_mv": max_err(res["run"][0], res["fp64"][0]),
                                "sensitivity_floor_mv": max_err(res["fp64_perturbed"][0], res["fp64"][0]),
                                "max_abs_err_mv_by_type": by_type,
                                "systems_compared": len(keep),
                                "at_ms": window,
                                "spikes_mixed_vs_fp64": compare_spikes(sp_of["fp64"], sp_of["run"]),
                                "spikes_fp64_floor": compare_spikes(sp_of["fp64"], sp_of["fp64_perturbed"]),
                                "stopped": {"fp64": res["fp64"][2], "fp64_perturbed": res["fp64_perturbed"][2]},
                                "floor": "the same FP64 run with every initial jitter + 1e-14"}}
    if rank == 0:
        counts = configs.type_counts(specs)
        out = {"metric": "compartment-updates/s", "value": units / wall, "unit": "compartment-updates/s",
               "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
               "ms_per_step": wall * 1e3 / args.steps, "higher_is_better": True, "scaling": "weak",
               "vs_baseline": None, "dtype": "f64 state+stages, f32 gating" if precision == "mixed" else "f64",
               "data": "synthetic (seeded cells, synapses, weights and delays)",
               "config": {"workload": "network: 2048 GrC x4 + 512 GoC x131 + 512 PC x1600 (a distinct seeded tree "
                                      "per GoC and per PC), 780404 synapses (MF->GrC Poisson 5-50 Hz, GrC->GoC, "
                                      "GoC->GrC, GrC->PC), lognormal weights (sigma 0.25: at 0.5 the mossy-fibre "
                                      "tail drives some granule cells non-finite), delays U[1,5] ms",
                          "window_ms": [0.0, window], "step_sim_ms": step_ms},
               "run": {"precision": precision, "cells": {k: v[0] for k, v in counts.items()}, "synapses": nsyn,
                       "synapses_with_activity": int(np.count_nonzero(n_spk)), "stopped_systems": len(stopped),
                       "stopped": stopped[:64], "setup_s": round(setup_s, 2),
                       "timing": "host wall clock; one persistent launch and one synapse launch per interval",
                       "sim_ms_per_wall_s": window / wall},
               "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                            "frac": achieved / peak, "traffic": None, "kernel": "k_mega + k_syn_update",
                            "peak_kind": f"{peak_kind} hbm_gbs", "bytes_per_update": bpu},
               "gpu_launches": 2 * args.steps * n_iv, "clocks": clk}
        if vs_fp64:
            out["vs_plain_fp64"] = vs_fp64
        print(json.dumps(out))
    if dist is not None:
        dist.destroy_process_group()


# ------------------------------------------------------------ helpers
def type_runs(specs, ids):
    """{cell type: (first system id, count, spec indices)}: every type's systems
    are one consecutive run of ids (configs.add_to registers them in order)."""
    runs = {}
    for k, sp in enumerate(specs):
        runs.setdefault(sp.cell_type, []).append(k)
    out = {}
    for ty, ks in runs.items():
        first = ids[ks[0]]
        if [ids[k] for k in ks] != list(range(first, first + len(ks))):
            raise RuntimeError("systems of one type are not consecutive")
        out[ty] = (first, len(ks), ks)
    return out


def cell_stim(specs, ks):
    """Per-cell (comp, amp, t0, t1) arrays of the given specs, concatenated."""
    cols = [[], [], [], []]
    for k in ks:
        sp = specs[k]
        for j, dt in enumerate((np.int32, np.float64, np.float64, np.float64)):
            cols[j].append(np.broadcast_to(np.asarray(sp.stim[j], dtype=dt), sp.n))
    return tuple(np.ascontiguousarray(np.concatenate(c)) for c in cols)


def apply_budgets(eng, specs, ids):
    """Per-system interval budgets (spec.extra["n_intervals"]), where given."""
    for sp, sid in zip(specs, ids):
        n = sp.extra.get("n_intervals")
        if n is not None:
            eng.set_budget(sid, 1, int(n))


def reset_to_start(eng, specs, ids):
    """Refill every system with its own initial cell (same jitter, stimulus and
    edge conductances): the state of a freshly built engine at t = 0, while
    the engine keeps its launch tuning.  The initialisation launch runs here,
    outside any timed region."""
    for ty, (first, n, ks) in type_runs(specs, ids).items():
        jit = np.concatenate([np.asarray(specs[k].jitter, dtype=np.float64) for k in ks])
        gg = None
        if all(specs[k].io_gap_g is not None for k in ks):
            gg = np.concatenate([np.asarray(specs[k].io_gap_g, dtype=np.float64) for k in ks])
        cc = None
        if all(specs[k].cond_scale_ch is not None for k in ks):
            cc = np.concatenate([np.asarray(specs[k].cond_scale_ch, dtype=np.float64).reshape(-1) for k in ks])
        eng.reset_systems(first, n, jit, stim=cell_stim(specs, ks), io_gap_g=gg, cond_scale_ch=cc)
    apply_budgets(eng, specs, ids)
    eng.advance(0.0, 0, tolerate_retire=True)


def stopped_systems(G, eng, specs, ids):
    """The systems that stopped: spec index, shape tag, cell type, status bits."""
    out = []
    for ty, (first, n, ks) in type_runs(specs, ids).items():
        st, _ = eng.run_status(first, n)
        for j in np.nonzero(st)[0]:
            k = ks[int(j)]
            out.append({"index": k, "tag": specs[k].tag, "type": int(ty), "status": int(st[j]),
                        "why": next((v for b, v in G.STATUS_BITS.items() if int(st[j]) & b), str(int(st[j])))})
    return out


RASTER_W = {0: 4, 3: 3}          # recorded compartments 0..w-1 per cell (granule, olive)
RASTER_AT = {0: 3, 1: 0, 2: 0, 3: 2}   # raster compartment within the record


def raster_traces(eng, n_iv):
    """Per cell type, [interval][cell] values of each cell's raster compartment
    at the interval ends (the soma record, widened for granule and olive)."""
    out = {}
    for ty in range(4):
        nc = eng.type_cells(ty)
        if nc == 0:
            continue
        w = RASTER_W.get(ty, 1)
        buf = np.empty((n_iv, nc, w), np.float64)
        eng.read_soma_type(ty, n_iv, buf)
        out[ty] = buf[:, :, RASTER_AT[ty]]
    return out


def spike_times(trace, t0=0.0, thresh=None, ty=0):
    """Threshold crossings of output_file's rule (value > threshold, previous
    <= threshold; GrC/GoC/IO 10 mV, PC -10 mV; the first previous value is 100,
    as main.cu:163-169), each timed by linear interpolation between the two
    interval-end samples: per cell, the list of times."""
    th = (-10.0 if ty == 2 else 10.0) if thresh is None else thresh
    n_iv, nc = trace.shape
    prev = np.concatenate([np.full((1, nc), 100.0), trace[:-1]])
    up = (trace > th) & (prev <= th)
    out = [[] for _ in range(nc)]
    for k, c in zip(*np.nonzero(up)):
        t1 = t0 + (k + 1) * H_MAX
        if k == 0:
            out[c].append(t1)          # crossing from the initial 100 mV sentinel: no interpolation
            continue
        a, b = prev[k, c], trace[k, c]
        out[c].append(t1 - H_MAX + H_MAX * (th - a) / (b - a))
    return out


def compare_spikes(a, b):
    """Spike counts and times of two runs (lists per cell)."""
    equal = sum(1 for x, y in zip(a, b) if len(x) == len(y))
    spiking = sum(1 for x, y in zip(a, b) if x or y)
    dts = [abs(p - q) for x, y in zip(a, b) if len(x) == len(y) for p, q in zip(x, y)]
    return {"spikes": [sum(len(x) for x in a), sum(len(y) for y in b)], "cells_spiking": spiking,
            "cells_with_equal_counts": equal, "cells": len(a),
            "max_spike_time_err_ms": max(dts) if dts else 0.0,
            "spikes_within_0.05ms": (sum(1 for d in dts if d <= 0.05), len(dts))}


# ------------------------------------------------------------ accuracy against FP64
TYPE_NAMES = {0: "gr", 1: "go", 2: "pkj", 3: "io"}
PERTURB = {1: 1e-14, 2: 1e-7}     # FP64 floor copies: initial jitter moved by this much


def accuracy_vs_fp64(G, configs, sample, horizon_ms=100.0, checkpoints=(1.0, 5.0, 20.0, 100.0)):
    """Mixed precision against plain FP64 on a sample of the workload, from
    t = 0, next to two FP64 sensitivity floors: the same FP64 run with every
    cell's initial jitter moved by 1e-14 (its initial voltage by a few units
    in the last place: V0 = V_init + 2..10 x jitter), and by 1e-7 (V0 by
    2e-7..1e-6 mV, under FP32's resolution of a membrane voltage, 3.8e-6 mV at
    -65 mV: the size of the rounding the mixed path's FP32 gating starts
    from).  The three FP64 copies share one engine.  Reports max |V - V_fp64|
    over every compartment at the checkpoints, in all and per cell type; the
    same split by whether a system took the FP64 run's step decisions (equal
    step, rejection, stage and power-iteration counts) up to the checkpoint;
    and the interpolated spike times of every cell (device raster rule) over
    the horizon."""
    import copy
    copies = [sample]
    for c in sorted(PERTURB):
        pert = []
        for sp in sample:
            q = copy.copy(sp)
            q.jitter = np.asarray(sp.jitter, dtype=np.float64) + PERTURB[c]
            pert.append(q)
        copies.append(pert)
    n_iv = int(round(horizon_ms / H_MAX))
    nsys = len(sample)
    ncopy = len(copies)
    # FP64 engine: every copy, ordered by cell type (each type one run of
    # ids), the unperturbed copy first within a type
    combo = sorted((sp.cell_type, c, k) for c in range(ncopy) for k, sp in enumerate(sample))
    res = {}
    for name, prec in (("fp64", G.FP64), ("mixed", G.MIXED)):
        keys = combo if name == "fp64" else [(sp.cell_type, 0, k) for k, sp in enumerate(sample)]
        specs = [copies[c][k] for _, c, k in keys]
        e = G.Engine(prec)
        ids = configs.add_to(e, specs)
        e.build()
        for ty, w in RASTER_W.items():
            if e.type_cells(ty):
                e.record_width(ty, w)
        e.record_soma(n_iv)
        v, st, t, done = [], [], 0.0, 0
        for cp in checkpoints:
            k = int(round(cp / H_MAX)) - done
            e.advance(t, k, tolerate_retire=True)
            t += k * H_MAX
            done += k
            v.append({(c, kk): e.read(i, G.F_VNEW) for (_, c, kk), i in zip(keys, ids)})
            st.append({(c, kk): e.ctl(i)[1] for (_, c, kk), i in zip(keys, ids)})
        tr = raster_traces(e, n_iv)
        stop = [dict(x, copy=keys[x["index"]][1], index=keys[x["index"]][2]) for x in stopped_systems(G, e, specs, ids)]
        res[name] = (v, st, tr, stop)
        e.close()
    ncomp = sum(sp.nc for sp in sample)
    v64, st64 = res["fp64"][0], res["fp64"][1]
    v32, st32 = res["mixed"][0], res["mixed"][1]
    runs = {"mixed": (v32, st32, 0), "floor": (v64, st64, 1), "floor_fp32_resolution": (v64, st64, 2)}

    def err(vv, c, j, kk):
        return float(np.max(np.abs(vv[j][(c, kk)] - v64[j][(0, kk)])))

    errs = {r: [[err(vv, c, j, kk) for kk in range(nsys)] for j in range(len(checkpoints))]
            for r, (vv, _, c) in runs.items()}
    out = {"sample": f"{nsys} systems, {ncomp} compartments, from t = 0 to {horizon_ms:g} ms",
           "max_abs_err_mv": {f"{cp:g}ms": max(errs["mixed"][j]) for j, cp in enumerate(checkpoints)},
           "sensitivity_floor_mv": {f"{cp:g}ms": max(errs["floor"][j]) for j, cp in enumerate(checkpoints)},
           "sensitivity_floor_fp32_resolution_mv": {f"{cp:g}ms": max(errs["floor_fp32_resolution"][j])
                                                    for j, cp in enumerate(checkpoints)}}
    by_type = {}
    for ty in sorted({sp.cell_type for sp in sample}):
        ks = [kk for kk, sp in enumerate(sample) if sp.cell_type == ty]
        by_type[TYPE_NAMES.get(ty, str(ty))] = {
            f"{cp:g}ms": {r: max(errs[r][j][kk] for kk in ks) for r in runs} for j, cp in enumerate(checkpoints)}
    out["max_abs_err_mv_by_type"] = by_type
    # split by whether the system took the FP64 run's step decisions
    dec = {}
    for j, cp in enumerate(checkpoints):
        row = {}
        for r, (_, ss, c) in runs.items():
            same = [kk for kk in range(nsys) if ss[j][(c, kk)] == st64[j][(0, kk)]]
            diff = [kk for kk in range(nsys) if kk not in set(same)]
            row[r] = {"same": len(same), "max_err_same_mv": max([errs[r][j][kk] for kk in same], default=0.0),
                      "differ": len(diff), "max_err_differ_mv": max([errs[r][j][kk] for kk in diff], default=0.0)}
        dec[f"{cp:g}ms"] = row
    out["by_step_decisions"] = dec
    tr64, tr32 = res["fp64"][2], res["mixed"][2]
    sp = {r: [] for r in ("fp64", "mixed", "floor", "floor_fp32_resolution")}
    for ty in sorted(tr64):
        h = tr64[ty].shape[1] // ncopy
        sp["fp64"] += spike_times(tr64[ty][:, :h], ty=ty)
        sp["floor"] += spike_times(tr64[ty][:, h:2 * h], ty=ty)
        sp["floor_fp32_resolution"] += spike_times(tr64[ty][:, 2 * h:3 * h], ty=ty)
        sp["mixed"] += spike_times(tr32[ty], ty=ty)
    out["spikes_mixed_vs_fp64"] = compare_spikes(sp["fp64"], sp["mixed"])
    out["spikes_fp64_floor"] = compare_spikes(sp["fp64"], sp["floor"])
    out["spikes_fp64_floor_fp32_resolution"] = compare_spikes(sp["fp64"], sp["floor_fp32_resolution"])
    out["stopped"] = {"fp64": [x for x in res["fp64"][3] if x["copy"] == 0],
                      "fp64_perturbed": [x for x in res["fp64"][3] if x["copy"] != 0],
                      "mixed": res["mixed"][3]}
    out["floor"] = ("the same FP64 run with every initial jitter + 1e-14 (V0 moved by a few units in the last "
                    "place); floor_fp32_resolution: + 1e-7 (V0 moved by 2e-7..1e-6 mV, under FP32's resolution "
                    "of a membrane voltage)")
    return out


# ------------------------------------------------------------ serving
def run_serve(G, precision, n_requests, seed=5, quantum=8, n_compare=8, slots_scale=1, ts_ms=(5.0, 25.0),
              compare_ms=None):
    """Serve a Poisson request stream (configs.serve_workload) through the
    request server on the wall clock: requests are submitted when their
    arrival time has passed, every round admits what fits and advances all
    resident requests one quantum.  Latency = completion - arrival.  Then a
    sample of the same requests runs one at a time, each in its own plain
    FP64 engine (build, advance, read back), for the throughput ratio and the
    served results' voltage error and spike counts against FP64."""
    import configs
    classes, reqs = configs.serve_workload(n_requests, seed=seed, slots_scale=slots_scale, ts_ms=ts_ms)
    prec = G.MIXED if precision == "mixed" else G.FP64
    srv = G.Server(prec, 0, quantum)
    cids = [srv.add_class(c.cell_type, c.nx, c.ny, c.rows, slots=c.slots, gap=c.gap) for c in classes]
    t_build = time.perf_counter()
    srv.start()
    build_s = time.perf_counter() - t_build

    def submit(r):
        return srv.submit(cids[r.cls], r.n_systems, r.n_intervals, r.jitter, stim=r.stim, cond_scale=r.cond_scale,
                          io_gap_g=r.io_gap_g)

    # warm-up: one short request per class, run to completion, not counted
    _, warm = configs.serve_workload(len(classes) * 4, seed=seed + 100, slots_scale=slots_scale)
    seen = set()
    for r in warm:
        if r.cls not in seen:
            seen.add(r.cls)
            r.n_intervals = 16
            submit(r)
    while srv.stats()["resident"] + srv.stats()["queued"] > 0:
        srv.advance()
    st0 = srv.stats()
    ids, arrive, done_at = [], [], {}
    nxt = 0
    t0 = time.perf_counter()
    while True:
        now = time.perf_counter() - t0
        while nxt < len(reqs) and reqs[nxt].arrival_s <= now:
            ids.append(submit(reqs[nxt]))
            arrive.append(reqs[nxt].arrival_s)
            nxt += 1
        st = srv.stats()
        if st["queued"] + st["resident"] == 0:
            if nxt == len(reqs):
                break
            time.sleep(max(0.0, reqs[nxt].arrival_s - (time.perf_counter() - t0)))
            continue
        srv.advance()
        tnow = time.perf_counter() - t0
        for k, rid in enumerate(ids):
            if k not in done_at and srv.state(rid)[0] in (G.REQ_DONE, G.REQ_FAILED):
                done_at[k] = tnow
    wall = time.perf_counter() - t0
    st = srv.stats()
    lat = np.array([(done_at[k] - arrive[k]) * 1e3 for k in range(len(ids))])
    cu = st["compartment_updates"] - st0["compartment_updates"]
    sim_cell_ms = sum(r.n_systems * classes[r.cls].nx * classes[r.cls].ny * r.n_intervals * H_MAX for r in reqs)
    failures = []
    for k, rid in enumerate(ids):
        state, _, status = srv.state(rid)
        if state == G.REQ_FAILED:
            r = reqs[k]
            failures.append({"class": classes[r.cls].name, "systems": r.n_systems, "intervals": r.n_intervals,
                             "status": status})
    out = {"requests": len(ids), "failed": st["failed"] - st0["failed"], "failures": failures, "wall_s": wall,
           "value": cu / wall, "unit": "compartment-updates/s",
           "latency_ms": {"p50": float(np.percentile(lat, 50, method="inverted_cdf")),
                          "p99": float(np.percentile(lat, 99, method="inverted_cdf")),
                          "mean": float(lat.mean()), "max": float(lat.max()),
                          "from": "arrival (Poisson, wall clock) to completion"},
           "rounds": st["rounds"] - st0["rounds"], "quantum_intervals": quantum,
           "engine_share": (st["advance_s"] - st0["advance_s"]) / wall,
           "hbm_reserved_gb": st["hbm_reserved"] / 1e9, "slots": st["slots"],
           "sim_cell_ms_per_wall_s": sim_cell_ms / wall, "arena_build_s": build_s,
           "workload": (f"{len(reqs)} requests, Poisson 200/s; 20% IO 4x4 network sets (1-8), else 1-4096 GrC x4 "
                        f"/ 1-128 GoC x131 (6 shapes) / 1-16 PC x1600 (5 shapes); {ts_ms[0]:g}-{ts_ms[1]:g} ms "
                        f"each; seed {seed}")}
    # one request at a time, plain FP64, on a sample of the same requests
    sample = []
    for ty in (0, 1, 2, 3):
        sample += [k for k, r in enumerate(reqs) if classes[r.cls].cell_type == ty][:max(1, n_compare // 4)]
    seq_cu, seq_wall, err, spk_same, spk_total = 0, 0.0, 0.0, 0, 0
    per_type = {}  # type -> [cell-ms, wall s]

    def cell_ms(r):
        c = classes[r.cls]
        return r.n_systems * c.nx * c.ny * r.n_intervals * H_MAX

    for k in sample:
        r, c = reqs[k], classes[reqs[k].cls]
        cells = c.nx * c.ny
        # with compare_ms, a long request runs alone only for its first
        # compare_ms (its rate is what the estimate needs); the served result
        # is then not compared
        n_run = r.n_intervals if compare_ms is None else min(r.n_intervals, int(round(compare_ms / H_MAX)))
        w0 = time.perf_counter()
        eng = G.Engine(G.FP64)
        for j in range(r.n_systems):
            sl = slice(j * cells, (j + 1) * cells)
            eng.add_system(c.cell_type, c.nx, c.ny, c.rows, r.jitter[sl], stim=tuple(a[sl] for a in r.stim),
                           gap=c.gap, cond_scale=r.cond_scale[sl],
                           io_gap_g=None if r.io_gap_g is None else r.io_gap_g[4 * j * cells:4 * (j + 1) * cells])
        eng.build()
        eng.record_spikes(1 << 20)
        eng.advance(0.0, n_run, tolerate_retire=True)
        v = np.concatenate([eng.read(j, G.F_VNEW) for j in range(r.n_systems)])
        dt = time.perf_counter() - w0
        seq_wall += dt
        seq_cu += eng.compartment_updates(-1)
        pt = per_type.setdefault(c.cell_type, [0.0, 0.0])
        pt[0] += cell_ms(r) * n_run / r.n_intervals
        pt[1] += dt
        ft, _, _ = eng.read_spikes(c.cell_type)
        eng.close()
        if n_run == r.n_intervals:
            got = srv.read(ids[k], v.size)
            err = max(err, float(np.max(np.abs(got - v))))
            gt, _ = srv.spikes(ids[k])
            spk_same += int(len(gt) == len(ft))
            spk_total += 1
    # the whole stream served one request at a time: each request's cell-ms
    # at its type's sampled sequential rate
    est = sum(cell_ms(r) * per_type[classes[r.cls].cell_type][1] / per_type[classes[r.cls].cell_type][0]
              for r in reqs)
    out["one_at_a_time_fp64"] = {"requests_sampled": len(sample), "value": seq_cu / seq_wall,
                                 "unit": "compartment-updates/s (sample)",
                                 "stream_makespan_s_est": est,
                                 "includes": "engine build, advance and read-back per request"}
    out["vs_one_at_a_time_fp64"] = est / wall
    out["served_vs_fp64"] = {"max_abs_err_mv": err, "spike_counts_equal": f"{spk_same}/{spk_total}",
                             "precision": precision, "requests_compared": spk_total}
    if compare_ms is not None:
        out["one_at_a_time_fp64"]["sampled_for_ms"] = compare_ms
    srv.close()
    return out


# ------------------------------------------------------------ CPU side
def _cpu_specs(cfg, fraction):
    import configs
    if cfg == "sweep":
        return configs.sweep_batch(n_gr=max(1, int(32768 * fraction)), n_go=max(1, int(32768 * fraction)))
    if cfg == "mixed":
        return configs.scaled_stated_batch(fraction)
    if cfg == "screened":
        return configs.scaled_mixed_batch(fraction)
    return workload(cfg)[0]


def _oracle_worker(conn, cfg, fraction, idx):
    """A process holding a slice of a workload sample in the oracle (reference
    arithmetic, FP64) and advancing it on command: ("advance", t0, n) ->
    (compartment-updates, seconds, systems stopped so far); ("reset",) rebuilds
    the slice at t = 0; ("stop",).  A system whose step fails is stopped and
    skipped from then on, as the GPU engine retires it."""
    sys.path.insert(0, PKG)
    sys.path.insert(0, ORACLE)
    import configs
    import oracle_py as O
    specs = _cpu_specs(cfg, fraction)

    def build():
        return [[specs[i], configs.add_to_oracle(O, specs[i], canon=False), True] for i in idx]

    systems = build()
    while True:
        cmd = conn.recv()
        if cmd[0] == "stop":
            break
        if cmd[0] == "reset":
            systems = build()
            conn.send(0)
            continue
        _, t, n = cmd
        before = sum((s.stats()["stages"] + s.stats()["steps"]) * sp.nc for sp, s, _ in systems)
        w0 = time.perf_counter()
        for _ in range(n):
            for rec in systems:
                if rec[2] and rec[1].advance(t) != 0:
                    rec[2] = False
            t += H_MAX
        dt = time.perf_counter() - w0
        after = sum((s.stats()["stages"] + s.stats()["steps"]) * sp.nc for sp, s, _ in systems)
        conn.send((after - before, dt, sum(1 for r in systems if not r[2])))


class OraclePool:
    """Worker processes (spawned) over a proportional sample of a workload;
    systems dealt out largest first."""

    def __init__(self, cfg, fraction, workers):
        import multiprocessing as mp
        specs = _cpu_specs(cfg, fraction)
        order = sorted(range(len(specs)), key=lambda i: -specs[i].nc)
        slices = [order[k::workers] for k in range(workers)]
        ctx = mp.get_context("spawn")
        self.conns, self.procs = [], []
        for sl in slices:
            if not sl:
                continue
            a, b = ctx.Pipe()
            p = ctx.Process(target=_oracle_worker, args=(b, cfg, fraction, sl), daemon=True)
            p.start()
            self.conns.append(a)
            self.procs.append(p)
        self.specs = specs

    def advance(self, t, n):
        """Advance every slice n intervals from t in parallel: (units, wall s, stopped)."""
        w0 = time.perf_counter()
        for c in self.conns:
            c.send(("advance", t, n))
        res = [c.recv() for c in self.conns]
        return sum(r[0] for r in res), time.perf_counter() - w0, sum(r[2] for r in res)

    def reset(self):
        for c in self.conns:
            c.send(("reset",))
        for c in self.conns:
            c.recv()

    def close(self):
        for c in self.conns:
            c.send(("stop",))
        for p in self.procs:
            p.join(timeout=10)

    def describe(self):
        import configs
        counts = configs.type_counts(self.specs)
        return ", ".join(f"{v[0]} {k}" for k, v in counts.items())


def cpu_baseline_single(args):
    """The oracle on one host thread, on a small sample of the same workload
    from t = 0, for about --cpu-seconds."""
    frac = {"mixed": 1.0 / 256, "screened": 1.0 / 256, "sweep": 1.0 / 4096}.get(args.config, 1.0)
    pool = OraclePool(args.config, frac, 1)
    try:
        units, wall, n_iv = 0, 0.0, 0
        probe_u, probe_w, _ = pool.advance(0.0, 2)
        per_iv = max(probe_w / 2, 1e-4)
        n = int(max(4, min(4000, args.cpu_seconds / per_iv)))
        pool.reset()
        units, wall, stopped = pool.advance(0.0, n)
    finally:
        pool.close()
    return {"value": units / wall, "unit": "compartment-updates/s", "cores": 1, "kind": "port",
            "cpu": cpu_model(), "nproc": os.cpu_count(),
            "sample": f"{pool.describe()}; [0, {n * H_MAX:g}] ms (oracle, reference arithmetic, FP64, one thread)"}


def run_reference(args):
    """The reference arm: the reference's RKC path restated on the CPU (the
    oracle, reference arithmetic, FP64) on all host cores, over a
    proportional sample of the same workload and the same window [0, window]
    split into the same K steps.  Warm-up steps advance one interval each;
    the sample is then rebuilt at t = 0.  Rank 0 only."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    cores = os.cpu_count() or 1
    cfg = args.config
    window = args.window_ms
    n_iv = int(round(window / args.steps / H_MAX))
    frac = {"mixed": 1.0 / 16, "screened": 1.0 / 16, "sweep": 1.0 / 256}.get(cfg, 1.0)
    pool = OraclePool(cfg, frac, cores)
    try:
        for k in range(args.warmup):
            pool.advance(k * H_MAX, 1)
        pool.reset()
        units, wall, stopped = 0, 0.0, 0
        for k in range(args.steps):
            u, w, stopped = pool.advance(k * n_iv * H_MAX, n_iv)
            units += u
            wall += w
        desc = pool.describe()
    finally:
        pool.close()
    v = units / wall
    _, wl = workload(cfg)
    out = {"impl": "reference", "metric": "compartment-updates/s", "value": v, "unit": "compartment-updates/s",
           "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
           "ms_per_step": 1e3 * wall / max(1, args.steps), "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded morphologies, jitter and step currents)",
           "config": config_key(args, wl),
           "cpu_baseline": {"value": v, "unit": "compartment-updates/s", "cores": cores, "kind": "port",
                            "cpu": cpu_model(),
                            "sample": f"{desc} (x{frac:g} of every population); the same window in the same "
                                      f"{args.steps} steps; {stopped} systems stopped; oracle, reference "
                                      "arithmetic, FP64"},
           "e2e": {"value": v, "unit": "compartment-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out))


# ------------------------------------------------------------ GPU side
def dist_init(n):
    if n <= 1 and "RANK" not in os.environ:
        return 0, 1, None
    import torch
    import torch.distributed as dist
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if torch.cuda.is_available():
        torch.cuda.set_device(local)
    dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    return rank, world, dist


def _reduce_device(dist):
    # NCCL reduces device tensors, gloo host tensors
    return "cuda" if dist.get_backend() == "nccl" else "cpu"


def barrier_max(dist, x):
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64, device=_reduce_device(dist))
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier_sum(dist, x):
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64, device=_reduce_device(dist))
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gbrkc", choices=["gbrkc", "reference"])
    ap.add_argument("--config", default="mixed",
                    choices=["mixed", "screened", "pkj3x3", "sweep", "serve", "network"])
    ap.add_argument("--precision", default=None, choices=["mixed", "fp64"])
    ap.add_argument("--window-ms", type=float, default=None,
                    help="simulated window timed from t = 0, split into the steps (default: the workload's own, "
                         "500 ms mixed, 200 ms pkj3x3)")
    ap.add_argument("--accuracy-ms", type=float, default=100.0, help="horizon of the mixed-vs-FP64 accuracy sample")
    ap.add_argument("--no-accuracy", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--scale", type=float, default=1.0,
                    help="population fraction of the mixed batch (small profiling cases; 1 = the benchmark)")
    ap.add_argument("--no-fp64-compare", action="store_true")
    ap.add_argument("--no-pkj3x3", action="store_true",
                    help="leave out the Purkinje 3x3 record that the mixed workload's line carries")
    ap.add_argument("--serve-slots", type=int, default=1, help="multiplier on the serving arenas' slot counts")
    ap.add_argument("--serve-ts", type=float, nargs=2, default=None, metavar=("LO", "HI"),
                    help="request durations U[LO, HI] ms (default 5 25 beside the mixed workload, 50 1000 for "
                         "--config serve)")
    ap.add_argument("--serve-requests", type=int, default=None,
                    help="requests of the serving stream (default 48 beside the mixed workload, 128 for "
                         "--config serve; 0: none)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.window_ms is None:
        args.window_ms = WINDOW_MS.get(args.config, 500.0)
    if args.impl == "reference":
        run_reference(args)
        return
    precision = args.precision or ("fp64" if args.config == "pkj3x3" else "mixed")
    rank, world, dist = dist_init(args.gpus)
    import torch
    import gbrkc as G
    import configs
    if args.config == "network":
        run_network(args, G, configs, torch, precision, rank, world, dist)
        return
    if args.config == "serve":
        # the serving stream on its own: value = compartment-updates/s over the stream's wall time
        ts = tuple(args.serve_ts) if args.serve_ts else (50.0, 1000.0)
        sv = run_serve(G, precision, args.serve_requests or 24, slots_scale=args.serve_slots, ts_ms=ts,
                       compare_ms=25.0 if ts[1] > 100.0 else None)
        if rank == 0:
            out = {"metric": "compartment-updates/s", "value": sv["value"], "unit": "compartment-updates/s",
                   "n_gpus": world, "steps": 1, "warmup": args.warmup, "ms_per_step": sv["wall_s"] * 1e3,
                   "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                   "dtype": "f64 state+stages, f32 gating" if precision == "mixed" else "f64",
                   "data": "synthetic (seeded request stream)",
                   "config": {"workload": sv["workload"], "precision": precision}, "serving": sv,
                   "gpu_launches": sv["rounds"]}
            print(json.dumps(out))
        if dist is not None:
            dist.destroy_process_group()
        return
    specs, wl = workload(args.config, args.scale)
    out = run_batch(args, G, configs, torch, specs, wl, precision, rank, world, dist)
    if rank == 0 and args.config == "mixed" and args.scale == 1.0 and not args.no_pkj3x3:
        out["pkj3x3"] = pkj3x3_record(args, G, configs, torch)
    if rank == 0:
        print(json.dumps(out))
    if dist is not None:
        dist.destroy_process_group()


def run_batch(args, G, configs, torch, specs, wl, precision, rank, world, dist):
    """The batch workloads (mixed, pkj3x3): a fixed simulated window from t = 0,
    split into the timed steps.

    Warm-up: W steps of the same length from t = 0 (kernel loading, clocks, the
    engine's CTA split between cell types settles); then every system is
    refilled with its own initial cell (reset_to_start), so the K timed steps
    cover exactly [0, window] whatever K is.  Each timed step, end to end
    through the C ABI: upload every cell's stimulus table from pinned host
    memory, advance one launch (device time from CUDA events on its stream:
    `value`), read back every cell's recorded compartments of every interval
    into pinned host memory (`e2e` = host wall time of the whole step).  L2 is
    flushed (a 256 MB write) before each step, outside both timings."""
    window = args.window_ms
    n_iv = int(round(window / args.steps / H_MAX))
    if n_iv < 1 or abs(n_iv * args.steps * H_MAX - window) > 1e-9:
        raise SystemExit(f"--window-ms {window} is not {args.steps} steps of whole 0.125 ms intervals")
    step_ms = n_iv * H_MAX
    prec = G.MIXED if precision == "mixed" else G.FP64
    eng = G.Engine(prec)
    ids = configs.add_to(eng, specs)
    t_setup = time.perf_counter()
    eng.build()
    apply_budgets(eng, specs, ids)
    setup_s = time.perf_counter() - t_setup
    eng.record_soma(n_iv)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")  # > L2 (129 MB)
    # pinned host buffers: per type the stimulus table (inputs) and the soma record (outputs)
    bufs = {}
    for ty, (first, n, ks) in type_runs(specs, ids).items():
        nc = eng.type_cells(ty)
        stim = cell_stim(specs, ks)
        pins = [torch.empty(nc, dtype=torch.int32 if j == 0 else torch.float64, pin_memory=True) for j in range(4)]
        for p, a in zip(pins, stim):
            p.numpy()[:] = a
        soma = torch.empty((n_iv, nc), dtype=torch.float64, pin_memory=True)
        bufs[ty] = (pins, soma)
    h2d = sum(p[0].numel() * 4 + 3 * p[1].numel() * 8 for p, _ in bufs.values())
    d2h = sum(sm.numel() * 8 for _, sm in bufs.values())

    def step(t):
        for ty, (pins, soma) in bufs.items():
            eng.set_stim_type(ty, *(p.numpy() for p in pins))
        eng.rewind_soma()
        eng.advance(t, n_iv, tolerate_retire=True)
        for ty, (pins, soma) in bufs.items():
            eng.read_soma_type(ty, n_iv, soma.numpy())

    t = 0.0
    for _ in range(args.warmup):
        step(t)
        t += step_ms
    # granule systems per warp, measured on a replay of the next 1 ms
    tune_s = time.perf_counter()
    lanes = eng.autotune(t, 8)
    tune_s = time.perf_counter() - tune_s
    reset_to_start(eng, specs, ids)
    torch.cuda.synchronize()
    clocks = ClockSampler(int(os.environ.get("LOCAL_RANK", "0")))
    clocks.start()
    dev_ms, e2e_s, kern_ms = 0.0, 0.0, {k: 0.0 for k in range(4)}
    step_ms_dev, step_units, retired_at = [], [], []
    stop_ms = {}             # spec index -> end of the timed step after which it was found stopped
    units0 = eng.compartment_updates(-1)
    units_t0 = {k: eng.compartment_updates(k) for k in range(4)}
    if dist is not None:
        dist.barrier()
    torch.cuda.synchronize()
    t = 0.0
    for k in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        u0 = eng.compartment_updates(-1)
        w0 = time.perf_counter()
        step(t)
        e2e_s += time.perf_counter() - w0
        t += step_ms
        dev_ms += eng.last_advance_ms()
        step_ms_dev.append(eng.last_advance_ms())
        step_units.append(eng.compartment_updates(-1) - u0)
        if eng.retired() > (retired_at[-1] if retired_at else 0):
            for x in stopped_systems(G, eng, specs, ids):
                stop_ms.setdefault(x["index"], t)
        retired_at.append(eng.retired())
        for ty in range(4):
            kern_ms[ty] += eng.last_kernel_ms(ty)
    torch.cuda.synchronize()
    if dist is not None:
        dist.barrier()
    clk = clocks.stop()
    units = eng.compartment_updates(-1) - units0
    units_t = {k: eng.compartment_updates(k) - units_t0[k] for k in range(4)}
    t_max_ms = barrier_max(dist, dev_ms)
    units_all = barrier_sum(dist, units)
    value = units_all / (t_max_ms * 1e-3)
    e2e_value = units_all / barrier_max(dist, e2e_s)
    persistent, role_ctas = eng.launch_layout()
    launches = args.steps if persistent else args.steps * sum(1 for k in range(4) if eng.type_cells(k) > 0)
    stopped = stopped_systems(G, eng, specs, ids)
    for x in stopped:
        x["stopped_by_ms"] = stop_ms.get(x["index"])
    n_compartments = eng.total_compartments()
    names = {0: "gr", 1: "go", 2: "pkj", 3: "io"}
    peak, peak_kind = peaks()
    bpu = ALG_BYTES[precision]
    if persistent:
        kname, key = "k_mega", "mega"
        per_launch_units, per_launch_ms = units / args.steps, dev_ms / args.steps
    else:
        dom = max(range(4), key=lambda k: kern_ms[k])
        team = eng.type_team(dom)
        base = {"grid": "k_advance_grid", "cluster": "k_advance_cluster"}.get(team, "k_advance")
        kname, key = f"{base}<{names[dom]}>", names[dom]
        per_launch_units, per_launch_ms = units_t[dom] / args.steps, kern_ms[dom] / args.steps
    achieved = bpu * per_launch_units / (per_launch_ms * 1e-3) / 1e9 if per_launch_ms > 0 else 0.0
    traffic, fp64_ncu = None, None
    tfile = os.path.join(ROOT, "profiles", f"traffic_{args.config}_{precision}.json")
    if os.path.exists(tfile):
        try:
            tr = json.load(open(tfile))
            if key in tr:
                traffic = tr[key] * per_launch_units     # DRAM bytes per update from one capture, scaled
            fp64_ncu = tr.get("fp64_pipe_active")
        except Exception:
            pass
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "traffic": traffic, "kernel": kname, "peak_kind": f"{peak_kind} hbm_gbs", "bytes_per_update": bpu,
                "role_ms_per_step" if persistent else "kernel_ms_per_step":
                    {names[k]: kern_ms[k] / args.steps for k in range(4)}}
    if persistent:
        roofline["role_ctas"] = {names[k]: role_ctas[k] for k in range(4)}
    if fp64_ncu is not None:
        roofline["fp64_pipe_active_ncu"] = fp64_ncu
    try:
        roofline["fp64_peak_tflops_dgemm"] = fp64_peak_tflops(torch)
    except Exception as ex:      # a measurement beside the line, never a reason to fail it
        roofline["fp64_peak_tflops_dgemm"] = f"unmeasured: {ex}"
    eng.close()
    del flush

    # plain FP64 on the same systems over the first steps of the same window
    vs_fp64 = None
    if precision == "mixed" and rank == 0 and not args.no_fp64_compare:
        k = max(1, args.steps // 5)
        e = G.Engine(G.FP64)
        ids64 = configs.add_to(e, specs)
        e.build()
        apply_budgets(e, specs, ids64)
        for _ in range(args.warmup):
            e.advance(0.0, min(n_iv, 40), tolerate_retire=True)
        reset_to_start(e, specs, ids64)
        ms64, u64 = 0.0, 0
        for j in range(k):
            u0 = e.compartment_updates(-1)
            e.advance(j * step_ms, n_iv, tolerate_retire=True)
            ms64 += e.last_advance_ms()
            u64 += e.compartment_updates(-1) - u0
        e.close()
        mixed_v = sum(step_units[:k]) / (sum(step_ms_dev[:k]) * 1e-3)
        vs_fp64 = {"fp64_value": u64 / (ms64 * 1e-3), "mixed_value": mixed_v, "ratio": mixed_v / (u64 / (ms64 * 1e-3)),
                   "window_ms": [0.0, k * step_ms], "unit": "compartment-updates/s (same systems, same window)"}
        if args.config in ("mixed", "screened", "sweep") and not args.no_accuracy:
            sample = {"mixed": lambda: configs.scaled_stated_batch(1.0 / 16),
                      "screened": lambda: configs.scaled_mixed_batch(1.0 / 16),
                      "sweep": lambda: configs.sweep_batch(n_gr=512, n_go=512)}[args.config]()
            vs_fp64["accuracy"] = accuracy_vs_fp64(G, configs, sample, horizon_ms=args.accuracy_ms)
    serving = None
    n_serve = 48 if args.serve_requests is None else args.serve_requests
    if n_serve > 0 and rank == 0 and args.config in ("mixed", "screened"):
        serving = run_serve(G, precision, n_serve, slots_scale=args.serve_slots,
                            ts_ms=tuple(args.serve_ts) if args.serve_ts else (5.0, 25.0))
    cpu = None
    if not args.no_cpu and rank == 0:
        cpu = cpu_baseline_single(args)
    counts = configs.type_counts(specs)
    cfg = config_key(args, wl)
    res = {"metric": "compartment-updates/s", "value": value, "unit": "compartment-updates/s",
           "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
           "ms_per_step": t_max_ms / args.steps, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f64 state+stages, f32 gating" if precision == "mixed" else "f64",
           "data": "synthetic (seeded morphologies, jitter and step currents)",
           "config": cfg,
           "run": {"precision": precision, "cells": {k: v[0] for k, v in counts.items()},
                   "compartments": n_compartments, "l2": "flushed (256 MB write) before each timed step",
                   "parallelism": f"replicas x{world}" if world > 1 else "single GPU", "setup_s": round(setup_s, 2),
                   "sim_ms_per_wall_s": window / (t_max_ms * 1e-3), "units_per_step": units / args.steps,
                   "units_per_step_list": step_units, "stopped_systems": len(stopped),
                   "autotune": {"granule_systems_per_warp": lanes, "seconds": round(tune_s, 2),
                                "how": "the launch after the warm-up replayed for 1 ms with 32, 16 and 8 "
                                       "granule systems per warp from a device snapshot; fastest kept"},
                   "stopped": stopped[:64]},
           "roofline": roofline, "gpu_launches": launches, "clocks": clk,
           "e2e": {"value": e2e_value, "unit": "compartment-updates/s", "h2d_bytes_per_step": h2d,
                   "d2h_bytes_per_step": d2h,
                   "timing": "host wall clock of each timed step: stimulus upload (pinned), launch, soma read-back"}}
    if serving:
        res["serving"] = serving
    if vs_fp64:
        res["vs_plain_fp64"] = vs_fp64
    if cpu:
        res["cpu_baseline"] = cpu
    return res


def pkj3x3_record(args, G, configs, torch, steps=5):
    """The Purkinje 3x3 workload (one 14 400-compartment system, plain FP64,
    [0, 200] ms) timed beside the mixed workload on rank 0: the same timing
    rules as its own line (`--config pkj3x3`), in `steps` timed steps after
    the warm-up."""
    import copy
    a = copy.copy(args)
    a.config, a.window_ms, a.steps = "pkj3x3", WINDOW_MS["pkj3x3"], steps
    a.no_cpu, a.no_fp64_compare, a.serve_requests = True, True, 0
    specs, wl = workload("pkj3x3", 1.0)
    r = run_batch(a, G, configs, torch, specs, wl, "fp64", 0, 1, None)
    return {"metric": r["metric"], "value": r["value"], "unit": r["unit"], "e2e": r["e2e"]["value"],
            "ms_per_step": r["ms_per_step"], "steps": steps, "warmup": a.warmup, "dtype": r["dtype"],
            "config": r["config"], "wall_s_window": r["ms_per_step"] * steps * 1e-3,
            "kernel": r["roofline"]["kernel"], "gpu_launches": r["gpu_launches"],
            "stopped_systems": r["run"]["stopped_systems"], "clocks": r["clocks"]}


def config_key(args, wl):
    """The workload description shared by this arm's line and the reference arm's."""
    return {"workload": wl, "window_ms": [0.0, args.window_ms], "step_sim_ms": args.window_ms / args.steps}


if __name__ == "__main__":
    main()
