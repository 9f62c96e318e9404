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
def workload(name, scale=1.0):
    import configs
    if name == "mixed" and scale < 1.0:
        specs = configs.scaled_mixed_batch(scale)
        c = configs.type_counts(specs)
        return specs, (f"mixed-type batch scaled x{scale:g}: {c['gr'][0]} GrC x4 + {c['go'][0]} GoC x131 + "
                       f"{c['pkj'][0]} PC x1600 + IO 16x16 net x3 (small profiling case)")
    if name == "mixed":
        return configs.mixed_batch(), "mixed-type batch: 4096 GrC x4 + 1024 GoC x131 + 256 PC x1600 + IO 16x16 net x3"
    if name == "pkj3x3":
        return configs.pkj_grid(3, 3), "Purkinje 3x3 grid, one RKC system, x-neighbour gap junctions, 0.5 nA"
    raise SystemExit(f"unknown config {name}")


# ------------------------------------------------------------ network
def run_network(args, G, configs, torch, precision, rank, world, dist):
    """The network workload: 2048 GrC, 512 GoC, 512 PC as independent systems
    coupled by 780 404 chemical synapses with delays (configs.network_batch).
    Network mode advances every system one interval per launch, then updates
    every synapse; a step is --step-ms of simulated time, timed on the host
    wall clock around the synchronous advance (launches included)."""
    specs, groups = configs.network_batch()
    eng = G.Engine(G.MIXED if precision == "mixed" else G.FP64)
    configs.add_network(eng, specs, groups)
    t0 = time.perf_counter()
    eng.build()
    setup_s = time.perf_counter() - t0
    n_iv = int(round(args.step_ms / H_MAX))
    t = 0.0
    for _ in range(args.warmup):
        eng.advance(t, n_iv, tolerate_retire=True)
        t += n_iv * H_MAX
    clocks = ClockSampler(int(os.environ.get("LOCAL_RANK", "0")))
    clocks.start()
    u0 = eng.compartment_updates(-1)
    torch.cuda.synchronize()
    w0 = time.perf_counter()
    for _ in range(args.steps):
        eng.advance(t, n_iv, tolerate_retire=True)
        t += n_iv * H_MAX
    torch.cuda.synchronize()
    wall = barrier_max(dist, time.perf_counter() - w0)
    clk = clocks.stop()
    units = barrier_sum(dist, eng.compartment_updates(-1) - u0)
    nsyn = sum(len(g["post_system"]) for g in groups)
    n_spk = eng.read_synapses(G.SYNF_S0, nsyn)
    peak, peak_kind = peaks()
    bpu = ALG_BYTES[precision]
    achieved = bpu * units / wall / 1e9
    if rank == 0:
        counts = configs.type_counts(specs)
        out = {"metric": "compartment-updates/s", "value": units / wall, "unit": "compartment-updates/s",
               "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
               "ms_per_step": wall * 1e3 / args.steps, "higher_is_better": True, "scaling": "weak",
               "vs_baseline": None, "dtype": "f64 state+stages, f32 gating" if precision == "mixed" else "f64",
               "data": "synthetic (seeded cells, synapses, weights and delays)",
               "config": {"workload": "network: 2048 GrC x4 + 512 GoC x131 + 512 PC x1600, 780404 synapses "
                                      "(MF->GrC Poisson 5-50 Hz, GrC->GoC, GoC->GrC, GrC->PC), lognormal weights, "
                                      "delays U[1,5] ms", "precision": precision, "step_sim_ms": args.step_ms,
                          "cells": {k: v[0] for k, v in counts.items()}, "synapses": nsyn,
                          "synapses_with_activity": int(np.count_nonzero(n_spk)),
                          "retired_systems": eng.retired(), "setup_s": round(setup_s, 2),
                          "timing": "host wall clock; one persistent launch and one synapse launch per interval",
                          "sim_ms_per_wall_s": args.steps * args.step_ms / wall},
               "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                            "frac": achieved / peak, "traffic": None, "kernel": "k_mega + k_syn_update",
                            "peak_kind": f"{peak_kind} hbm_gbs", "bytes_per_update": bpu},
               "gpu_launches": 2 * args.steps * n_iv, "clocks": clk}
        print(json.dumps(out))
    eng.close()
    if dist is not None:
        dist.destroy_process_group()


# ------------------------------------------------------------ FP64 comparison
def fp64_compare(G, configs, specs, n_iv, warmup, k, step_ms, step_units, flush, torch):
    """Plain FP64 on the same systems and time window as the first k timed
    mixed steps (throughput ratio), then the mixed precision's accuracy on
    a 1/16 sample of the workload: max |V_mixed - V_fp64| over every
    compartment after 1 ms and after 5 ms, and the device raster's spike
    counts over 20 ms."""
    eng = G.Engine(G.FP64)
    configs.add_to(eng, specs)
    eng.build()
    t = 0.0
    for _ in range(warmup):
        eng.advance(t, n_iv, tolerate_retire=True)
        t += n_iv * H_MAX
    ms, units = 0.0, 0
    for _ in range(k):
        flush.zero_()
        torch.cuda.synchronize()
        u0 = eng.compartment_updates(-1)
        eng.advance(t, n_iv, tolerate_retire=True)
        t += n_iv * H_MAX
        ms += eng.last_advance_ms()
        units += eng.compartment_updates(-1) - u0
    eng.close()
    fp64 = units / (ms * 1e-3)
    mixed = sum(step_units[:k]) / (sum(step_ms[:k]) * 1e-3)
    sample = configs.scaled_mixed_batch(1.0 / 16)
    res = {}
    for prec in (G.FP64, G.MIXED):
        e = G.Engine(prec)
        ids = configs.add_to(e, sample)
        e.build()
        e.record_spikes(1 << 20)
        v = []
        tt = 0.0
        for n in (8, 32, 120):          # to 1 ms, 5 ms, 20 ms
            e.advance(tt, n, tolerate_retire=True)
            tt += n * H_MAX
            v.append(np.concatenate([e.read(i, G.F_VNEW) for i in ids]))
        counts = {}
        for ty in range(4):
            _, sy, ce = e.read_spikes(ty)
            for a, b in zip(sy.tolist(), ce.tolist()):
                counts[(a, b)] = counts.get((a, b), 0) + 1
        res[prec] = (v, counts, e.retired())
        e.close()
    (v64, s64, r64), (v32, s32, r32) = res[G.FP64], res[G.MIXED]
    return {"fp64_value": fp64, "mixed_value": mixed, "ratio": mixed / fp64, "steps": k,
            "unit": "compartment-updates/s (same systems, same window)",
            "accuracy_sample": "mixed batch x1/16 (256 GrC, 64 GoC, 16 PC, IO 16x16), from t = 0",
            "max_abs_err_mv": {"1ms": float(np.max(np.abs(v32[0] - v64[0]))),
                               "5ms": float(np.max(np.abs(v32[1] - v64[1]))),
                               "20ms": float(np.max(np.abs(v32[2] - v64[2])))},
            "spikes_20ms": {"fp64": sum(s64.values()), "mixed": sum(s32.values()),
                            "cells_with_equal_counts": sum(1 for c in set(s64) | set(s32) if s64.get(c) == s32.get(c)),
                            "cells_spiking": len(set(s64) | set(s32))},
            "stopped_systems": {"fp64": r64, "mixed": r32}}


# ------------------------------------------------------------ serving
def run_serve(G, precision, n_requests, seed=5, quantum=8, n_compare=8, slots_scale=1):
    """Serve a Poisson request stream (configs.serve_workload) through the
    request server on the wall clock: requests are submitted when their
    arrival time has passed, every round admits what fits and advances all
    resident requests one quantum.  Latency = completion - arrival.  Then a
    sample of the same requests runs one at a time, each in its own plain
    FP64 engine (build, advance, read back), for the throughput ratio and the
    served results' voltage error and spike counts against FP64."""
    import configs
    classes, reqs = configs.serve_workload(n_requests, seed=seed, slots_scale=slots_scale)
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
                        f"/ 1-128 GoC x131 (6 shapes) / 1-16 PC x1600 (5 shapes); 5-25 ms each; seed {seed}")}
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
        w0 = time.perf_counter()
        eng = G.Engine(G.FP64)
        for j in range(r.n_systems):
            sl = slice(j * cells, (j + 1) * cells)
            eng.add_system(c.cell_type, c.nx, c.ny, c.rows, r.jitter[sl], stim=tuple(a[sl] for a in r.stim),
                           gap=c.gap, cond_scale=r.cond_scale[sl],
                           io_gap_g=None if r.io_gap_g is None else r.io_gap_g[4 * j * cells:4 * (j + 1) * cells])
        eng.build()
        eng.record_spikes(1 << 20)
        eng.advance(0.0, r.n_intervals, tolerate_retire=True)
        v = np.concatenate([eng.read(j, G.F_VNEW) for j in range(r.n_systems)])
        dt = time.perf_counter() - w0
        seq_wall += dt
        seq_cu += eng.compartment_updates(-1)
        pt = per_type.setdefault(c.cell_type, [0.0, 0.0])
        pt[0] += cell_ms(r)
        pt[1] += dt
        ft, _, _ = eng.read_spikes(c.cell_type)
        eng.close()
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
                             "precision": precision}
    srv.close()
    return out


# ------------------------------------------------------------ CPU side
def _oracle_worker(args):
    """Run a slice of a sampled workload in the oracle (reference arithmetic)."""
    cfg, fraction, idx, t_begin, n_iv, warm_iv = args
    sys.path.insert(0, PKG)
    sys.path.insert(0, ORACLE)
    import configs
    import oracle_py as O
    specs = configs.scaled_mixed_batch(fraction) if cfg == "mixed" else configs.pkj_grid(3, 3)
    systems = [(specs[i], configs.add_to_oracle(O, specs[i], canon=False)) for i in idx]
    t = 0.0
    for _ in range(warm_iv):
        for sp, s in systems:
            s.advance(t)
        t += H_MAX
    before = sum((s.stats()["stages"] + s.stats()["steps"]) * sp.nc for sp, s in systems)
    t0 = time.perf_counter()
    for _ in range(n_iv):
        for sp, s in systems:
            if s.advance(t) != 0:
                raise RuntimeError("oracle step failed")
        t += H_MAX
    dt = time.perf_counter() - t0
    after = sum((s.stats()["stages"] + s.stats()["steps"]) * sp.nc for sp, s in systems)
    return after - before, dt


def cpu_sample(cfg, fraction, n_iv, warm_iv, workers):
    """Time the oracle on a bounded, proportional sample of the workload."""
    import configs
    specs = configs.scaled_mixed_batch(fraction) if cfg == "mixed" else configs.pkj_grid(3, 3)
    order = sorted(range(len(specs)), key=lambda i: -specs[i].nc)
    slices = [order[k::workers] for k in range(workers)]
    jobs = [(cfg, fraction, sl, 0.0, n_iv, warm_iv) for sl in slices if sl]
    if workers == 1:
        res = [_oracle_worker(j) for j in jobs]
    else:
        import multiprocessing as mp
        with mp.get_context("spawn").Pool(len(jobs)) as pool:
            res = pool.map(_oracle_worker, jobs)
    units = sum(r[0] for r in res)
    wall = max(r[1] for r in res)
    counts = configs.type_counts(specs)
    desc = ", ".join(f"{v[0]} {k}" for k, v in counts.items())
    return units, wall, f"{desc}; {n_iv} intervals ({n_iv * H_MAX:g} ms) after {warm_iv} warm-up intervals"


def run_reference(args):
    """The reference arm: the CPU restatement of the reference's RKC path (the
    reference's own CUDA code cannot travel: its sources are not part of this
    repository), on all host cores, over a bounded sample of the workload."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    cores = os.cpu_count() or 1
    cfg = args.config
    fraction = 1.0 / 16 if cfg == "mixed" else 1.0
    n_iv = 8 if cfg == "mixed" else 4
    vals = []
    for k in range(args.warmup + args.steps):
        units, wall, sample = cpu_sample(cfg, fraction, n_iv, 0, cores)
        if k >= args.warmup:
            vals.append((units, wall))
    units = sum(u for u, _ in vals)
    wall = sum(w for _, w in vals)
    v = units / wall
    _, wl = workload(cfg)
    out = {"impl": "reference", "metric": "compartment-updates/s", "value": v, "unit": "compartment-updates/s",
           "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
           "ms_per_step": 1e3 * wall / max(1, len(vals)), "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded morphologies and stimuli)",
           "config": {"workload": wl, "precision": "fp64 (reference arithmetic)"},
           "cpu_baseline": {"value": v, "unit": "compartment-updates/s", "cores": cores, "kind": "port",
                            "cpu": cpu_model(),
                            "sample": sample},
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
    ap.add_argument("--config", default="mixed", choices=["mixed", "pkj3x3", "serve", "network"])
    ap.add_argument("--precision", default=None, choices=["mixed", "fp64"])
    ap.add_argument("--step-ms", type=float, default=5.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--scale", type=float, default=1.0,
                    help="population fraction of the mixed batch (small profiling cases; 1 = the benchmark)")
    ap.add_argument("--no-fp64-compare", action="store_true")
    ap.add_argument("--serve-slots", type=int, default=1, help="multiplier on the serving arenas' slot counts")
    ap.add_argument("--serve-requests", type=int, default=None,
                    help="requests of the serving stream (default 48 beside the mixed workload, 128 for "
                         "--config serve; 0: none)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
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
        sv = run_serve(G, precision, args.serve_requests or 128, slots_scale=args.serve_slots)
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
    eng = G.Engine(G.MIXED if precision == "mixed" else G.FP64)
    configs.add_to(eng, specs)
    t_setup = time.perf_counter()
    eng.build()
    setup_s = time.perf_counter() - t_setup
    n_iv = int(round(args.step_ms / H_MAX))
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")  # > L2 (129 MB)
    t = 0.0
    for _ in range(args.warmup):
        eng.advance(t, n_iv, tolerate_retire=True)
        t += n_iv * H_MAX
    torch.cuda.synchronize()
    clocks = ClockSampler(int(os.environ.get("LOCAL_RANK", "0")))
    clocks.start()
    dev_ms, kern_ms = 0.0, {k: 0.0 for k in range(4)}
    step_ms, step_units = [], []
    units0 = eng.compartment_updates(-1)
    units_t0 = {k: eng.compartment_updates(k) for k in range(4)}
    if dist is not None:
        dist.barrier()
    torch.cuda.synchronize()
    wall0 = time.perf_counter()
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        u0 = eng.compartment_updates(-1)
        eng.advance(t, n_iv, tolerate_retire=True)
        t += n_iv * H_MAX
        dev_ms += eng.last_advance_ms()
        step_ms.append(eng.last_advance_ms())
        step_units.append(eng.compartment_updates(-1) - u0)
        for k in range(4):
            kern_ms[k] += eng.last_kernel_ms(k)
    torch.cuda.synchronize()
    wall = time.perf_counter() - wall0
    if dist is not None:
        dist.barrier()
    clk = clocks.stop()
    units = eng.compartment_updates(-1) - units0
    units_t = {k: eng.compartment_updates(k) - units_t0[k] for k in range(4)}
    t_max_ms = barrier_max(dist, dev_ms)
    units_all = barrier_sum(dist, units)
    value = units_all / (t_max_ms * 1e-3)
    persistent, role_ctas = eng.launch_layout()
    if persistent:
        launches = args.steps
    else:
        launches = args.steps * sum(1 for k in range(4) if eng.type_cells(k) > 0)

    # roofline of the dominant kernel: the one persistent launch, or the
    # longest per-type launch
    names = {0: "gr", 1: "go", 2: "pkj", 3: "io"}
    peak, peak_kind = peaks()
    bpu = ALG_BYTES[precision]
    if persistent:
        kname, key = "k_mega", "mega"
        per_launch_units = units / args.steps
        per_launch_ms = dev_ms / args.steps
    else:
        dom = max(range(4), key=lambda k: kern_ms[k])
        kname, key = f"k_advance<{names[dom]}>", names[dom]
        per_launch_units = units_t[dom] / args.steps
        per_launch_ms = kern_ms[dom] / args.steps
    per_launch_bytes = bpu * per_launch_units
    achieved = per_launch_bytes / (per_launch_ms * 1e-3) / 1e9 if per_launch_ms > 0 else 0.0
    traffic = None
    tfile = os.path.join(ROOT, "profiles", f"traffic_{args.config}_{precision}.json")
    if os.path.exists(tfile):
        try:
            tr = json.load(open(tfile))
            # bytes per compartment-update from one capture, scaled to this launch
            if key in tr:
                traffic = tr[key] * per_launch_units
        except Exception:
            traffic = None
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "traffic": traffic, "kernel": kname,
                "peak_kind": f"{peak_kind} hbm_gbs", "bytes_per_update": bpu,
                "role_ms_per_step" if persistent else "kernel_ms_per_step":
                    {names[k]: kern_ms[k] / args.steps for k in range(4)}}
    if persistent:
        roofline["role_ctas"] = {names[k]: role_ctas[k] for k in range(4)}
    # what bounds the kernel instead: the FP64 pipe, as ncu reported it for the
    # same kernel (profiles/), beside the HBM fraction above
    if os.path.exists(tfile):
        try:
            tr = json.load(open(tfile))
            if "fp64_pipe_active" in tr:
                roofline["fp64_pipe_active_ncu"] = tr["fp64_pipe_active"]
        except Exception:
            pass

    # end to end through the C ABI with host buffers: per step, upload every
    # cell's stimulus table -- the workload's own protocol, so the dynamics
    # match the device-timed steps -- (pinned host -> device) and read back
    # every cell's soma voltage at every interval (device -> pinned host)
    e2e = None
    if not args.no_e2e:
        # a second engine with the same systems runs the same warm-up and
        # steps, so e2e covers exactly the device-timed work plus the copies
        eng.close()
        eng = G.Engine(G.MIXED if precision == "mixed" else G.FP64)
        configs.add_to(eng, specs)
        eng.build()
        ncell = {k: eng.type_cells(k) for k in range(4)}
        eng.record_soma(n_iv)
        bufs = {}
        cell_specs = {k: [] for k in range(4)}
        for s in specs:
            cell_specs[s.cell_type].append(s)
        for k in range(4):
            if ncell[k] == 0:
                continue
            comp = torch.empty(ncell[k], dtype=torch.int32, pin_memory=True)
            amp, t0v, t1v = (torch.empty(ncell[k], dtype=torch.float64, pin_memory=True) for _ in range(3))
            cs, am, a0, a1 = [], [], [], []
            for s in cell_specs[k]:
                cs.append(np.broadcast_to(np.asarray(s.stim[0]), s.n))
                am.append(np.broadcast_to(np.asarray(s.stim[1], dtype=np.float64), s.n))
                a0.append(np.broadcast_to(np.asarray(s.stim[2], dtype=np.float64), s.n))
                a1.append(np.broadcast_to(np.asarray(s.stim[3], dtype=np.float64), s.n))
            comp.numpy()[:] = np.concatenate(cs)
            amp.numpy()[:] = np.concatenate(am)
            t0v.numpy()[:] = np.concatenate(a0)
            t1v.numpy()[:] = np.concatenate(a1)
            soma = torch.empty((n_iv, ncell[k]), dtype=torch.float64, pin_memory=True)
            bufs[k] = (comp, amp, t0v, t1v, soma)
        h2d = sum(b[0].numel() * 4 + 3 * b[1].numel() * 8 for b in bufs.values())
        d2h = sum(b[4].numel() * 8 for b in bufs.values())
        t = 0.0

        def e2e_step(t):
            for k, (comp, amp, t0v, t1v, soma) in bufs.items():
                eng.set_stim_type(k, comp.numpy(), amp.numpy(), t0v.numpy(), t1v.numpy())
            eng.rewind_soma()
            eng.advance(t, n_iv, tolerate_retire=True)
            for k, (comp, amp, t0v, t1v, soma) in bufs.items():
                eng.read_soma_type(k, n_iv, soma.numpy())

        for _ in range(args.warmup):
            e2e_step(t)
            t += n_iv * H_MAX
        e_units0 = eng.compartment_updates(-1)
        torch.cuda.synchronize()
        w0 = time.perf_counter()
        for _ in range(args.steps):
            e2e_step(t)
            t += n_iv * H_MAX
        torch.cuda.synchronize()
        e_wall = time.perf_counter() - w0
        e_units = eng.compartment_updates(-1) - e_units0
        e_wall = barrier_max(dist, e_wall)
        e_units = barrier_sum(dist, e_units)
        e2e = {"value": e_units / e_wall, "unit": "compartment-updates/s", "h2d_bytes_per_step": h2d,
               "d2h_bytes_per_step": d2h, "timing": "host wall clock incl. pinned copies"}

    n_compartments, n_retired = eng.total_compartments(), eng.retired()

    # the same systems in plain FP64 over the first timed steps (same warm-up),
    # and the mixed precision's voltage error and spike counts against FP64
    vs_fp64 = None
    if precision == "mixed" and rank == 0 and not args.no_fp64_compare and args.config == "mixed":
        eng.close()
        vs_fp64 = fp64_compare(G, configs, specs, n_iv, args.warmup, min(3, args.steps), step_ms, step_units,
                               flush, torch)
    serving = None
    n_serve = 48 if args.serve_requests is None else args.serve_requests
    if n_serve > 0 and rank == 0 and args.config == "mixed":
        eng.close()
        serving = run_serve(G, precision, n_serve, slots_scale=args.serve_slots)

    cpu = None
    if not args.no_cpu and rank == 0:
        # bounded single-thread sample of the same workload in the oracle
        frac = 1.0 / 256 if args.config == "mixed" else 1.0
        probe_units, probe_wall, _ = cpu_sample(args.config, frac, 2, 0, 1)
        per_iv = max(probe_wall / 2, 1e-3)
        n_cpu = int(max(4, min(4000, args.cpu_seconds / per_iv)))
        units_c, wall_c, sample = cpu_sample(args.config, frac, n_cpu, 0, 1)
        cpu = {"value": units_c / wall_c, "unit": "compartment-updates/s", "cores": 1, "kind": "port",
               "cpu": cpu_model(), "nproc": os.cpu_count(),
               "sample": sample + " (oracle, reference arithmetic, FP64, one thread)"}

    if rank == 0:
        counts = configs.type_counts(specs)
        out = {"metric": "compartment-updates/s", "value": value, "unit": "compartment-updates/s",
               "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
               "ms_per_step": t_max_ms / args.steps, "higher_is_better": True, "scaling": "weak",
               "vs_baseline": None, "dtype": "f64 state+stages, f32 gating" if precision == "mixed" else "f64",
               "data": "synthetic (seeded morphologies, jitter and step currents)",
               "config": {"workload": wl, "precision": precision, "step_sim_ms": args.step_ms,
                          "cells": {k: v[0] for k, v in counts.items()},
                          "compartments": n_compartments,
                          "l2": "flushed (256 MB write) between timed steps",
                          "parallelism": f"replicas x{world}" if world > 1 else "single GPU",
                          "setup_s": round(setup_s, 2), "wall_s": round(wall, 3),
                          "retired_systems": n_retired,
                          "sim_ms_per_wall_s": args.steps * args.step_ms / (t_max_ms * 1e-3),
                          "units_per_step": units / args.steps},
               "roofline": roofline, "gpu_launches": launches, "clocks": clk}
        if e2e:
            out["e2e"] = e2e
        if serving:
            out["serving"] = serving
        if vs_fp64:
            out["vs_plain_fp64"] = vs_fp64
        if cpu:
            out["cpu_baseline"] = cpu
        print(json.dumps(out))
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
