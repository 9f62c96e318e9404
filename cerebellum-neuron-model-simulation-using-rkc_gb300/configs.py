"""Benchmark and test workloads as seeded synthetic inputs.

A workload is a list of system specs; ``add_to(engine, specs)`` registers them
with a gbrkc Engine and ``add_to_oracle`` builds the same systems in the CPU
oracle.  No dataset is involved: every morphology, jitter and stimulus comes
from a documented seed.

* ``pkj_grid``: the reference-style plain run -- nx x ny Purkinje cells of one
  synthetic tree, x-neighbour gap junctions, one RKC system (every cell shares
  one step size), constant somatic current.  3x3 at 0.5 nA for 200 ms is the
  plain-FP64 drop-in case.
* ``mixed_batch``: 4096 reduced granule cells (4 compartments), 1024 Golgi
  cells (131), 256 Purkinje cells (1600) and one 16x16 inferior-olive
  gap-junction network (768 compartments, edge conductances G_C x U[0.5,1.5]);
  every cell but the olive network is its own RKC system; per-cell step
  currents switched on at U[0, 20] ms.  Amplitudes: the batch is held in the
  regime where the reference's frozen-current splitting stays finite for
  500 ms (screened on the GPU in both precisions): Purkinje U[0, 0.4] nA on
  trees 7, 8, 9, 12, 13; Golgi U[0, 0.4] nA on six tree variants; granule
  U[0, 0.05] nA (the reference drives it with 0.01 nA); olive U[0, 6]
  uA/cm^2 (its reference units; the reference uses 5.5).  At 0.6 nA some
  Purkinje and Golgi trees diverge (NaN) in the reference scheme itself.
"""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import Optional

import numpy as np

import morph as M

G_C_IO = 0.04


@dataclass
class Spec:
    cell_type: int
    nx: int
    ny: int
    rows: np.ndarray
    jitter: np.ndarray
    stim: Optional[tuple] = None
    gap: bool = False
    gj_pairs: Optional[np.ndarray] = None
    io_gap_g: Optional[np.ndarray] = None
    tol: float = 0.0
    cond_scale_ch: Optional[np.ndarray] = None   # per cell and channel density factors
    tag: str = ""
    extra: dict = field(default_factory=dict)

    @property
    def n(self):
        return self.nx * self.ny

    @property
    def nc(self):
        return self.n * self.rows.shape[0]


def _jitter(rng, n):
    # same range as the reference's init_v_rand: (-0.5, 0.5)
    return rng.uniform(-0.5, 0.5, n)


def reference_jitter(cell_type: int, n: int, seed: int = 0) -> np.ndarray:
    """The reference's own initial jitter of n cells of one type: libc srand
    (seed) then one rand() per cell, (rand() + 1) / (RAND_MAX + 2) - 0.5 for
    GrC and PC (gr_ion.cu:642, pkj_ion.cu:367), rand() / RAND_MAX - 0.5 for
    GoC and IO (go_ion.cu:598, io_ion.cu:172), as a run of main.cu (srand(0)
    at main.cu:38) with only this type draws it."""
    import ctypes
    libc = ctypes.CDLL(None)
    libc.srand(ctypes.c_uint(seed))
    rand_max = 2147483647.0   # glibc RAND_MAX
    r = np.array([libc.rand() for _ in range(n)], dtype=np.float64)
    if cell_type in (M.GR, M.PKJ):
        return ((r + 1.0) / (rand_max + 2.0)) - 0.5
    return (r / rand_max) - 0.5


# Purkinje trees whose cells stay finite for 500 ms at 0.1-0.4 nA under the
# reference's frozen-current splitting, in FP64 and in mixed precision
# (screened on the GPU); Golgi tree variants likewise.
PKJ_STABLE_SEEDS = (7, 8, 9, 12, 13)
GO_STABLE_VARIANTS = (0, 1, 3, 5, 6, 7)


def pkj_grid(nx=3, ny=3, seed=2, amp=0.5e-3, tree_seed=None, gap=True, jitter="reference"):
    """Reference-style Purkinje grid (one RKC system) of one seeded synthetic
    tree (PKJ_STABLE_SEEDS[0] unless given), a constant somatic current.  The
    initial jitter is the reference's own rand() sequence (srand(0)), so its
    CUDA build runs exactly this system from the same model file; with
    jitter="seeded" it is drawn from numpy with seed."""
    rows = M.pkj_synthetic(tree_seed if tree_seed is not None else PKJ_STABLE_SEEDS[0])
    n = nx * ny
    jit = reference_jitter(M.PKJ, n) if jitter == "reference" else _jitter(np.random.default_rng(seed), n)
    return [Spec(M.PKJ, nx, ny, rows, jit, stim=(rows.shape[0] - 1, amp, 0.0, 1e9),
                 gap=gap, gj_pairs=M.PKJ_GJ_PAIRS, tag=f"pkj{nx}x{ny}")]


AMP_MAX = {M.GR: 0.05e-3, M.GO: 0.4e-3, M.PKJ: 0.4e-3, M.IO: 6.0}


def mixed_batch(seed=2, n_gr=4096, n_go=1024, n_pkj=256, io_side=16, amp_max=None, go_variants=GO_STABLE_VARIANTS,
                pkj_seeds=PKJ_STABLE_SEEDS, pkj_taper=True):
    """The mixed-type batch.  amp_max (per type) bounds the step currents;
    go_variants / pkj_seeds pick the tree shapes, cycled over the cells;
    pkj_taper=False gives untapered Purkinje trees.  Each spec's tag names
    its type and shape ("pkj7", "go3", ...)."""
    amp = dict(AMP_MAX if amp_max is None else amp_max)
    rng = np.random.default_rng(seed)
    specs = []
    gr_rows = M.gr_reduced4()
    for i in range(n_gr):
        specs.append(Spec(M.GR, 1, 1, gr_rows, _jitter(rng, 1),
                          stim=(1, rng.uniform(0, amp[M.GR]), rng.uniform(0, 20.0), 1e9), tag="gr"))
    go_rows = [M.go_synthetic(seed * 1000 + k) for k in go_variants]
    for i in range(n_go):
        specs.append(Spec(M.GO, 1, 1, go_rows[i % len(go_rows)], _jitter(rng, 1),
                          stim=(30, rng.uniform(0, amp[M.GO]), rng.uniform(0, 20.0), 1e9),
                          tag=f"go{go_variants[i % len(go_rows)]}"))
    pk_rows = [M.pkj_synthetic(s, taper=pkj_taper) for s in pkj_seeds]
    for i in range(n_pkj):
        r = pk_rows[i % len(pk_rows)]
        specs.append(Spec(M.PKJ, 1, 1, r, _jitter(rng, 1),
                          stim=(r.shape[0] - 1, rng.uniform(0, amp[M.PKJ]), rng.uniform(0, 20.0), 1e9),
                          tag=f"pkj{pkj_seeds[i % len(pk_rows)]}"))
    if io_side > 0:
        n = io_side * io_side
        specs.append(Spec(M.IO, io_side, io_side, M.io_rows(), _jitter(rng, n),
                          stim=(np.zeros(n, np.int32), rng.uniform(0, amp[M.IO], n), rng.uniform(0, 20.0, n),
                                np.full(n, 1e9)),
                          gap=True, io_gap_g=G_C_IO * rng.uniform(0.5, 1.5, 4 * n), tag="io"))
    return specs


# The mixed batch's per-type current bounds as its specification states them
# (U[0, 0.6] nA for every cell), in each model's units: mA for GrC / GoC / PC;
# for the olive, whose injected current is a density (uA/cm^2, io.cu:247),
# 0.6 nA = 6e-4 uA over its dendrite's lateral area (pi x 6 um x 53.07 um =
# 1.0e-5 cm^2): 60 uA/cm^2.
IO_DEND_AREA_CM2 = np.pi * 6.0e-4 * 53.07e-4
STATED_AMP = {M.GR: 0.6e-3, M.GO: 0.6e-3, M.PKJ: 0.6e-3, M.IO: 0.6e-3 / IO_DEND_AREA_CM2}


def stated_mixed_batch(seed=2, n_gr=4096, n_go=1024, n_pkj=256, io_side=16):
    """The mixed batch with the stated currents (STATED_AMP), a distinct seeded
    Golgi tree per Golgi cell and a distinct seeded Purkinje tree per Purkinje
    cell (tapered diameters: untapered trees go non-finite within
    milliseconds under the reference's frozen-current splitting, in its own
    build too)."""
    rng = np.random.default_rng(seed)
    specs = []
    gr_rows = M.gr_reduced4()
    for i in range(n_gr):
        specs.append(Spec(M.GR, 1, 1, gr_rows, _jitter(rng, 1),
                          stim=(1, rng.uniform(0, STATED_AMP[M.GR]), rng.uniform(0, 20.0), 1e9), tag="gr"))
    for i in range(n_go):
        rows = M.go_synthetic(seed * 100000 + i)
        specs.append(Spec(M.GO, 1, 1, rows, _jitter(rng, 1),
                          stim=(30, rng.uniform(0, STATED_AMP[M.GO]), rng.uniform(0, 20.0), 1e9), tag=f"go#{i}"))
    for i in range(n_pkj):
        rows = M.pkj_synthetic(seed * 100000 + i)
        specs.append(Spec(M.PKJ, 1, 1, rows, _jitter(rng, 1),
                          stim=(rows.shape[0] - 1, rng.uniform(0, STATED_AMP[M.PKJ]), rng.uniform(0, 20.0), 1e9),
                          tag=f"pkj#{i}"))
    if io_side > 0:
        n = io_side * io_side
        specs.append(Spec(M.IO, io_side, io_side, M.io_rows(), _jitter(rng, n),
                          stim=(np.zeros(n, np.int32), rng.uniform(0, STATED_AMP[M.IO], n), rng.uniform(0, 20.0, n),
                                np.full(n, 1e9)),
                          gap=True, io_gap_g=G_C_IO * rng.uniform(0.5, 1.5, 4 * n), tag="io"))
    return specs


def scaled_stated_batch(fraction: float, seed=2):
    """stated_mixed_batch with every population but the olive network scaled
    (bounded CPU samples and accuracy samples)."""
    return stated_mixed_batch(seed=seed, n_gr=max(1, int(4096 * fraction)), n_go=max(1, int(1024 * fraction)),
                              n_pkj=max(1, int(256 * fraction)), io_side=16)


def scaled_mixed_batch(fraction: float, seed=2):
    """The mixed batch with every population scaled (for bounded CPU samples)."""
    return mixed_batch(seed=seed, n_gr=max(1, int(4096 * fraction)), n_go=max(1, int(1024 * fraction)),
                       n_pkj=max(1, int(256 * fraction)), io_side=16)


def sweep_batch(seed=4, n_gr=32768, n_go=32768, amp_max=0.4e-3, ts_ms=(100.0, 1000.0)):
    """Parameter-sweep batch: n_gr reduced granule cells and n_go Golgi cells
    (one seeded tree), every instance its own RKC system, no gap junctions.
    Each instance scales every channel density by its own U[0.8, 1.2]
    (cond_scale_ch, the per-compartment conductances the reference builds
    from its model rows, gr.cu:31-35, go.cu:33-38), takes a step current
    U[0, amp_max] switched on at t = 0 at the reference's stimulated
    compartment, and runs for its own duration U[ts_ms] (whole intervals,
    kept in spec.extra["n_intervals"]: the engine's per-system interval
    budget)."""
    rng = np.random.default_rng(seed)
    gr_rows, go_rows = M.gr_reduced4(), M.go_synthetic(seed * 1000)
    specs = []
    for t, n, rows, comp, ncond in ((M.GR, n_gr, gr_rows, 1, 10), (M.GO, n_go, go_rows, 30, 13)):
        for i in range(n):
            sp = Spec(t, 1, 1, rows, _jitter(rng, 1), stim=(comp, rng.uniform(0, amp_max), 0.0, 1e9),
                      cond_scale_ch=rng.uniform(0.8, 1.2, ncond), tag="gr" if t == M.GR else "go")
            sp.extra["n_intervals"] = int(round(rng.uniform(*ts_ms) / 0.125))
            specs.append(sp)
    return specs


@dataclass
class ServeClass:
    name: str
    cell_type: int
    nx: int
    ny: int
    rows: np.ndarray
    slots: int
    max_systems: int     # largest request of this class
    stim_comp: int
    gap: bool = False


@dataclass
class Request:
    cls: int             # index into the class list
    n_systems: int
    n_intervals: int
    arrival_s: float     # wall-clock arrival after the start
    jitter: np.ndarray
    stim: tuple
    cond_scale: np.ndarray
    io_gap_g: Optional[np.ndarray] = None


def serve_workload(n_requests=64, seed=5, rate_hz=200.0, ts_ms=(5.0, 25.0), io_fraction=0.2, slots_scale=1):
    """Request stream of the serving benchmark: Poisson arrivals at rate_hz;
    each request is either an inferior-olive 4x4 gap-junction network set
    (io_fraction; 1-8 networks, edge conductances G_C x U[0.5,1.5]) or
    U{1..max} cells of one granule / Golgi / Purkinje shape; duration
    U[ts_ms] rounded to whole 0.125 ms intervals; per-cell step currents
    U[0, AMP_MAX] from t = 0 and channel densities x U[0.8, 1.2].  Request
    sizes and durations are scaled down from 1-4096 cells and 50-1000 ms so
    that the whole stream finishes in tens of seconds.  The arenas hold about
    half the stream's cells at once (32768 granule slots, 768 per Golgi
    shape, 96 per Purkinje shape, 128 olive networks; 0.42 GB of HBM);
    slots_scale multiplies them.  A quarter of that queues more and halves
    the throughput (measured on the GB300: 3.5e9 against 6.5e9
    compartment-updates/s, p99 12.6 s against 6.7 s)."""
    rng = np.random.default_rng(seed)
    classes = [ServeClass("gr", M.GR, 1, 1, M.gr_reduced4(), 32768 * slots_scale, 4096, 1)]
    for k in GO_STABLE_VARIANTS:
        classes.append(ServeClass(f"go{k}", M.GO, 1, 1, M.go_synthetic(2000 + k), 768 * slots_scale, 128, 30))
    for k in PKJ_STABLE_SEEDS:
        r = M.pkj_synthetic(k)
        classes.append(ServeClass(f"pkj{k}", M.PKJ, 1, 1, r, 96 * slots_scale, 16, r.shape[0] - 1))
    classes.append(ServeClass("io4x4", M.IO, 4, 4, M.io_rows(), 128 * slots_scale, 8, 0, gap=True))
    by_type = {t: [i for i, c in enumerate(classes) if c.cell_type == t] for t in (M.GR, M.GO, M.PKJ, M.IO)}
    reqs = []
    t = 0.0
    for _ in range(n_requests):
        t += rng.exponential(1.0 / rate_hz)
        if rng.uniform() < io_fraction:
            ci = by_type[M.IO][0]
        else:
            ty = (M.GR, M.GO, M.PKJ)[rng.integers(0, 3)]
            ci = by_type[ty][rng.integers(0, len(by_type[ty]))]
        c = classes[ci]
        n_sys = int(rng.integers(1, c.max_systems + 1))
        cells = n_sys * c.nx * c.ny
        n_iv = int(round(rng.uniform(*ts_ms) / 0.125))
        amp = rng.uniform(0, AMP_MAX[c.cell_type], cells)
        stim = (np.full(cells, c.stim_comp, np.int32), amp, np.zeros(cells), np.full(cells, 1e9))
        gg = G_C_IO * rng.uniform(0.5, 1.5, 4 * cells) if c.cell_type == M.IO else None
        reqs.append(Request(ci, n_sys, n_iv, t, _jitter(rng, cells), stim, rng.uniform(0.8, 1.2, cells), gg))
    return classes, reqs


# mossy fibre -> granule, granule -> Golgi, Golgi -> granule, granule -> Purkinje
SYN_MFGR, SYN_GRGO, SYN_GOGR, SYN_GRPKJ = 0, 1, 2, 3


# Shapes that stay finite in the network workload (screened on the GPU in
# both precisions over 12 ms): Golgi variant 3 and Purkinje tree 9 diverge
# under its synaptic drive in the reference scheme itself.
NET_GO_VARIANTS = (0, 1, 5, 6, 7)
NET_PKJ_SEEDS = (7, 8, 12, 13)


def network_batch(seed=3, n_gr=2048, n_go=512, n_pkj=512, n_syn=780404, mf_groups=8, sigma=0.25,
                  scale=(1.0, 1.0, 1.0, 1.0), distinct_trees=True):
    """Network workload: n_gr reduced granule cells, n_go Golgi cells and
    n_pkj Purkinje cells, each its own system -- with distinct_trees a
    distinct seeded tree per Golgi and per Purkinje cell (tapered Purkinje
    diameters), else the shapes NET_GO_VARIANTS / NET_PKJ_SEEDS -- coupled by
    n_syn chemical synapses with the reference's
    kinetics: 4 mossy fibres per granule cell (Poisson, groups at 5-50 Hz),
    100 granule cells onto each Golgi soma, 4 Golgi cells onto each granule
    soma, and the rest granule -> Purkinje onto random dendritic
    compartments.  Weights are lognormal (sigma 0.25; at 0.5 the mossy-fibre
    tail drives some granule cells to divergence) around the reference's,
    scaled by the postsynaptic cell's input count as syn.cu:57, 175, 328, 511
    do (W_MFGR / 4, W_GRGO / (n / 4), W_GOGR / (4 n), W_GRPKJ / (512 n / 10)
    with the constants of syn.cuh:54-58); every synapse has a transmission
    delay of U[1, 5] ms
    (8-40 intervals).  No injected current.  Returns (specs, groups); each
    group is the keyword arguments of Engine.add_synapses with system
    indices into specs."""
    rng = np.random.default_rng(seed)
    gr_rows = M.gr_reduced4()
    if distinct_trees:
        go_rows = [M.go_synthetic(seed * 100000 + i) for i in range(n_go)]
        pk_rows = [M.pkj_synthetic(seed * 100000 + 50000 + i) for i in range(n_pkj)]
    else:
        go_rows = [M.go_synthetic(2000 + k) for k in NET_GO_VARIANTS]
        pk_rows = [M.pkj_synthetic(k) for k in NET_PKJ_SEEDS]
    specs = [Spec(M.GR, 1, 1, gr_rows, _jitter(rng, 1), tag="gr") for _ in range(n_gr)]
    specs += [Spec(M.GO, 1, 1, go_rows[i % len(go_rows)], _jitter(rng, 1), tag=f"go#{i}") for i in range(n_go)]
    specs += [Spec(M.PKJ, 1, 1, pk_rows[i % len(pk_rows)], _jitter(rng, 1), tag=f"pkj#{i}") for i in range(n_pkj)]
    gr = np.arange(n_gr)
    go = n_gr + np.arange(n_go)
    pk = n_gr + n_go + np.arange(n_pkj)

    def lognormal(median, n):
        return median * np.exp(sigma * rng.standard_normal(n))

    def delay(n):
        return rng.integers(8, 41, n)

    groups = []
    per = n_gr // mf_groups
    for g in range(mf_groups):
        cells = gr[g * per:(g + 1) * per] if g < mf_groups - 1 else gr[g * per:]
        n = 4 * len(cells)
        groups.append(dict(kind=SYN_MFGR, post_system=np.repeat(cells, 4), post_comp=np.tile(np.arange(4), len(cells)),
                           weight=scale[0] * lognormal(10000.0, n), rates=(5.0 + 45.0 * g / max(1, mf_groups - 1), 0.0, 0.0, 0.0),
                           seed=1000 + g, delay=delay(n)))
    n = 100 * n_go
    groups.append(dict(kind=SYN_GRGO, post_system=np.repeat(go, 100), post_comp=0, weight=scale[1] * lognormal(16.0 / (100 / 4.0), n),
                       pre_system=rng.choice(gr, n), pre_comp=3, delay=delay(n)))
    n = 4 * n_gr
    groups.append(dict(kind=SYN_GOGR, post_system=np.repeat(gr, 4), post_comp=1,
                       weight=scale[2] * lognormal(640000.0 / (4 * 4.0), n),
                       pre_system=rng.choice(go, n), pre_comp=30, delay=delay(n)))
    n = n_syn - sum(len(g["post_system"]) for g in groups)
    post = rng.choice(pk, n)
    n_in = np.bincount(post - pk[0], minlength=n_pkj)[post - pk[0]]
    groups.append(dict(kind=SYN_GRPKJ, post_system=post, post_comp=rng.integers(0, 1599, n),
                       weight=scale[3] * 300000.0 / (512 * n_in / 10.0) * np.exp(sigma * rng.standard_normal(n)),
                       pre_system=rng.choice(gr, n), pre_comp=3, delay=delay(n)))
    return specs, groups


def add_network(engine, specs, groups):
    ids = np.asarray(add_to(engine, specs))
    for g in groups:
        kw = dict(g)
        kw["post_system"] = ids[np.asarray(kw["post_system"])]
        if "pre_system" in kw:
            kw["pre_system"] = ids[np.asarray(kw["pre_system"])]
        engine.add_synapses(kw.pop("kind"), kw.pop("post_system"), kw.pop("post_comp"), kw.pop("weight"), **kw)
    return ids


def add_to(engine, specs):
    ids = []
    for s in specs:
        ids.append(engine.add_system(s.cell_type, s.nx, s.ny, s.rows, s.jitter, stim=s.stim,
                                     gj_pairs=s.gj_pairs, gap=s.gap, io_gap_g=s.io_gap_g, tol=s.tol,
                                     cond_scale_ch=s.cond_scale_ch))
    return ids


def add_to_oracle(O, s: Spec, canon=False):
    sysm = O.System(s.cell_type, s.nx, s.ny, s.rows, s.jitter, stim=s.stim, gj_pairs=s.gj_pairs,
                    io_gap=s.gap, go_gj=s.gap, pkj_gj=s.gap, io_gap_g=s.io_gap_g, tol=s.tol, canon=canon,
                    cond_scale_ch=s.cond_scale_ch)
    rc = sysm.init()
    if rc != 0:
        raise RuntimeError(f"oracle init failed ({rc})")
    return sysm


def type_counts(specs):
    out = {}
    for s in specs:
        c = out.setdefault(M.TYPE_NAMES[s.cell_type], [0, 0])
        c[0] += s.n
        c[1] += s.nc
    return out
