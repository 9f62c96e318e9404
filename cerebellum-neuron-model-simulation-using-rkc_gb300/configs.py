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


# Purkinje trees whose cells stay finite for 500 ms at 0.1-0.4 nA under the
# reference's frozen-current splitting, in FP64 and in mixed precision
# (screened on the GPU); Golgi tree variants likewise.
PKJ_STABLE_SEEDS = (7, 8, 9, 12, 13)
GO_STABLE_VARIANTS = (0, 1, 3, 5, 6, 7)


def pkj_grid(nx=3, ny=3, seed=2, amp=0.5e-3, tree_seed=None, gap=True):
    """Reference-style Purkinje grid (one RKC system); the tree is the first
    screened-stable one unless given."""
    rng = np.random.default_rng(seed)
    rows = M.pkj_synthetic(tree_seed if tree_seed is not None else PKJ_STABLE_SEEDS[0])
    n = nx * ny
    return [Spec(M.PKJ, nx, ny, rows, _jitter(rng, n), stim=(rows.shape[0] - 1, amp, 0.0, 1e9),
                 gap=gap, gj_pairs=M.PKJ_GJ_PAIRS, tag=f"pkj{nx}x{ny}")]


AMP_MAX = {M.GR: 0.05e-3, M.GO: 0.4e-3, M.PKJ: 0.4e-3, M.IO: 6.0}


def mixed_batch(seed=2, n_gr=4096, n_go=1024, n_pkj=256, io_side=16):
    rng = np.random.default_rng(seed)
    specs = []
    gr_rows = M.gr_reduced4()
    for i in range(n_gr):
        specs.append(Spec(M.GR, 1, 1, gr_rows, _jitter(rng, 1),
                          stim=(1, rng.uniform(0, AMP_MAX[M.GR]), rng.uniform(0, 20.0), 1e9), tag="gr"))
    go_rows = [M.go_synthetic(seed * 1000 + k) for k in GO_STABLE_VARIANTS]
    for i in range(n_go):
        specs.append(Spec(M.GO, 1, 1, go_rows[i % len(go_rows)], _jitter(rng, 1),
                          stim=(30, rng.uniform(0, AMP_MAX[M.GO]), rng.uniform(0, 20.0), 1e9), tag="go"))
    pk_rows = [M.pkj_synthetic(s) for s in PKJ_STABLE_SEEDS]
    for i in range(n_pkj):
        r = pk_rows[i % len(pk_rows)]
        specs.append(Spec(M.PKJ, 1, 1, r, _jitter(rng, 1),
                          stim=(r.shape[0] - 1, rng.uniform(0, AMP_MAX[M.PKJ]), rng.uniform(0, 20.0), 1e9),
                          tag="pkj"))
    if io_side > 0:
        n = io_side * io_side
        specs.append(Spec(M.IO, io_side, io_side, M.io_rows(), _jitter(rng, n),
                          stim=(np.zeros(n, np.int32), rng.uniform(0, AMP_MAX[M.IO], n), rng.uniform(0, 20.0, n),
                                np.full(n, 1e9)),
                          gap=True, io_gap_g=G_C_IO * rng.uniform(0.5, 1.5, 4 * n), tag="io"))
    return specs


def scaled_mixed_batch(fraction: float, seed=2):
    """The mixed batch with every population scaled (for bounded CPU samples)."""
    return mixed_batch(seed=seed, n_gr=max(1, int(4096 * fraction)), n_go=max(1, int(1024 * fraction)),
                       n_pkj=max(1, int(256 * fraction)), io_side=16)


def add_to(engine, specs):
    ids = []
    for s in specs:
        ids.append(engine.add_system(s.cell_type, s.nx, s.ny, s.rows, s.jitter, stim=s.stim,
                                     gj_pairs=s.gj_pairs, gap=s.gap, io_gap_g=s.io_gap_g, tol=s.tol))
    return ids


def add_to_oracle(O, s: Spec, canon=False):
    sysm = O.System(s.cell_type, s.nx, s.ny, s.rows, s.jitter, stim=s.stim, gj_pairs=s.gj_pairs,
                    io_gap=s.gap, go_gj=s.gap, pkj_gj=s.gap, io_gap_g=s.io_gap_g, tol=s.tol, canon=canon)
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
