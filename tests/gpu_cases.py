"""Seeded test systems shared by the GPU parity tests, smoke() and bench.py.

Each case is (cell_type, nx, ny, rows, stim, gj_pairs, gap): one RKC system
exactly as the reference would integrate it (all nx*ny cells with one step
size), built from seeded synthetic morphologies in the reference formats.
"""
import numpy as np

import morph as M

# (type, nx, ny, rows factory, stim (comp, amp, t0, t1), gap junctions)
CASES = {
    "io_net4x4": (M.IO, 4, 4, lambda: M.io_rows(), (0, 5.5, 1.0, 6.0), True),
    "io_single": (M.IO, 1, 1, lambda: M.io_rows(), (0, 3.0, 0.0, 1e9), False),
    "pkj_cell": (M.PKJ, 1, 1, lambda: M.pkj_synthetic(2), (1599, 0.5e-3, 0.0, 1e9), False),
    "pkj_2x1_gj": (M.PKJ, 2, 1, lambda: M.pkj_synthetic(4), (1599, 0.5e-3, 0.0, 1e9), True),
    "go_cell": (M.GO, 1, 1, lambda: M.go_synthetic(2), (30, 0.4e-3, 0.0, 1e9), False),
    "go_2x2_gj": (M.GO, 2, 2, lambda: M.go_synthetic(3), (30, 0.4e-3, 0.0, 1e9), True),
    "gr_reduced": (M.GR, 1, 1, lambda: M.gr_reduced4(), (1, 0.01e-3, 0.0, 1e9), False),
    "gr_full": (M.GR, 1, 1, lambda: M.gr_synthetic(11), (16, 0.01e-3, 0.0, 1e9), False),
}


def jitter_for(O, t, n, seed=0):
    O.libc_srand(seed)
    return O.draw_jitter(t, n)


def make_oracle(O, name, canon=True, seed=0):
    t, nx, ny, rows, stim, gap = CASES[name]
    r = rows()
    jit = jitter_for(O, t, nx * ny, seed)
    s = O.System(t, nx, ny, r, jit, stim=stim, gj_pairs=M.PKJ_GJ_PAIRS if t == M.PKJ else None,
                 io_gap=gap, go_gj=gap, pkj_gj=gap, canon=canon)
    assert s.init() == 0
    return s


def add_to_engine(G, O, eng, name, seed=0):
    t, nx, ny, rows, stim, gap = CASES[name]
    r = rows()
    jit = jitter_for(O, t, nx * ny, seed)
    return eng.add_system(t, nx, ny, r, jit, stim=stim,
                          gj_pairs=M.PKJ_GJ_PAIRS if t == M.PKJ else None, gap=gap)
