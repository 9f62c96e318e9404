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


# ---------------------------------------------------------------- network
NET_NGR, NET_NGO, NET_NPK_SYN = 8, 2, 5


def build_network(O, target, seed=5, mf_rate=400.0, delays=False):
    """A small network in the reference's topology: 8 reduced granule cells,
    2 Golgi cells and 1 Purkinje cell, each its own system; mossy fibres onto
    every granule compartment, granule axon -> Golgi soma, Golgi comp 30 ->
    granule soma, granule axon -> 5 random Purkinje compartments per cell,
    with weights scaled like the reference's (W_* / counts, syn.cuh:46-50).
    `target` is an oracle Network or a gbrkc Engine; returns the system ids.
    delays: seeded transmission delays of 1-40 intervals (0.125-5 ms) per
    synapse instead of the reference's same-interval rule."""
    import numpy as np
    rng = np.random.default_rng(seed)
    O.libc_srand(0)
    ids = []
    gr_rows, go_rows, pk_rows = M.gr_reduced4(), M.go_synthetic(3), M.pkj_synthetic(7)
    specs = [(M.GR, gr_rows)] * NET_NGR + [(M.GO, go_rows)] * NET_NGO + [(M.PKJ, pk_rows)]
    for t, rows in specs:
        jit = O.draw_jitter(t, 1)
        if hasattr(target, "systems"):  # oracle network
            s = O.System(t, 1, 1, rows, jit, canon=True)
            assert s.init() == 0
            ids.append(target.add_system(s))
        else:
            ids.append(target.add_system(t, 1, 1, rows, jit))
    gr, go, pk = ids[:NET_NGR], ids[NET_NGR:NET_NGR + NET_NGO], ids[-1]
    drng = np.random.default_rng(seed + 100)

    def dl(n):
        return drng.integers(1, 41, n) if delays else None

    target.add_synapses(0, np.repeat(gr, 4), np.tile(np.arange(4), NET_NGR), 10000.0,
                        rates=(mf_rate, 0.0, 0.0, 0.0), seed=7, delay=dl(4 * NET_NGR))
    target.add_synapses(1, np.tile(go, NET_NGR), 0, 16.0 / (NET_NGR / 4.0), pre_system=np.repeat(gr, NET_NGO),
                        pre_comp=3, delay=dl(NET_NGR * NET_NGO))
    target.add_synapses(2, np.tile(gr, NET_NGO), 1, 640000.0 / (NET_NGO * 4.0), pre_system=np.repeat(go, NET_NGR),
                        pre_comp=30, delay=dl(NET_NGR * NET_NGO))
    target.add_synapses(3, np.full(NET_NGR * NET_NPK_SYN, pk), rng.integers(0, 1599, NET_NGR * NET_NPK_SYN),
                        300000.0 / (512 * NET_NGR / 10.0), pre_system=np.repeat(gr, NET_NPK_SYN), pre_comp=3,
                        delay=dl(NET_NGR * NET_NPK_SYN))
    return ids
