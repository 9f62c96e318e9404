"""The reference's network wiring rules (syn.cu: mfgr_create, grgo_create,
gogr_create, grpkj_create) as synapse lists for Engine.add_synapses, and the
Purkinje compartment-location file they read (Pkj_location_info.csv).

Cells sit on grids: granule cell i at (16 (i mod nx_gr), 16 (i div nx_gr)) um,
Golgi and Purkinje cells at (32 (i mod nx) + 8, 32 (i div nx) + 8).  The rules,
in the reference's enumeration order (which fixes the synapse ids):

* MF -> GrC (syn.cu:43-84): four fibres per granule cell, onto compartments
  0-3, weight W_MFGR / 4.
* GrC -> GoC (syn.cu:146-262): every pair with |dx| < 16 and |dy| < 220,
  granule-major; from axon compartment 250 + 77 - int((8 + 32 iy_go -
  16 iy_gr) / 10) to the Golgi soma (compartment 0); weight W_GRGO / (n / 4),
  n = the Golgi cell's input count.
* GoC -> GrC (syn.cu:295-410): every pair with |dx| < 32 and |dy| < 32,
  Golgi-major; from Golgi compartment 30 (GO_COMP_DEND * 3) to the granule
  soma (compartment 16); weight W_GOGR / (4 n), n = the granule cell's input
  count.
* GrC -> PC (syn.cu:455-619): every pair with |dx| < 120 and |dy| < 220,
  granule-major, 25 synapses each (N_Syn_Per_GRPKJ); from axon compartment
  250 + 77 + int(dy / 10) (dy = 16 iy_gr - (8 + 32 iy_pkj)); onto the
  Purkinje compartment minimising |x - dx + 10 f| (x from the location file,
  dx = 16 ix_gr - (8 + 32 ix_pkj), f uniform in (-0.5, 0.5]), the running
  minimum carried across the connection's 25 draws as the reference does;
  weight W_GRPKJ / (512 n / 10), n = the Purkinje cell's connection count.

The reference draws f with cuRAND; here f comes from the caller's numpy
Generator, or from splitmix_uniform(seed, k) -- the draws the drop-in's
network mode makes (k counts the draws in order).  Weight constants:
syn.cuh:54-58.
"""
from __future__ import annotations

import numpy as np

W_MFGR = 40000.0
W_GRGO = 64.0 / 4.0
W_GOGR = 160000.0 * 4.0
W_GRPKJ = 1000000.0 * 0.3
N_SYN_PER_GRPKJ = 25
GR_AXON0 = 250 + 77          # granule axon compartment level with the soma row
GR_SOMA, GO_SOMA, GO_OUT = 16, 0, 30
SYN_MFGR, SYN_GRGO, SYN_GOGR, SYN_GRPKJ = 0, 1, 2, 3


_M64 = (1 << 64) - 1


def splitmix_uniform(seed: int, idx: int, counter: int = 0) -> float:
    """The SplitMix64 finaliser over (seed, index, counter) as a double in
    (0, 1] -- the same formula as the library's splitmix.h."""
    z = (seed ^ ((idx * 0xD1B54A32D192ED03) & _M64) ^ ((counter * 0x9E3779B97F4A7C15) & _M64)) & _M64
    z = (z + 0x9E3779B97F4A7C15) & _M64
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & _M64
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & _M64
    z ^= z >> 31
    return float((z >> 11) + 1) * 2.0 ** -53


def read_pkj_location(path: str):
    """Pkj_location_info.csv: one row per Purkinje compartment,
    'index,x,y,z,type' (syn.cu:536-553).  Returns (x, z, type) arrays."""
    rows = np.loadtxt(path, delimiter=",", ndmin=2)
    return rows[:, 1].copy(), rows[:, 3].copy(), rows[:, 4].astype(np.int32)


def _gr_xy(i, nx):
    return float(int(i % nx) * 16.0), float(int(i // nx) * 16.0)


def _big_xy(i, nx):
    return float(int(i % nx) * 32.0 + 8.0), float(int(i // nx) * 32.0 + 8.0)


def reference_synapses(nx_gr, ny_gr, nx_go, ny_go, nx_pkj, ny_pkj, pkj_x=None, rng=None, uniform=None):
    """Synapse groups of the reference network, keyed by kind: dicts of
    pre_cell, pre_comp, post_cell, post_comp, weight (cell = index within its
    type's grid; compartments within the cell).  uniform(k), if given, is the
    k-th draw in (0, 1] of the Purkinje targets (else rng)."""
    n_gr, n_go, n_pkj = nx_gr * ny_gr, nx_go * ny_go, nx_pkj * ny_pkj
    out = {}
    # MF -> GrC
    post = np.repeat(np.arange(n_gr), 4)
    out[SYN_MFGR] = dict(pre_cell=np.full(4 * n_gr, -1), pre_comp=np.zeros(4 * n_gr, int), post_cell=post,
                         post_comp=np.tile(np.arange(4), n_gr), weight=np.full(4 * n_gr, W_MFGR / 4.0))
    # GrC -> GoC
    pairs = []
    for i_gr in range(n_gr if n_go else 0):
        xg, yg = _gr_xy(i_gr, nx_gr)
        for i_go in range(n_go):
            xo, yo = _big_xy(i_go, nx_go)
            if abs(xo - xg) < 16.0 and abs(yo - yg) < 220.0:
                pairs.append((i_gr, i_go))
    cnt_go = np.bincount([p[1] for p in pairs], minlength=n_go) if pairs else np.zeros(n_go, int)
    pre_comp, w = [], []
    for i_gr, i_go in pairs:
        # a float distance divided by the double 10.0, truncated (syn.cu:165-166)
        diff = float(np.float32(8.0 + (i_go // nx_go) * 32.0 - (i_gr // nx_gr) * 16.0))
        pre_comp.append(GR_AXON0 - int(diff / 10.0))
        w.append(W_GRGO / (cnt_go[i_go] * 1.0 / 4.0))
    out[SYN_GRGO] = dict(pre_cell=np.array([p[0] for p in pairs], int), pre_comp=np.array(pre_comp, int),
                         post_cell=np.array([p[1] for p in pairs], int), post_comp=np.full(len(pairs), GO_SOMA),
                         weight=np.array(w, float))
    # GoC -> GrC
    pairs = []
    for i_go in range(n_go if n_gr else 0):
        xo, yo = _big_xy(i_go, nx_go)
        for i_gr in range(n_gr):
            xg, yg = _gr_xy(i_gr, nx_gr)
            if abs(xo - xg) < 32.0 and abs(yo - yg) < 32.0:
                pairs.append((i_go, i_gr))
    cnt_gr = np.bincount([p[1] for p in pairs], minlength=n_gr) if pairs else np.zeros(n_gr, int)
    out[SYN_GOGR] = dict(pre_cell=np.array([p[0] for p in pairs], int), pre_comp=np.full(len(pairs), GO_OUT),
                         post_cell=np.array([p[1] for p in pairs], int), post_comp=np.full(len(pairs), GR_SOMA),
                         weight=np.array([W_GOGR / (cnt_gr[g] * 4.0) for _, g in pairs], float))
    # GrC -> PC
    pairs = []
    for i_gr in range(n_gr if n_pkj else 0):
        xg, yg = _gr_xy(i_gr, nx_gr)
        for i_pkj in range(n_pkj):
            xp, yp = _big_xy(i_pkj, nx_pkj)
            if abs(xp - xg) < 120.0 and abs(yp - yg) < 220.0:
                pairs.append((i_gr, i_pkj))
    if pairs and pkj_x is None:
        raise ValueError("granule -> Purkinje wiring needs the compartment locations (Pkj_location_info.csv)")
    cnt_pkj = np.bincount([p[1] for p in pairs], minlength=n_pkj) if pairs else np.zeros(n_pkj, int)
    rng = rng if rng is not None else np.random.default_rng(0)
    pre_cell, pre_comp, post_cell, post_comp, w = [], [], [], [], []
    x = None if pkj_x is None else np.asarray(pkj_x, float)
    k_draw = 0
    for i_gr, i_pkj in pairs:
        dx = (i_gr % nx_gr) * 16.0 - (8.0 + (i_pkj % nx_pkj) * 32.0)
        dy = (i_gr // nx_gr) * 16.0 - (8.0 + (i_pkj // nx_pkj) * 32.0)
        ax = GR_AXON0 + int(dy / 10.0)
        best, min_x = -1, 1000000.0
        for _ in range(N_SYN_PER_GRPKJ):
            u = uniform(k_draw) if uniform is not None else 1.0 - rng.random()   # (0, 1] like curand_uniform
            k_draw += 1
            f = u - 0.5
            d = np.abs(x - dx + 10.0 * f)
            k = int(np.argmin(d))                    # first of the smallest, as the strict < scan
            if d[k] < min_x:
                min_x, best = float(d[k]), k
            pre_cell.append(i_gr)
            pre_comp.append(ax)
            post_cell.append(i_pkj)
            post_comp.append(best)
            w.append(W_GRPKJ / (512.0 * cnt_pkj[i_pkj] * 1.0 * 1 / 10.0))
    out[SYN_GRPKJ] = dict(pre_cell=np.array(pre_cell, int), pre_comp=np.array(pre_comp, int),
                          post_cell=np.array(post_cell, int), post_comp=np.array(post_comp, int),
                          weight=np.array(w, float))
    return out


def add_reference_network(engine, groups, cell_system, rates=(0.0, 0.0, 0.0, 0.0), seed=0, delay=None):
    """Add the groups to an Engine (or oracle Network).  cell_system(type,
    cell) -> (system id, compartment offset of the cell in that system): one
    system per cell, or the reference's one block per type."""
    pre_type = {SYN_GRGO: 0, SYN_GOGR: 1, SYN_GRPKJ: 0}
    post_type = {SYN_MFGR: 0, SYN_GRGO: 1, SYN_GOGR: 0, SYN_GRPKJ: 2}
    first = {}
    for kind in (SYN_MFGR, SYN_GRGO, SYN_GOGR, SYN_GRPKJ):
        g = groups[kind]
        if len(g["post_cell"]) == 0:
            continue
        loc = [cell_system(post_type[kind], int(c)) for c in g["post_cell"]]
        post_sys = np.array([s for s, _ in loc], np.int32)
        post_comp = np.array([o for _, o in loc], np.int32) + g["post_comp"]
        kw = dict(delay=delay) if delay is not None else {}
        if kind == SYN_MFGR:
            first[kind] = engine.add_synapses(kind, post_sys, post_comp, g["weight"], rates=rates, seed=seed, **kw)
        else:
            ploc = [cell_system(pre_type[kind], int(c)) for c in g["pre_cell"]]
            pre_sys = np.array([s for s, _ in ploc], np.int32)
            pre_comp = np.array([o for _, o in ploc], np.int32) + g["pre_comp"]
            first[kind] = engine.add_synapses(kind, post_sys, post_comp, g["weight"], pre_system=pre_sys,
                                              pre_comp=pre_comp, **kw)
    return first
