"""Cell morphologies in the reference simulator's file formats.

A morphology is a float64 array of rows, one row per compartment, laid out
exactly as the reference's parameter files are read (one row per line):

* GR  (``Gr.txt``, read at gr.cu:31-35):     i1 i2 d1 d2 d3 d4 i3 + 10 densities
* GO  (``Go_131.txt``, read at go.cu:33-38): i1 i2 d1 d2 d3 d4 i3 + 13 densities
* PKJ (``Pkj.txt``, read at pkj.cu:35-40):   i1 i2 x y z d i3
* IO  (``IO.txt``, read at io.cu:28-33):     i1 i2 d1 d2 d4 i3

(i1 = index, i2 = parent or -1, d1 = diameter um, d2 = length um, d3 = Ra
ohm cm, d4 = Cm uF/cm^2, i3 = compartment type; PKJ stores the segment vector
x y z instead of a length.)

The reference ships fixed morphologies; the benchmark workloads use seeded
synthetic trees in the same formats, generated here.  ``parse_rows`` and
``write_rows`` read and write the text formats, so a synthetic cell can be fed
to the reference's own loader.
"""
from __future__ import annotations

import numpy as np

GR, GO, PKJ, IO = 0, 1, 2, 3
TYPE_NAMES = {GR: "gr", GO: "go", PKJ: "pkj", IO: "io"}
ROW_FIELDS = {GR: 17, GO: 20, PKJ: 7, IO: 6}

# Soma (voltage output) and raster compartments of the reference cells
# (gr.cu:264,270; go.cu:280,286; pkj.cu:382,404; io.cu:271-283).
REF_NCOMP = {GR: 578, GO: 131, PKJ: 1600, IO: 3}

# Inferior olive three-compartment cell: dendrite -> soma -> axon hillock,
# 6 um x 53.07 um, Cm 1 uF/cm^2 (the reference IO.txt values).
_IO_ROWS = np.array([[0, 1, 6.0, 53.07, 1.0, 0],
                     [1, 2, 6.0, 53.07, 1.0, 1],
                     [2, -1, 6.0, 53.07, 1.0, 2]], dtype=np.float64)

# Granule-cell compartment classes used by the reduced cell, with the channel
# densities the reference assigns to those classes (Gr.txt rows of types 0, 4,
# 6, 7): d um, L um, Ra ohm cm, Cm, type, then
# g_leak1 g_leak2 g_leak3 g_Na g_KV g_KA g_KCa g_KM g_KIR g_Ca (mS/cm^2).
_GR_CLASSES = {
    "dend": (0.75, 2.5, 100.0, 1.0, 0, [0.0223, 0.0476, 0, 0, 0, 0, 14, 0, 0, 0]),
    "soma": (5.8, 5.8, 100.0, 1.0, 4, [0.0916, 0, 0, 0, 0, 40, 0, 6, 2, 0]),
    "ais": (0.15, 2.3367, 500.0, 1.0, 6, [0, 0, 1, 800, 10000, 0, 0, 0, 0, 0]),
    "axon": (0.15, 2.3367, 100.0, 1.0, 7, [0, 0, 0.05, 900, 1000, 0, 0, 0, 0, 0]),
}

# Golgi-cell compartment classes (Go_131.txt rows of types 0, 1, 2): d, L,
# Ra, Cm, type, then g_leak g_NaT g_NaR g_NaP g_KV g_KA g_KC g_Kslow g_CaHVA
# g_CaLVA g_HCN1 g_HCN2 g_KAHP (mS/cm^2).
_GO_DEND = (3.0, 11.7, 100.0, 1.0, 0, [0.021] + [0.0] * 12)
_GO_SOMA = (27.0, 27.0, 100.0, 1.0, 1,
            [0.021, 48.0, 1.7, 0.19, 32.0, 8.0, 3.0, 1.0, 0.46, 0.25, 0.05, 0.08, 38.0])
_GO_AXON = (2.4, 12.0, 100.0, 1.0, 2, [0.021] + [0.0] * 12)

# Purkinje gap-junction compartment pairs between x-neighbour cells
# (pre compartment in cell x, post compartment in cell x+1; Pkj_GJ.csv).
PKJ_GJ_PAIRS = np.array([
    [61, 151], [161, 471], [194, 52], [238, 31], [321, 138], [381, 139],
    [471, 539], [595, 598], [635, 286], [658, 1022], [668, 885], [717, 987],
    [889, 1053], [905, 1030], [966, 1205], [974, 1244], [975, 1088], [1082, 924],
    [1090, 1088], [1194, 918], [1243, 1379], [1249, 758], [1301, 1327],
    [1411, 1151], [1470, 1457], [1516, 1367]], dtype=np.int32)


def io_rows() -> np.ndarray:
    """The reference three-compartment IO cell."""
    return _IO_ROWS.copy()


def soma_comp(cell_type: int, ncomp: int) -> int:
    """Compartment written to the voltage CSV (reference cells: 16/30/1599/1)."""
    if cell_type == PKJ:
        return ncomp - 1
    if cell_type == GO:
        return 30
    if cell_type == GR:
        return 16 if ncomp == REF_NCOMP[GR] else 1
    return 1


def raster_comp(cell_type: int, ncomp: int) -> int:
    """Compartment whose threshold crossing is a spike (77/30/1599/2)."""
    if cell_type == PKJ:
        return ncomp - 1
    if cell_type == GO:
        return 30
    if cell_type == GR:
        return 77 if ncomp == REF_NCOMP[GR] else ncomp - 1
    return 2


def raster_threshold(cell_type: int) -> float:
    return -10.0 if cell_type == PKJ else 10.0


def _lognormal_diam(rng, median=1.5, sigma=0.5, lo=0.5, hi=8.0):
    return float(np.clip(median * np.exp(sigma * rng.standard_normal()), lo, hi))


def _random_binary_tree(rng, n_nodes: int, root_children: int):
    """Random recursive tree with out-degree <= 2 under a virtual root.

    Returns (parent list with -1 for children of the root, depth list), nodes
    numbered in creation order (every parent precedes its children)."""
    parent = []
    depth = []
    nchild = []
    open_slots = []           # nodes that can still take a child
    root_slots = root_children
    for i in range(n_nodes):
        choices = len(open_slots) + (1 if root_slots > 0 else 0)
        k = int(rng.integers(choices))
        if root_slots > 0 and k == choices - 1:
            parent.append(-1)
            depth.append(1)
            root_slots -= 1
        else:
            p = open_slots[k]
            parent.append(p)
            depth.append(depth[p] + 1)
            nchild[p] += 1
            # a node takes at most two children
            if nchild[p] >= 2:
                open_slots.pop(k)
        nchild.append(0)
        open_slots.append(i)
    return parent, depth


def pkj_synthetic(seed: int, ncomp: int = 1600, taper: bool = True) -> np.ndarray:
    """Seeded synthetic Purkinje cell in ``Pkj.txt`` layout.

    Soma at index ncomp-1 (diameter 29.8 um, type 0) and a binary-branching
    dendrite of ncomp-1 segments: segment length U[5,20] um along a random
    direction, diameter lognormal (median 1.5 um, sigma_ln 0.5) clipped to
    [0.5, 8] um; compartment type by depth: main (1) for depth <= 3, smooth (2)
    for depth <= 8, spiny (3) beyond.  The lognormal median is tapered by
    class like the reference tree (main x5.5, smooth x3, spiny x1: mean
    diameters 8.4 / 4.6 / 1.5 um in Pkj.txt); without the thick trunk the soma
    is too weakly loaded for the frozen-current RKC splitting at 0.5 nA.
    Parents always carry a higher index than their children, as in the
    reference file.  taper=False draws every diameter from the untapered
    lognormal (median 1.5 um)."""
    rng = np.random.default_rng(seed)
    nd = ncomp - 1
    parent, depth = _random_binary_tree(rng, nd, root_children=1)
    # creation order has parents first; reverse it so parents get higher indices
    new_index = {old: nd - 1 - old for old in range(nd)}
    rows = np.zeros((ncomp, 7), dtype=np.float64)
    for old in range(nd):
        i = new_index[old]
        p = parent[old]
        pi = ncomp - 1 if p < 0 else new_index[p]
        L = rng.uniform(5.0, 20.0)
        u = rng.standard_normal(3)
        u /= np.linalg.norm(u)
        x, y, z = (L * u).tolist()
        dep = depth[old]
        ctype = 1 if dep <= 3 else (2 if dep <= 8 else 3)
        dd = _lognormal_diam(rng, median=1.5 * ({1: 5.5, 2: 3.0, 3: 1.0}[ctype] if taper else 1.0))
        rows[i] = [i, pi, x, y, z, dd, ctype]
    rows[ncomp - 1] = [ncomp - 1, -1, 0.0, 0.0, 0.0, 29.8, 0]
    return rows


def go_synthetic(seed: int, ndend: int = 30, naxon: int = 100) -> np.ndarray:
    """Seeded synthetic Golgi cell in ``Go_131.txt`` layout (131 compartments).

    Compartments 0..ndend-1 form a binary-branching dendritic tree rooted on
    the soma (three primary dendrites; segment length U[5,20] um, diameter
    lognormal median 1.5 um clipped to [0.5, 8]); the soma is compartment
    ndend (reference index 30) and is the parent of the first axon
    compartment chain ndend+1 .. ndend+naxon, whose last compartment is the
    root, as in the reference file.  Channel densities per class as in the
    reference (leak only in dendrite and axon)."""
    rng = np.random.default_rng(seed)
    parent, depth = _random_binary_tree(rng, ndend, root_children=3)
    n = ndend + 1 + naxon
    soma = ndend
    rows = np.zeros((n, 20), dtype=np.float64)
    for i in range(ndend):
        p = soma if parent[i] < 0 else parent[i]
        L = rng.uniform(5.0, 20.0)
        dd = _lognormal_diam(rng)
        d1, d2, d3, d4, t, g = _GO_DEND
        rows[i] = [i, p, dd, L, d3, d4, t] + g
    d1, d2, d3, d4, t, g = _GO_SOMA
    rows[soma] = [soma, soma + 1, d1, d2, d3, d4, t] + g
    for k in range(naxon):
        i = soma + 1 + k
        p = i + 1 if k < naxon - 1 else -1
        d1, d2, d3, d4, t, g = _GO_AXON
        rows[i] = [i, p, d1, d2, d3, d4, t] + g
    return rows


def gr_reduced4() -> np.ndarray:
    """Reduced four-compartment granule cell: dendrite -> soma -> AIS -> axon
    (root), geometry and densities of the reference's classes."""
    order = ["dend", "soma", "ais", "axon"]
    rows = np.zeros((4, 17), dtype=np.float64)
    for i, cls in enumerate(order):
        d1, d2, d3, d4, t, g = _GR_CLASSES[cls]
        rows[i] = [i, i + 1 if i < 3 else -1, d1, d2, d3, d4, t] + g
    return rows


_GR_FULL_CLASSES = {
    0: (0.75, 2.5, 100.0, [0.0223, 0.0476, 0, 0, 0, 0, 14, 0, 0, 0]),
    1: (0.75, 2.5, 100.0, [0.0223, 0.0476, 0, 0, 0, 0, 14, 0, 0, 0]),
    2: (0.75, 5.0, 100.0, [0.0451, 0.0953, 0, 0, 0, 0, 14, 0, 0, 0]),
    3: (0.75, 5.0, 100.0, [0.0451, 0.0953, 0, 0, 0, 0, 14, 0, 0, 0]),
    4: (5.8, 5.8, 100.0, [0.0916, 0, 0, 0, 0, 40, 0, 6, 2, 0]),
    5: (2.0, 0.5, 500.0, [0, 0, 0, 500, 30000, 0, 0, 0, 0, 0]),
    6: (0.15, 2.3367, 500.0, [0, 0, 1, 800, 10000, 0, 0, 0, 0, 0]),
    7: (0.15, 2.3367, 100.0, [0, 0, 0.05, 900, 1000, 0, 0, 0, 0, 0]),
    8: (0.15, 10.0, 100.0, [0, 0, 0.05, 300, 30, 0, 0, 0, 0, 0]),
}


def gr_synthetic(seed: int) -> np.ndarray:
    """Seeded full-size (578-compartment) granule cell in ``Gr.txt`` layout.

    Topology of the reference file: four 4-compartment dendrites (types 0-3,
    distal to proximal) on the soma (16), hillock 17-21, AIS 22-24, axon 25-77
    joining a 500-compartment parallel fibre 78..577 at 328 (root 577).
    Geometry per class with seeded x U[0.8, 1.2] perturbations."""
    rng = np.random.default_rng(seed)
    n = 578
    rows = np.zeros((n, 17), dtype=np.float64)
    for i in range(n):
        if i < 16:
            t, p = i // 4, (i + 4 if i < 12 else 16)
        elif i == 16:
            t, p = 4, 17
        elif i <= 21:
            t, p = 5, i + 1
        elif i <= 24:
            t, p = 6, i + 1
        elif i <= 77:
            t, p = 7, (i + 1 if i < 77 else 328)
        else:
            t, p = 8, (i + 1 if i < 577 else -1)
        d1, d2, d3, g = _GR_FULL_CLASSES[t]
        rows[i] = [i, p, d1 * rng.uniform(0.8, 1.2), d2 * rng.uniform(0.8, 1.2), d3, 1.0, t] + g
    return rows


def parse_rows(text: str, cell_type: int) -> np.ndarray:
    """Parse a reference-format parameter file (whitespace separated)."""
    nf = ROW_FIELDS[cell_type]
    vals = np.array(text.split(), dtype=np.float64)
    if vals.size % nf:
        raise ValueError(f"row table size {vals.size} is not a multiple of {nf}")
    return vals.reshape(-1, nf)


def write_rows(rows: np.ndarray, cell_type: int) -> str:
    """Format rows like the reference files (ints for index/parent/type)."""
    int_cols = {0, 1, 6} if cell_type in (GR, GO, PKJ) else {0, 1, 5}
    out = []
    for r in rows:
        out.append("\t".join(str(int(v)) if j in int_cols else repr(float(v))
                             for j, v in enumerate(r)))
    return "\n".join(out) + "\n"
