"""The oracle against the reference's only checked-in result:
io_raster_by_RKC.csv -- 8x8 inferior-olive cells solved by RKC with the
default stimulus (5.5 at the dendrite for 800 <= t < 820 ms, io.cu:247-257),
libc srand(0) for the initial jitter (main.cu:38).  Every cell spikes exactly
once; spike times are on the 0.125 ms output grid (main.cu:214)."""
import os

import numpy as np

import morph as M

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "io_raster_8x8_ref.csv")


def load_gold():
    out = []
    for line in open(GOLD):
        if line.startswith("#") or not line.strip():
            continue
        t, c = line.strip().split(",")
        out.append((float(t), int(c)))
    return out


def run_io_raster(O, t_end=809.0):
    O.libc_srand(0)
    jit = O.draw_jitter(O.IO, 64)
    s = O.System(O.IO, 8, 8, M.io_rows(), jit, stim=(0, 5.5, 800.0, 820.0))
    assert s.init() == 0
    prev = np.full(64, 100.0)
    raster = []
    t = 0.0
    while t < t_end:
        assert s.advance(t) == 0
        vs = s.vnew()[2::3]
        for j in np.nonzero((vs > 10.0) & (prev <= 10.0))[0]:
            raster.append((t + 0.125, int(j)))
        prev = vs
        t += 0.125
    return raster


def test_io_raster_matches_reference(oracle):
    gold = {c: t for t, c in load_gold()}
    mine = run_io_raster(oracle)
    cells = [c for _, c in mine]
    assert sorted(cells) == list(range(64)), "every cell spikes exactly once"
    times = {c: t for t, c in mine}
    exact = sum(times[c] == gold[c] for c in range(64))
    # The reference was run on a V100 (FMA contraction, CUDA libm); cells
    # whose upstroke crosses 10 mV within ~1 us of a sample may land one
    # 0.125 ms sample apart.
    assert all(abs(times[c] - gold[c]) <= 0.125 for c in range(64))
    assert exact >= 62, f"only {exact}/64 spike times identical"
