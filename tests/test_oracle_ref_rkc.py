"""The oracle's integrator against the reference's own CUDA RKC path.

tests/golden/ref_rkc/*.npz hold every compartment's v_new at every 0.125 ms
interval of the reference simulator's code (solve_rkc.cu's controller,
stages and power method, the *_ion.cu gating, gap.cu, and its setup),
compiled from its sources for sm_103a and run on a GB300 by
tests/golden/make_ref_rkc_vectors.py: seeded synthetic cells, the
reference's own initial jitter (srand(0) and rand() in main.cu's order),
a constant current at the compartment each type's X_set_current
stimulates.  Here the oracle integrates the same cells in reference
arithmetic (libm, no canonical choices) and must match:

* the initial membrane voltages bit for bit;
* after the first interval, every voltage to 1e-12 relative to the largest
  |v| for Golgi and Purkinje cells (or 30 x the floor below, for the trees
  whose first steps already turn last bits into different decisions)
  -- the reference's GPU arithmetic (CUDA's
  device exp and fused multiply-adds, cuBLAS and atomic summation order)
  differs from the oracle's only in last bits.  The granule cell (tolerance
  1e-9: every accepted step carries a local error of that order) is held to
  3e-9 and the olive network to 3e-7: already in its first interval a
  last-bit change of the power method's rho can flip the stage count
  m = 1 + floor(sqrt(1.54 h rho + 1)), and the oracle's own two arithmetics
  (reference, canonical) differ by 2e-8 there;
* every later interval within max(1e-4, 30 x floor) relative, where floor
  is the largest difference so far between the oracle in reference
  arithmetic and two runs that differ from it only in last bits: its
  canonical arithmetic, and reference arithmetic with every initial jitter
  moved by 1e-15.  The reference's deviation grows at the rate of that
  envelope, about ten times above it (its last-bit differences are in every
  operation), until a discrete controller decision (an accept, a stage
  count, an ion-update step) comes out differently; 1e-4 (6 uV of 60 mV)
  bounds the difference two valid trajectories keep after such a flip
  over these windows;
* the reference's raster (its own output_file lines) equals the oracle's
  threshold crossings at the interval ends;
* where the reference's run goes non-finite (untapered Purkinje trees under
  its frozen-current splitting), the oracle's does too, within one interval.
"""
import glob
import json
import os
import sys

import numpy as np
import pytest

import morph as M

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import make_ref_rkc_vectors as G  # noqa: E402

CASES = sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(HERE, "golden", "ref_rkc", "*.npz")))
STIM_COMP = {M.GR: 16, M.GO: 30, M.PKJ: 1599, M.IO: 0}
THRESH = {M.GR: 10.0, M.GO: 10.0, M.PKJ: -10.0, M.IO: 10.0}
RASTER_COMP = {M.GR: 77, M.GO: 30, M.PKJ: 1599, M.IO: 2}
FIRST_INTERVAL = {M.GR: 3e-9, M.GO: 1e-12, M.PKJ: 1e-12, M.IO: 3e-7}


def _system(O, c, canon, nudge=0.0):
    t, n = c["type"], c["nx"] * c["ny"]
    O.libc_srand(0)
    jit = O.draw_jitter(t, n) + nudge
    s = O.System(t, c["nx"], c["ny"], G.rows_for(c["rows"]), jit,
                 stim=(np.full(n, STIM_COMP[t], np.int32), np.full(n, c["amp"]), np.zeros(n), np.full(n, 1e9)),
                 gj_pairs=M.PKJ_GJ_PAIRS if t == M.PKJ else None, io_gap=True, go_gj=True, pkj_gj=True, canon=canon)
    assert s.init() == 0
    return s


@pytest.mark.parametrize("name", CASES)
def test_oracle_matches_reference_cuda_build(oracle, name):
    z = np.load(os.path.join(HERE, "golden", "ref_rkc", f"{name}.npz"))
    meta = json.loads(str(z["meta"]))
    c = G.CASES[name]
    t = c["type"]
    ref = _system(oracle, c, False)
    variants = [_system(oracle, c, True), _system(oracle, c, False, 1e-15)]
    np.testing.assert_array_equal(ref.elem_v(), z["v0"])
    vnew = z["vnew"]
    floor, tt, crossings = 0.0, 0.0, []
    ncomp = vnew.shape[1] // (c["nx"] * c["ny"])
    prev = np.full(c["nx"] * c["ny"], 100.0)
    for k in range(vnew.shape[0]):
        want = vnew[k]
        if not np.all(np.isfinite(want)):
            # the reference went non-finite: so does the oracle, within one interval
            for _ in range(2):
                if ref.advance(tt) != 0 or not np.all(np.isfinite(ref.vnew())):
                    return
                tt += 0.125
            raise AssertionError(f"the reference went non-finite at interval {k + 1}, the oracle did not")
        rc = ref.advance(tt)
        if rc != 0 and k + 1 < vnew.shape[0] and not np.all(np.isfinite(vnew[k + 1])):
            return          # the oracle stopped one interval before the reference
        assert rc == 0, f"interval {k + 1}"
        for w in variants:
            assert w.advance(tt) == 0, f"interval {k + 1}"
        tt += 0.125
        got = ref.vnew()
        scale = np.max(np.abs(want))
        floor = max([floor] + [np.max(np.abs(got - w.vnew())) / scale for w in variants])
        err = np.max(np.abs(got - want)) / scale
        if k == 0:
            assert err < max(FIRST_INTERVAL[t], 30.0 * floor), f"first interval: {err:.3e}, floor {floor:.3e}"
        assert err <= max(1e-4, 30.0 * floor), f"interval {k + 1}: {err:.3e} against floor {floor:.3e}"
        x = got[np.arange(c["nx"] * c["ny"]) * ncomp + RASTER_COMP[t]]
        for cell in np.nonzero((x > THRESH[t]) & (prev <= THRESH[t]))[0]:
            crossings.append((round(tt, 6), int(cell)))
        prev = x
    lines = [ln.split(",") for ln in meta["raster"].splitlines() if ln.strip()]
    assert sorted((round(float(a), 6), int(b)) for a, b in lines) == sorted(crossings)
