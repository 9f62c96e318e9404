"""Plain-FP64 parity at the workloads' own sizes and horizons, bit for bit
against the oracle in canonical arithmetic:

* the Purkinje 3x3 grid -- one RKC system of 14 400 compartments with
  x-neighbour gap junctions, on the engine's default path for a system that
  large (a thread-block cluster) -- for its whole 200 ms;
* a 1/16 sample of the mixed batch (256 granule, 64 Golgi and 16 Purkinje
  cells, one 16x16 olive network; stated currents, distinct trees) in one
  persistent launch per advance, for 20 ms.

The oracle runs in worker processes started with spawn (this process
already holds a CUDA context)."""
import multiprocessing as mp
import os
import sys

import numpy as np
import pytest

import configs
import gbrkc as G

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def _oracle_run(args):
    """Worker: the given specs of a workload in the oracle (canonical), each
    advanced through the checkpoints; returns per spec the v_new at each
    checkpoint and the final statistics."""
    which, idx, checkpoints = args
    sys.path.insert(0, os.path.join(ROOT, "cerebellum-neuron-model-simulation-using-rkc_gb300"))
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import configs as C
    import oracle_py as O
    specs = C.pkj_grid(3, 3) if which == "pkj3x3" else C.scaled_stated_batch(1.0 / 16)
    out = []
    for i in idx:
        s = C.add_to_oracle(O, specs[i], canon=True)
        t, done, vs, rc = 0.0, 0, [], 0
        for cp in checkpoints:
            for _ in range(cp - done):
                if rc == 0:
                    rc = s.advance(t)    # a stopped system keeps its state, as the engine's does
                t += 0.125
            done = cp
            vs.append(s.vnew())
        out.append((i, vs, (s.stats(), rc)))
    return out


def _oracle(which, n_specs, checkpoints, workers):
    chunks = [list(range(k, n_specs, workers)) for k in range(workers)]
    with mp.get_context("spawn").Pool(len([c for c in chunks if c])) as pool:
        res = pool.map(_oracle_run, [(which, c, checkpoints) for c in chunks if c])
    return {i: (vs, st) for part in res for i, vs, st in part}


def _gpu(specs, checkpoints):
    eng = G.Engine(G.FP64)
    ids = configs.add_to(eng, specs)
    eng.build()
    t, done, out = 0.0, 0, {k: [] for k in range(len(specs))}
    for cp in checkpoints:
        eng.advance(t, cp - done, tolerate_retire=True)
        t += (cp - done) * G.H_MAX
        done = cp
        for k, sid in enumerate(ids):
            out[k].append(eng.vnew(sid))
    stats = {k: eng.ctl(sid)[1:] for k, sid in enumerate(ids)}
    layout = eng.launch_layout()
    eng.close()
    return out, stats, layout


def _compare(gpu, stats, orc):
    for k, (vs, (st, rc)) in orc.items():
        g_st, status = stats[k]
        assert (status != 0) == (rc != 0), (k, status, rc)
        if rc != 0:
            continue            # stopped in both (the reference's scheme diverged); states not compared
        for j, v in enumerate(vs):
            np.testing.assert_array_equal(gpu[k][j], v, err_msg=f"system {k}, checkpoint {j}")
        for key, val in st.items():
            assert g_st[key] == val, (k, key, g_st[key], val)


def test_pkj3x3_fp64_bit_exact_200ms():
    specs = configs.pkj_grid(3, 3)
    checkpoints = [8, 160, 800, 1600]          # 1, 20, 100, 200 ms
    gpu, stats, (persistent, _) = _gpu(specs, checkpoints)
    assert not persistent                        # a cluster launch, the path for a system this large
    _compare(gpu, stats, _oracle("pkj3x3", 1, checkpoints, 1))


def test_mixed_sample_fp64_bit_exact_20ms():
    specs = configs.scaled_stated_batch(1.0 / 16)
    checkpoints = [8, 40, 160]                   # 1, 5, 20 ms
    gpu, stats, (persistent, _) = _gpu(specs, checkpoints)
    assert persistent
    _compare(gpu, stats, _oracle("mixed16", len(specs), checkpoints, max(1, min(16, os.cpu_count() or 1))))
