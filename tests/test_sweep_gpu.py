"""The parameter-sweep workload on the GPU: independent granule and Golgi
instances, each channel density scaled by its own factor (cond_scale_ch),
each running for its own number of intervals (the engine's per-system
interval budget), all in one persistent launch.

Plain FP64 is bit-identical to the oracle (canonical arithmetic) system by
system, every system stops exactly at its own budget, and mixed precision
keeps the FP64 spike counts."""
import numpy as np
import pytest

import configs
import gbrkc as G

pytestmark = pytest.mark.gpu


def _sweep(n_gr=24, n_go=8):
    return configs.sweep_batch(n_gr=n_gr, n_go=n_go, amp_max=0.4e-3, ts_ms=(0.5, 3.0))


def _engine(prec, specs):
    eng = G.Engine(prec)
    ids = configs.add_to(eng, specs)
    eng.build()
    for sid, sp in zip(ids, specs):
        eng.set_budget(sid, 1, sp.extra["n_intervals"])
    return eng, ids


def test_sweep_fp64_matches_oracle_per_system_budgets(oracle):
    specs = _sweep()
    eng, ids = _engine(G.FP64, specs)
    longest = max(sp.extra["n_intervals"] for sp in specs)
    eng.advance(0.0, longest + 4)          # every system stops at its own budget
    for sid, sp in zip(ids, specs):
        n = sp.extra["n_intervals"]
        s = configs.add_to_oracle(oracle, sp, canon=True)
        t = 0.0
        for _ in range(n):
            assert s.advance(t) == 0
            t += G.H_MAX
        np.testing.assert_array_equal(eng.vnew(sid), s.vnew(), err_msg=f"system {sid} ({sp.tag})")
        ctl, st, status = eng.ctl(sid)
        assert status == 0
        assert ctl["tend"] == s.ctl()["tend"] == n * G.H_MAX + G.H_MAX
        for k, v in s.stats().items():
            assert st[k] == v, (sid, k, st[k], v)
    eng.close()


def test_sweep_mixed_keeps_fp64_spike_counts():
    specs = _sweep(64, 16)
    counts = {}
    for prec in (G.FP64, G.MIXED):
        eng, ids = _engine(prec, specs)
        eng.record_spikes(1 << 16)
        eng.advance(0.0, max(sp.extra["n_intervals"] for sp in specs))
        c = {}
        for ty in (G.GR, G.GO):
            _, sy, _ = eng.read_spikes(ty)
            for x in sy.tolist():
                c[x] = c.get(x, 0) + 1
        counts[prec] = c
        assert eng.retired() == 0
        eng.close()
    assert counts[G.FP64] == counts[G.MIXED]
