"""GPU parity: the plain-FP64 CUDA path against the oracle, bit for bit.

The oracle runs in canonical mode (the agreed exp/log/pow, explicit fused
multiply-adds in the vector updates, pairwise-tree sums, 1/Cm as a multiply;
everything else in the reference's literal order).  The GPU path is built to
the same arithmetic, so voltages, gates, calcium, the current vector, the
controller scalars and every counter must be identical -- through spikes,
rejections and power iterations, across several launches.
"""
import numpy as np
import pytest

import gbrkc as G
from gpu_cases import CASES, add_to_engine, make_oracle

pytestmark = pytest.mark.gpu

HORIZON = {"pkj_2x1_gj": 24, "gr_full": 24}   # shorter for the costliest oracle cases


def oracle_state(s, t):
    out = {"vnew": s.vnew(), "v": s.elem_v(), "ca": s.ca(), "b": s.b()}
    for k in range(s.nion()):
        out[f"ion{k}"] = s.ion(k)
    return out


def gpu_state(eng, sid, nion):
    out = {"vnew": eng.read(sid, G.F_VNEW), "v": eng.read(sid, G.F_V), "ca": eng.read(sid, G.F_CA),
           "b": eng.read(sid, G.F_B)}
    for k in range(nion):
        out[f"ion{k}"] = eng.read(sid, G.F_ION, k)
    return out


def compare(a, b, where):
    for k in a:
        np.testing.assert_array_equal(a[k], b[k], err_msg=f"{where}: {k}")


def run_pair(O, name, chunks):
    s = make_oracle(O, name, canon=True)
    eng = G.Engine(G.FP64)
    sid = add_to_engine(G, O, eng, name)
    eng.build()
    t = 0.0
    for n_iv in chunks:
        eng.advance(t, n_iv)
        for _ in range(n_iv):
            assert s.advance(t) == 0
            t += G.H_MAX
        compare(oracle_state(s, t), gpu_state(eng, sid, s.nion()), f"{name} t={t}")
        ctl_g, st_g, status = eng.ctl(sid)
        assert status == 0
        ctl_o, st_o = s.ctl(), s.stats()
        for k in ctl_o:
            assert ctl_g[k] == ctl_o[k], (name, t, k, ctl_g[k], ctl_o[k])
        for k in st_o:
            assert st_g[k] == st_o[k], (name, t, k, st_g[k], st_o[k])
    return s, eng, sid


@pytest.mark.parametrize("name", sorted(CASES))
def test_fp64_bit_exact(oracle, name):
    n = HORIZON.get(name, 64)
    run_pair(oracle, name, [1, n // 2 - 1, n // 2])


def test_batch_equals_alone(oracle):
    """Every system gives the same bits alone and packed with all others."""
    names = sorted(CASES)
    alone = {}
    for nm in names:
        eng = G.Engine(G.FP64)
        sid = add_to_engine(G, oracle, eng, nm)
        eng.build()
        eng.advance(0.0, 16)
        alone[nm] = eng.vnew(sid)
        eng.close()
    eng = G.Engine(G.FP64)
    ids = {nm: add_to_engine(G, oracle, eng, nm) for nm in names}
    eng.build()
    eng.advance(0.0, 16)
    for nm in names:
        np.testing.assert_array_equal(eng.vnew(ids[nm]), alone[nm], err_msg=nm)


def test_soma_recording(oracle):
    name = "io_net4x4"
    s = make_oracle(oracle, name, canon=True)
    eng = G.Engine(G.FP64)
    sid = add_to_engine(G, oracle, eng, name)
    eng.build()
    eng.record_soma(32)
    eng.advance(0.0, 32)
    rec = eng.read_soma(sid, 32)
    t = 0.0
    for k in range(32):
        s.advance(t)
        t += G.H_MAX
        np.testing.assert_array_equal(rec[k], s.vnew()[1::3])


@pytest.mark.parametrize("precision", [G.FP64, G.MIXED])
def test_persistent_equals_per_type(monkeypatch, precision):
    """The one persistent launch (every CTA a cell-type role pulling systems
    from a queue, with the role split re-tuned after every launch) gives the
    same bits as one launch per cell type."""
    import configs
    specs = configs.scaled_mixed_batch(1.0 / 64)
    out = {}
    for mode in ("persistent", "per_type"):
        if mode == "per_type":
            monkeypatch.setenv("GBRKC_NO_MEGA", "1")
        else:
            monkeypatch.delenv("GBRKC_NO_MEGA", raising=False)
        eng = G.Engine(precision)
        ids = configs.add_to(eng, specs)
        eng.build()
        persistent, ctas = eng.launch_layout()
        assert persistent == (mode == "persistent"), ctas
        if persistent:
            assert all(c > 0 for c in ctas), ctas
        t = 0.0
        for n_iv in (8, 8, 16):
            eng.advance(t, n_iv, tolerate_retire=True)
            t += n_iv * G.H_MAX
        out[mode] = [eng.vnew(i) for i in ids]
        out[mode + "_units"] = eng.compartment_updates(-1)
        eng.close()
    for k, (a, b) in enumerate(zip(out["persistent"], out["per_type"])):
        np.testing.assert_array_equal(a, b, err_msg=f"system {k}")
    assert out["persistent_units"] == out["per_type_units"]
