"""Slot reuse and the request server on the GPU.

A system refilled in place, and every request served among others (admitted
late, into slots other requests used before, next to requests of other
types, cut into quanta, stopped at its own interval count), must give the
same bits as a fresh engine that holds only that request's systems and
starts at t = 0.  The device raster must equal the reference's output_file
rule applied to the oracle's voltages, and the final voltages the oracle's,
in the plain-FP64 form.
"""
import numpy as np
import pytest

import gbrkc as G
import morph as M

pytestmark = pytest.mark.gpu

FIELDS = (G.F_VNEW, G.F_V, G.F_CA)

# class shapes: type, nx, ny, rows, stimulus compartment, amplitude range, gap junctions
SHAPES = {
    "gr": (M.GR, 1, 1, M.gr_reduced4, 1, (0.0, 0.05e-3), False),
    "go": (M.GO, 1, 1, lambda: M.go_synthetic(3), 30, (0.0, 0.4e-3), False),
    "pkj": (M.PKJ, 1, 1, lambda: M.pkj_synthetic(2), 1599, (0.3e-3, 0.5e-3), False),
    "io": (M.IO, 4, 4, M.io_rows, 0, (3.0, 5.5), True),
}
ROWS = {}


def rows(name):
    if name not in ROWS:
        ROWS[name] = SHAPES[name][3]()
    return ROWS[name]


def inputs(name, n_sys, rng):
    """Per-cell inputs of a request: jitter, stimulus, conductance scales (and IO edges)."""
    t, nx, ny, _, comp, (a0, a1), gap = SHAPES[name]
    cells = n_sys * nx * ny
    d = {
        "jitter": rng.uniform(-0.5, 0.5, cells),
        "stim": (np.full(cells, comp), rng.uniform(a0, a1, cells), np.full(cells, 0.5), np.full(cells, 1e9)),
        "cond_scale": rng.uniform(0.8, 1.2, cells),
    }
    if t == M.IO:
        d["io_gap_g"] = 5e-3 * rng.uniform(0.5, 1.5, 4 * cells)
        d["stim"] = (np.full(cells, comp), rng.uniform(a0, a1, cells), np.full(cells, 0.25), np.full(cells, 1.5))
    return d


def fresh(precision, name, n_sys, n_iv, inp, spikes=False):
    """The request alone: its systems in an engine of their own, from t = 0."""
    t, nx, ny, _, _, _, gap = SHAPES[name]
    cells = nx * ny
    eng = G.Engine(precision)
    for k in range(n_sys):
        sl = slice(k * cells, (k + 1) * cells)
        comp, amp, t0, t1 = inp["stim"]
        eng.add_system(t, nx, ny, rows(name), inp["jitter"][sl], stim=(comp[sl], amp[sl], t0[sl], t1[sl]),
                       gap=gap, cond_scale=inp["cond_scale"][sl],
                       io_gap_g=inp["io_gap_g"][4 * k * cells:4 * (k + 1) * cells] if "io_gap_g" in inp else None)
    eng.build()
    if spikes:
        eng.record_spikes(1 << 16)
    eng.advance(0.0, n_iv)
    out = {f: np.concatenate([eng.read(s, f) for s in range(n_sys)]) for f in FIELDS}
    if spikes:
        st, ss, sc = eng.read_spikes(t)
        out["spikes"] = (st, ss * cells + sc)
    eng.close()
    return out


@pytest.mark.parametrize("precision", [G.FP64, G.MIXED])
@pytest.mark.parametrize("name", ["gr", "go", "pkj", "io"])
def test_reset_equals_fresh(precision, name):
    """Engine level: systems refilled mid-run (new cells, budget) match fresh ones; the others go on."""
    rng = np.random.default_rng(11)
    t, nx, ny, _, _, _, gap = SHAPES[name]
    first = inputs(name, 3, rng)
    eng = G.Engine(precision)
    cells = nx * ny
    for k in range(3):
        sl = slice(k * cells, (k + 1) * cells)
        comp, amp, t0, t1 = first["stim"]
        eng.add_system(t, nx, ny, rows(name), first["jitter"][sl], stim=(comp[sl], amp[sl], t0[sl], t1[sl]),
                       gap=gap)
    eng.build()
    eng.advance(0.0, 6)
    second = inputs(name, 2, rng)
    T = 6 * G.H_MAX
    comp, amp, t0, t1 = second["stim"]
    eng.reset_systems(1, 2, second["jitter"], stim=(comp, amp, t0 + T, t1 + T), cond_scale=second["cond_scale"],
                      io_gap_g=second.get("io_gap_g"), n_intervals=11)
    eng.advance(T, 8)
    eng.advance(T + 8 * G.H_MAX, 8)   # the reset systems stop after 3 of these
    got = {f: np.concatenate([eng.read(s, f) for s in (1, 2)]) for f in FIELDS}
    ref = fresh(precision, name, 2, 11, second)
    for f in FIELDS:
        np.testing.assert_array_equal(got[f], ref[f], err_msg=f"{name} field {f}")
    # system 0 ran all 22 intervals, untouched by its neighbours' reset
    eng0 = G.Engine(precision)
    c, a, s0, s1 = (x[:cells] for x in first["stim"])
    eng0.add_system(t, nx, ny, rows(name), first["jitter"][:cells], stim=(c, a, s0, s1), gap=gap)
    eng0.build()
    eng0.advance(0.0, 22)
    np.testing.assert_array_equal(eng.read(0, G.F_VNEW), eng0.read(0, G.F_VNEW))
    assert [eng.ctl(s)[2] for s in (0, 1, 2)] == [0, 0, 0]


def serve_plan():
    # round -> [(class, systems, intervals)]; the arenas are small enough that
    # requests queue, backfill and reuse slots that others held
    return {
        0: [("gr", 25, 13), ("go", 4, 9), ("pkj", 1, 20), ("io", 2, 12), ("gr", 20, 7)],
        1: [("gr", 10, 17), ("go", 3, 5)],
        3: [("gr", 30, 8), ("pkj", 2, 6), ("io", 1, 19), ("go", 6, 4)],
        4: [("gr", 5, 3)],
    }


@pytest.mark.parametrize("precision", [G.FP64, G.MIXED])
def test_served_requests_equal_fresh(precision):
    rng = np.random.default_rng(7)
    srv = G.Server(precision, hbm_budget=0, quantum=8)
    slots = {"gr": 40, "go": 6, "pkj": 2, "io": 3}
    cid = {}
    for name, (t, nx, ny, _, _, _, gap) in SHAPES.items():
        cid[name] = srv.add_class(t, nx, ny, rows(name), slots=slots[name], gap=gap)
    srv.start()
    plan = serve_plan()
    reqs = []
    cancelled_queued = cancelled_resident = None
    for rnd in range(40):
        for name, n_sys, n_iv in plan.get(rnd, []):
            inp = inputs(name, n_sys, rng)
            rid = srv.submit(cid[name], n_sys, n_iv, inp["jitter"], stim=inp["stim"], cond_scale=inp["cond_scale"],
                             io_gap_g=inp.get("io_gap_g"))
            reqs.append((rid, name, n_sys, n_iv, inp))
        if rnd == 1:
            # one request cancelled while queued, one while resident (its slots are reused later)
            junk = inputs("gr", 39, rng)
            cancelled_queued = srv.submit(cid["gr"], 39, 50, junk["jitter"])
            junk = inputs("go", 1, rng)
            cancelled_resident = srv.submit(cid["go"], 1, 50, junk["jitter"], stim=junk["stim"])
        srv.advance()
        if rnd == 2:
            assert srv.state(cancelled_queued)[0] == G.REQ_QUEUED
            srv.destroy(cancelled_queued)
            assert srv.state(cancelled_resident)[0] == G.REQ_RESIDENT
            srv.destroy(cancelled_resident)
        st = srv.stats()
        if rnd > max(plan) and st["queued"] == 0 and st["resident"] == 0:
            break
    st = srv.stats()
    assert st["completed"] == len(reqs) and st["failed"] == 0 and st["cancelled"] == 2, st
    assert st["queued"] == 0 and st["resident"] == 0 and st["free_slots"] == st["slots"]
    assert 0 < st["p50_ms"] <= st["p99_ms"] <= st["max_ms"]
    assert st["compartment_updates"] > 0 and st["lost_spike_reads"] == 0
    n_spikes = 0
    for rid, name, n_sys, n_iv, inp in reqs:
        state, lat, status = srv.state(rid)
        assert state == G.REQ_DONE and status == 0 and lat > 0
        nc = n_sys * SHAPES[name][1] * SHAPES[name][2] * rows(name).shape[0]
        got = srv.read(rid, nc)
        ref = fresh(precision, name, n_sys, n_iv, inp, spikes=True)
        np.testing.assert_array_equal(got, ref[G.F_VNEW], err_msg=f"request {rid} ({name})")
        t, c = srv.spikes(rid)
        rt, rc = ref["spikes"]
        np.testing.assert_array_equal(t, rt, err_msg=f"request {rid} spike times")
        np.testing.assert_array_equal(c, rc, err_msg=f"request {rid} spike cells")
        n_spikes += len(t)
    assert n_spikes > 0
    with pytest.raises(G.GbrkcError):
        srv.submit(cid["pkj"], 3, 5, np.zeros(3))   # more systems than the class holds
    srv.close()


def test_served_request_matches_oracle(oracle):
    """Plain FP64: a served granule request's final voltages and raster equal the oracle's."""
    O = oracle
    rng = np.random.default_rng(5)
    name, n_sys, n_iv = "gr", 3, 60
    srv = G.Server(G.FP64, hbm_budget=0, quantum=8)
    c = srv.add_class(M.GR, 1, 1, rows(name), slots=8, gap=False)
    srv.start()
    # a first request occupies and frees the slots
    warm = inputs(name, 8, rng)
    srv.submit(c, 8, 5, warm["jitter"], stim=warm["stim"])
    srv.advance()
    inp = inputs(name, n_sys, rng)
    inp["stim"] = (inp["stim"][0], np.full(n_sys, 0.05e-3), inp["stim"][2], inp["stim"][3])
    rid = srv.submit(c, n_sys, n_iv, inp["jitter"], stim=inp["stim"], cond_scale=inp["cond_scale"])
    while srv.state(rid)[0] != G.REQ_DONE:
        srv.advance()
    got = srv.read(rid, n_sys * 4)
    st, sc = srv.spikes(rid)
    ref_v, ref_t, ref_c = [], [], []
    comp, amp, t0, t1 = inp["stim"]
    for k in range(n_sys):
        s = O.System(M.GR, 1, 1, rows(name), inp["jitter"][k:k + 1], stim=(comp[k], amp[k], t0[k], t1[k]),
                     canon=True, cond_scale=inp["cond_scale"][k:k + 1])
        assert s.init() == 0
        prev, t = 100.0, 0.0
        for _ in range(n_iv):
            assert s.advance(t) == 0
            t += G.H_MAX
            x = s.vnew()[3]            # reduced granule cell: the last compartment
            if x > 10.0 and prev <= 10.0:
                ref_t.append(t)
                ref_c.append(k)
            prev = x
        ref_v.append(s.vnew())
    np.testing.assert_array_equal(got, np.concatenate(ref_v))
    order = np.lexsort((ref_c, ref_t))
    np.testing.assert_array_equal(st, np.array(ref_t)[order])
    np.testing.assert_array_equal(sc, np.array(ref_c)[order])
    assert len(st) > 0, "the stimulus should make the granule cells fire"
    srv.close()


@pytest.mark.parametrize("precision", [G.FP64, G.MIXED])
def test_reset_then_noalloc_advance(precision):
    """The allocation-free advance initialises refilled systems the same way."""
    rng = np.random.default_rng(21)
    engines = []
    for _ in range(2):
        eng = G.Engine(precision)
        for name in ("gr", "go", "pkj"):
            t, nx, ny, _, _, _, gap = SHAPES[name]
            for k in range(2):
                eng.add_system(t, nx, ny, rows(name), np.zeros(nx * ny), gap=gap, idle=True)
        eng.build()
        engines.append(eng)
    inp = {name: inputs(name, 2, np.random.default_rng(5)) for name in ("gr", "go", "pkj")}
    for eng in engines:
        for j, name in enumerate(("gr", "go", "pkj")):
            d = inp[name]
            eng.reset_systems(2 * j, 2, d["jitter"], stim=d["stim"], cond_scale=d["cond_scale"], n_intervals=12)
    a, b = engines
    a.advance(0.0, 8)
    b.advance_noalloc(0.0, 8)
    a.advance(1.0, 8)
    b.advance_noalloc(1.0, 8)
    for s in range(6):
        np.testing.assert_array_equal(a.vnew(s), b.vnew(s), err_msg=f"system {s}")
        assert a.ctl(s)[1] == b.ctl(s)[1]
    ref = fresh(precision, "go", 2, 12, inp["go"])
    np.testing.assert_array_equal(np.concatenate([b.vnew(2), b.vnew(3)]), ref[G.F_VNEW])
    for eng in engines:
        eng.close()


def test_failed_request_is_reported_and_its_slots_reused():
    """A request whose cells blow up (a 1000x stimulus: non-finite voltages,
    a solver stop on the device) ends FAILED with the stop status; the
    request beside it completes, and the freed slots serve the next one."""
    rng = np.random.default_rng(31)
    srv = G.Server(G.MIXED, hbm_budget=0, quantum=8)
    c = srv.add_class(M.GR, 1, 1, rows("gr"), slots=8, gap=False)
    srv.start()
    good = srv.submit(c, 4, 12, rng.uniform(-0.5, 0.5, 4), stim=(1, 0.02e-3, 0.0, 1e9))
    bad = srv.submit(c, 2, 12, rng.uniform(-0.5, 0.5, 2), stim=(1, 1.0, 0.0, 1e9))
    for _ in range(10):
        srv.advance()
        if srv.stats()["resident"] == 0:
            break
    st_bad, _, status = srv.state(bad)
    assert st_bad == G.REQ_FAILED and status != 0
    assert srv.state(good)[0] == G.REQ_DONE
    st = srv.stats()
    assert st["failed"] == 1 and st["completed"] == 1 and st["free_slots"] == st["slots"]
    inp = inputs("gr", 8, rng)
    nxt = srv.submit(c, 8, 10, inp["jitter"], stim=inp["stim"], cond_scale=inp["cond_scale"])
    while srv.state(nxt)[0] in (G.REQ_QUEUED, G.REQ_RESIDENT):
        srv.advance()
    assert srv.state(nxt)[0] == G.REQ_DONE
    ref = fresh(G.MIXED, "gr", 8, 10, inp)
    np.testing.assert_array_equal(srv.read(nxt, 8 * 4), ref[G.F_VNEW])
    srv.close()
