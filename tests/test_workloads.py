"""The benchmark's seeded synthetic workloads (configs.py) on the CPU: shapes,
sizes and value ranges as the bench line reports them, and reproducible from
their seeds."""
import numpy as np

import configs
import morph as M


def test_mixed_batch():
    specs = configs.mixed_batch()
    counts = configs.type_counts(specs)
    assert counts == {"gr": [4096, 16384], "go": [1024, 134144], "pkj": [256, 409600], "io": [256, 768]}
    assert sum(c[1] for c in counts.values()) == 560896
    again = configs.mixed_batch()
    for a, b in zip(specs, again):
        np.testing.assert_array_equal(a.jitter, b.jitter)
        for x, y in zip(a.stim, b.stim):
            np.testing.assert_array_equal(x, y)
    for s in specs:
        comp, amp, t0, t1 = (np.broadcast_to(x, s.n) for x in s.stim)
        assert np.all((comp >= 0) & (comp < s.rows.shape[0]))
        assert np.all((amp >= 0) & (amp <= configs.AMP_MAX[s.cell_type]))
        assert np.all((t0 >= 0) & (t0 <= 20.0)) and np.all(t1 > t0)


def test_serve_workload():
    classes, reqs = configs.serve_workload()
    assert len(reqs) == 64 and len(classes) == 1 + len(configs.GO_STABLE_VARIANTS) + len(configs.PKJ_STABLE_SEEDS) + 1
    arrivals = np.array([r.arrival_s for r in reqs])
    assert np.all(np.diff(arrivals) > 0)
    for r in reqs:
        c = classes[r.cls]
        cells = r.n_systems * c.nx * c.ny
        assert 1 <= r.n_systems <= c.max_systems <= c.slots
        assert 40 <= r.n_intervals <= 200                       # 5-25 ms
        assert r.jitter.size == cells and r.cond_scale.size == cells
        assert np.all((r.cond_scale >= 0.8) & (r.cond_scale <= 1.2))
        assert np.all(r.stim[0] == c.stim_comp) and np.all(r.stim[1] <= configs.AMP_MAX[c.cell_type])
        assert (r.io_gap_g is not None) == (c.cell_type == M.IO)
        if r.io_gap_g is not None:
            assert r.io_gap_g.size == 4 * cells
    _, again = configs.serve_workload()
    assert [(r.cls, r.n_systems, r.n_intervals) for r in reqs] == [(r.cls, r.n_systems, r.n_intervals) for r in again]


def test_network_batch():
    specs, groups = configs.network_batch()
    types = np.array([s.cell_type for s in specs])
    assert [int((types == t).sum()) for t in (M.GR, M.GO, M.PKJ)] == [2048, 512, 512]
    assert sum(len(g["post_system"]) for g in groups) == 780404
    pre_t = {configs.SYN_GRGO: M.GR, configs.SYN_GOGR: M.GO, configs.SYN_GRPKJ: M.GR}
    post_t = {configs.SYN_MFGR: M.GR, configs.SYN_GRGO: M.GO, configs.SYN_GOGR: M.GR, configs.SYN_GRPKJ: M.PKJ}
    for g in groups:
        post = np.asarray(g["post_system"])
        assert np.all(types[post] == post_t[g["kind"]])
        comp = np.broadcast_to(g["post_comp"], post.size)
        ncomp = np.array([specs[i].rows.shape[0] for i in post])
        assert np.all((comp >= 0) & (comp < ncomp))
        if "pre_system" in g:
            assert np.all(types[np.asarray(g["pre_system"])] == pre_t[g["kind"]])
        w = np.asarray(g["weight"])
        assert np.all(np.isfinite(w) & (w > 0))
        d = np.asarray(g["delay"])
        assert np.all((d >= 8) & (d <= 40))                    # 1-5 ms
