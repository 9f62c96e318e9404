"""The reference's network wiring rules (connectivity.py, after syn.cu's
*_create functions), checked on the CPU against the rules restated pair by
pair, and the Purkinje location-file reader."""
import numpy as np

import connectivity as CN


def grid_gr(i, nx):
    return (i % nx) * 16.0, (i // nx) * 16.0


def grid_big(i, nx):
    return (i % nx) * 32.0 + 8.0, (i // nx) * 32.0 + 8.0


def test_wiring_rules(tmp_path):
    nx_gr, ny_gr, nx_go, ny_go, nx_pk, ny_pk = 8, 6, 2, 2, 2, 1
    x = np.random.default_rng(1).uniform(-150, 150, 1600)
    rows = np.column_stack([np.arange(1600), x, np.zeros(1600), np.zeros(1600), np.full(1600, 3)])
    path = tmp_path / "Pkj_location_info.csv"
    np.savetxt(path, rows, delimiter=",", fmt=["%d", "%.3f", "%.3f", "%.3f", "%d"])
    px, pz, pt = CN.read_pkj_location(str(path))
    assert px.shape == (1600,) and pt[0] == 3
    g = CN.reference_synapses(nx_gr, ny_gr, nx_go, ny_go, nx_pk, ny_pk, px, np.random.default_rng(2))
    n_gr, n_go, n_pk = nx_gr * ny_gr, nx_go * ny_go, nx_pk * ny_pk
    mf = g[CN.SYN_MFGR]
    assert len(mf["post_cell"]) == 4 * n_gr and set(mf["post_comp"]) == {0, 1, 2, 3}
    assert np.all(mf["weight"] == 10000.0)
    # GrC -> GoC: every pair within the window, granule-major
    want = [(a, b) for a in range(n_gr) for b in range(n_go)
            if abs(grid_big(b, nx_go)[0] - grid_gr(a, nx_gr)[0]) < 16 and
            abs(grid_big(b, nx_go)[1] - grid_gr(a, nx_gr)[1]) < 220]
    gg = g[CN.SYN_GRGO]
    assert list(zip(gg["pre_cell"], gg["post_cell"])) == want
    cnt = np.bincount(gg["post_cell"], minlength=n_go)
    np.testing.assert_array_equal(gg["weight"], 16.0 / (cnt[gg["post_cell"]] / 4.0))
    assert np.all(gg["post_comp"] == 0) and gg["pre_comp"].min() >= 300 and gg["pre_comp"].max() <= 577
    # GoC -> GrC
    want = [(b, a) for b in range(n_go) for a in range(n_gr)
            if abs(grid_big(b, nx_go)[0] - grid_gr(a, nx_gr)[0]) < 32 and
            abs(grid_big(b, nx_go)[1] - grid_gr(a, nx_gr)[1]) < 32]
    og = g[CN.SYN_GOGR]
    assert list(zip(og["pre_cell"], og["post_cell"])) == want
    cnt = np.bincount(og["post_cell"], minlength=n_gr)
    np.testing.assert_array_equal(og["weight"], 640000.0 / (cnt[og["post_cell"]] * 4.0))
    assert np.all(og["pre_comp"] == 30) and np.all(og["post_comp"] == 16)
    # GrC -> PC: 25 synapses per pair within the window
    want = [(a, b) for a in range(n_gr) for b in range(n_pk)
            if abs(grid_big(b, nx_pk)[0] - grid_gr(a, nx_gr)[0]) < 120 and
            abs(grid_big(b, nx_pk)[1] - grid_gr(a, nx_gr)[1]) < 220]
    pk = g[CN.SYN_GRPKJ]
    assert len(pk["post_cell"]) == 25 * len(want)
    assert list(zip(pk["pre_cell"][::25], pk["post_cell"][::25])) == want
    cnt = np.bincount([b for _, b in want], minlength=n_pk)
    np.testing.assert_allclose(pk["weight"], 300000.0 / (512.0 * cnt[pk["post_cell"]] / 10.0), rtol=0)
    # the target compartment's location is within 5 um of the connection's dx
    # (f in (-0.5, 0.5]), and the running minimum never moves away from it
    for k, (a, b) in enumerate(want):
        dx = (a % nx_gr) * 16.0 - (8.0 + (b % nx_pk) * 32.0)
        comps = pk["post_comp"][25 * k:25 * (k + 1)]
        assert np.all(np.abs(px[comps] - dx) <= 5.0 + np.min(np.abs(px - dx)) + 1e-9)
