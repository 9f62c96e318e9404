"""The parameter-sweep workload on the CPU: its shape (counts, per-channel
factor ranges, currents, per-system durations) and that per-channel
conductance factors reach the oracle's conductances."""
import numpy as np

import configs
import morph as M


def test_sweep_workload_shape():
    specs = configs.sweep_batch(n_gr=300, n_go=200)
    gr = [s for s in specs if s.cell_type == M.GR]
    go = [s for s in specs if s.cell_type == M.GO]
    assert len(gr) == 300 and len(go) == 200
    for group, ncond, comp in ((gr, 10, 1), (go, 13, 30)):
        f = np.array([s.cond_scale_ch for s in group])
        assert f.shape == (len(group), ncond) and f.min() >= 0.8 and f.max() <= 1.2
        assert len({s.rows.tobytes() for s in group}) == 1          # one morphology per type
        assert all(s.stim[0] == comp and 0 <= s.stim[1] <= 0.4e-3 and s.stim[2] == 0.0 for s in group)
    n_iv = np.array([s.extra["n_intervals"] for s in specs])
    assert n_iv.min() >= 800 and n_iv.max() <= 8000 and len(set(n_iv.tolist())) > 100
    full = configs.sweep_batch()
    assert len(full) == 65536


def test_sweep_channel_scales_change_the_cells(oracle):
    """Per-channel factors reach the conductances: all factors equal to x give
    the per-cell scale x exactly; distinct factors give a different cell."""
    sp = configs.sweep_batch(n_gr=1, n_go=0)[0]
    x = 1.1
    a = oracle.System(sp.cell_type, 1, 1, sp.rows, sp.jitter, stim=sp.stim, cond_scale_ch=np.full(10, x))
    b = oracle.System(sp.cell_type, 1, 1, sp.rows, sp.jitter, stim=sp.stim, cond_scale=np.full(1, x))
    for k in range(a.ncond()):
        np.testing.assert_array_equal(a.cond(k), b.cond(k))
    c = oracle.System(sp.cell_type, 1, 1, sp.rows, sp.jitter, stim=sp.stim, cond_scale_ch=sp.cond_scale_ch)
    d = oracle.System(sp.cell_type, 1, 1, sp.rows, sp.jitter, stim=sp.stim)
    for k in range(c.ncond()):
        np.testing.assert_array_equal(c.cond(k), d.cond(k) * sp.cond_scale_ch[k])


