"""The Markov-scheme solvers never swap rows.

The GR 12-state Na and GoC KAHP Crank-Nicolson matrices are -(Q + 2/DT I)
with Q a rate generator, i.e. strictly diagonally dominant by columns, so the
reference's partial pivoting (gr_ion.cu:141-190, go_ion.cu:152-200) always
keeps the diagonal.  The CUDA path eliminates without swaps (and checks each
pivot); this pins the premise on the oracle across spiking runs of both cell
types, at the step currents of the mixed workload and above.
"""
import numpy as np

import morph as M


def run(O, cell_type, rows, comp, amp, ms, tol=0.0):
    O.libc_srand(0)
    jit = O.draw_jitter(cell_type, 1)
    s = O.System(cell_type, 1, 1, rows, jit, stim=(comp, amp, 0.0, 1e9), tol=tol)
    assert s.init() == 0
    t = 0.0
    spikes, prev = 0, s.vnew().copy()
    for _ in range(int(ms / 0.125)):
        assert s.advance(t) == 0
        t += 0.125
        v = s.vnew()
        spikes += int(np.any((prev < 0.0) & (v >= 0.0)))
        prev = v.copy()
    return s, spikes


def test_no_row_swaps(oracle):
    O = oracle
    before = O.pivot_swaps()
    s, sp_gr = run(O, M.GR, M.gr_reduced4(), 1, 0.05e-3, 60.0)
    assert s.stats()["ion_updates"] > 100
    s, sp_go = run(O, M.GO, M.go_synthetic(2), 30, 0.4e-3, 30.0)
    assert s.stats()["ion_updates"] > 20
    assert sp_gr + sp_go > 0, "the runs should cross spike threshold"
    assert O.pivot_swaps() == before


def test_markov_states_conserved(oracle):
    """The Markov schemes keep their occupancies summing to 1 through the
    same spiking runs (the reference's own check: gr_ion.cu:204, within
    0.99..1.01; go_ion.cu:208, within 1e-4); here to 1e-9."""
    O = oracle
    for cell_type, rows, comp, amp, ms, slots in ((M.GR, M.gr_reduced4(), 1, 0.05e-3, 30.0, range(8, 20)),
                                                   (M.GO, M.go_synthetic(2), 30, 0.4e-3, 15.0, range(18, 24))):
        s, _ = run(O, cell_type, rows, comp, amp, ms)
        total = sum(s.ion(k) for k in slots)
        used = total > 0.5                       # compartments that carry the scheme
        assert used.any()
        assert np.max(np.abs(total[used] - 1.0)) < 1e-9, (cell_type, np.max(np.abs(total[used] - 1.0)))
