"""Known answer for the whole RKC path on the CPU oracle: a passive granule
cable (the 578-compartment tree with every channel but the first leak set to
0, so its voltage obeys the linear system C dV/dt = -(L V + g_L (V - E_L) - I))
against the matrix exponential of that system.

L is the axial conductance Laplacian of gr_solve.cu:26-45 (between a
compartment and its parent, g = 2 / (R_a l / (pi r^2) summed over both)); the
areas, capacitances and leak conductances are gr.cu:36-60's.  The oracle
freezes the leak current between ion updates (every 2^{log10 tol} ms), so it
matches the exact solution to within that splitting: a few uV after a 13 mV
excursion at the granule tolerance (1e-9), and less as a tighter tolerance
brings the ion updates closer."""
import numpy as np
import pytest

import morph as M

scipy_linalg = pytest.importorskip("scipy.linalg")

V_LEAK1_GR = -16.5           # gr.cuh:15
STIM = (16, 0.01e-3)         # soma, 0.01 nA (gr.cu:244-253)


def passive_rows():
    rows = M.gr_synthetic(11)
    rows[:, 8:] = 0.0        # every conductance but leak 1
    return rows


def exact(rows, v0, t_ms):
    n = rows.shape[0]
    rad, ln, ra = 0.5 * rows[:, 2] * 1e-4, rows[:, 3] * 1e-4, rows[:, 4] * 1e-3
    area = 2.0 * np.pi * rad * ln
    cm, gl = rows[:, 5] * area, rows[:, 7] * area
    lap = np.zeros((n, n))
    for i in range(n):
        p = int(rows[i, 1])
        if p < 0:
            continue
        g = 2.0 / (ra[i] * ln[i] / (rad[i] ** 2 * np.pi) + ra[p] * ln[p] / (rad[p] ** 2 * np.pi))
        lap[i, i] += g
        lap[p, p] += g
        lap[i, p] -= g
        lap[p, i] -= g
    cur = np.zeros(n)
    cur[STIM[0]] = STIM[1]
    a = lap + np.diag(gl)
    v_star = np.linalg.solve(a, gl * V_LEAK1_GR + cur)
    m = -a / cm[:, None]
    return v_star + scipy_linalg.expm(m * t_ms) @ (v0 - v_star)


def max_error(O, rows, tol):
    O.libc_srand(0)
    s = O.System(M.GR, 1, 1, rows, O.draw_jitter(M.GR, 1), stim=(STIM[0], STIM[1], 0.0, 1e9), tol=tol)
    assert s.init() == 0
    v0 = s.vnew().copy()
    assert np.ptp(v0) == 0.0                       # a uniform start: the axial currents come from the stimulus
    t = 0.0
    for k in range(16):                            # 2 ms
        assert s.advance(t) == 0
        t += 0.125
    want = exact(rows, v0, 2.0)
    assert np.ptp(want) > 10.0, "the stimulus should spread a voltage gradient"
    return np.max(np.abs(s.vnew() - want))


def test_passive_cable_matches_matrix_exponential(oracle):
    rows = passive_rows()
    err = max_error(oracle, rows, 0.0)             # the granule default, 1e-9
    assert err < 1e-2, f"max |V - V_exact| = {err:.3g} mV"
    # the remainder is the frozen-current splitting: it shrinks with the ion-update interval
    assert max_error(oracle, rows, 1e-11) < 0.5 * err
