"""Large systems on a thread-block cluster (8 or 16 CTAs, workspace spread
block-cyclically over their shared memory, neighbour reads through
distributed shared memory): bit for bit with the oracle, like every other
team.  A low size threshold (GBRKC_CLUSTER_MIN_NC) sends the test cases down
that path; GBRKC_CLUSTER_SIZE picks the cluster size."""
import numpy as np
import pytest

import gbrkc as G
import morph as M
from test_gpu_parity import HORIZON, run_pair

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("csize", [8, 16])
@pytest.mark.parametrize("name", ["pkj_cell", "pkj_2x1_gj", "gr_full"])
def test_cluster_team_bit_exact(oracle, monkeypatch, name, csize):
    monkeypatch.setenv("GBRKC_CLUSTER_MIN_NC", "500")
    monkeypatch.setenv("GBRKC_CLUSTER_SIZE", str(csize))
    n = HORIZON.get(name, 64)
    s, eng, sid = run_pair(oracle, name, [1, n // 2 - 1, n // 2])
    persistent, ctas = eng.launch_layout()
    assert persistent is False and max(ctas) == csize, ctas
    eng.close()


@pytest.mark.parametrize("csize", [8, 16])
def test_cluster_io_network(oracle, monkeypatch, csize):
    """A 12x12 olive network (432 compartments, nonlinear gap junctions
    crossing CTA boundaries) on a cluster, against the oracle."""
    monkeypatch.setenv("GBRKC_CLUSTER_MIN_NC", "400")
    monkeypatch.setenv("GBRKC_CLUSTER_SIZE", str(csize))
    O = oracle
    O.libc_srand(0)
    jit = O.draw_jitter(O.IO, 144)
    stim = (0, 5.5, 1.0, 30.0)
    s = O.System(O.IO, 12, 12, M.io_rows(), jit, stim=stim, canon=True)
    assert s.init() == 0
    eng = G.Engine(G.FP64)
    sid = eng.add_system(M.IO, 12, 12, M.io_rows(), jit, stim=stim, gap=True)
    eng.build()
    assert max(eng.launch_layout()[1]) == csize
    t = 0.0
    for chunk in (1, 15, 16):
        eng.advance(t, chunk)
        for _ in range(chunk):
            assert s.advance(t) == 0
            t += G.H_MAX
        np.testing.assert_array_equal(eng.vnew(sid), s.vnew(), err_msg=f"t={t}")
        np.testing.assert_array_equal(eng.read(sid, G.F_B), s.b(), err_msg=f"b t={t}")
    ctl, st, status = eng.ctl(sid)
    assert status == 0 and st == s.stats()
    eng.close()
