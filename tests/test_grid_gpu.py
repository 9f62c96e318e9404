"""A system alone in its engine and larger than a cluster holds efficiently
runs as one grid team: every CTA of a cooperative launch takes a slice of
its workspace (kept in global memory, in L2), and a bounded software grid
barrier separates the stages.  Bit for bit with the oracle like every other
team: the reductions combine chunk sums (a power-of-two chunk per CTA) in the
same pairwise order.  GBRKC_GRID_MIN_NC lowers the size threshold so that
small cases take the path; GBRKC_GRID_BW and GBRKC_GRID_CTAS force a shape."""
import numpy as np
import pytest

import gbrkc as G
import morph as M
from gpu_cases import jitter_for
from test_gpu_parity import HORIZON, run_pair

pytestmark = pytest.mark.gpu


def _sms():
    import torch
    return torch.cuda.get_device_properties(0).multi_processor_count


def grid_shape(nc, cap, want_bw=0, want_ctas=0):
    """The engine's choice of (element-owning threads per CTA, CTAs): the
    smallest busiest-CTA load, then the fewest CTAs, within 256 chunks and 8
    rows per thread."""
    best = None
    for bw in (32, 64, 128, 256):
        if want_bw and bw != want_bw:
            continue
        chunks = -(-nc // bw)
        if chunks > 256:
            continue
        ctas = min(cap, want_ctas) if want_ctas else min(cap, chunks)
        rows = -(-chunks // ctas)
        if rows > 8:
            continue
        key = (rows * bw, ctas)
        if best is None or key < best[0]:
            best = (key, bw, ctas)
    return best[1], best[2]


def test_grid_shape_rule():
    assert grid_shape(14400, 152) == (128, 113)      # the Purkinje 3x3 system
    assert grid_shape(57600, 152) == (256, 152)
    assert grid_shape(1600, 152) == (32, 50)


@pytest.mark.parametrize("name", ["pkj_cell", "pkj_2x1_gj", "gr_full", "go_2x2_gj"])
def test_grid_team_bit_exact(oracle, monkeypatch, name):
    monkeypatch.setenv("GBRKC_GRID_MIN_NC", "300")
    n = HORIZON.get(name, 64)
    s, eng, sid = run_pair(oracle, name, [1, n // 2 - 1, n // 2])
    persistent, ctas = eng.launch_layout()
    assert persistent is False and max(ctas) == grid_shape(s.nc, _sms())[1], ctas
    eng.close()


@pytest.mark.parametrize("bw,ctas,rows_smem", [(32, 0, 1), (64, 0, 1), (128, 0, 1), (256, 0, 1), (64, 7, 1),
                                                (256, 3, 1), (128, 0, 0), (64, 7, 0)])
def test_grid_team_shapes_bit_exact(oracle, monkeypatch, bw, ctas, rows_smem):
    """Every element-owning width, few CTAs (several rows per thread), and
    the operator's rows read from shared memory or (GBRKC_GRID_ROWS_SMEM=0)
    from global memory."""
    monkeypatch.setenv("GBRKC_GRID_MIN_NC", "300")
    monkeypatch.setenv("GBRKC_GRID_BW", str(bw))
    monkeypatch.setenv("GBRKC_GRID_ROWS_SMEM", str(rows_smem))
    if ctas:
        monkeypatch.setenv("GBRKC_GRID_CTAS", str(ctas))
    s, eng, sid = run_pair(oracle, "pkj_2x1_gj", [1, 15, 16])
    persistent, got = eng.launch_layout()
    assert persistent is False and max(got) == grid_shape(s.nc, _sms(), bw, ctas)[1], got
    eng.close()


@pytest.mark.parametrize("name", ["pkj_2x1_gj", "go_2x2_gj"])
def test_grid_team_sc_fence_barrier_bit_exact(oracle, monkeypatch, name):
    """The grid barrier with sequentially consistent fences on both sides of
    the wait (GBRKC_GRID_FENCE=sc) instead of fence.acq_rel and acquire
    polls."""
    monkeypatch.setenv("GBRKC_GRID_MIN_NC", "300")
    monkeypatch.setenv("GBRKC_GRID_FENCE", "sc")
    s, eng, sid = run_pair(oracle, name, [1, 15, 16])
    assert eng.launch_layout()[0] is False
    eng.close()


@pytest.mark.parametrize("name", ["pkj_2x1_gj", "go_2x2_gj"])
def test_grid_team_grid_barrier_stages_bit_exact(oracle, monkeypatch, name):
    """Every stage barrier a grid barrier (GBRKC_GRID_LOCAL=0) instead of a
    wait for the neighbouring CTAs only."""
    monkeypatch.setenv("GBRKC_GRID_MIN_NC", "300")
    monkeypatch.setenv("GBRKC_GRID_LOCAL", "0")
    s, eng, sid = run_pair(oracle, name, [1, 15, 16])
    assert eng.launch_layout()[0] is False
    eng.close()


def test_grid_io_network(oracle, monkeypatch):
    """A 12x12 olive network (nonlinear gap junctions across CTAs)."""
    monkeypatch.setenv("GBRKC_GRID_MIN_NC", "400")
    O = oracle
    O.libc_srand(0)
    jit = O.draw_jitter(O.IO, 144)
    stim = (0, 5.5, 1.0, 30.0)
    s = O.System(O.IO, 12, 12, M.io_rows(), jit, stim=stim, canon=True)
    assert s.init() == 0
    eng = G.Engine(G.FP64)
    sid = eng.add_system(M.IO, 12, 12, M.io_rows(), jit, stim=stim, gap=True)
    eng.build()
    assert max(eng.launch_layout()[1]) == grid_shape(s.nc, _sms())[1]
    t = 0.0
    for chunk in (1, 15, 16):
        eng.advance(t, chunk)
        for _ in range(chunk):
            assert s.advance(t) == 0
            t += G.H_MAX
        np.testing.assert_array_equal(eng.vnew(sid), s.vnew(), err_msg=f"t={t}")
    ctl, st, status = eng.ctl(sid)
    assert status == 0 and st == s.stats()
    eng.close()


def test_grid_system_beyond_cluster_capacity(oracle):
    """6 x 6 Purkinje cells of 1600 compartments (57 600; two rows of the
    grid's threads): the default path for it is now the grid team."""
    rows = M.pkj_synthetic(4, 1600)
    stim = (1599, 0.5e-3, 0.0, 1e9)
    jit = jitter_for(oracle, M.PKJ, 36)
    s = oracle.System(M.PKJ, 6, 6, rows, jit, stim=stim, gj_pairs=M.PKJ_GJ_PAIRS, pkj_gj=True, canon=True)
    assert s.init() == 0
    eng = G.Engine(G.FP64)
    sid = eng.add_system(M.PKJ, 6, 6, rows, jit, stim=stim, gj_pairs=M.PKJ_GJ_PAIRS, gap=True)
    eng.build()
    persistent, ctas = eng.launch_layout()
    assert not persistent and ctas[M.PKJ] == _sms(), ctas
    assert eng.type_team(M.PKJ) == "grid" and eng.type_team(M.GR) == ""
    t = 0.0
    for chunk in (1, 2):
        eng.advance(t, chunk)
        for _ in range(chunk):
            assert s.advance(t) == 0
            t += G.H_MAX
        np.testing.assert_array_equal(eng.vnew(sid), s.vnew())
    ctl, st, status = eng.ctl(sid)
    assert status == 0
    for k, v in s.stats().items():
        assert st[k] == v, (k, st[k], v)
    eng.close()
