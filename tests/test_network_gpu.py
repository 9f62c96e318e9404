"""Network mode (chemical synapses between systems) on the GPU against the
oracle in canonical mode, bit for bit: every system's voltages and every
synapse's states and conductance, through spikes that travel granule ->
Golgi, Golgi -> granule and granule -> Purkinje."""
import numpy as np
import pytest

import gbrkc as G
from gpu_cases import build_network

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("delays", [False, True])
@pytest.mark.parametrize("checkpoints", [(40, 100, 160)])
def test_network_fp64_bit_exact(oracle, checkpoints, delays):
    """delays: every synapse acts 1-40 intervals after its event (bit rings)."""
    O = oracle
    net = O.Network()
    ids_o = build_network(O, net, delays=delays)
    net.build()
    eng = G.Engine(G.FP64)
    ids_g = build_network(O, eng, delays=delays)
    eng.build()
    nsyn = len(net.syn(0))
    t, done = 0.0, 0
    for cp in checkpoints:
        eng.advance(t, cp - done)
        for _ in range(cp - done):
            assert net.advance(t) == 0
            t += G.H_MAX
        done = cp
        for a, b in zip(ids_o, ids_g):
            np.testing.assert_array_equal(eng.vnew(b), net.systems[a].vnew(), err_msg=f"interval {cp} system {a}")
        for f in range(5):
            np.testing.assert_array_equal(eng.read_synapses(f, nsyn), net.syn(f), err_msg=f"interval {cp} field {f}")
    s0 = net.syn(1)
    n_mf, n_grgo, n_gogr = 32, 16, 16
    assert s0[:n_mf].max() > 0, "mossy fibres fired"
    assert s0[n_mf + n_grgo:n_mf + n_grgo + n_gogr].max() > 0, "a Golgi spike reached the granule cells"
    assert s0[n_mf + n_grgo + n_gogr:].max() > 0, "a granule spike reached the Purkinje cell"
    eng.close()


def test_network_mixed_runs():
    """Mixed precision steps the same network; synapses see spikes."""
    import oracle_py as O
    eng = G.Engine(G.MIXED)
    build_network(O, eng)
    eng.build()
    eng.advance(0.0, 160)
    s0 = eng.read_synapses(G.SYNF_S0, 32 + 16 + 16 + 40)
    assert np.all(np.isfinite(s0)) and s0[:32].max() > 0
    eng.close()


def test_reference_wiring_network_bit_exact(oracle):
    """Full-size cells wired by the reference's rules (connectivity.py):
    8 granule cells (578 compartments), one Golgi cell, one Purkinje cell
    with synthetic compartment locations, one system each; FP64 against the
    oracle, bit for bit."""
    import connectivity as CN
    import morph as M
    O = oracle
    g = CN.reference_synapses(4, 2, 1, 1, 1, 1, np.random.default_rng(3).uniform(-150, 150, 1600),
                              np.random.default_rng(4))
    assert all(len(g[k]["post_cell"]) > 0 for k in g)
    shapes = [(M.GR, M.gr_synthetic(11), 8), (M.GO, M.go_synthetic(3), 1), (M.PKJ, M.pkj_synthetic(2), 1)]
    net, eng = O.Network(), G.Engine(G.FP64)
    O.libc_srand(0)
    jit = [O.draw_jitter(t, n) for t, _, n in shapes]
    first = {}
    for target in (net, eng):
        k = 0
        for (t, rows, n), j in zip(shapes, jit):
            first[(id(target), t)] = k
            for c in range(n):
                if target is net:
                    s = O.System(t, 1, 1, rows, j[c:c + 1], canon=True)
                    assert s.init() == 0
                    target.add_system(s)
                else:
                    target.add_system(t, 1, 1, rows, j[c:c + 1])
                k += 1
        CN.add_reference_network(target, g, lambda ty, c, tg=target: (first[(id(tg), ty)] + c, 0),
                                 rates=(400.0, 0.0, 0.0, 0.0), seed=9)
    net.build()
    eng.build()
    nsyn = len(net.syn(0))
    eng.advance(0.0, 24)
    t = 0.0
    for _ in range(24):
        assert net.advance(t) == 0
        t += G.H_MAX
    for a in range(len(net.systems)):
        np.testing.assert_array_equal(eng.vnew(a), net.systems[a].vnew(), err_msg=f"system {a}")
    for f in range(5):
        np.testing.assert_array_equal(eng.read_synapses(f, nsyn), net.syn(f), err_msg=f"field {f}")
    assert net.syn(1)[:32].max() > 0, "mossy fibres fired"
    eng.close()
