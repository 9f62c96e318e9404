"""The oracle's network mode on its own (CPU): synaptic events propagate
and a run is deterministic (the Poisson draws are a pure function of seed,
synapse and interval)."""
import numpy as np

from gpu_cases import build_network


def run(O, n_iv):
    net = O.Network()
    build_network(O, net)
    net.build()
    t = 0.0
    for _ in range(n_iv):
        assert net.advance(t) == 0
        t += 0.125
    return net


def test_network_activity_and_determinism(oracle):
    a = run(oracle, 120)
    b = run(oracle, 120)
    for f in range(5):
        np.testing.assert_array_equal(a.syn(f), b.syn(f))
    for sa, sb in zip(a.systems, b.systems):
        np.testing.assert_array_equal(sa.vnew(), sb.vnew())
    s0 = a.syn(1)
    assert s0[:32].max() > 0
    # some granule cell spiked: its outgoing synapses stepped
    assert s0[32:48].max() > 0 or s0[64:].max() > 0


def test_delay_ring_shifts_events(oracle):
    """A delay of d intervals shifts a synapse's event train by d: mossy-fibre
    states (their Poisson draws do not depend on the cells) after k
    intervals with delay 3 equal those after k - 3 without, bit for bit."""
    import pytest
    import morph as M
    O = oracle

    def mf_states(delay, n_iv):
        net = O.Network()
        O.libc_srand(0)
        ids = [net.add_system(_cell(O, M)) for _ in range(2)]
        net.add_synapses(0, np.repeat(ids, 4), np.tile(np.arange(4), 2), 10000.0, rates=(800.0, 0.0, 0.0, 0.0),
                         seed=11, delay=delay)
        net.build()
        t = 0.0
        for _ in range(n_iv):
            assert net.advance(t) == 0
            t += 0.125
        return net.syn(1), net.syn(2)

    s0, s1 = mf_states(3, 40)
    r0, r1 = mf_states(0, 37)
    assert r0.max() > 0
    np.testing.assert_array_equal(s0, r0)
    np.testing.assert_array_equal(s1, r1)
    np.testing.assert_array_equal(mf_states(None, 37)[0], r0)   # delay 0 is the reference's rule
    with pytest.raises(ValueError):
        mf_states(64, 1)


def _cell(O, M):
    s = O.System(M.GR, 1, 1, M.gr_reduced4(), O.draw_jitter(M.GR, 1), canon=True)
    assert s.init() == 0
    return s
