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
