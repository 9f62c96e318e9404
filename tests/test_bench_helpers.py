"""The benchmark's host-side measurement helpers on the CPU: threshold
crossings timed by interpolation at the device raster's rule, the spike
comparison, and the grouping of systems into one run of ids per cell type."""
import numpy as np
import pytest

import bench


def test_spike_times_rule_and_interpolation():
    # two cells, 4 intervals; cell 0 crosses 10 mV between intervals 1 and 2
    tr = np.array([[-60.0, 20.0], [0.0, 30.0], [20.0, -70.0], [-50.0, 15.0]])
    sp = bench.spike_times(tr, ty=0)
    # cell 0: from 0 mV at t = 0.25 to 20 mV at t = 0.375, crossing 10 mV half way
    assert sp[0] == [pytest.approx(0.3125)]
    # cell 1: the first value is above threshold but the previous one is the
    # 100 mV sentinel (no crossing); it crosses again at interval 4 (from -70)
    assert sp[1] == [pytest.approx(0.375 + 0.125 * 80.0 / 85.0)]


def test_spike_times_purkinje_threshold():
    tr = np.array([[-60.0], [-5.0]])
    assert bench.spike_times(tr, ty=2)[0] == [pytest.approx(0.125 + 0.125 * 50.0 / 55.0)]
    assert bench.spike_times(tr, ty=0)[0] == []


def test_compare_spikes():
    a = [[1.0, 2.0], [3.0], []]
    b = [[1.01, 2.2], [3.0, 4.0], []]
    r = bench.compare_spikes(a, b)
    assert r["spikes"] == [3, 4]
    assert r["cells_spiking"] == 2 and r["cells_with_equal_counts"] == 2
    assert r["max_spike_time_err_ms"] == pytest.approx(0.2)
    assert r["spikes_within_0.05ms"] == (1, 2)


def test_type_runs_needs_consecutive_ids():
    class S:
        def __init__(self, t):
            self.cell_type = t
    specs = [S(0), S(0), S(1), S(2)]
    runs = bench.type_runs(specs, [0, 1, 2, 3])
    assert runs[0][:2] == (0, 2) and runs[1][:2] == (2, 1) and runs[2][:2] == (3, 1)
    with pytest.raises(RuntimeError):
        bench.type_runs([S(0), S(1), S(0)], [0, 1, 2])
