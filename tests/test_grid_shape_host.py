"""The grid team's launch-shape rule (gbrkc_grid_shape, host only): CTAs of a
power-of-two thread count, every thread owning elements; the smallest
busiest-CTA load, then the fewest CTAs, within 256 chunks and 8 elements a
thread.  Checked against a restatement of the rule and on the workloads'
sizes."""
import pytest

import gbrkc as G


def rule(nc, cap):
    best = None
    for bw in (32, 64, 128, 256):
        chunks = -(-nc // bw)
        if chunks > 256:
            continue
        ctas = min(cap, chunks)
        rows = -(-chunks // ctas)
        if rows > 8:
            continue
        key = (rows * bw, ctas)
        if best is None or key < best[0]:
            best = (key, bw, ctas)
    return None if best is None else (best[1], best[2])


def test_workload_sizes():
    assert G.grid_shape(14400, 152) == (128, 113)     # the Purkinje 3x3 system: one element a thread
    assert G.grid_shape(57600, 152) == (256, 152)     # 6x6 Purkinje cells: two elements a thread
    assert G.grid_shape(1600, 152) == (32, 50)
    assert G.grid_shape(4096 * 16, 152) == (256, 152)


@pytest.mark.parametrize("cap", [1, 7, 113, 152])
def test_matches_the_rule(cap):
    for nc in list(range(1, 600, 7)) + [4095, 4096, 4097, 14400, 32768, 65535, 65536]:
        want = rule(nc, cap)
        if want is None:
            with pytest.raises(G.GbrkcError):
                G.grid_shape(nc, cap)
            continue
        bw, n = G.grid_shape(nc, cap)
        assert (bw, n) == want, (nc, cap)
        assert n * bw * 8 >= nc and n <= cap


def test_too_large_or_invalid():
    with pytest.raises(G.GbrkcError):
        G.grid_shape(256 * 256 + 1, 152)              # more than 256 chunks of 256
    with pytest.raises(G.GbrkcError):
        G.grid_shape(0, 152)
    with pytest.raises(G.GbrkcError):
        G.grid_shape(100, 0)
