"""The request server's host-side checks on the CPU: arguments rejected before
any device call, calls out of order, and a start that fails (here: no CUDA
device) leaving the server as it was, so that it can be retried."""
import re

import numpy as np
import pytest

import gbrkc as G
import morph as M

EINVAL, ECUDA, ESTATE, ENOMEM = -1, -2, -3, -4


def expect(code, fn, *a, **k):
    with pytest.raises(G.GbrkcError) as ei:
        fn(*a, **k)
    got = int(re.search(r"error (-?\d+)", str(ei.value)).group(1))
    assert got == code, str(ei.value)


def test_server_rejects_bad_arguments_and_order():
    expect(EINVAL, G.Server, 7)                        # no such precision
    expect(EINVAL, G.Server, G.MIXED, -1)              # negative HBM budget
    expect(EINVAL, G.Server, G.MIXED, 0, 0)            # empty quantum
    srv = G.Server(G.MIXED, hbm_budget=1 << 30)
    rows = M.gr_reduced4()
    expect(EINVAL, srv.add_class, 9, 1, 1, rows, slots=4)
    expect(EINVAL, srv.add_class, M.GR, 0, 1, rows, slots=4)
    expect(EINVAL, srv.add_class, M.GR, 1, 1, rows)             # neither slots nor a share
    expect(EINVAL, srv.add_class, M.GR, 1, 1, rows, slots=-1)
    cid = srv.add_class(M.GR, 1, 1, rows, slots=4)
    expect(ESTATE, srv.submit, cid, 1, 8, np.zeros(1))          # not started
    expect(ESTATE, srv.advance)
    srv.close()
    srv = G.Server(G.MIXED, hbm_budget=1 << 10)                 # 1 KB holds no granule slot
    srv.add_class(M.GR, 1, 1, rows, slots=64)
    expect(ENOMEM, srv.start)
    srv.close()


def test_failed_start_leaves_the_server_restartable():
    srv = G.Server(G.MIXED, hbm_budget=1 << 30)
    rows = M.gr_reduced4()
    srv.add_class(M.GR, 1, 1, rows, slots=4)
    try:
        srv.start()
    except G.GbrkcError as e:
        assert "error -2" in str(e), str(e)          # no CUDA device on this host
    else:
        srv.close()
        pytest.skip("a CUDA device is present: start succeeded")
    # not started: classes can still be added, and start fails the same way again
    srv.add_class(M.GR, 1, 1, rows, slots=2)
    expect(ECUDA, srv.start)
    assert G.lib().gbrkc_server_engine(srv.h) is None
    srv.close()
