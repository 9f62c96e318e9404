"""Known-answer test of the RKC stage coefficients the kernels use
(gbrkc_rkc_coefficients: the host table built by solve_rkc.cu:816-906's
recurrences) against the published formulas of Sommeijer, Shampine & Verwer
(1998), evaluated independently in 50-digit arithmetic through the closed
forms of the Chebyshev polynomials at w0 > 1:

  theta = acosh(w0),  T_j = cosh(j theta),  T_j' = j sinh(j theta) / sinh(theta),
  T_j'' = j (j cosh(j theta) sinh(theta) - sinh(j theta) cosh(theta)) / sinh(theta)^3,

with w0 = 1 + (2/13) / s^2, w1 = T_s'/T_s'', b_j = T_j''/T_j'^2 (b_0 = b_1 = b_2),
mu~_1 = b_1 w1, mu_j = 2 b_j w0 / b_{j-1}, nu_j = -b_j / b_{j-2},
mu~_j = 2 b_j w1 / b_{j-1}, a_j = 1 - b_j T_j.  Needs no GPU."""
import ctypes as C
import os

import numpy as np
import pytest

mp = pytest.importorskip("mpmath")

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB = os.path.join(ROOT, "cerebellum-neuron-model-simulation-using-rkc_gb300", "libgbrkc.so")


@pytest.fixture(scope="module")
def table():
    if not os.path.exists(LIB):
        import build as B
        B.build()
    L = C.CDLL(LIB)
    L.gbrkc_rkc_coefficients.restype = C.c_long
    L.gbrkc_rkc_coefficients.argtypes = [C.c_int, C.POINTER(C.c_double), C.c_long]

    def get(m):
        out = np.zeros(1 + 5 * (m - 1))
        n = L.gbrkc_rkc_coefficients(m, out.ctypes.data_as(C.POINTER(C.c_double)), out.size)
        assert n == out.size
        return out
    return L, get


def published(s):
    mp.mp.dps = 50
    w0 = 1 + mp.mpf(2) / 13 / s ** 2
    th = mp.acosh(w0)
    sh, ch = mp.sinh(th), mp.cosh(th)

    def T(j):
        return mp.cosh(j * th)

    def dT(j):
        return j * mp.sinh(j * th) / sh

    def d2T(j):
        return j * (j * mp.cosh(j * th) * sh - mp.sinh(j * th) * ch) / sh ** 3

    w1 = dT(s) / d2T(s)
    b = {j: d2T(j) / dT(j) ** 2 for j in range(2, s + 1)}
    b[0] = b[1] = b.get(2, 1 / (4 * w0 ** 2))
    out = [b[1] * w1]
    for j in range(2, s + 1):
        mu = 2 * b[j] * w0 / b[j - 1]
        nu = -b[j] / b[j - 2]
        a_prev = 1 - b[j - 1] * T(j - 1)
        out += [mu, nu, 1 - mu - nu, 2 * b[j] * w1 / b[j - 1], a_prev]
    return np.array([float(x) for x in out])


# m >= 2: rkclow takes m = 1 + int(sqrt(1.54 h rho + 1)) stages, and w1 = T_1'/T_1'' has no value at s = 1
@pytest.mark.parametrize("m", [2, 3, 4, 7, 16, 100, 400, 1024])
def test_against_published_formulas(table, m):
    _, get = table
    got, want = get(m), published(m)
    assert got.shape == want.shape
    np.testing.assert_allclose(got, want, rtol=1e-9, atol=1e-14)


def test_arguments(table):
    L, _ = table
    buf = np.zeros(4)
    p = buf.ctypes.data_as(C.POINTER(C.c_double))
    assert L.gbrkc_rkc_coefficients(0, p, 4) == -1
    assert L.gbrkc_rkc_coefficients(1025, p, 4) == -1
    assert L.gbrkc_rkc_coefficients(3, p, 4) == -1          # needs 11 values
