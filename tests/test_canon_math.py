"""The canonical exp / log / pow (oracle/canon_math.h, and its device copy
csrc/canon_math.cuh) against correctly rounded values.

The canonical functions exist so that the GPU path and the oracle agree bit
for bit (the platform libm differs between glibc and CUDA); they must still
be accurate.  Reference values come from exact rational arithmetic
(fractions + a high-precision series), so the error is measured in ulps of
the true result.  The device copy is checked against this one bit for bit by
the GPU parity tests, whose trajectories call exp / log / pow millions of
times."""
import math
from decimal import Decimal, getcontext

import numpy as np
import pytest

getcontext().prec = 60


def ulp_err(got, exact):
    exact_f = float(exact)
    if exact_f == 0.0:
        return abs(got)
    return abs(Decimal(got) - exact) / Decimal(math.ulp(exact_f))


def exact_exp(x):
    return Decimal(x).exp()


def exact_log(x):
    return Decimal(x).ln()


@pytest.fixture(scope="module")
def O(oracle):
    return oracle


def test_exp_accuracy(O):
    rng = np.random.default_rng(1)
    xs = np.concatenate([rng.uniform(-700, 700, 300), rng.uniform(-1, 1, 300), rng.uniform(-0.35, 0.35, 200),
                         [0.0, 1e-300, -1e-300, 0.5, -0.5, 1.0, -1.0, 709.7, -708.0]])
    worst = max(ulp_err(O.cm_exp(float(x)), exact_exp(float(x))) for x in xs)
    assert worst <= 2, f"exp: {worst} ulp"


def test_log_accuracy(O):
    rng = np.random.default_rng(2)
    xs = np.concatenate([np.exp(rng.uniform(-700, 700, 300)), rng.uniform(0.5, 2.0, 300),
                         [1.0, 2.0, 0.5, 1e-300, 1e300, math.sqrt(2.0), 1.0 + 1e-12]])
    worst = 0
    for x in xs:
        x = float(x)
        ex = exact_log(x)
        got = O.cm_log(x)
        if float(ex) == 0.0:
            assert got == 0.0
            continue
        worst = max(worst, ulp_err(got, ex))
    assert worst <= 2, f"log: {worst} ulp"


def test_pow_cube_root_as_the_controller_uses_it(O):
    # err^(1/3) over the error norms the step controller sees
    rng = np.random.default_rng(3)
    xs = np.concatenate([np.exp(rng.uniform(-40, 10, 500)), [1.0, 8.0, 0.125, 1e-12, 1e6]])
    third = 1.0 / 3.0
    worst = 0
    for x in xs:
        x = float(x)
        ex = (Decimal(x).ln() * Decimal(third)).exp()
        worst = max(worst, ulp_err(O.cm_pow(x, third), ex))
    assert worst <= 8, f"pow(x, 1/3): {worst} ulp"


def test_special_values(O):
    assert O.cm_exp(800.0) == math.inf
    assert O.cm_exp(-800.0) == 0.0
    assert math.isnan(O.cm_exp(math.nan))
    assert O.cm_log(0.0) == -math.inf
    assert math.isnan(O.cm_log(-1.0))
    assert O.cm_log(math.inf) == math.inf
    assert O.cm_exp(0.0) == 1.0
    assert O.cm_log(1.0) == 0.0


def test_cbrt_accuracy(O):
    """The controller's err^(1/3): within 4 ulp of the exact cube root over
    the error norms the controller sees, and exact at 0, inf and NaN."""
    rng = np.random.default_rng(3)
    xs = list(10.0 ** rng.uniform(-12, 6, 3000)) + [1.0, 8.0, 0.125, 2.0, 3.0, 1e-300, 1e-310, 5e-324, 1e300]
    worst = 0.0
    for x in xs:
        got = O.lib().orc_cm_cbrt(float(x))
        exact = Decimal(float(x)) ** (Decimal(1) / Decimal(3))
        worst = max(worst, float(ulp_err(got, exact)))
    assert worst <= 4.0, worst
    assert O.lib().orc_cm_cbrt(0.0) == 0.0
    assert O.lib().orc_cm_cbrt(math.inf) == math.inf
    assert math.isnan(O.lib().orc_cm_cbrt(math.nan))
