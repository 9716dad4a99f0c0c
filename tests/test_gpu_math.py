"""The device functions that stand in for most divisions and square roots in the
kernels (physics.cuh: rcp, the hardware reciprocal refined by the series
y (1 + e + e^2); rsq, the hardware reciprocal square root refined by
y (1 + e/2 + 3e^2/8); sq(x) = x rsq(x)) against correctly rounded results,
through fvgb_math_eval: within one ulp (rcp, rsq) and two ulp (sq) over the
normal range, exact where the result is a power of two, and the library
function's result for zero, subnormal, negative, infinite and NaN arguments.
That bound is what lets them replace the reference's divisions and square roots
inside the 1e-12 parity tolerance."""
import ctypes
from decimal import Decimal, getcontext

import numpy as np
import pytest

import cfd_solver_2d_gpu_gb300 as fv

pytestmark = pytest.mark.gpu


def evaluate(op, x):
    L = fv.lib()
    L.fvgb_math_eval.restype = ctypes.c_int
    L.fvgb_math_eval.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
    x = np.ascontiguousarray(x, dtype=np.float64)
    out = np.full(len(x), np.nan)
    assert L.fvgb_math_eval(0, op, len(x), x.ctypes.data, out.ctypes.data) == 0, L.fvgb_last_error().decode()
    return out


def _samples(seed, positive=False):
    rng = np.random.default_rng(seed)
    x = np.concatenate([
        10.0 ** rng.uniform(-250, 250, 20000),           # the normal range the kernels can meet
        10.0 ** rng.uniform(-10, np.log10(4e7), 20000),  # densities, pressures, volumes
        1.0 + rng.uniform(-1e-6, 1e-6, 2000),            # near one
        np.nextafter(np.ldexp(1.0, np.arange(-60, 61)), 0.0),
        np.nextafter(np.ldexp(1.0, np.arange(-60, 61)), np.inf),
    ])
    return x if positive else np.concatenate([x, -x[:1000]])


def _ulps(got, exact):
    return np.abs(got - exact) / np.spacing(np.abs(exact))


def test_reciprocal_within_an_ulp():
    x = _samples(20261203)
    got = evaluate(0, x)
    getcontext().prec = 50
    exact = np.array([float(1 / Decimal(v)) for v in x])
    assert _ulps(got, exact).max() <= 1.0
    p2 = np.ldexp(1.0, np.arange(-200, 201))
    assert np.array_equal(evaluate(0, p2), 1.0 / p2)


def test_reciprocal_square_root_and_square_root():
    x = _samples(7, positive=True)
    getcontext().prec = 50
    roots = [Decimal(v).sqrt() for v in x]
    r_exact = np.array([float(1 / r) for r in roots])
    s_exact = np.array([float(r) for r in roots])
    assert _ulps(evaluate(1, x), r_exact).max() <= 1.0
    assert _ulps(evaluate(2, x), s_exact).max() <= 2.0
    p4 = np.ldexp(1.0, 2 * np.arange(-200, 201))  # even powers of two: exact roots
    assert np.array_equal(evaluate(1, p4), 1.0 / np.sqrt(p4))
    assert np.array_equal(evaluate(2, p4), np.sqrt(p4))
    special = np.array([0.0, -0.0, 5e-324, 2e-310, -1.0, np.inf, -np.inf, np.nan])
    with np.errstate(all="ignore"):
        want_s = np.sqrt(special)
        want_r = 1.0 / np.sqrt(special)
    for got, want in ((evaluate(2, special), want_s), (evaluate(1, special), want_r)):
        same = (got == want) | (np.isnan(got) & np.isnan(want))
        with np.errstate(invalid="ignore"):
            close = np.isfinite(want) & (np.abs(got - want) <= 2 * np.spacing(np.abs(want)))
        assert np.all(same | close), (got, want)
