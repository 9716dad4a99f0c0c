"""The device reciprocal that stands in for most divisions in the kernels
(physics.cuh: rcp, the hardware approximation refined by the series
y (1 + e + e^2)) against correctly rounded results, through fvgb_math_eval:
within one ulp over the normal range, exact on powers of two.  That bound is what
lets it replace the reference's divisions inside the 1e-12 parity tolerance."""
import ctypes
from decimal import Decimal, getcontext

import numpy as np
import pytest

import cfd_solver_2d_gpu_gb300 as fv

pytestmark = pytest.mark.gpu


def reciprocal(x):
    L = fv.lib()
    L.fvgb_math_eval.restype = ctypes.c_int
    L.fvgb_math_eval.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
    x = np.ascontiguousarray(x, dtype=np.float64)
    out = np.full(len(x), np.nan)
    assert L.fvgb_math_eval(0, len(x), x.ctypes.data, out.ctypes.data) == 0, L.fvgb_last_error().decode()
    return out


def test_reciprocal_within_an_ulp():
    rng = np.random.default_rng(20261203)
    x = np.concatenate([
        10.0 ** rng.uniform(-250, 250, 20000),           # the normal range the kernels can meet
        10.0 ** rng.uniform(-10, np.log10(4e7), 20000),  # densities, pressures, volumes
        1.0 + rng.uniform(-1e-6, 1e-6, 2000),            # near one
        np.nextafter(np.ldexp(1.0, np.arange(-60, 61)), 0.0),
    ])
    x = np.concatenate([x, -x[:1000]])
    got = reciprocal(x)
    getcontext().prec = 50
    exact = np.array([float(1 / Decimal(v)) for v in x])
    assert (np.abs(got - exact) / np.spacing(np.abs(exact))).max() <= 1.0
    p2 = np.ldexp(1.0, np.arange(-200, 201))
    assert np.array_equal(reciprocal(p2), 1.0 / p2)
