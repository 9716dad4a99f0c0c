"""The correctly rounded FP64 multiply and add that run on the integer pipes
(csrc/softfp64.cuh).  They must give the IEEE 754 round-to-nearest-even result
bit for bit, since the kernels use them in place of the hardware instruction
without changing any result: on the CPU, the host build of the same code against
numpy (the host's IEEE arithmetic); on the GPU, the device build against the
hardware instruction on the same pairs, and the throughput of both side by side."""
import ctypes

import numpy as np
import pytest

import cfd_solver_2d_gpu_gb300 as fv


def _pairs(seed, n):
    """Random normal operands over the full exponent range and over the range the kernels
    meet, operands whose products and sums round at or next to ties, sums that cancel,
    and every pair of special values."""
    rng = np.random.default_rng(seed)
    u = rng.integers(0, 2**63, (6, n), dtype=np.uint64)
    frac = u & np.uint64(0x000FFFFFFFFFFFFF)
    sign = (u >> np.uint64(62)) << np.uint64(63)
    full = lambda i: (frac[i] | (rng.integers(1, 2047, n, dtype=np.uint64) << np.uint64(52)) | sign[i]).view(np.float64)
    near = lambda i: (frac[i] | (rng.integers(1023 - 60, 1023 + 60, n, dtype=np.uint64) << np.uint64(52)) |
                      sign[i]).view(np.float64)
    short = (np.uint64(1023) << np.uint64(52)) | (rng.integers(0, 64, n, dtype=np.uint64) << rng.integers(
        0, 46, n, dtype=np.uint64).astype(np.uint64))
    short = short.view(np.float64) * np.ldexp(1.0, rng.integers(-5, 5, n))
    a = np.concatenate([full(0), near(1), short, near(2)])
    b = np.concatenate([full(3), near(4), short[::-1], -near(2) * (1 + np.ldexp(1.0, -rng.integers(1, 53, n)))])
    sp = np.array([0.0, -0.0, 1.0, -1.0, np.inf, -np.inf, np.nan, 5e-324, -5e-324, 2.2250738585072014e-308,
                   1.7976931348623157e308, 1e-300, 1e300, 0.5, 3.0, 1.0000000000000002, 0.9999999999999999])
    sa, sb = np.meshgrid(sp, sp)
    return np.concatenate([a, sa.ravel()]), np.concatenate([b, sb.ravel()])


def _same(x, y):
    xb, yb = x.view(np.uint64), y.view(np.uint64)
    return bool(np.all((xb == yb) | (np.isnan(x) & np.isnan(y))))


@pytest.mark.parametrize("op", [0, 1])
def test_host_build_is_ieee_exact(op):
    L = fv.lib()
    L.fvgb_softfp64_host.restype = ctypes.c_int
    L.fvgb_softfp64_host.argtypes = [ctypes.c_int, ctypes.c_int] + [ctypes.c_void_p] * 3
    a, b = _pairs(7 + op, 400000)
    out = np.empty_like(a)
    assert L.fvgb_softfp64_host(op, len(a), a.ctypes.data, b.ctypes.data, out.ctypes.data) == 0
    with np.errstate(all="ignore"):
        want = a * b if op == 0 else a + b
    assert _same(out, want)


@pytest.mark.gpu
@pytest.mark.parametrize("op", [0, 1])
def test_device_build_matches_the_hardware_instruction(op):
    L = fv.lib()
    L.fvgb_softfp64_eval.restype = ctypes.c_int
    L.fvgb_softfp64_eval.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int] + [ctypes.c_void_p] * 4
    a, b = _pairs(11 + op, 2000000)
    soft, hw = np.empty_like(a), np.empty_like(a)
    assert L.fvgb_softfp64_eval(0, op, len(a), a.ctypes.data, b.ctypes.data, soft.ctypes.data, hw.ctypes.data) == 0
    assert _same(soft, hw)
    with np.errstate(all="ignore"):
        want = a * b if op == 0 else a + b
    assert _same(hw, want)


@pytest.mark.gpu
def test_rates_are_reported():
    L = fv.lib()
    L.fvgb_softfp64_rate.restype = ctypes.c_int
    L.fvgb_softfp64_rate.argtypes = [ctypes.c_int, ctypes.c_void_p]
    out = np.zeros(10)
    assert L.fvgb_softfp64_rate(0, out.ctypes.data) == 0, L.fvgb_last_error().decode()
    sms, mhz = out[8], out[9]
    names = ["mul fp64 pipe", "mul integer pipes", "mul 4 + 4", "mul 2 + 6",
             "add fp64 pipe", "add integer pipes", "add 4 + 4", "add 6 + 2"]
    for nm, g in zip(names, out[:8]):
        print(f"{nm}: {g:.1f} Gop/s = {g * 1e9 / (sms * mhz * 1e6):.2f} per SM per cycle at {mhz:.0f} MHz")
    assert np.all(out[:8] > 0)
