"""The kernels' square root and division (sqrt_rn and div_tk in
csrc/common.cuh) against CUDA's IEEE sqrt and division, bit for bit, through
the C ABI (fteik_sqrt_rn, fteik_div_rn).

Every traveltime operator of the reference takes a correctly rounded square
root (`x ** 0.5`) and divides by a constant (fteikpy/_fteik/_fteik3d.py:
113-117,155-158).  The kernels compute the root with a float seed, a
fixed-point Newton step, one coupled FP64 Newton step and Tuckerman's
rounding test, and the quotient with a product by the rounded reciprocal and
the same test.  The inputs cover the whole range, exact results and their
neighbours, values whose exact result lies just beside a rounding midpoint
(the hardest cases for the rounding test), and the special values that take
the fallback.
"""

import numpy as np
import pytest
import torch

from fteikpy_gb300 import _device, _lib

pytestmark = pytest.mark.gpu


def _check(x):
    lib = _lib.load()
    xd = torch.as_tensor(np.ascontiguousarray(x, dtype=np.float64)).to(_device.device())
    out = torch.empty_like(xd)
    assert lib.fteik_sqrt_rn(_device.ptr(xd), xd.numel(), _device.ptr(out), _device.stream()) == _lib.OK
    ref = torch.sqrt(xd)
    a = out.view(torch.int64)
    b = ref.view(torch.int64)
    bad = (a != b) & ~(torch.isnan(out) & torch.isnan(ref))
    nbad = int(bad.sum())
    if nbad:
        i = int(torch.nonzero(bad)[0])
        raise AssertionError(f"{nbad} mismatches, e.g. sqrt_rn({float(xd[i])!r}) = "
                             f"{float(out[i])!r}, IEEE {float(ref[i])!r}")


def _check_div(x, c):
    lib = _lib.load()
    xd = torch.as_tensor(np.ascontiguousarray(x, dtype=np.float64)).to(_device.device())
    out = torch.empty_like(xd)
    assert lib.fteik_div_rn(_device.ptr(xd), xd.numel(), float(c), _device.ptr(out),
                            _device.stream()) == _lib.OK
    # IEEE division by a tensor divisor (a tensor divided by a Python scalar is
    # computed as a product with the scalar's reciprocal)
    ref = xd / torch.full_like(xd, c)
    sample = np.random.default_rng(len(x)).integers(0, len(x), size=min(len(x), 1 << 16))
    host = np.asarray(x, dtype=np.float64)[sample] / c
    assert np.array_equal(ref.cpu().numpy()[sample].view(np.int64), host.view(np.int64)) or \
        np.isnan(host).any()
    bad = (out.view(torch.int64) != ref.view(torch.int64)) & ~(torch.isnan(out) & torch.isnan(ref))
    nbad = int(bad.sum())
    if nbad:
        i = int(torch.nonzero(bad)[0])
        raise AssertionError(f"{nbad} mismatches, e.g. div({float(xd[i])!r}, {c!r}) = "
                             f"{float(out[i])!r}, IEEE {float(ref[i])!r}")


def _ulp_neighbours(v, k):
    """v's bit patterns shifted by -k..k (positive doubles)."""
    b = v.view(np.int64)
    return np.concatenate([(b + d).view(np.float64) for d in range(-k, k + 1)])


def test_sqrt_rn_random_bit_patterns():
    rng = np.random.default_rng(0)
    for _ in range(4):
        # every positive finite double is equally likely per bit pattern
        bits = rng.integers(1, 0x7FF0000000000000, size=1 << 24, dtype=np.int64)
        _check(bits.view(np.float64))
    # the ranges the solvers use: radicands of traveltime operators
    _check(10.0 ** rng.uniform(-12.0, 2.0, size=1 << 24))


def test_sqrt_rn_squares_and_neighbours():
    rng = np.random.default_rng(1)
    y = np.ldexp(1.0 + rng.random(1 << 21), rng.integers(-500, 500, size=1 << 21))
    _check(_ulp_neighbours(y * y, 3))
    # exact squares of short significands (their roots are representable)
    m = rng.integers(1, 1 << 26, size=1 << 21).astype(np.float64)
    _check(_ulp_neighbours(np.ldexp(m * m, 2 * rng.integers(-200, 200, size=1 << 21)), 2))


def test_sqrt_rn_near_midpoints():
    # g + ulp/2 is a rounding midpoint; the doubles next to its square have
    # roots within about 2^-106 relative of it
    rng = np.random.default_rng(2)
    g = 1.0 + rng.integers(0, 1 << 52, size=1 << 21, dtype=np.int64) * 2.0**-52
    # (g + ulp/2)^2 = g^2 + g ulp + ulp^2/4, ulp = 2^-52
    x = np.concatenate([g * g, g * g + g * 2.0**-52])
    x = np.concatenate([x, 4.0 * x])  # both halves of the exponent parity
    _check(_ulp_neighbours(x, 4))


def test_sqrt_rn_special_values():
    tiny = np.nextafter(0.0, 1.0)
    x = np.array([0.0, -0.0, tiny, 2.2250738585072014e-308, np.nextafter(2.2250738585072014e-308, 0.0),
                  1.0, np.nextafter(1.0, 2.0), np.nextafter(1.0, 0.0), 4.0, np.nextafter(4.0, 0.0),
                  2.0, 0.25, np.finfo(np.float64).max, np.inf, -1.0, np.nan, 1e-300, 1e300])
    _check(np.concatenate([x, np.ldexp(1.0, np.arange(-1074, 1024))]))


# the constants the kernels divide by: sums of inverse squared spacings,
# spacings, diagonals, cell volumes; and arbitrary ones
DIVISORS = [0.02, 0.03, 0.01, 10.0, 7.0, 14.142135623730951, 1000.0, 1.0 / 3.0, 3.0,
            0.0002, 123.456, 2.0**-30 * 1.75, 5.0e7]


def test_div_rn_random():
    rng = np.random.default_rng(3)
    for c in DIVISORS + list(10.0 ** rng.uniform(-6.0, 6.0, size=3)):
        x = rng.standard_normal(1 << 21) * 10.0 ** rng.uniform(-8.0, 8.0, size=1 << 21)
        _check_div(x, c)
    bits = rng.integers(1, 0x7FF0000000000000, size=1 << 23, dtype=np.int64)
    x = bits.view(np.float64) * np.where(rng.random(1 << 23) < 0.5, -1.0, 1.0)
    for c in (0.02, 7.0, 1.0 / 3.0):
        _check_div(x, c)


def test_div_rn_exact_and_near_midpoint_quotients():
    rng = np.random.default_rng(4)
    q = 1.0 + rng.integers(0, 1 << 52, size=1 << 20, dtype=np.int64) * 2.0**-52
    q = np.ldexp(q, rng.integers(-30, 30, size=1 << 20))
    for c in DIVISORS:
        # x = c q (quotient next to a double) and x = c (q + ulp/2) (quotient
        # next to a midpoint), each with its neighbours
        ulp = np.ldexp(1.0, np.frexp(q)[1] - 53)
        x = np.concatenate([c * q, c * (q + 0.5 * ulp), -(c * q)])
        _check_div(_ulp_neighbours(np.abs(x), 3) * np.sign(np.tile(x, 7)), c)


def test_div_rn_special_values():
    tiny = np.nextafter(0.0, 1.0)
    x = np.array([0.0, -0.0, tiny, -tiny, 2.2250738585072014e-308, 1.0, -1.0,
                  np.finfo(np.float64).max, -np.finfo(np.float64).max, np.inf, -np.inf, np.nan,
                  1e-300, 1e300, 4.0, 0.5])
    x = np.concatenate([x, np.ldexp(1.0, np.arange(-1074, 1024)), -np.ldexp(1.0, np.arange(-1074, 1024))])
    for c in DIVISORS:
        _check_div(x, c)


def _check_recip(x):
    lib = _lib.load()
    xd = torch.as_tensor(np.ascontiguousarray(x, dtype=np.float64)).to(_device.device())
    out = torch.empty_like(xd)
    assert lib.fteik_recip_rn(_device.ptr(xd), xd.numel(), _device.ptr(out), _device.stream()) == _lib.OK
    ref = torch.ones_like(xd) / xd  # IEEE division (tensor by tensor)
    bad = (out.view(torch.int64) != ref.view(torch.int64)) & ~(torch.isnan(out) & torch.isnan(ref))
    nbad = int(bad.sum())
    if nbad:
        i = int(torch.nonzero(bad)[0])
        raise AssertionError(f"{nbad} mismatches, e.g. 1/{float(xd[i])!r} = {float(out[i])!r}, "
                             f"IEEE {float(ref[i])!r}")


def test_recip_rn():
    """The gradient post-pass's reciprocal (recip_rn): random bit patterns
    over the whole range, gradient-norm-like values, the neighbours of
    reciprocals of short significands (results next to a double or a
    midpoint), and the special values."""
    rng = np.random.default_rng(5)
    bits = rng.integers(1, 0x7FF0000000000000, size=1 << 24, dtype=np.int64)
    _check_recip(bits.view(np.float64))
    _check_recip(10.0 ** rng.uniform(-6.0, 1.0, size=1 << 22))
    m = rng.integers(1, 1 << 26, size=1 << 20).astype(np.float64)
    q = np.ldexp(1.0 + rng.integers(0, 1 << 52, size=1 << 20, dtype=np.int64) * 2.0**-52, 0)
    x = np.concatenate([m, 1.0 / q, 1.0 / (q + 2.0**-53), np.ldexp(m, rng.integers(-300, 300, 1 << 20))])
    _check_recip(_ulp_neighbours(x, 3))
    tiny = np.nextafter(0.0, 1.0)
    s = np.array([0.0, -0.0, tiny, 2.2250738585072014e-308, 1.0, 2.0, 0.5, -1.0, -3.0,
                  np.finfo(np.float64).max, np.inf, -np.inf, np.nan, 1e-300, 1e300])
    _check_recip(np.concatenate([s, np.ldexp(1.0, np.arange(-1074, 1024)),
                                 np.ldexp(1.5, np.arange(-1074, 1023))]))
