"""Arithmetic identities the CUDA kernels rely on to stay bit-exact with the
single-precision restatement, checked on the CPU."""
import ctypes as C

import numpy as np

from oracle import oracle as O


def test_division_by_six_as_fused_multiply_add():
    lib = O.load()
    lib.ko_check_div6.restype = C.c_long
    # every float of two binades: the identity then holds for all finite |x| > 2^-98
    assert lib.ko_check_div6() == 0


def test_power_of_two_division_is_multiplication():
    rng = np.random.Generator(np.random.Philox(key=5))
    x = rng.uniform(-4, 4, 200_000).astype(np.float32)
    for d in (0.125, 0.0625, 0.03125, 1.0, 2.0):
        d32 = np.float32(d)
        assert np.array_equal((x / d32).view(np.uint32), (x * np.float32(1.0 / d)).view(np.uint32))


def test_portable_sincos_accuracy():
    xs = np.linspace(-60, 60, 40001).astype(np.float32)
    err_s = max(abs(O.sincos(float(v))[0] - np.sin(np.float64(v))) for v in xs[::4])
    err_c = max(abs(O.sincos(float(v))[1] - np.cos(np.float64(v))) for v in xs[::4])
    # about one ulp of values in [-1, 1]
    assert err_s < 2.4e-7 and err_c < 2.4e-7


def test_sincos_quadrant_from_integer_bits():
    """The kernels take the sine/cosine quadrant as (int)n & 3 (0 when
    |n| >= 2^31, NaN or infinite); the oracle as n - 4 floor(n / 4) clamped
    to [0, 3].  The two agree for every n = rint(x * 2/pi) (checked here over
    random reductions, every integer near the float-spacing changes, and the
    special values), so both sides pick the same polynomial and signs."""
    rng = np.random.default_rng(7)
    x = np.concatenate([rng.uniform(-1e4, 1e4, 200_000), rng.uniform(-3e9, 3e9, 50_000),
                        rng.standard_normal(50_000) * 1e12]).astype(np.float32)
    n = np.rint(x * np.float32(float.fromhex('0x1.45f306p-1'))).astype(np.float32)
    edges = []
    for e in (24, 25, 30, 31, 32):
        for sgn in (1.0, -1.0):
            for direction in (np.inf, -np.inf):
                v = np.float32(sgn * 2.0 ** e)
                for _ in range(9):
                    edges.append(v)
                    v = np.nextafter(v, np.float32(direction))
    n = np.concatenate([n, np.float32(edges), np.arange(-100, 101, dtype=np.float32),
                        np.float32([np.nan, np.inf, -np.inf, 0.0, -0.0])])
    with np.errstate(invalid="ignore"):
        qf = (n - np.float32(4.0) * np.floor(n * np.float32(0.25))).astype(np.float32)
        q_float = np.where((qf >= 0) & (qf <= 3), np.nan_to_num(qf).astype(np.int64), 0)
        small = np.abs(n) < np.float32(2.0 ** 31)
        q_int = np.where(small, np.where(small, n, 0).astype(np.int64) & 3, 0)
    assert np.array_equal(q_float, q_int)
