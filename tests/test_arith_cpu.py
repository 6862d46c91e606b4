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
