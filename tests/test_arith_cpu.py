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


def test_sincos_rounding_by_magic_addition():
    """Both sides take n = rint(x * 2/pi) as (x * 2/pi + 1.5 * 2^23) - 1.5 * 2^23
    and the quadrant as the sum's two lowest bits.  While |x * 2/pi| < 2^22
    (every angle the planners meet) that is rintf's round-to-nearest-even and
    n mod 4 exactly: checked over random and hand-picked reductions, the ties
    and the ends of the range."""
    rng = np.random.default_rng(7)
    f32 = np.float32
    two_over_pi = f32(float.fromhex('0x1.45f306p-1'))
    magic = f32(1.5 * 2.0 ** 23)
    x = np.concatenate([rng.uniform(-1e4, 1e4, 200_000), rng.uniform(-6.5e6, 6.5e6, 100_000),
                        np.arange(-200, 201) * (np.pi / 4)]).astype(f32)
    y = (x * two_over_pi).astype(f32)
    # ties and the range ends, as products
    ties = np.concatenate([np.arange(-64, 64) + f32(0.5), np.float32([2.0 ** 22 - 1, -(2.0 ** 22 - 1), 2.0 ** 22 - 0.5, -(2.0 ** 22 - 0.5)])])
    y = np.concatenate([y, ties.astype(f32)])
    y = y[np.abs(y) < f32(2.0 ** 22)]
    t = (y + magic).astype(f32)
    n = (t - magic).astype(f32)
    assert np.array_equal(n, np.rint(y).astype(f32))
    q = t.view(np.uint32) & 3
    assert np.array_equal(q.astype(np.int64), np.rint(y).astype(np.int64) & 3)


def test_sincos_coefficients_come_from_the_fit():
    """The minimax coefficients in the oracle (and, operation for operation,
    in the kernels) are the float roundings of the Lawson fit in
    oracle/fit_sincos.py, and that fit stays under 4e-9 / 2e-10 relative
    error before rounding."""
    import re
    from pathlib import Path
    import importlib.util
    root = Path(__file__).resolve().parents[1]
    spec = importlib.util.spec_from_file_location("fit_sincos", root / "oracle" / "fit_sincos.py")
    fit = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(fit)
    half = np.pi / 8
    x = np.cos(np.linspace(0.0, np.pi, 20001)) * half + half
    x = x[x > 1e-6]
    basis = np.stack([np.ones_like(x), x ** 2, x ** 4], 1)
    cs, es = fit.lawson(basis, (np.sin(x) - x) / x ** 3, x ** 3 / np.sin(x))
    cc, ec = fit.lawson(basis, (np.cos(x) - 1.0 + x ** 2 / 2.0) / x ** 4, x ** 4 / np.cos(x))
    assert es < 4e-9 and ec < 2e-10
    src = (root / "oracle" / "kgmt_oracle.c").read_text()
    def const(name):
        m = re.search(r"#define %s \(?(-?0x[0-9a-fp.+-]+)f\)?" % name, src)
        return np.float32(float.fromhex(m.group(1)))
    assert [const(n) for n in ("KO_S1", "KO_S2", "KO_S3")] == [np.float32(v) for v in cs]
    assert [const(n) for n in ("KO_C2", "KO_C3", "KO_C4")] == [np.float32(v) for v in cc]
    assert const("KO_C1") == np.float32(-0.5)
    # the kernels' portable sine/cosine uses the same literals
    dev = (root / "kgmt_gb300" / "csrc" / "kgmt_device.cuh").read_text()
    body = dev[dev.index("void sincos_portable("):]
    body = body[:body.index("\n}\n")]
    lits = {np.float32(float.fromhex(m)) for m in re.findall(r"(-?0x[0-9a-f]\.[0-9a-f]+p[+-]?[0-9]+)f", body)}
    for name in ("KO_S1", "KO_S2", "KO_S3", "KO_C1", "KO_C2", "KO_C3", "KO_C4"):
        assert const(name) in lits, name
