"""The fixed-point conversions of the Q1/Q2 cell-kernel contractions
(include/prismspf/gpu/fixed_point.cuh) against exact rational arithmetic, on the CPU: the
header compiles as plain C++ (tests/fixed_point_shim.cc) and every result is compared with
Python's correctly rounded Fraction -> float conversion."""
from __future__ import annotations

import ctypes as C
import math
import shutil
import subprocess
from fractions import Fraction
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]

pytestmark = pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")

ONE = 1 << 63


@pytest.fixture(scope="module")
def fx(tmp_path_factory):
    out = tmp_path_factory.mktemp("fx_shim") / "libfx_shim.so"
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-I", str(ROOT / "include"),
           str(ROOT / "tests" / "fixed_point_shim.cc"), "-o", str(out)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    lib = C.CDLL(str(out))
    lib.fxs_exponent.restype = C.c_int
    lib.fxs_exponent.argtypes = [C.c_double]
    lib.fxs_to_fixed.restype = C.c_longlong
    lib.fxs_to_fixed.argtypes = [C.c_double, C.c_int, C.c_int]
    lib.fxs_to_double.restype = C.c_double
    lib.fxs_to_double.argtypes = [C.c_longlong, C.c_int, C.c_ulonglong]
    lib.fxs_make_scale.argtypes = [C.c_double, C.POINTER(C.c_ulonglong), C.POINTER(C.c_int)]
    for f in (lib.fxs_line_derivative, lib.fxs_line_integral):
        f.restype = C.c_longlong
        f.argtypes = [C.c_int, C.c_int, C.c_longlong, C.c_longlong, C.c_longlong]
    lib.fxs_fastdiv.restype = C.c_uint
    lib.fxs_fastdiv.argtypes = [C.c_uint, C.c_uint]
    lib.fxs_to_fixed_fast.restype = C.c_longlong
    lib.fxs_to_fixed_fast.argtypes = [C.c_double, C.c_int, C.c_int]
    lib.fxs_to_fixed_scaled.restype = C.c_longlong
    lib.fxs_to_fixed_scaled.argtypes = [C.c_double, C.c_int, C.c_ulonglong, C.c_int]
    lib.fxs_to_double_fast.restype = C.c_double
    lib.fxs_to_double_fast.argtypes = [C.c_longlong, C.c_int, C.c_ulonglong, C.c_int]
    return lib


def exact_fixed(v: float, E: int, top: int) -> int:
    """round(v * 2^(1023 + top - E)), ties away from zero; 0 for subnormals."""
    if v == 0.0 or abs(v) < 2.0 ** -1022:
        return 0
    q = Fraction(v) * Fraction(2) ** (1023 + top - E)
    a = abs(q)
    n = int(a)
    if a - n >= Fraction(1, 2):
        n += 1
    return -n if v < 0 else n


def exact_double(x: int, lsb: int, sig: int = ONE) -> float:
    """x * 2^lsb * sig / 2^63, correctly rounded; flushed below the normal range."""
    if x == 0:
        return 0.0
    q = Fraction(x) * Fraction(2) ** lsb * Fraction(sig, ONE)
    if abs(q) < Fraction(2) ** -1022:
        return math.copysign(0.0, x)
    try:
        return float(q)
    except OverflowError:
        return math.copysign(math.inf, x)


def scale(fx, s):
    sig, k = C.c_ulonglong(), C.c_int()
    fx.fxs_make_scale(s, C.byref(sig), C.byref(k))
    return sig.value, k.value


def test_exponent(fx):
    assert fx.fxs_exponent(1.0) == 1023
    assert fx.fxs_exponent(-0.75) == 1022
    assert fx.fxs_exponent(0.0) == 0
    assert fx.fxs_exponent(5e-324) == 0
    assert fx.fxs_exponent(math.inf) == 2047
    assert fx.fxs_exponent(math.nan) == 2047


def test_to_fixed_exact(fx):
    rng = np.random.default_rng(1)
    for _ in range(4000):
        top = int(rng.choice([53, 58, 60]))
        v = float(rng.standard_normal() * 10.0 ** rng.integers(-30, 30))
        e = fx.fxs_exponent(v)
        E = e + int(rng.integers(0, 70))  # the block maximum is at least as large
        assert fx.fxs_to_fixed(v, E, top) == exact_fixed(v, E, top), (v, E, top)
    for v in (0.0, -0.0, 5e-324, -2.2e-308, 1.0, -1.0, 0.5, 1.5, 2.0 ** 52 + 1):
        E = max(fx.fxs_exponent(v), 1)
        assert fx.fxs_to_fixed(v, E, 58) == exact_fixed(v, E, 58)


def test_round_trip_keeps_every_bit(fx):
    rng = np.random.default_rng(2)
    for _ in range(2000):
        v = float(rng.uniform(-1, 1) * 10.0 ** rng.integers(-20, 20))
        e = fx.fxs_exponent(v)
        for drop in range(0, 7):  # block maxima up to 6 binades above v lose nothing at top 58
            E = e + drop
            x = fx.fxs_to_fixed(v, E, 58)
            assert fx.fxs_to_double(x, E - 1023 - 58, ONE) == v


def test_to_double_correctly_rounded(fx):
    rng = np.random.default_rng(3)
    for _ in range(4000):
        bits = int(rng.integers(1, 63))
        x = int(rng.integers(0, 2 ** 62)) >> (62 - bits)
        if rng.random() < 0.5:
            x = -x
        lsb = int(rng.integers(-1100, 1000))
        assert fx.fxs_to_double(x, lsb, ONE) == exact_double(x, lsb), (x, lsb)
    # ties to even, carries into the exponent, overflow, underflow
    for x, lsb in [((1 << 53) + 1, 0), ((1 << 53) + 3, 0), ((1 << 54) - 1, 0), ((1 << 62) - 1, 0),
                   (-((1 << 53) + 1), -10), (1, 1023), (3, 1023), (1, -1022), (1, -1023), (1, -1080),
                   ((1 << 62) - 1, 962), ((1 << 62) - 1, 961)]:
        assert fx.fxs_to_double(x, lsb, ONE) == exact_double(x, lsb), (x, lsb)


def test_to_double_scaled(fx):
    rng = np.random.default_rng(4)
    for _ in range(4000):
        s = float(rng.uniform(0.001, 1000.0))
        sig, k = scale(fx, s)
        assert Fraction(sig, ONE) * Fraction(2) ** k == Fraction(s)
        x = int(rng.integers(-(2 ** 62), 2 ** 62))
        lsb = int(rng.integers(-200, 200))
        got = fx.fxs_to_double(x, lsb + k, sig)
        want = exact_double(x, lsb, sig) * 2.0 ** k
        exact = Fraction(x) * Fraction(sig, ONE) * Fraction(2) ** (lsb + k)
        # rounded to nearest from floor(|x| sigma): at most half a unit in the last place plus
        # 2^(lsb + k), the fraction dropped below the block resolution
        err = abs(Fraction(got) - exact)
        assert err <= Fraction(float(np.spacing(abs(want)))) / 2 + Fraction(2) ** (lsb + k), (x, lsb, s)
        if abs(x) >= 2 ** 60:  # 61+ bits kept: within 129/256 of a unit in the last place
            assert err <= Fraction(float(np.spacing(abs(want)))) * Fraction(129, 256)


def test_contraction_matches_fp64(fx):
    """A Q2 derivative through the fixed path against the same sum in exact arithmetic and in
    FP64: the fixed result is the exact sum of the quantised values rounded once."""
    D = [[-3, 4, -1], [-1, 0, 1], [1, -4, 3]]
    rng = np.random.default_rng(5)
    for _ in range(2000):
        u = rng.uniform(-1, 1, 3) * 10.0 ** rng.integers(-8, 8)
        h = float(rng.uniform(0.01, 10.0))
        sig, k = scale(fx, 1.0 / h)
        E = max(fx.fxs_exponent(float(a)) for a in u)
        xs = [fx.fxs_to_fixed(float(a), E, 58) for a in u]
        for q in range(3):
            s = sum(D[q][j] * xs[j] for j in range(3))
            got = fx.fxs_to_double(s, E - 1023 - 58 + k, sig)
            exact = sum(Fraction(D[q][j]) * Fraction(float(u[j])) for j in range(3)) / Fraction(h)
            fp64 = sum(D[q][j] / h * float(u[j]) for j in range(3))
            ulp = 2.0 ** (E - 1023 - 52) / h  # rounding unit of the largest term
            res_ulp = float(np.spacing(abs(float(exact))))
            assert abs(got - float(exact)) <= res_ulp + ulp
            assert abs(fp64 - float(exact)) <= 2 * res_ulp + 16 * ulp


def test_fast_division(fx):
    rng = np.random.default_rng(6)
    ds = [1, 2, 3, 5, 7, 64, 65, 129, 255, 256, 257, 1000, 4097, 65535, 65537, 2 ** 30 - 1, 2 ** 30, 2 ** 30 + 1,
          2 ** 31 - 1] + [int(v) for v in rng.integers(1, 2 ** 31, 200)]
    for d in ds:
        ns = [0, 1, d - 1, d, d + 1, 2 ** 31 - 1, 2 ** 31 - 2] + [int(v) for v in rng.integers(0, 2 ** 31, 200)]
        for n in ns:
            if 0 <= n < 2 ** 31:
                assert fx.fxs_fastdiv(n, d) == n // d, (n, d)


def test_line_formulas_match_the_gauss_lobatto_matrices(fx):
    """The closed-form line contractions against D (derivatives of the Lagrange basis at the
    Gauss-Lobatto nodes of [0, 1]) and D w (weights times 2 for Q1, 6 for Q2), computed here."""
    for n, W in ((2, 2), (3, 6)):
        x = np.linspace(0.0, 1.0, n)
        w = np.array([0.5, 0.5]) if n == 2 else np.array([1, 4, 1]) / 6.0
        D = np.zeros((n, n))
        for j in range(n):
            c = np.poly1d([1.0])
            for m in range(n):
                if m != j:
                    c *= np.poly1d([1.0, -x[m]]) / (x[j] - x[m])
            D[:, j] = c.deriv()(x)
        Di = np.rint(D).astype(np.int64)
        assert np.allclose(D, Di)
        Wi = np.rint(w * W).astype(np.int64)
        rng = np.random.default_rng(7)
        for _ in range(300):
            u = [int(v) for v in rng.integers(-(2 ** 58), 2 ** 58, 3)]
            for q in range(n):
                want = sum(int(Di[q][j]) * u[j] for j in range(n))
                assert fx.fxs_line_derivative(n, q, *u) == want
            for j in range(n):
                g = [v >> 4 for v in u]  # integration terms sit 4 bits lower (headroom)
                want = sum(int(Di[q][j]) * int(Wi[q]) * g[q] for q in range(n))
                assert fx.fxs_line_integral(n, j, *g) == want


# --- the lane kernel's conversions ----------------------------------------------------------


def round_half_away(q: Fraction) -> int:
    a = abs(q)
    n = int(a)
    if a - n >= Fraction(1, 2):
        n += 1
    return -n if q < 0 else n


def test_to_fixed_fast_equals_to_fixed(fx):
    rng = np.random.default_rng(11)
    for _ in range(6000):
        top = int(rng.choice([52, 53, 58, 60]))
        v = float(rng.standard_normal() * 10.0 ** rng.integers(-300, 300))
        e = fx.fxs_exponent(v)
        E = e + int(rng.integers(0, 80))
        assert fx.fxs_to_fixed_fast(v, E, top) == fx.fxs_to_fixed(v, E, top) == exact_fixed(v, E, top), (v, E, top)
    for v in (0.0, -0.0, 5e-324, -2.2e-308, 1.0, -1.0, 0.5, 1.5, -(2.0 ** 52 + 1), 1.7976931348623157e308):
        E = max(fx.fxs_exponent(v), 1)
        for top in (52, 58):
            assert fx.fxs_to_fixed_fast(v, E, top) == exact_fixed(v, E, top)


def test_to_fixed_scaled_within_half_a_unit(fx):
    """h v in fixed point for a scale h that is not a power of two: the significands' 64-bit
    product floor, rounded; within half a unit plus 2^-10 of the exact value."""
    rng = np.random.default_rng(12)
    for _ in range(4000):
        h = float(rng.uniform(0.001, 1000.0))
        sig, k = scale(fx, h)
        v = float(rng.standard_normal() * 10.0 ** rng.integers(-100, 100))
        e = fx.fxs_exponent(v)
        E = e + k + 1 + int(rng.integers(0, 60))
        got = fx.fxs_to_fixed_scaled(v, E, sig, k)
        exact = Fraction(v) * Fraction(sig, ONE) * Fraction(2) ** (k + 1023 + 52 - E)
        assert abs(got) < 2 ** 53
        assert abs(Fraction(got) - exact) <= Fraction(1, 2) + Fraction(1, 1024), (v, h, E)
    for v in (0.0, -0.0, 5e-324):
        assert fx.fxs_to_fixed_scaled(v, 1000, scale(fx, 3.0)[0], 1) == 0


def test_to_double_fast_rounds_to_nearest(fx):
    rng = np.random.default_rng(13)
    for _ in range(6000):
        bits = int(rng.integers(1, 62))
        x = int(rng.integers(0, 2 ** 61)) >> (61 - bits)
        if rng.random() < 0.5:
            x = -x
        lsb = int(rng.integers(-1150, 1000))
        got = fx.fxs_to_double_fast(x, lsb, ONE, 0)
        want = exact_double(x, lsb)
        exact = Fraction(x) * Fraction(2) ** lsb
        if x != 0 and 2.0 ** -1022 <= abs(want) < math.inf:
            # nearest, ties away from zero (to_double breaks ties to even)
            assert abs(Fraction(got) - exact) <= Fraction(float(np.spacing(abs(want)))) / 2, (x, lsb)
            if Fraction(got) != exact and abs(Fraction(got) - exact) * 2 != Fraction(float(np.spacing(abs(want)))):
                assert got == want
        else:
            assert got == fx.fxs_to_double(x, lsb, ONE), (x, lsb)
    assert fx.fxs_to_double_fast(0, -60, ONE, 0) == 0.0
    assert math.copysign(1.0, fx.fxs_to_double_fast(0, -60, ONE, 0)) == 1.0
    # ties away from zero, carries into the exponent, both range ends
    assert fx.fxs_to_double_fast((1 << 53) + 1, 0, ONE, 0) == float((1 << 53) + 2)
    assert fx.fxs_to_double_fast(-((1 << 53) + 1), 0, ONE, 0) == -float((1 << 53) + 2)
    assert fx.fxs_to_double_fast((1 << 54) - 1, 0, ONE, 0) == float(1 << 54)
    for x, lsb in [(1, 1023), (3, 1023), ((1 << 61) - 1, 962), (1, -1022), (1, -1023), (1, -1080), (3, -1075)]:
        assert fx.fxs_to_double_fast(x, lsb, ONE, 0) == fx.fxs_to_double(x, lsb, ONE), (x, lsb)


def test_to_double_fast_scaled(fx):
    rng = np.random.default_rng(14)
    for _ in range(4000):
        s = float(rng.uniform(0.001, 1000.0))
        sig, k = scale(fx, s)
        x = int(rng.integers(-(2 ** 61), 2 ** 61))
        lsb = int(rng.integers(-200, 200))
        got = fx.fxs_to_double_fast(x, lsb + k, sig, 1)
        exact = Fraction(x) * Fraction(sig, ONE) * Fraction(2) ** (lsb + k)
        want = float(exact) if exact != 0 else 0.0
        err = abs(Fraction(got) - exact)
        assert err <= Fraction(float(np.spacing(abs(want)))) / 2 + Fraction(2) ** (lsb + k), (x, lsb, s)
