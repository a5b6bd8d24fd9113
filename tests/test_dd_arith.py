"""Float-float arithmetic (nalu-wind_gb300/csrc/dd.h) against its stated
error bounds, on the CPU, in x87 extended precision (64-bit significand):

  split of a double:  |hi + lo - x| <= 2^-48 |x|
  a + b, a - b:       |err| <= 2^-46 (|a| + |b|)
  a * b:              |err| <= 2^-45 |a b|
  1 / a:              |err| <= 2^-45 / |a|
  widen(float):       exact
  dd -> double:       hi + lo correctly rounded (ties to even)

The edge-assembly kernels evaluate their FP64 formulas in this arithmetic;
the GPU parity tests then bound the assembled entries by 1e-12 times their
running magnitude.
"""
import ctypes as C
import platform
import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent

pytestmark = pytest.mark.skipif(platform.machine() not in ("x86_64", "AMD64"),
                                reason="needs x87 extended precision for the reference sums")


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    out = tmp_path_factory.mktemp("dd") / "libddhost.so"
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-shared", "-fPIC",
                    "-I", str(ROOT / "nalu-wind_gb300" / "csrc"), str(ROOT / "tests" / "dd_host.cpp"),
                    "-o", str(out)], check=True)
    return C.CDLL(str(out))


def _p(a, t):
    return a.ctypes.data_as(C.POINTER(t))


def _split(lib, x):
    n = len(x)
    hi, lo = np.zeros(n, np.float32), np.zeros(n, np.float32)
    lib.dd_split(C.c_int64(n), _p(x, C.c_double), _p(hi, C.c_float), _p(lo, C.c_float))
    return hi, lo


def _op(lib, op, a, b):
    n = len(a[0])
    rh, rl = np.zeros(n, np.float32), np.zeros(n, np.float32)
    lib.dd_binop(C.c_int(op), C.c_int64(n), _p(a[0], C.c_float), _p(a[1], C.c_float),
                 _p(b[0], C.c_float), _p(b[1], C.c_float), _p(rh, C.c_float), _p(rl, C.c_float))
    return rh, rl


def _ld(pair):
    return pair[0].astype(np.longdouble) + pair[1].astype(np.longdouble)


def _samples(rng, n):
    mag = 10.0 ** rng.uniform(-18, 30, n)
    x = rng.choice([-1.0, 1.0], n) * mag * rng.uniform(1, 2, n)
    x[:5] = [0.0, -0.0, 1.0, -3.0, 2.0 ** -62]
    return x


def test_split_and_back(lib):
    rng = np.random.default_rng(0)
    x = np.concatenate([_samples(rng, 20000), [1e-300, -1e-200, 1e300, 5e-324]])
    hi, lo = _split(lib, x)
    err = np.abs(_ld((hi, lo)) - x.astype(np.longdouble))
    inrange = (np.abs(x) >= 2.0 ** -62) & (np.abs(x) < 2.0 ** 127)
    assert np.all(err[inrange] <= 2.0 ** -48 * np.abs(x[inrange]))
    assert np.all(hi[x == 0] == 0) and np.all(lo[x == 0] == 0)
    back = np.zeros(len(x))
    lib.dd_back(C.c_int64(len(x)), _p(hi, C.c_float), _p(lo, C.c_float), _p(back, C.c_double))
    np.testing.assert_array_equal(back, (hi.astype(np.float64) + lo.astype(np.float64)))


def test_widen_is_exact(lib):
    rng = np.random.default_rng(1)
    f = np.concatenate([rng.normal(0, 1, 5000) * 10.0 ** rng.uniform(-37, 37, 5000),
                        [0.0, -0.0, 1e-45, -1e-40, np.inf, -np.inf]]).astype(np.float32)
    out = np.zeros(len(f))
    lib.dd_widen(C.c_int64(len(f)), _p(f, C.c_float), _p(out, C.c_double))
    np.testing.assert_array_equal(out, f.astype(np.float64))
    assert np.array_equal(np.signbit(out), np.signbit(f.astype(np.float64)))


def test_add_mul_rcp_bounds(lib):
    rng = np.random.default_rng(2)
    n = 20000
    a = _split(lib, rng.choice([-1, 1], n) * 10.0 ** rng.uniform(-10, 10, n))
    b = _split(lib, rng.choice([-1, 1], n) * 10.0 ** rng.uniform(-10, 10, n))
    # near-cancelling pairs
    c = _split(lib, -(a[0].astype(np.float64) + a[1]) * (1 + 1e-9 * rng.normal(size=n)))
    A, B, Cc = _ld(a), _ld(b), _ld(c)
    for (x, X), (y, Y) in [((a, A), (b, B)), ((a, A), (c, Cc))]:
        s = _ld(_op(lib, 0, x, y))
        assert np.all(np.abs(s - (X + Y)) <= 2.0 ** -46 * (np.abs(X) + np.abs(Y)))
        d = _ld(_op(lib, 1, x, y))
        assert np.all(np.abs(d - (X - Y)) <= 2.0 ** -46 * (np.abs(X) + np.abs(Y)))
    p = _ld(_op(lib, 2, a, b))
    assert np.all(np.abs(p - A * B) <= 2.0 ** -45 * np.abs(A * B))
    r = _ld(_op(lib, 3, a, b))
    assert np.all(np.abs(r - 1 / A) <= 2.0 ** -45 / np.abs(A))
    q = _ld(_op(lib, 4, a, b))
    Bh = b[0].astype(np.longdouble)
    assert np.all(np.abs(q - A * Bh) <= 2.0 ** -45 * np.abs(A * Bh))


def test_pair_to_double_is_correctly_rounded(lib):
    from fractions import Fraction
    rng = np.random.default_rng(3)
    n = 4000
    hi = (rng.choice([-1, 1], n) * 10.0 ** rng.uniform(-30, 30, n)).astype(np.float32)
    # lo a few to many binades below hi, either sign, including exact ties
    k = rng.integers(1, 80, n)
    lo = (hi.astype(np.float64) * rng.choice([-1, 1], n) * 2.0 ** (-k.astype(np.float64))
          * rng.uniform(0.5, 1.0, n)).astype(np.float32)
    lo[:100] = (hi[:100].astype(np.float64) * 2.0 ** -53).astype(np.float32)   # half-ulp ties
    lo[100:200] = (hi[100:200].astype(np.float64) * 3.0 * 2.0 ** -54).astype(np.float32)
    lo[200:300] = -lo[200:300]
    lo[300:310] = 0.0
    out = np.zeros(n)
    lib.dd_back(C.c_int64(n), _p(hi, C.c_float), _p(lo, C.c_float), _p(out, C.c_double))
    for h, l, o in zip(hi.tolist(), lo.tolist(), out.tolist()):
        exact = float(Fraction(h) + Fraction(l))
        assert o == exact, (h, l, o, exact)


def test_integer_widening_rounds_like_the_fp64_add(lib):
    """dd_to_double_int (no FP64 instruction, used by the row kernels): for
    normalised pairs, including a power-of-two hi with a lo of the other
    sign (the sum drops below hi's binade) and half-unit ties, the same bits
    as the FP64 add of the widened halves (hi + lo correctly rounded); other
    pairs take that path."""
    from fractions import Fraction
    import math
    rng = np.random.default_rng(7)
    n = 20000
    hi = (rng.choice([-1, 1], n) * 10.0 ** rng.uniform(-30, 30, n)).astype(np.float32)
    hi[:500] = (np.sign(rng.normal(size=500)) * 2.0 ** rng.integers(-60, 60, 500)).astype(np.float32)
    ulp = np.spacing(np.abs(hi)).astype(np.float64)
    lo = (rng.uniform(-0.5, 0.5, n) * ulp * 2.0 ** -rng.integers(0, 40, n)).astype(np.float32)
    lo[:250] = -np.sign(hi[:250]) * np.abs(lo[:250])  # power of two hi, lo of the other sign
    lo[250:260] = 0.0
    # exact ties: odd multiples of half a double unit of hi's binade (a quarter
    # unit below a power-of-two hi, where the lower binade's unit is half)
    ud = np.spacing(np.abs(hi[260:600]).astype(np.float64))
    odd = 2 * rng.integers(0, 4, 340) + 1
    lo[260:600] = (rng.choice([-1, 1], 340) * ud * odd / 2).astype(np.float32)
    lo[260:400] = (-np.sign(hi[260:400]) * ud[:140] * odd[:140] / 4).astype(np.float32)
    hi[260:400] = (np.sign(hi[260:400]) * 2.0 ** rng.integers(-60, 60, 140)).astype(np.float32)
    lo[260:400] = (-np.sign(hi[260:400]) * np.spacing(np.abs(hi[260:400]).astype(np.float64))
                   * odd[:140] / 4).astype(np.float32)
    extra_hi = np.array([0.0, -0.0, 1e-40, np.inf, 1.0, 1.0], np.float32)
    extra_lo = np.array([0.0, 1e-44, 0.0, 0.0, np.float32(2.0 ** -24), -np.float32(2.0 ** -23)], np.float32)
    hi = np.concatenate([hi, extra_hi])
    lo = np.concatenate([lo, extra_lo])
    out = np.zeros(len(hi))
    ref = np.zeros(len(hi))
    lib.dd_back_int(C.c_int64(len(hi)), _p(hi, C.c_float), _p(lo, C.c_float), _p(out, C.c_double))
    lib.dd_back(C.c_int64(len(hi)), _p(hi, C.c_float), _p(lo, C.c_float), _p(ref, C.c_double))
    for h, l, o, r in zip(hi.tolist(), lo.tolist(), out.tolist(), ref.tolist()):
        if not math.isfinite(h):
            assert o == r or (math.isnan(o) and math.isnan(r))
            continue
        assert o == r, (h, l, o, r)
        exact = Fraction(h) + Fraction(l)
        assert abs(Fraction(o) - exact) <= Fraction(np.spacing(abs(r))) / 2


@pytest.mark.parametrize("k", [2, 7, 30])
def test_deferred_accumulator_bound(lib, k):
    """dd_acc (the row kernels' running sums): the sum of k pairs within
    k^2 u^2 of the sum of |terms|, with mixed signs and heavy cancellation."""
    rng = np.random.default_rng(11 + k)
    groups = 4000
    x = rng.normal(size=groups * k) * 10.0 ** rng.uniform(-3, 3, groups * k)
    x[: groups * k // 2] *= rng.choice([-1.0, 1.0], groups * k // 2)
    # every fifth group: terms that cancel to a small remainder
    for g in range(0, groups, 5):
        seg = x[g * k:(g + 1) * k]
        seg[-1] = -np.sum(seg[:-1]) * (1 + 1e-9)
    hi, lo = _split(lib, x)
    rh, rl = np.zeros(groups, np.float32), np.zeros(groups, np.float32)
    lib.dd_accsum(C.c_int64(groups), C.c_int(k), _p(hi, C.c_float), _p(lo, C.c_float),
                  _p(rh, C.c_float), _p(rl, C.c_float))
    terms = hi.astype(np.longdouble) + lo.astype(np.longdouble)
    exact = terms.reshape(groups, k).sum(1)
    mag = np.abs(terms).reshape(groups, k).sum(1)
    got = rh.astype(np.longdouble) + rl.astype(np.longdouble)
    assert np.all(np.abs(got - exact) <= k * k * 2.0 ** -48 * mag)
