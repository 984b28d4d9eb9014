"""The FP64 pow / log / cos that the FP64 kernels and the oracle share
(imex_sflow2d_dev_gb300/csrc/sflow_math.h), evaluated on the host through
the oracle library: its double-double constants recomputed from exact
arithmetic, its results against correctly rounded values (Python's decimal
at 60 digits) on the argument ranges of the settling, hindered-settling and
entrainment closures (constitutive_2d.f90:5370-5392, 4850-4851, 5046-5057)
and at random, and the C99 special values."""
import math
import os
import re
from decimal import Decimal, getcontext
from fractions import Fraction

import numpy as np
import pytest

import oracle

HDR = os.path.join(os.path.dirname(__file__), "..", "imex_sflow2d_dev_gb300", "csrc", "sflow_math.h")


def _pi():
    getcontext().prec = 80

    def atan_inv(n):
        x = Decimal(1) / n
        x2, s, t, k = x * x, x, x, 1
        while True:
            t *= -x2
            k += 2
            d = t / k
            if abs(d) < Decimal(10) ** -78:
                return s
            s += d
    return 16 * atan_inv(5) - 4 * atan_inv(239)


def _split(v):
    hi = float(v)
    return hi, float(v - Fraction(hi))


def test_double_double_constants_are_the_exact_values_split():
    getcontext().prec = 80
    text = open(HDR).read()
    defs = dict(re.findall(r"#define (SFM_\w+) (0x[0-9a-fp.+-]+)", text))
    ln2 = Fraction(Decimal(2).ln())
    pi = Fraction(_pi())
    assert (float.fromhex(defs["SFM_LN2_HI"]), float.fromhex(defs["SFM_LN2_LO"])) == _split(ln2)
    assert (float.fromhex(defs["SFM_PIO2_HI"]), float.fromhex(defs["SFM_PIO2_LO"])) == _split(pi / 2)
    assert float.fromhex(defs["SFM_INV_LN2"]) == float(1 / ln2)
    assert float.fromhex(defs["SFM_TWO_OVER_PI"]) == float(2 / pi)
    assert float.fromhex(defs["SFM_SQRT2"]) == math.sqrt(2.0)
    # every (hi, lo) pair of the series coefficients is 1/n or 1/n! split
    pairs = re.findall(r"sfm_mk\((-?0x[0-9a-fp.+-]+), (-?0x[0-9a-fp.+-]+)\)", text)
    exact = {}
    for n in (3, 5, 7):
        exact[_split(Fraction(1, n))] = n
    for n in range(2, 22):
        exact[_split(Fraction(1, math.factorial(n)))] = -n
        hi, lo = _split(Fraction(1, math.factorial(n)))
        exact[(-hi, -lo)] = -n
    assert len(pairs) >= 10
    for h, l in pairs:
        assert (float.fromhex(h), float.fromhex(l)) in exact, (h, l)
    # single-double coefficients: 1/n (log series) and 1/n! (exp, sin, cos)
    singles = {float(Fraction(1, n)) for n in range(9, 28, 2)}
    singles |= {float(Fraction(1, math.factorial(n))) for n in range(7, 22)}
    for h in re.findall(r"(?:SFM_MUL\(\w, \w+\), |double [vw] = )(-?0x[0-9a-fp.+-]+)", text):
        assert abs(float.fromhex(h)) in singles, h


def _cr_pow(x, y):
    getcontext().prec = 60
    return float(Decimal(x) ** Decimal(y))


@pytest.mark.parametrize("case", ["rey_0.687", "ri_2.4", "hindered_4.65", "random"])
def test_pow_is_correctly_rounded_on_the_closure_ranges(case):
    rng = np.random.default_rng({"rey_0.687": 1, "ri_2.4": 2, "hindered_4.65": 3, "random": 4}[case])
    n = 1500
    if case == "rey_0.687":
        x, y = 10 ** rng.uniform(-4, 3, n), np.full(n, 0.687)
    elif case == "ri_2.4":
        x, y = 10 ** rng.uniform(-6, 15, n), np.full(n, 2.4)
    elif case == "hindered_4.65":
        x, y = rng.uniform(0, 1, n), np.full(n, 4.65)
    else:
        x, y = 10 ** rng.uniform(-300, 300, n), rng.uniform(-1, 1, n)
    got = oracle.eval_math("pow", x, y)
    want = np.array([_cr_pow(a, b) for a, b in zip(x, y)])
    assert np.array_equal(got, want)


def test_log_is_correctly_rounded():
    getcontext().prec = 60
    rng = np.random.default_rng(5)
    x = np.concatenate([10 ** rng.uniform(-300, 300, 2000), rng.uniform(0.5, 2.0, 1000),
                        [5e-324, 1e-310, 1.0, 2.0, 0.5, 1e300]])
    got = oracle.eval_math("log", x)
    want = np.array([float(Decimal(v).ln()) for v in x])
    assert np.array_equal(got, want)


def test_cos_within_one_ulp_of_correct_rounding():
    getcontext().prec = 60

    def dcos(v):
        v = Decimal(v)
        s = t = Decimal(1)
        n = 0
        while True:
            n += 2
            t = -t * v * v / (n * (n - 1))
            if abs(t) < Decimal(10) ** -70:
                return float(s)
            s += t
    rng = np.random.default_rng(6)
    x = np.concatenate([rng.uniform(0, 3.2, 3000), rng.uniform(-60, 60, 1000)])
    got = oracle.eval_math("cos", x)
    want = np.array([dcos(v) for v in x])
    ulp = np.array([math.ulp(w) for w in want])
    assert np.all(np.abs(got - want) <= ulp)
    assert np.mean(got == want) >= 0.999


def test_special_values():
    inf, nan = float("inf"), float("nan")
    cases = [(0.0, 2.0, 0.0), (-0.0, 3.0, -0.0), (-0.0, -3.0, -inf), (0.0, -1.0, inf), (-2.0, 3.0, -8.0),
             (inf, 2.0, inf), (inf, -2.0, 0.0), (2.0, inf, inf), (0.5, inf, 0.0), (1.0, nan, 1.0),
             (nan, 0.0, 1.0), (2.0, 1024.0, inf), (2.0, -1075.0, 0.0), (2.0, -1074.0, 5e-324),
             (10.0, 308.0, 1e308), (-1.0, -inf, 1.0), (4.0, 0.5, 2.0), (1e300, 1e10, inf), (1e-300, 1e10, 0.0)]
    for x, y, want in cases:
        got = float(oracle.eval_math("pow", [x], [y])[0])
        assert got == want and math.copysign(1, got) == math.copysign(1, want), (x, y, got)
    assert math.isnan(oracle.eval_math("pow", [-2.0], [0.5])[0])
    assert math.isnan(oracle.eval_math("pow", [nan], [2.0])[0])
    lg = oracle.eval_math("log", [0.0, -1.0, inf, nan])
    assert lg[0] == -inf and math.isnan(lg[1]) and lg[2] == inf and math.isnan(lg[3])
    assert math.isnan(oracle.eval_math("cos", [inf])[0])
