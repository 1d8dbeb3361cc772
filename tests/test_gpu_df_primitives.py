"""GPU: error bounds of the double-float primitives behind MWSEP_PLAIN_DF
(exp2 by a 2^(j/1024) table and one FP32 correction, sqrt and the quotient
by one Newton step from the SFU approximations, Dekker's add and the FMA
product), against numpy's FP64 results for the same split inputs.  Measured
maxima on GB300: exp2 1.9e-14, sqrt 1.5e-14, quotient 2.4e-14, product
1.2e-14, sum 8e-15 of |x| + |y|; the bounds below are 2^-45 (2.8e-14) and
2^-46 (1.4e-14).  The reference values ks*us*us are FP64 products: their own
rounding (~2^-52) is far below the bounds."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

EXP2, SQRT, DIV, MUL, ADD, SQ_SCALE_ADD, LOG2 = range(7)


def _split(x):
    """The pair a double becomes on the device, as its exact double value."""
    hi = np.asarray(x, dtype=np.float64).astype(np.float32)
    lo = (np.asarray(x, dtype=np.float64) - hi.astype(np.float64)).astype(np.float32)
    return hi.astype(np.float64) + lo.astype(np.float64)


def _eval(op, x, y=None, z=None):
    from milkywayathome_client_gb300 import native as N
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.ascontiguousarray(np.zeros_like(x) if y is None else y, dtype=np.float64)
    z = np.ascontiguousarray(np.zeros_like(x) if z is None else z, dtype=np.float64)
    out = np.zeros_like(x)
    P = C.POINTER(C.c_double)
    rc = N.lib().mwsep_df_eval(0, op, x.size, x.ctypes.data_as(P), y.ctypes.data_as(P), z.ctypes.data_as(P),
                               out.ctypes.data_as(P))
    assert rc == 0, rc
    return out


@pytest.fixture(scope="module")
def rng(built_library):
    return np.random.default_rng(20261203)


@pytest.fixture(params=[0, 10], ids=["scalar", "packed"])
def base(request):
    """Op offset: the scalar primitives (likelihood, tests) or the packed
    ones the integral kernel uses; both do the same roundings per value."""
    return request.param


def test_exp2(rng, base):
    x = np.concatenate([rng.uniform(-100.0, 2.0, 200000), rng.uniform(-1e-3, 1e-3, 20000),
                        np.arange(-100, 3, dtype=np.float64),
                        np.arange(-2048, 2049) / 1024.0,                    # table knots
                        (np.arange(-2048, 2048) + 0.5) / 1024.0])           # rounding ties
    got = _eval(base + EXP2, x)
    want = np.exp2(_split(x))
    rel = np.abs(got - want) / want
    assert rel.max() <= 2.0 ** -45, rel.max()
    # the bottom of FP32 range: the low part turns subnormal, a few bits go
    deep = rng.uniform(-126.0, -100.0, 20000)
    rel = np.abs(_eval(base + EXP2, deep) - np.exp2(_split(deep))) / np.exp2(_split(deep))
    assert rel.max() <= 2.0 ** -20, rel.max()
    # below range: exactly 0; NaN propagates
    below = np.array([-126.5, -127.0, -150.0, -1e6, -1e30, -np.inf])
    assert np.all(_eval(base + EXP2, below) == 0.0)
    assert np.isnan(_eval(base + EXP2, np.array([np.nan]))).all()


def test_sqrt(rng, base):
    x = np.exp(rng.uniform(np.log(1e-8), np.log(1e8), 200000))
    got = _eval(base + SQRT, x)
    want = np.sqrt(_split(x))
    err = (np.abs(got - want) / want).max()
    assert err <= 2.0 ** -45, err


def test_quotient(rng, base):
    x = np.exp(rng.uniform(np.log(1e-12), np.log(1e12), 200000))
    y = np.exp(rng.uniform(np.log(1e-12), np.log(1e12), 200000))
    got = _eval(base + DIV, x, y)
    want = _split(x) / _split(y)
    err = (np.abs(got - want) / want).max()
    assert err <= 2.0 ** -45, err
    assert np.all(_eval(base + DIV, np.zeros(4), np.array([1.0, 2.0, 1e-9, 1e9])) == 0.0)


def test_product_and_sum(rng, base):
    x = rng.uniform(-100.0, 100.0, 200000)
    y = rng.uniform(-100.0, 100.0, 200000)
    xs, ys = _split(x), _split(y)
    got = _eval(base + MUL, x, y)
    err = (np.abs(got - xs * ys) / np.abs(xs * ys)).max()
    assert err <= 2.0 ** -46, err
    # Dekker's add: 2^-48-ish of |x| + |y| (not of the sum, under cancellation)
    got = _eval(base + ADD, x, y)
    err = np.abs(got - (xs + ys)) / (np.abs(xs) + np.abs(ys))
    assert err.max() <= 2.0 ** -46, err.max()


def test_sq_scale_add(rng, base):
    """k u^2 + c, the exponent and halo quadratic: about five roundings of
    2^-47 of |k u^2| + |c| (measured 3.3e-14), also where the two cancel
    (c ~ -k u^2)."""
    k = -np.exp(rng.uniform(np.log(1e-3), np.log(10.0), 200000))
    u = rng.uniform(-30.0, 30.0, 200000)
    ks, us = _split(k), _split(u)
    ku2 = ks * us * us
    c = np.where(rng.random(200000) < 0.5, rng.uniform(-50.0, 0.0, 200000), -ku2 * rng.uniform(0.9, 1.1, 200000))
    got = _eval(base + SQ_SCALE_ADD, k, u, c)
    want = ku2 + _split(c)
    err = (np.abs(got - want) / (np.abs(ku2) + np.abs(_split(c)))).max()
    assert err <= 2.0 ** -44, err


def test_packed_equals_scalar(rng):
    """The packed primitives perform the scalar ones' roundings on each half:
    the same bits, element for element (odd counts included) -- except sqrt,
    whose FP32-refined reciprocal square root differs by an ulp between the
    two compiled forms for ~6.5% of inputs on GB300, moving the result by
    ~2^-48 (both stay within the bound test_sqrt checks)."""
    n = 100001
    cases = {EXP2: (rng.uniform(-130.0, 2.0, n),), SQRT: (np.exp(rng.uniform(-15, 15, n)),),
             DIV: (np.exp(rng.uniform(-20, 20, n)), np.exp(rng.uniform(-20, 20, n))),
             MUL: (rng.uniform(-100, 100, n), rng.uniform(-100, 100, n)),
             ADD: (rng.uniform(-100, 100, n), rng.uniform(-100, 100, n)),
             SQ_SCALE_ADD: (-np.exp(rng.uniform(-7, 2, n)), rng.uniform(-30, 30, n), rng.uniform(-60, 0, n)),
             LOG2: (np.exp(rng.uniform(-14, 14, n)),)}
    for op, args in cases.items():
        a, b = _eval(op, *args), _eval(10 + op, *args)
        if op == SQRT:
            assert (np.abs(a - b) / a).max() <= 2.0 ** -47
        else:
            np.testing.assert_array_equal(a, b, err_msg=str(op))


def test_log2(rng, base):
    """log2 for the general alpha/delta background: measured 9.2e-15 of
    |log2 x| + 1 (a few roundings of 2^-48 at the size of k + log2 c, the
    pair's resolution there); bound 2^-46."""
    x = np.concatenate([np.exp(rng.uniform(np.log(1e-6), np.log(1e6), 200000)),
                        1.0 + rng.uniform(-1e-3, 1e-3, 20000), np.array([1.0, 2.0, 0.5, 1024.0])])
    got = _eval(base + LOG2, x)
    want = np.log2(_split(x))
    err = np.abs(got - want) / (np.abs(want) + 1.0)
    assert err.max() <= 2.0 ** -46, err.max()


def test_fp64_exp(rng):
    """The FP64 integral kernel's e^x (Tang's table method, op 20) against
    numpy's FP64 exp: within 2^-51 relative over the normal range, within
    one subnormal step below it, and the range edges (0, underflow, NaN,
    +-inf, large positive) handled."""
    x = np.concatenate([rng.uniform(-708.0, 0.0, 400000), rng.uniform(-40.0, 0.0, 200000),
                        rng.uniform(-1e-6, 0.0, 20000), rng.uniform(0.0, 700.0, 20000),
                        -np.arange(0, 2049) * (np.log(2.0) / 256.0),        # table knots
                        np.array([-0.0, 0.0, -1.0, -708.39, 709.0])])
    got = _eval(20, x)
    want = np.exp(x)
    rel = np.abs(got - want) / want
    assert rel.max() <= 2.0 ** -51, (rel.max(), x[np.argmax(rel)])
    sub = np.concatenate([rng.uniform(-745.1, -708.4, 20000), np.array([-744.0, -745.0, -745.2])])
    assert np.abs(_eval(20, sub) - np.exp(sub)).max() <= 2.0 ** -1073
    edges = np.array([-745.3, -1000.0, -1e300, -np.inf, np.nan, 746.0, np.inf])
    got = _eval(20, edges)
    np.testing.assert_array_equal(got[:4], 0.0)
    assert np.isnan(got[4]) and got[5] == np.inf and got[6] == np.inf


def test_fp64_reciprocal(rng):
    """The FP64 integral kernel's 1/x (two Newton-Raphson steps from the
    SFU approximation, op 21) against the correctly rounded quotient:
    within 2^-51 relative for positive x with x and 1/x normal (the
    approximation flushes a subnormal reciprocal, e.g. of 1e308, to 0)."""
    x = np.concatenate([np.exp(rng.uniform(-700.0, 700.0, 200000)), rng.uniform(1.0, 2.0, 200000),
                        2.0 ** np.arange(-1021, 1022, dtype=np.float64), np.array([1.0, 3.0, 4.4e307, 2.3e-308])])
    got = _eval(21, x)
    want = 1.0 / x
    rel = np.abs(got - want) / want
    assert rel.max() <= 2.0 ** -51, (rel.max(), x[np.argmax(rel)])
