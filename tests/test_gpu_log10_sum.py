"""The compensated likelihood's log10 sum on the GPU (mwsep_log10_sum_eval):
a mantissa product with the binary exponents summed as integers and log10
taken once, against a correctly rounded sum of the per-term log10 values
(math.fsum over numpy's log10), with log10's semantics per term."""
import ctypes as C
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _gpu_sum(built_library, x):
    from milkywayathome_client_gb300 import native as N
    x = np.ascontiguousarray(x, dtype=np.float64)
    out = C.c_double()
    rc = N.lib().mwsep_log10_sum_eval(0, x.size, x.ctypes.data_as(C.POINTER(C.c_double)), C.byref(out))
    assert rc == 0
    return out.value


def _want(x):
    with np.errstate(divide="ignore", invalid="ignore"):
        terms = np.log10(np.asarray(x, dtype=np.float64))
    if np.isnan(terms).any() or (np.isposinf(terms).any() and np.isneginf(terms).any()):
        return math.nan
    if np.isposinf(terms).any():
        return math.inf
    if np.isneginf(terms).any():
        return -math.inf
    return math.fsum(terms), float(np.sum(np.abs(terms)))


@pytest.mark.parametrize("case", ["wide", "narrow", "subnormal", "one_term", "empty", "many"])
def test_finite_sums(built_library, case):
    rng = np.random.default_rng(11)
    x = {"wide": 10.0 ** rng.uniform(-300, 300, 5000),
         "narrow": rng.uniform(0.5, 2.0, 5000),
         "subnormal": np.array([5e-324, 1e-315, 2.2e-308, 1e-310, 3.0, 7e-320]),
         "one_term": np.array([0.001234]),
         "empty": np.array([], dtype=np.float64),
         "many": rng.lognormal(-3.0, 2.0, 200000)}[case]
    got = _gpu_sum(built_library, x)
    want, scale = _want(x) if x.size else (0.0, 0.0)
    # one rounding of 2^-53 per factor (~5e-17 per term in log10) plus the final sum
    assert abs(got - want) <= 1e-16 * x.size + 4e-16 * max(scale, 1.0), (got, want)


@pytest.mark.parametrize("special,want", [([0.0], -math.inf), ([-1.0], math.nan), ([math.inf], math.inf),
                                          ([math.nan], math.nan), ([0.0, math.inf], math.nan),
                                          ([-0.0], -math.inf), ([1e-320, -2.0, 0.0], math.nan)])
def test_special_terms(built_library, special, want):
    x = np.concatenate([np.full(1000, 3.25), np.array(special, dtype=np.float64)])
    got = _gpu_sum(built_library, x)
    if math.isnan(want):
        assert math.isnan(got)
    else:
        assert got == want
