"""The reciprocal inside the FP64 Newton step's LDL^T solve and the Green
operator's 3x3 inverse (rcp_nr: the hardware's approximate double reciprocal
refined by two Newton-Raphson steps, plain division outside
2^-99 <= |x| < 2^99), computed on the GPU through voce_diag_rcp and checked
against IEEE division: within 1 ulp inside that range, and the same bits as
1.0 / x outside it (subnormals, 0, infinities, NaN and the far exponents)."""
import numpy as np
import pytest

from voce_gb300 import capi

pytestmark = pytest.mark.gpu

LO, HI = 2.0 ** -99, 2.0 ** 99


def _inputs():
    rng = np.random.Generator(np.random.PCG64(5))
    mant = 1.0 + rng.random(40)
    xs = [np.ldexp(m, e) for e in range(-1074, 1024, 3) for m in mant[:4]]
    xs += list(np.ldexp(mant, 0))
    for edge in (LO, HI):
        xs += [edge, np.nextafter(edge, 0.0), np.nextafter(edge, np.inf),
               edge * (1 + 2 ** -52), edge * (1 - 2 ** -53)]
    xs += [5e-324, 1e-310, 2.2250738585072014e-308, np.nextafter(2.2250738585072014e-308, 0.0),
           1.7976931348623157e308, 0.0, np.inf, np.nan, 1.0, 3.0, 7.0, 0.1, 1.0 / 3.0]
    x = np.array(xs, dtype=np.float64)
    x = x[np.isfinite(x) | np.isinf(x) | np.isnan(x)]
    return np.concatenate([x, -x])


def test_rcp_nr_within_one_ulp_inside_range_and_exact_outside(voce_lib):
    x = _inputs()
    got = capi.diag_rcp(x)
    with np.errstate(divide="ignore", over="ignore", invalid="ignore"):
        want = 1.0 / x
    ax = np.abs(x)
    inside = (ax >= LO) & (ax < HI)
    assert inside.sum() > 200 and (~inside).sum() > 200
    ulp = np.spacing(np.abs(want[inside]))
    err = np.abs(got[inside] - want[inside]) / ulp
    assert err.max() <= 1.0, (x[inside][np.argmax(err)], err.max())
    # outside the range: the division itself, bit for bit (NaN stays NaN)
    o_got, o_want = got[~inside], want[~inside]
    assert np.array_equal(o_got.view(np.uint64)[~np.isnan(o_want)],
                          o_want.view(np.uint64)[~np.isnan(o_want)])
    assert np.all(np.isnan(o_got[np.isnan(o_want)]))
    # the sign of zero and of infinity follows the input's
    assert np.array_equal(np.signbit(got[~np.isnan(x)]), np.signbit(x[~np.isnan(x)]))


def test_sqrt_nr_of_the_mixed_ir_norms(voce_lib):
    """sqrt_nr (voce_diag_sqrt): within 1e-12 relative of the correctly
    rounded square root for 2^-99 <= x < 2^99, and sqrt itself outside
    (zero, subnormals, far exponents, infinity, NaN, negative values)."""
    x = _inputs()
    got = capi.diag_sqrt(x)
    with np.errstate(invalid="ignore"):
        want = np.sqrt(x)
    inside = (x >= LO) & (x < HI)
    assert inside.sum() > 200 and (~inside).sum() > 200
    rel = np.abs(got[inside] - want[inside]) / want[inside]
    print("sqrt_nr max relative error", rel.max())
    assert rel.max() <= 1e-12, (x[inside][np.argmax(rel)], rel.max())
    o_got, o_want = got[~inside], want[~inside]
    nan = np.isnan(o_want)
    assert np.array_equal(o_got.view(np.uint64)[~nan], o_want.view(np.uint64)[~nan])
    assert np.all(np.isnan(o_got[nan]))
