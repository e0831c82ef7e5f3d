"""The engine's own FP64 functions (csrc/hbt_math.cuh), run on the device
through hbt_check_math, against the host's libm (numpy): cos, used for the
same-event numerators, and exp, used by the radii fits.

Bounds: cos within 3e-16 absolute over |x| < 1000 (the phases of the pair
kernels are a few hundred at most) and 1e-15 absolute near 2^20, at scale 1
and at the pair kernels' scale 1/hbarC (against libm's cos of the exact
product, 3.5e-16); exp within 4 ulp relative over |x| < 700 and within 1e-15 relative
of libm outside (there it calls the device's exp())."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

_PD = ctypes.POINTER(ctypes.c_double)


def _dev(which, x):
    from hadronic_afterburner_toolkit_gb300 import engine
    L = engine.load()
    L.hbt_check_math.restype = ctypes.c_int32
    L.hbt_check_math.argtypes = [ctypes.c_int, ctypes.c_int32, ctypes.c_int64, _PD, _PD]
    x = np.ascontiguousarray(x, dtype=np.float64)
    out = np.empty_like(x)
    assert L.hbt_check_math(0, which, x.size, x.ctypes.data_as(_PD), out.ctypes.data_as(_PD)) == 0
    return out


def test_table_cos_against_libm():
    rng = np.random.default_rng(1)
    step = 2 * np.pi / 512
    k = np.arange(-4000, 4000)
    x = np.concatenate([rng.uniform(-1000, 1000, 200000), rng.uniform(-1, 1, 50000),
                        k * step, k * step + step / 2, np.nextafter(k * step + step / 2, 0),
                        [0.0, -0.0, 1e-300, 5e-324, np.pi, -np.pi, 2 * np.pi]])
    got = _dev(0, x)
    assert np.max(np.abs(got - np.cos(x))) < 3e-16
    big = rng.uniform(-1048575, 1048575, 20000)
    assert np.max(np.abs(_dev(0, big) - np.cos(big))) < 1e-15
    tail = np.array([1048576.0, -3e6, 1e10])
    np.testing.assert_array_equal(np.isnan(_dev(0, [np.nan, np.inf])), [True, True])
    assert np.max(np.abs(_dev(0, tail) - np.cos(tail))) < 1e-15


def test_table_exp_against_libm():
    rng = np.random.default_rng(2)
    ln2_64 = np.log(2) / 64
    k = np.arange(-64000, 64000, 7)
    x = np.concatenate([rng.uniform(-700, 700, 200000), rng.uniform(-1, 1, 50000),
                        -rng.exponential(30, 50000), k * ln2_64, k * ln2_64 + ln2_64 / 2,
                        [0.0, -0.0, 1e-300, -1e-300, 699.99, -699.99]])
    got = _dev(1, x)
    ref = np.exp(x)
    ulp = np.spacing(ref)
    assert np.max(np.abs(got - ref) / ulp) <= 4
    tail = np.array([700.0, -700.0, 709.7, -708.0, -800.0, 800.0, -np.inf, np.inf])
    with np.errstate(over="ignore"):
        want = np.exp(tail)
    got = _dev(1, tail)
    fin = np.isfinite(want)
    np.testing.assert_allclose(got[fin], want[fin], rtol=1e-15, atol=1e-320)
    np.testing.assert_array_equal(got[~fin], want[~fin])
    assert np.isnan(_dev(1, [np.nan])[0])


def test_df_cos_against_libm():
    """The double-float form's cos (csrc/hbt_tile.cuh df_cos) of x split into
    hi = (float)x, lo = (float)(x - hi), against libm's cos of hi + lo (exact
    in FP64): within 1e-14 absolute for |x| < 3200 (the table's 48-bit values
    and the reduction), quarter-period and table-point edges included;
    beyond, it calls the device's FP64 cos."""
    rng = np.random.default_rng(3)
    k = np.arange(-2000, 2000)
    x = np.concatenate([rng.uniform(-3200, 3200, 200000), rng.uniform(-1, 1, 50000),
                        k * (np.pi / 2), k * (np.pi / 2) + 1e-9, k * (np.pi / 2) + np.pi / 4,
                        np.arange(-51, 52) / 64.0 + 1 / 128.0,
                        [0.0, -0.0, 1e-30, -1e-30, np.pi, -np.pi, 3199.9, -3199.9]])
    h = x.astype(np.float32)
    xs = h.astype(np.float64) + (x - h.astype(np.float64)).astype(np.float32).astype(np.float64)
    got = _dev(2, x)
    assert np.max(np.abs(got - np.cos(xs))) < 1e-14
    far = np.concatenate([rng.uniform(3300, 1e5, 2000), -rng.uniform(3300, 1e5, 2000)])
    hf = far.astype(np.float32)
    xf = hf.astype(np.float64) + (far - hf.astype(np.float64)).astype(np.float32).astype(np.float64)
    assert np.max(np.abs(_dev(2, far) - np.cos(xf))) < 1e-15
    np.testing.assert_array_equal(np.isnan(_dev(2, [np.nan, np.inf])), [True, True])


HBARC = 0.197327053  # GeV fm, the pair kernels' constant


def _two_prod(a, b):
    """a * b = p + e exactly (Dekker's product with Veltkamp's split)."""
    p = a * b

    def split(v):
        c = 134217729.0 * v
        hi = c - (c - v)
        return hi, v - hi
    ah, al = split(a)
    bh, bl = split(b)
    return p, ((ah * bh - p) + ah * bl + al * bh) + al * bl


def _cos_scaled(h, x):
    """cos(h x) of the exact product: cos(p + e) = cos p - e sin p (e is
    below half an ulp of p, so the next term is below 1e-20)."""
    p, e = _two_prod(np.full_like(x, h), x)
    return np.cos(p) - np.sin(p) * e


def test_table_cos_at_the_pair_scale():
    """cos(ph / hbarC) of phases ph in GeV fm, the reduction done on ph
    itself, against libm's cos of the exact product (3.5e-16: the device's
    3e-16 at scale 1 plus the reference's own rounding)."""
    rng = np.random.default_rng(4)
    h = 1.0 / HBARC
    step = 2 * np.pi / 512 / h
    k = np.arange(-3000, 3000)
    x = np.concatenate([rng.uniform(-200, 200, 200000), rng.uniform(-0.5, 0.5, 50000),
                        k * step, k * step + step / 2, np.nextafter(k * step + step / 2, 0),
                        [0.0, -0.0, 1e-300, 5e-324, HBARC * np.pi]])
    assert np.max(np.abs(_dev(3, x) - _cos_scaled(h, x))) < 3.5e-16
    big = rng.uniform(-262143, 262143, 20000)  # the table's range at this scale
    assert np.max(np.abs(_dev(3, big) - _cos_scaled(h, big))) < 1e-15
    np.testing.assert_array_equal(np.isnan(_dev(3, [np.nan, np.inf])), [True, True])
    # beyond it the device's cos of the rounded product h * x
    tail = np.array([262144.0, -3e6, 1e10])
    assert np.max(np.abs(_dev(3, tail) - np.cos(h * tail))) < 1e-15
