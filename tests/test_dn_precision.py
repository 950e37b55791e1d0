"""Precision of the mixed path's D_n recurrence (CPU emulation).

The mixed coefficient kernel (geosmie_gb300/csrc/gbmie_table_tc.cu,
homog_core_mixed) runs the downward log-derivative recurrence
    D_k = (k+1)/z - 1 / (D_{k+1} + (k+1)/z),   z = m x,
of pymiecoated/mie_coeffs.py:101,119-121 in double-float arithmetic (pairs of
FP32 numbers, geosmie_gb300/csrc/df.cuh) and shortens the warm-up above nmax
to an e^-23 damping where |z| < nmax + 1.  This test restates those steps in
numpy float32 (two-sum, fast two-sum, FMA two-product, one Newton step of the
reciprocal; an FMA is emulated by one float64 evaluation rounded to float32,
and the seed reciprocal is the correctly rounded float32 one rather than the
GPU's approximate instruction) and compares D_k at every order with the
reference's FP64 recurrence from its own start, zero at
round(max(nmax, |m x|) + 16).

Bounds (relative to |D_k|, every order 1..nmax):
  dust-like indices (Im m 1e-4 .. 1e-2), x up to 630: 1e-10 (measured 1.6e-11);
  weakly absorbing indices (Im m 1e-9 .. 1e-8), x up to 630: 2e-8 (measured
  5.2e-9 at x = 630, m = 1.333 + 1e-9 i, where |m x| > nmax and near-pole
  orders amplify the rounding of either arithmetic).
Both lie far below the FP32 coefficients the mixed path emits.
"""
import numpy as np
import pytest

f32 = np.float32


def _two_sum(a, b):
    s = f32(a + b)
    bb = f32(s - a)
    return s, f32(f32(a - f32(s - bb)) + f32(b - bb))


def _fast_two_sum(a, b):
    s = f32(a + b)
    return s, f32(b - f32(s - a))


def _fma(a, b, c):
    return f32(np.float64(a) * np.float64(b) + np.float64(c))


def _add(a, b):
    s, e = _two_sum(a[0], b[0])
    return _fast_two_sum(s, f32(e + f32(a[1] + b[1])))


def _mul(a, b):
    p = f32(a[0] * b[0])
    e = _fma(a[1], b[0], _fma(a[0], b[1], _fma(a[0], b[0], -p)))
    return _fast_two_sum(p, e)


def _mul_f(a, b):
    p = f32(a[0] * b)
    return _fast_two_sum(p, _fma(a[1], b, _fma(a[0], b, -p)))


def _dfma(a, b, c):
    p = f32(a[0] * b[0])
    e = _fma(a[1], b[0], _fma(a[0], b[1], _fma(a[0], b[0], -p)))
    s = _two_sum(p, c[0])
    return _fast_two_sum(s[0], f32(s[1] + f32(e + c[1])))


def _rcp(a):
    y = f32(f32(1) / a[0])
    r = _fma(-a[1], y, _fma(-a[0], y, f32(1)))
    return _fast_two_sum(y, f32(y * r))


def _from64(d):
    hi = f32(d)
    return hi, f32(d - np.float64(hi))


def dn_mixed(m, x, nmax):
    """D_1..D_nmax as the mixed kernel forms them."""
    z = m * x
    hz = x / z
    xi = _from64(1.0 / x)
    zinv = (_mul(_from64(hz.real), xi), _mul(_from64(hz.imag), xi))
    az = f32(f32(abs(z) / x) * f32(x))
    nmx = int(np.rint(max(f32(nmax), az) + f32(16)))
    warm = nmx - 1 - nmax
    if az < nmax + 1:
        q = 2.0 * np.log((2.0 * (nmax + 1) + 1.0) / az)
        warm = min(warm, int(np.ceil(23.0 / q)) + 2)

    def step(D, kk):
        r = (_mul_f(zinv[0], f32(kk)), _mul_f(zinv[1], f32(kk)))
        w = (_add(D[0], r[0]), _add(D[1], r[1]))
        iw = _rcp(_dfma(w[0], w[0], _mul(w[1], w[1])))
        return _dfma((-w[0][0], -w[0][1]), iw, r[0]), _dfma(w[1], iw, r[1])
    zero = (f32(0), f32(0))
    D = (zero, zero)
    for k in range(nmax + warm, nmax, -1):
        D = step(D, k + 1)
    out = np.zeros(nmax, complex)
    for k in range(nmax, 0, -1):
        D = step(D, k + 1)
        out[k - 1] = complex(np.float64(D[0][0]) + np.float64(D[0][1]), np.float64(D[1][0]) + np.float64(D[1][1]))
    return out


def dn_reference(m, x, nmax):
    """The reference's FP64 recurrence from zero at its nmx."""
    z = m * x
    D = 0j
    out = np.zeros(nmax, complex)
    for j in range(int(np.rint(max(nmax, abs(z)) + 16)) - 1, 0, -1):
        D = (j + 1) / z - 1.0 / (D + (j + 1) / z)
        if j <= nmax:
            out[j - 1] = D
    return out


def _nmax(x):
    return int(np.rint(2.0 + x + 4.0 * np.cbrt(x)))


XS = [1e-3, 0.05, 1.0, 7.3, 40.0, 157.0, 314.0, 630.0]


@pytest.mark.parametrize("m,tol", [(1.45 + 1e-4j, 1e-10), (1.6 + 1e-2j, 1e-10), (1.53 + 0.008j, 1e-10),
                                   (1.5 + 1e-8j, 2e-8), (1.43 + 1e-8j, 2e-8), (1.333 + 1e-9j, 2e-8)])
def test_dn_double_float_against_fp64_cpu(m, tol):
    for x in XS:
        nm = _nmax(x)
        a = dn_mixed(m, x, nm)
        b = dn_reference(m, x, nm)
        err = np.max(np.abs(a - b) / np.abs(b))
        assert err < tol, (m, x, err)


def test_dn_dust_draws_cpu():
    """Seeded dust-like indices (m_r 1.45-1.60, log10 m_i -4..-2) at the dust
    workload's largest sizes (x up to 314)."""
    rng = np.random.default_rng(20261203)
    for _ in range(6):
        m = rng.uniform(1.45, 1.60) + 1j * 10.0 ** rng.uniform(-4.0, -2.0)
        for x in (3.1, 52.0, 314.0):
            nm = _nmax(x)
            err = np.max(np.abs(dn_mixed(m, x, nm) - dn_reference(m, x, nm)) / np.abs(dn_reference(m, x, nm)))
            assert err < 1e-10, (m, x, err)
