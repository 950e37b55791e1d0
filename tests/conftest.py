import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300, sm_103a)")


def load_golden(name):
    return np.load(os.path.join(GOLDEN, name), allow_pickle=False)


def relerr(a, b):
    """Element-wise |a - b| / |b| (complex-aware), with b == 0 -> |a|."""
    a = np.asarray(a)
    b = np.asarray(b)
    d = np.abs(a - b)
    s = np.abs(b)
    return np.where(s > 0, d / np.where(s > 0, s, 1.0), d)


@pytest.fixture(scope="session")
def golden():
    return load_golden


DBL_EPS = np.finfo(np.float64).eps


def eff_tolerance(ref, x, an=None, bn=None):
    """Per-instance tolerances of (qext, qsca, qabs, qb, asy, qratio).

    1e-10 relative for qext and qsca and 1e-10 relative for the asymmetry
    parameter g, widened by the conditioning of the reference's own formulas:
      * g: + 1e3 eps / x^2.  The numerator of b_n in mie_coeffs.py:124-128
        cancels to O(x^2) of its terms, so the reference's b_n (and g) carry
        about 1e2 eps / x^2 of relative error at small x; 50-digit mpmath
        values in tests/golden/mie_exact_small_x.npz show it.
      * qabs = qext - qsca: 1e-10 of qext (absolute).
      * qb: 1e-9 + 1e3 eps * sum|(2n+1)(a_n - b_n)| / |sum (2n+1)(-1)^n (a_n - b_n)|,
        the condition number of the alternating back-scattering sum.
    Returns an array [6] of absolute tolerances.
    """
    qext, qsca, qabs, qb, g, qr = ref
    tol = np.empty(6)
    tol[0] = 1e-10 * abs(qext)
    tol[1] = 1e-10 * abs(qsca)
    tol[2] = 1e-10 * abs(qext)
    cond = 1.0
    if an is not None:
        n = np.arange(1, an.size + 1)
        t = (2 * n + 1) * (an - bn)
        den = abs(np.sum(t * (-1.0) ** n))
        cond = np.sum(np.abs(t)) / den if den > 0 else 1e300
    tol[3] = (1e-9 + 1e3 * DBL_EPS * cond) * abs(qb)
    tol[4] = (1e-10 + 1e3 * DBL_EPS / x ** 2) * abs(g) + 1e-15
    tol[5] = (1e-9 + 1e3 * DBL_EPS * cond + 1e-10) * abs(qr)
    return tol
