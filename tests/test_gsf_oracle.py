"""Known-answer checks of the GSF restatement (oracle/spher_expan.c), CPU only.

gsf/spher_expan.f has no test or golden file in the reference and cannot be
compiled here (no Fortran compiler), so the restatement is pinned by known
answers: Gauss-Legendre nodes, Henyey-Greenstein moments, and the MATR
reconstruction of the expanded matrix.
"""
import numpy as np
import pytest

from oracle import gsf


@pytest.mark.parametrize("n", [3, 4, 64, 129, 960])
def test_gauss_matches_leggauss(n):
    z, w = gsf.gauss(n)
    zr, wr = np.polynomial.legendre.leggauss(n)
    assert np.max(np.abs(z - zr)) < 1e-14
    # IND1 = 0 doubles PA^2 (1 - x^2), which is half the standard weight
    assert np.max(np.abs(w - wr)) < 1e-13


def _hg(g, mu):
    return (1 - g * g) / (1 + g * g - 2 * g * mu) ** 1.5


@pytest.mark.parametrize("g", [0.2, 0.6])
def test_henyey_greenstein_moments(g):
    ang = np.linspace(0.0, 180.0, 20001)
    mu = np.cos(np.radians(ang))
    p11 = _hg(g, mu)
    F = np.zeros((1, 6, ang.size))
    F[0, 0] = p11
    F[0, 1] = p11          # F22 = F11, F33 = F44 = 0, F12 = F34 = 0
    coef, cnorm = gsf.expand(ang, F, 64)
    l = np.arange(64)
    want = (2 * l + 1) * g ** l
    assert np.max(np.abs(coef[0, 0] - want)) < 2e-5
    assert abs(coef[0, 0, 0] - 1.0) < 1e-15


def test_matr_round_trip():
    ang = np.linspace(0.0, 180.0, 4001)
    mu = np.cos(np.radians(ang))
    P2 = 0.5 * (3 * mu * mu - 1)
    F = np.zeros((1, 6, ang.size))
    F[0, 0] = 1.0 + 0.4 * mu + 0.3 * P2
    # F22 + F33 ~ (1 + mu)^2 and F22 - F33 ~ (1 - mu)^2, as the generalized
    # spherical functions d^l_{2,2} and d^l_{2,-2} require
    S = 0.45 * (1 + mu) ** 2
    D = 0.1 * (1 - mu) ** 2
    F[0, 1] = 0.5 * (S + D)
    F[0, 2] = 0.5 * (S - D)
    F[0, 3] = 0.5 * mu + 0.1
    F[0, 4] = -0.2 * (1 - mu * mu)
    F[0, 5] = 0.1 * (1 - mu * mu) * mu
    coef, cnorm = gsf.expand(ang, F, 32)
    back = gsf.matr(coef[0], np.radians(ang)) / cnorm[0]
    want = F[0, [0, 1, 2, 3, 4, 5]]
    assert np.max(np.abs(back - want)) < 1e-5
