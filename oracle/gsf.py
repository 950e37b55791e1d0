"""ctypes front end of oracle/spher_expan.c -- oracle only.

TEST INFRASTRUCTURE: imported by tests/, __graft_entry__.smoke() and bench.py.
The shared object is built by :func:`build` (called from
``__graft_entry__.build()``) into ``oracle/_build``.
"""
import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_SRC = os.path.join(_HERE, "spher_expan.c")
_OUT = os.path.join(_HERE, "_build", "libspher_expan.so")
_lib = None


def build(force=False):
    """Compile spher_expan.c with gcc (no FMA contraction: same results on x86 and Arm)."""
    os.makedirs(os.path.dirname(_OUT), exist_ok=True)
    if not force and os.path.exists(_OUT) and os.path.getmtime(_OUT) >= os.path.getmtime(_SRC):
        return _OUT
    subprocess.check_call(["gcc", "-O2", "-ffp-contract=off", "-fPIC", "-shared", _SRC,
                           "-o", _OUT, "-lm"])
    return _OUT


def _load():
    global _lib
    if _lib is None:
        build()
        lib = ctypes.CDLL(_OUT)
        d = ctypes.POINTER(ctypes.c_double)
        lib.gsf_expand.argtypes = [ctypes.c_int, ctypes.c_int, d, d, ctypes.c_int, d, d]
        lib.gsf_expand.restype = ctypes.c_int
        lib.gsf_gauss.argtypes = [ctypes.c_int, d, d]
        lib.gsf_matr.argtypes = [d, d, d, d, d, d, ctypes.c_int, ctypes.c_int, d, d]
        _lib = lib
    return _lib


def _p(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def gauss(n):
    """Gauss-Legendre nodes (ascending) and weights, spher_expan.f:520-579."""
    z = np.zeros(n)
    w = np.zeros(n)
    _load().gsf_gauss(n, _p(z), _p(w))
    return z, w


def expand(ang_deg, F, ng):
    """Expansion coefficients of many table entries.

    ang_deg [nang] ascending degrees; F [ntab, 6, nang] as F11 F22 F33 F44 F12
    F34 (the reference's input order, convertncdf.py:177); returns
    (coef [ntab, 6, ng] as alpha1..alpha4, beta1, beta2 normalised so that
    alpha1(0) = 1, cnorm [ntab]).
    """
    ang = np.ascontiguousarray(ang_deg, dtype=np.float64)
    F = np.ascontiguousarray(F, dtype=np.float64)
    ntab = F.shape[0]
    coef = np.zeros((ntab, 6, ng))
    cnorm = np.zeros(ntab)
    rc = _load().gsf_expand(ntab, ang.size, _p(ang), _p(F), ng, _p(coef), _p(cnorm))
    if rc != 0:
        raise RuntimeError("gsf_expand failed (%d)" % rc)
    return coef, cnorm


def matr(coef, angl_rad):
    """Reconstruct [6, nang] F11 F22 F33 F44 F12 F34 from [6, L] coefficients."""
    coef = np.ascontiguousarray(coef, dtype=np.float64)
    ang = np.ascontiguousarray(angl_rad, dtype=np.float64)
    out = np.zeros((6, ang.size))
    L = coef.shape[1]
    _load().gsf_matr(*[_p(coef[i]) for i in range(6)], L - 1, ang.size, _p(ang), _p(out))
    return out


def quantize(coef):
    """The reference writes coefficients as F17.10 (spher_expan.f:104)."""
    return np.round(np.asarray(coef), 10)
