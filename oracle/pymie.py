"""CPU restatement of pymiecoated (homogeneous and coated Mie) -- oracle only.

TEST INFRASTRUCTURE: imported by tests/, __graft_entry__.smoke() and bench.py
(CPU baseline / reference arm).  Never imported by the product package.

Every function follows the reference algorithm step by step (same recurrences,
same start indices, same Bessel source -- scipy.special.jv/yv, the AMOS
routines the reference calls), so its results agree with the reference to
rounding.  Citations are paths inside the GEOSmie source tree.
"""
import numpy as np
from scipy.special import jv, yv

__all__ = [
    "nmax_of", "coeffs_homog", "coeffs_coated", "mie_coeffs", "props",
    "pitau", "s12_pt", "s12", "size_range", "batch_coeffs_homog",
    "batch_props", "batch_s12", "mueller",
]


def nmax_of(x):
    """Number of partial waves, round(2 + x + 4 x^(1/3)).

    pymiecoated/mie_coeffs.py:99,148,203 and mie_coated.py:131,166.  Python's
    round() is round-half-to-even, which is also what rint() does.
    """
    return int(round(2 + x + 4 * x ** (1.0 / 3.0)))


def coeffs_homog(eps, mu, x, ajv=None, ayv=None):
    """Homogeneous-sphere a_n, b_n (n = 1..nmax).

    Follows pymiecoated/mie_coeffs.py:132-180 (``single_mie_coeff``; the numba
    variant at :83-130 is the same arithmetic with caller-supplied jv/yv):
    psi_n = sqrt(pi x/2) J_{n+1/2}(x), chi_n = -sqrt(pi x/2) Y_{n+1/2}(x),
    xi_n = psi_n - i chi_n; D_n(z) by downward recurrence from zero at
    nmx = round(max(nmax, |z|) + 16); a_n = (da psi_n - psi_{n-1}) /
    (da xi_n - xi_{n-1}) with da = D_n/m + n/x, and b_n with db = D_n m + n/x.
    """
    eps = complex(eps)
    mu = complex(mu)
    x = float(x)
    z = np.sqrt(eps * mu) * x
    m = np.sqrt(eps / mu)
    nmax = nmax_of(x)
    nmx = int(round(max(nmax, abs(z)) + 16))
    n = np.arange(nmax)
    nu = n + 1.5
    sx = np.sqrt(0.5 * np.pi * x)
    if ajv is None or len(ajv) == 0:
        ajv = jv(nu, x)
    if ayv is None or len(ayv) == 0:
        ayv = yv(nu, x)
    px = sx * np.asarray(ajv)
    p1x = np.hstack((np.sin(x), px[: nmax - 1]))
    chx = -sx * np.asarray(ayv)
    ch1x = np.hstack((np.cos(x), chx[: nmax - 1]))
    gsx = px - 1j * chx
    gs1x = p1x - 1j * ch1x
    dnx = np.zeros(nmx, dtype=np.complex128)
    for j in range(nmx - 1, 0, -1):
        r = (j + 1.0) / z
        dnx[j - 1] = r - 1.0 / (dnx[j] + r)
    dn = dnx[:nmax]
    n1 = n + 1
    da = dn / m + n1 / x
    db = dn * m + n1 / x
    an = (da * px - p1x) / (da * gsx - gs1x)
    bn = (db * px - p1x) / (db * gsx - gs1x)
    return an, bn, nmax


def coeffs_coated(eps1, eps2, x, y):
    """Coated-sphere a_n, b_n (core size x, eps1; shell size y, eps2).

    Follows pymiecoated/mie_coeffs.py:183-251: D_n at u = m1 x, v = m2 x and
    w = m2 y from one start nmx = round(max(nmax, max(|m1 y|, |m2 y|)) + 16);
    Riccati-Bessel functions of the complex arguments v, w and the real y from
    scipy jv/yv; the ratio chain uu, vv, fv, fw, ku1, kv1, pt, prat, ku2, kv2
    gives the shell log-derivatives dns, gns, and a_n, b_n at y.
    """
    m1 = np.sqrt(complex(eps1))
    m2 = np.sqrt(complex(eps2))
    m = m2 / m1
    u = m1 * x
    v = m2 * x
    w = m2 * y
    nmax = nmax_of(y)
    mx = max(abs(m1 * y), abs(w))
    nmx = int(round(max(nmax, mx) + 16))
    n = np.arange(nmax)
    dns_list = []
    for zz in (u, v, w):
        dnx = np.zeros(nmx, dtype=np.complex128)
        for j in range(nmx - 1, 0, -1):
            r = (j + 1.0) / zz
            dnx[j - 1] = r - 1.0 / (dnx[j] + r)
        dns_list.append(dnx[:nmax].copy())
    dnu, dnv, dnw = dns_list
    nu = n + 1.5
    vwy = [v, w, y]
    sx = [np.sqrt(0.5 * np.pi * xx) for xx in vwy]
    pv, pw, py = [s * jv(nu, xx) for (s, xx) in zip(sx, vwy)]
    chv, chw, chy = [-s * yv(nu, xx) for (s, xx) in zip(sx, vwy)]
    p1y = np.hstack((np.sin(y), py[: nmax - 1]))
    ch1y = np.hstack((np.cos(y), chy[: nmax - 1]))
    gsy = py - 1j * chy
    gs1y = p1y - 1j * ch1y
    uu = m * dnu - dnv
    vv = dnu / m - dnv
    fv = pv / chv
    fw = pw / chw
    ku1 = uu * fv / pw
    kv1 = vv * fv / pw
    pt = pw - chw * fv
    prat = pw / pv / chv
    ku2 = uu * pt + prat
    kv2 = vv * pt + prat
    dns1 = ku1 / ku2
    gns1 = kv1 / kv2
    dns = dns1 + dnw
    gns = gns1 + dnw
    nrat = (n + 1) / y
    a1 = dns / m2 + nrat
    b1 = m2 * gns + nrat
    an = (py * a1 - p1y) / (gsy * a1 - gs1y)
    bn = (py * b1 - p1y) / (gsy * b1 - gs1y)
    return an, bn, nmax


def mie_coeffs(eps, x, mu=None, y=None, eps2=None):
    """Validation and dispatch, pymiecoated/mie_coeffs.py:36-73.

    Coated only if x != y and eps != eps2; shell-only when x == 0.
    """
    if x is None or eps is None:
        raise ValueError("Must specify x and either eps or m.")
    mu = complex(mu) if mu is not None else complex(1.0)
    coated = y is not None
    if coated == (eps2 is None):
        raise ValueError("Must specify both y and m2 for coated particles.")
    if coated and mu != complex(1.0):
        raise ValueError("Multilayer calculations for magnetic particles "
                         "are not currently supported.")
    if not coated:
        y = x
        eps2 = eps
    if x == y or eps == eps2:
        return coeffs_homog(eps, mu, y)
    if x == 0:
        return coeffs_homog(eps2, mu, y)
    return coeffs_coated(eps, eps2, x, y)


def props(an, bn, nmax, y):
    """Efficiencies (qext, qsca, qabs, qb, asy, qratio).

    pymiecoated/mie_props.py:28-70, including the zero-padded n+1 term of the
    asymmetry sum (:61-64) and qb = |sum (2n+1)(-1)^n (a_n - b_n)|^2 / y^2.
    """
    anp, anpp, bnp, bnpp = an.real, an.imag, bn.real, bn.imag
    n = np.arange(1.0, nmax + 1.0)
    cn = 2 * n + 1
    c1n = n * (n + 2) / (n + 1)
    c2n = cn / (n * (n + 1))
    y2 = y ** 2
    qext = 2 * (cn * (anp + bnp)).sum() / y2
    qsca = 2 * (cn * (anp ** 2 + anpp ** 2 + bnp ** 2 + bnpp ** 2)).sum() / y2
    qabs = qext - qsca
    q = ((an - bn) * cn * (-1) ** n).sum()
    qb = (q.real ** 2 + q.imag ** 2) / y2
    g1 = np.zeros((4, nmax))
    g1[:, : nmax - 1] = np.vstack((anp[1:nmax], anpp[1:nmax], bnp[1:nmax], bnpp[1:nmax]))
    asy1 = c1n * (anp * g1[0] + anpp * g1[1] + bnp * g1[2] + bnpp * g1[3])
    asy2 = c2n * (anp * bnp + anpp * bnpp)
    asy = 4 / y2 * (asy1 + asy2).sum() / qsca
    qratio = qb / qsca
    return qext, qsca, qabs, qb, asy, qratio


def pitau(u, nmax):
    """Scaled angular functions pi~_n(u), tau~_n(u), n = 1..nmax.

    pymiecoated/mie_props.py:166-192 (mie_p, mie_t) and :217-231 (scaling by
    (2n+1)/(n(n+1))).  Upward recurrences.
    """
    u = float(u)
    p = np.zeros(nmax)
    t = np.zeros(nmax)
    p[0] = 1.0
    p[1] = 3 * u
    for k in range(2, nmax):
        n = float(k)
        p[k] = (2 * n + 1) / n * p[k - 1] * u - (n + 1) / n * p[k - 2]
    t[0] = u
    t[1] = 6 * u ** 2 - 3
    for k in range(2, nmax):
        n = float(k)
        t[k] = (n + 1) * u * p[k] - (n + 2) * p[k - 1]
    i = np.arange(1, nmax + 1)
    n2 = (2.0 * i + 1) / (i * (i + 1))
    return p * n2, t * n2


def s12_pt(an, bn, pin, tin):
    """S1 = sum a_n pi~_n + b_n tau~_n, S2 = sum a_n tau~_n + b_n pi~_n.

    pymiecoated/mie_props.py:133-149 (mie_S12_backend_pt).
    """
    s1 = np.dot(an, pin) + np.dot(bn, tin)
    s2 = np.dot(an, tin) + np.dot(bn, pin)
    return s1, s2


def s12(an, bn, nmax, u):
    """S1, S2 at one cosine, pi/tau on the fly (mie_props.py:108-131)."""
    if abs(u) > 1:
        raise ValueError("The cosine u must be between -1 and 1.")
    pin, tin = pitau(u, nmax)
    return s12_pt(an, bn, pin, tin)


def mueller(s1, s2):
    """The six Mueller elements s11, s12, s22, s33, s34, s44.

    geosmie/dointegration.py:1044-1050 (calculateScatVals), including the sign
    of s34 = -Im(conj(S1) S2).
    """
    a1 = np.abs(s1) ** 2
    a2 = np.abs(s2) ** 2
    s11 = 0.5 * (a1 + a2)
    s12v = 0.5 * (a2 - a1)
    s33 = (s1 * np.conj(s2)).real
    s34 = -(np.conj(s1) * s2).imag
    return np.stack([s11, s12v, s11.copy(), s33, s34, s33.copy()])


def size_range(x_arr, costarr, mr, mi):
    """MultipleMie(xArr, None, costarr).calculateS12SizeRange(mr, mi).

    pymiecoated/mie_coated.py:61-89 with the pi/tau tables of :160-179:
    eps = (mr + i mi)^2, mu = 1; per x: coefficients, S1/S2 at every cosine,
    efficiencies.  Returns a dict with 's12' (list of lists of (S1, S2)) and
    the six efficiency lists.
    """
    eps = complex(mr, mi) ** 2
    keys = ["qext", "qsca", "qabs", "asy", "qb", "qratio"]
    ret = {k: [] for k in ["s12"] + keys}
    pt_cache = {}
    for x in x_arr:
        an, bn, nmax = coeffs_homog(eps, 1.0, x)
        if nmax not in pt_cache:
            pt_cache[nmax] = [pitau(c, nmax) for c in costarr]
        ret["s12"].append([s12_pt(an, bn, p, t) for (p, t) in pt_cache[nmax]])
        qext, qsca, qabs, qb, asy, qratio = props(an, bn, nmax, x)
        for k, v in zip(["qext", "qsca", "qabs", "qb", "asy", "qratio"],
                        [qext, qsca, qabs, qb, asy, qratio]):
            ret[k].append(v)
    return ret


# ---------------------------------------------------------------------------
# Vectorised forms of the same arithmetic (one numpy pass over many
# instances).  Used by tests at sizes where the per-instance loop is slow.
# ---------------------------------------------------------------------------

def batch_coeffs_homog(x, eps, mu=None):
    """a_n, b_n for many instances at once; returns (list of an, list of bn, nmax).

    Same arithmetic as :func:`coeffs_homog` (mie_coeffs.py:132-180): the
    downward D_n recurrence runs for all instances together, each instance
    starting from zero at its own nmx, so every instance sees exactly the
    operations of the scalar form.
    """
    x = np.asarray(x, dtype=np.float64)
    eps = np.asarray(eps, dtype=np.complex128) * np.ones_like(x)
    mu = np.ones_like(eps) if mu is None else np.asarray(mu, np.complex128) * np.ones_like(x)
    ninst = x.size
    z = np.sqrt(eps * mu) * x
    m = np.sqrt(eps / mu)
    nmax = np.array([nmax_of(v) for v in x], dtype=np.int64)
    nmx = np.array([int(round(max(nm, abs(zz)) + 16)) for nm, zz in zip(nmax, z)], np.int64)
    kmax = int(nmax.max())
    dn = np.zeros((ninst, kmax), dtype=np.complex128)
    d = np.zeros(ninst, dtype=np.complex128)
    for j in range(int(nmx.max()) - 1, 0, -1):
        act = j <= nmx - 1
        r = (j + 1.0) / z
        d = np.where(act, r - 1.0 / (d + r), 0.0)
        if j - 1 < kmax:
            keep = act & (j - 1 < nmax)
            dn[keep, j - 1] = d[keep]
    nidx = np.arange(kmax)
    nu = nidx + 1.5
    sx = np.sqrt(0.5 * np.pi * x)[:, None]
    n1 = (nidx + 1)[None, :]
    with np.errstate(all="ignore"):   # padded orders beyond an instance's nmax overflow
        px = sx * jv(nu[None, :], x[:, None])
        chx = -sx * yv(nu[None, :], x[:, None])
        p1x = np.concatenate([np.sin(x)[:, None], px[:, :-1]], axis=1)
        ch1x = np.concatenate([np.cos(x)[:, None], chx[:, :-1]], axis=1)
        gsx = px - 1j * chx
        gs1x = p1x - 1j * ch1x
        da = dn / m[:, None] + n1 / x[:, None]
        db = dn * m[:, None] + n1 / x[:, None]
        an = (da * px - p1x) / (da * gsx - gs1x)
        bn = (db * px - p1x) / (db * gsx - gs1x)
    ans = [an[i, : nmax[i]].copy() for i in range(ninst)]
    bns = [bn[i, : nmax[i]].copy() for i in range(ninst)]
    return ans, bns, nmax


def batch_props(ans, bns, nmax, y):
    """:func:`props` for every instance; returns an array [n, 6]."""
    return np.array([props(a, b, int(k), float(yy)) for a, b, k, yy in zip(ans, bns, nmax, y)])


def batch_s12(ans, bns, nmax, costarr):
    """S1, S2 [n, nang] from one pi/tau table of the largest nmax.

    pi~_n, tau~_n at index n do not depend on nmax (mie_props.py:166-192), so
    a single table truncated per instance reproduces mie_coated.py:160-179.
    """
    costarr = np.asarray(costarr, dtype=np.float64)
    kmax = int(np.max(nmax))
    tab = [pitau(c, max(kmax, 2)) for c in costarr]
    P = np.array([t[0] for t in tab])  # [nang, kmax]
    T = np.array([t[1] for t in tab])
    s1 = np.empty((len(ans), costarr.size), np.complex128)
    s2 = np.empty_like(s1)
    for i, (a, b) in enumerate(zip(ans, bns)):
        k = a.size
        s1[i] = P[:, :k] @ a + T[:, :k] @ b
        s2[i] = T[:, :k] @ a + P[:, :k] @ b
    return s1, s2
