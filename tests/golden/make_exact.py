"""Generate tests/golden/mie_exact_small_x.npz: 50-digit mpmath values of the
asymmetry parameter g (and qsca, qb) for small size parameters, where the
reference's formula (pymiecoated/mie_coeffs.py:124-128) loses about eps/x^2
of relative accuracy to cancellation in the numerator of b_n.  Used to show
that the GPU result is at least as close to the exact value as the reference.

    python tests/golden/make_exact.py
"""
import os

import mpmath as mp
import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
mp.mp.dps = 50


def psi(n, t):
    return mp.sqrt(mp.pi * t / 2) * mp.besselj(n + mp.mpf(1) / 2, t)


def chi(n, t):
    return -mp.sqrt(mp.pi * t / 2) * mp.bessely(n + mp.mpf(1) / 2, t)


def coeffs(m, x, nmax):
    m = mp.mpc(m)
    x = mp.mpf(x)
    z = m * x
    an, bn = [], []
    for n in range(1, nmax + 1):
        D = mp.diff(lambda s: psi(n, s), z) / psi(n, z)
        da = D / m + n / x
        db = D * m + n / x

        def xi(k):
            return psi(k, x) - 1j * chi(k, x)
        an.append((da * psi(n, x) - psi(n - 1, x)) / (da * xi(n) - xi(n - 1)))
        bn.append((db * psi(n, x) - psi(n - 1, x)) / (db * xi(n) - xi(n - 1)))
    return an, bn


def props(an, bn, x):
    x = mp.mpf(x)
    nmax = len(an)
    s = q = 0
    qb = 0
    for i in range(nmax):
        n = i + 1
        a1 = an[i + 1] if i + 1 < nmax else 0
        b1 = bn[i + 1] if i + 1 < nmax else 0
        s += mp.mpf(n * (n + 2)) / (n + 1) * mp.re(an[i] * mp.conj(a1) + bn[i] * mp.conj(b1)) \
            + mp.mpf(2 * n + 1) / (n * (n + 1)) * mp.re(an[i] * mp.conj(bn[i]))
        q += (2 * n + 1) * (abs(an[i]) ** 2 + abs(bn[i]) ** 2)
        qb += (2 * n + 1) * (-1) ** n * (an[i] - bn[i])
    qsca = 2 * q / x ** 2
    return float(4 / x ** 2 * s / qsca), float(qsca), float(abs(qb) ** 2 / x ** 2)


def main():
    xs, ms, g, qsca, qb = [], [], [], [], []
    for m in [1.33 + 1e-9j, 1.5 + 1e-8j, 1.53 + 0.008j, 1.95 + 0.79j]:
        for x in [1e-4, 3e-4, 1e-3, 3e-3, 1e-2, 3e-2, 0.1]:
            nmax = int(round(2 + x + 4 * x ** (1.0 / 3.0)))
            an, bn = coeffs(m, x, nmax)
            gg, qs, qbb = props(an, bn, x)
            xs.append(x)
            ms.append(m)
            g.append(gg)
            qsca.append(qs)
            qb.append(qbb)
    np.savez_compressed(os.path.join(HERE, "mie_exact_small_x.npz"), x=np.array(xs),
                        m=np.array(ms, dtype=np.complex128), g=np.array(g), qsca=np.array(qsca),
                        qb=np.array(qb))
    print("mie_exact_small_x: %d cases" % len(xs))


if __name__ == "__main__":
    main()
