/*
 * C restatement of gsf/spher_expan.f (GEOSmie) -- ORACLE / TEST INFRASTRUCTURE.
 *
 * Used by tests/, __graft_entry__.smoke() and bench.py's CPU legs only; the
 * product library never links it.  The reference is a Fortran 77 program run
 * once per table entry through text files (gsf/convertncdf.py:173-189); no
 * Fortran compiler exists in this image, so the algorithm is restated here
 * routine by routine, in double precision, with the same loop bounds:
 *
 *   gsf_gauss      GAUSS       spher_expan.f:520-579  (IND1 = 0: nodes on
 *                                                      [-1,1], weights x2)
 *   gsf_linterpol  LINTERPOL   spher_expan.f:593-623  (IEX = 1: linear
 *                                                      extrapolation)
 *   gsf_gener      GENER       spher_expan.f:363-407  (loop to LMAX = L1MAX-1,
 *                                                      fills index L1MAX)
 *   gsf_expand_one one_calc + SPHER_EXPAN + the 1/alpha1(0) normalisation of
 *                  the main program, spher_expan.f:93-107,120-180,269-358
 *   gsf_matr       MATR        spher_expan.f:419-517  (reconstruction)
 *
 * Element order in and out follows the reference: input F = [F11, F22, F33,
 * F44, F12, F34] on the table angles (degrees), output coefficients
 * [alpha1, alpha2, alpha3, alpha4, beta1, beta2] for l = 0..L1MAX-1.
 * NANG_MAX (1000) and NG_MAX are not imposed: arrays are sized by the caller.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

/* GAUSS(N, IND1=0, IND2=0, Z, W): Newton iteration on the Legendre
 * polynomial, nodes ascending (Z(1) ~ -1), weights multiplied by 2. */
void gsf_gauss(int n, double *z, double *w)
{
    const double A = 1.0, B = 2.0, C = 3.0;
    int ind = n % 2;
    int k = n / 2 + ind;
    double f = (double)n;
    for (int i = 1; i <= k; ++i) {
        int m = n + 1 - i;
        double x = 0.0, pa, pb, pc, dj, check;
        if (i == 1) x = A - B / ((f + A) * f);
        if (i == 2) x = (z[n - 1] - A) * 4.0 + z[n - 1];
        if (i == 3) x = (z[n - 2] - z[n - 1]) * 1.6 + z[n - 2];
        if (i > 3) x = (z[m] - z[m + 1]) * C + z[m + 2];
        if (i == k && ind == 1) x = 0.0;
        int niter = 0;
        check = 1e-16;
        for (;;) {
            pb = 1.0;
            niter++;
            if (niter > 100) check *= 10.0;
            pc = x;
            dj = A;
            for (int j = 2; j <= n; ++j) {
                dj += A;
                pa = pb;
                pb = pc;
                pc = x * pb + (x * pb - pa) * (dj - A) / dj;
            }
            pa = A / ((pb - x * pc) * f);
            pb = pa * pc * (A - x * x);
            x = x - pb;
            if (!(fabs(pb) > check * fabs(x))) break;
        }
        z[m - 1] = x;
        w[m - 1] = pa * pa * (A - x * x);
        w[m - 1] = B * w[m - 1];
        if (i == k && ind == 1) continue;
        z[i - 1] = -z[m - 1];
        w[i - 1] = w[m - 1];
    }
}

/* LINTERPOL with IEX = 1. */
double gsf_linterpol(int nn, const double *xx, const double *yy, double x)
{
    if (x < xx[0])
        return (yy[0] - yy[1]) / (xx[0] - xx[1]) * (x - xx[0]) + yy[0];
    if (x > xx[nn - 1])
        return (yy[nn - 1] - yy[nn - 2]) / (xx[nn - 1] - xx[nn - 2]) * (x - xx[nn - 1]) + yy[nn - 1];
    int i;
    for (i = 2; i <= nn; ++i)
        if (xx[i - 1] > x) break;
    if (i > nn) i = nn; /* DO-loop exit value when no XX(I) > X */
    return (yy[i - 1] - yy[i - 2]) / (xx[i - 1] - xx[i - 2]) * (x - xx[i - 2]) + yy[i - 2];
}

/* Recurrence coefficients, SPHER_EXPAN loop 150 (1-based index L1 = 3..L1MAX). */
static void gsf_coefs(int l1max, double *c /* [8][l1max+2] */)
{
    int s = l1max + 2;
    for (int l1 = 3; l1 <= l1max; ++l1) {
        int l = l1 - 1;
        c[0 * s + l1] = 1.0 / (double)(l + 1);
        c[1 * s + l1] = (double)(2 * l + 1);
        c[2 * s + l1] = 1.0 / sqrt((double)((l + 1) * (l + 1) - 4));
        c[3 * s + l1] = sqrt((double)(l * l - 4));
        c[4 * s + l1] = 1.0 / ((double)l * (double)((l + 1) * (l + 1) - 4));
        c[5 * s + l1] = (double)(2 * l + 1) * (double)(l * (l + 1));
        c[6 * s + l1] = (double)((2 * l + 1) * 4);
        c[7 * s + l1] = (double)(l + 1) * (double)(l * l - 4);
    }
}

/* GENER(U, L1MAX): P1..P4 at 1-based indices 1..L1MAX (arrays sized l1max+2). */
void gsf_gener(double u, int l1max, const double *c, double *p1, double *p2, double *p3, double *p4)
{
    int s = l1max + 2;
    const double d6 = 0.25 * sqrt(6.0);
    double dup = 1.0 + u, dum = 1.0 - u, du = u * u;
    p1[1] = 1.0; p1[2] = u; p1[3] = 0.5 * (3.0 * du - 1.0);
    p2[1] = 0.0; p2[2] = 0.0; p2[3] = 0.25 * dup * dup;
    p3[1] = 0.0; p3[2] = 0.0; p3[3] = 0.25 * dum * dum;
    p4[1] = 0.0; p4[2] = 0.0; p4[3] = d6 * (du - 1.0);
    int lmax = l1max - 1;
    for (int l1 = 3; l1 <= lmax; ++l1) {
        double c1 = c[0 * s + l1], c2 = c[1 * s + l1], c3 = c[2 * s + l1], c4 = c[3 * s + l1];
        double c5 = c[4 * s + l1], c6 = c[5 * s + l1], c7 = c[6 * s + l1], c8 = c[7 * s + l1];
        double cu1 = c2 * u, cu2 = c6 * u;
        int l2 = l1 + 1, l3 = l1 - 1;
        double dl = (double)l3;
        p1[l2] = c1 * (cu1 * p1[l1] - dl * p1[l3]);
        p2[l2] = c5 * ((cu2 - c7) * p2[l1] - c8 * p2[l3]);
        p3[l2] = c5 * ((cu2 + c7) * p3[l1] - c8 * p3[l3]);
        p4[l2] = c3 * (cu1 * p4[l1] - c4 * p4[l3]);
    }
}

/* One table entry: nodes/weights (ng), interpolation from the table angles
 * (degrees, ascending) to acos(node), expansion, normalisation by alpha1(0).
 * f: [6][nang] in order F11 F22 F33 F44 F12 F34.  coef: [6][ng].
 * Returns CNORM = 1/alpha1(0) (written by the reference as the header line). */
double gsf_expand_one(int nang, const double *ang_deg, const double *f, int ng,
                      const double *x, const double *w, const double *c,
                      double *work, double *coef)
{
    int l1max = ng;
    int s = l1max + 2;
    double *angl = work;              /* nang */
    double *p1 = angl + nang, *p2 = p1 + s, *p3 = p2 + s, *p4 = p3 + s;
    const double d2r = acos(-1.0) / 180.0;
    for (int i = 0; i < nang; ++i) angl[i] = ang_deg[i] * d2r;
    double *al1 = coef, *al2 = coef + ng, *al3 = coef + 2 * ng, *al4 = coef + 3 * ng;
    double *be1 = coef + 4 * ng, *be2 = coef + 5 * ng;
    memset(coef, 0, sizeof(double) * 6 * ng);
    for (int i = 0; i < ng; ++i) {
        double ang = acos(x[i]);
        double F[6];
        for (int e = 0; e < 6; ++e) F[e] = gsf_linterpol(nang, angl, f + e * nang, ang);
        gsf_gener(x[i], l1max, c, p1, p2, p3, p4);
        double wi = w[i];
        double ff11 = F[0] * wi, ff22 = F[1] * wi, ff33 = F[2] * wi, ff44 = F[3] * wi;
        double ff12 = F[4] * wi, ff34 = F[5] * wi;
        double fp = ff22 + ff33, fm = ff22 - ff33;
        for (int l1 = 1; l1 <= l1max; ++l1) {
            double p1l1 = p1[l1], p4l1 = p4[l1];
            al1[l1 - 1] += ff11 * p1l1;
            al4[l1 - 1] += ff44 * p1l1;
            al2[l1 - 1] += fp * p2[l1];
            al3[l1 - 1] += fm * p3[l1];
            be1[l1 - 1] += ff12 * p4l1;
            be2[l1 - 1] += ff34 * p4l1;
        }
    }
    for (int l1 = 1; l1 <= l1max; ++l1) {
        double cl = (double)(l1 - 1) + 0.5;
        al1[l1 - 1] *= cl;
        double a2 = al2[l1 - 1] * cl * 0.5, a3 = al3[l1 - 1] * cl * 0.5;
        al2[l1 - 1] = a2 + a3;
        al3[l1 - 1] = a2 - a3;
        al4[l1 - 1] *= cl;
        be1[l1 - 1] *= cl;
        be2[l1 - 1] *= cl;
    }
    double cnorm = 1.0 / al1[0];
    for (int k = 0; k < 6 * ng; ++k) coef[k] *= cnorm;
    return cnorm;
}

/* Batched driver: ntab entries sharing one angle grid and one node count. */
int gsf_expand(int ntab, int nang, const double *ang_deg, const double *f,
               int ng, double *coef, double *cnorm)
{
    if (ntab < 0 || nang < 2 || ng < 3) return 1;
    double *x = (double *)malloc(sizeof(double) * ng);
    double *w = (double *)malloc(sizeof(double) * ng);
    double *c = (double *)calloc((size_t)8 * (ng + 2), sizeof(double));
    double *work = (double *)malloc(sizeof(double) * (nang + 4 * (ng + 2)));
    if (!x || !w || !c || !work) { free(x); free(w); free(c); free(work); return 2; }
    gsf_gauss(ng, x, w);
    gsf_coefs(ng, c);
    for (int t = 0; t < ntab; ++t) {
        double cn = gsf_expand_one(nang, ang_deg, f + (size_t)t * 6 * nang, ng, x, w, c,
                                   work, coef + (size_t)t * 6 * ng);
        if (cnorm) cnorm[t] = cn;
    }
    free(x); free(w); free(c); free(work);
    return 0;
}

/* MATR: reconstruct F11 F22 F33 F44 F12 F34 at angles (radians) from the
 * coefficients a1..b2 (l = 0..lmax).  out: [6][nang]. */
void gsf_matr(const double *a1, const double *a2, const double *a3, const double *a4,
              const double *b1, const double *b2, int lmax, int nang, const double *angl,
              double *out)
{
    int l1max = lmax + 1;
    double d6 = sqrt(6.0) * 0.25;
    for (int i1 = 0; i1 < nang; ++i1) {
        double u = cos(angl[i1]);
        double f11 = 0, f2 = 0, f3 = 0, f44 = 0, f12 = 0, f34 = 0;
        double pp1 = 1.0, pp2 = 0.25 * (1 + u) * (1 + u), pp3 = 0.25 * (1 - u) * (1 - u);
        double pp4 = d6 * (u * u - 1.0);
        double q1 = 0, q2 = 0, q3 = 0, q4 = 0, p;
        for (int l1 = 1; l1 <= l1max; ++l1) {
            int l = l1 - 1;
            double dl = (double)l, dl1 = (double)l1;
            f11 += a1[l1 - 1] * pp1;
            f44 += a4[l1 - 1] * pp1;
            double pl1 = (double)(2 * l + 1);
            if (l != lmax) {
                p = (pl1 * u * pp1 - dl * q1) / dl1;
                q1 = pp1;
                pp1 = p;
            }
            if (l < 2) continue;
            f2 += (a2[l1 - 1] + a3[l1 - 1]) * pp2;
            f3 += (a2[l1 - 1] - a3[l1 - 1]) * pp3;
            f12 += b1[l1 - 1] * pp4;
            f34 += b2[l1 - 1] * pp4;
            if (l == lmax) continue;
            double pl2 = dl * dl1 * u, pl3 = dl1 * (dl * dl - 4.0);
            double pl4 = 1.0 / (dl * (dl1 * dl1 - 4.0));
            p = (pl1 * (pl2 - 4.0) * pp2 - pl3 * q2) * pl4;
            q2 = pp2; pp2 = p;
            p = (pl1 * (pl2 + 4.0) * pp3 - pl3 * q3) * pl4;
            q3 = pp3; pp3 = p;
            p = (pl1 * u * pp4 - sqrt(dl * dl - 4.0) * q4) / sqrt(dl1 * dl1 - 4.0);
            q4 = pp4; pp4 = p;
        }
        out[0 * nang + i1] = f11;
        out[1 * nang + i1] = (f2 + f3) * 0.5;
        out[2 * nang + i1] = (f2 - f3) * 0.5;
        out[3 * nang + i1] = f44;
        out[4 * nang + i1] = f12;
        out[5 * nang + i1] = f34;
    }
}
