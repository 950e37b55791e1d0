// Per-instance Mie device functions (FP64): Riccati-Bessel rows, homogeneous
// and coated coefficients with fused efficiency sums.
#pragma once
#include "df.cuh"
#include "common.cuh"

// ---------------------------------------------------------------------------
// Riccati-Bessel psi_n(z) = z j_n(z) by Miller's algorithm.
//
// The reference takes psi_n = sqrt(pi z/2) J_{n+1/2}(z) from scipy
// (pymiecoated/mie_coeffs.py:154-164, :223).  Here the three-term recurrence
// psi_{n-1} = (2n+1)/z psi_n - psi_{n+1} runs DOWNWARD (the stable direction
// for this minimal solution) from psi^_{N+1} = 0, psi^_N = 1 at
// N = max(nmax, |z|) + 16 + 4 |z|^(1/3), and the unnormalised sequence is
// scaled by the least-squares fit of (psi^_0, psi^_1) to the closed forms
// psi_0 = sin z, psi_1 = sin z / z - cos z.  Those two never vanish together,
// so the scale is well conditioned at every z -- including the zeros of
// psi_n (e.g. x = k pi), where an upward product of ratios psi_n/psi_{n-1}
// loses all accuracy.  Values grow downward where n > |z|; they are rescaled
// by 1e-100 whenever they pass 1e100.  Checked against 40-digit mpmath: error
// below 4e-15 of the local magnitude for real and complex z up to |z| = 630.
// ---------------------------------------------------------------------------
__device__ __forceinline__ int miller_start(double az, int nmax)
{
    const int top = nmax > (int)ceil(az) ? nmax : (int)ceil(az);
    return psi_start(az, top);
}

// Real argument: psi_n(x), chi_n(x) for n = 1..nmax written to row1[n-1]
// (order 0 is (sin x, cos x) and is not stored); chi_n = -x y_n(x) by the
// upward recurrence from chi_0 = cos x, chi_{-1} = -sin x (stable: chi is
// the dominant solution).  row1 may alias the coefficient output (the
// homogeneous kernels overwrite it in place).
// pair (or NULL): the same rows also as FP32 pairs (psi hi, lo, chi hi, lo)
// at pair[(n - 1) * pstride], for the mixed recurrences.  row1 == NULL (with
// pair): no FP64 rows; the unnormalised psi values are parked in the first
// 8 bytes of each pair slot instead.
__device__ __forceinline__ void psi_chi_row(double x, int nmax, double2 *row1, float4 *pair = nullptr, int pstride = 1)
{
    const int N = miller_start(x, nmax);
    const double xinv = 1.0 / x;
    // the unnormalised psi of order k (1..nmax)
    auto park = [&](int k) -> double & {
        return row1 ? row1[k - 1].x : *(double *)(pair + (size_t)(k - 1) * pstride);
    };
    double pn1 = 0.0, pn = 1.0;   // psi^_{n+1}, psi^_n
    for (int n = N; n >= 1; --n) {
        const double pm = (double)(2 * n + 1) * xinv * pn - pn1;
        pn1 = pn;
        pn = pm;
        if (n - 1 >= 1 && n - 1 <= nmax) park(n - 1) = pm;
        if (fabs(pm) > 1e100) {
            pn *= 1e-100;
            pn1 *= 1e-100;
            for (int k = (n - 1 >= 1 ? n - 1 : 1); k <= nmax; ++k) park(k) *= 1e-100;
        }
    }
    double s, c;
    sincos(x, &s, &c);
    const double psi1 = s * xinv - c;
    const double scale = (pn * s + pn1 * psi1) / (pn * pn + pn1 * pn1);
    double chi = c, chim1 = -s;
    // the unnormalised psi values are read back in groups of 8 independent
    // loads ahead of their use: read one at a time, each order waited for a
    // round trip to L2 (the row was just written), and rows of a few hundred
    // orders took that many round trips in sequence
    for (int n0 = 1; n0 <= nmax; n0 += 8) {
        double pr[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) pr[j] = park(min(n0 + j, nmax));
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const int n = n0 + j;
            if (n > nmax) continue;
            const double chin = (double)(2 * n - 1) * xinv * chi - chim1;
            chim1 = chi;
            chi = chin;
            const double psi = scale * pr[j];
            if (row1) row1[n - 1] = make_double2(psi, chi);
            if (pair) {
                const float ph = __double2float_rn(psi), ch = __double2float_rn(chi);
                pair[(size_t)(n - 1) * pstride] = make_float4(ph, __double2float_rn(psi - (double)ph), ch,
                                                              __double2float_rn(chi - (double)ch));
            }
        }
    }
}

// Complex argument: psi_n(z), n = 1..nmax, to out[(n-1) * stride].
__device__ __forceinline__ void psi_row_complex(cplx z, int nmax, double2 *out, int stride)
{
    const int N = miller_start(cabs(z), nmax);
    const cplx zinv = cinv(z);
    cplx pn1 = cx(0.0, 0.0), pn = cx(1.0, 0.0);
    for (int n = N; n >= 1; --n) {
        const cplx pm = zinv * (double)(2 * n + 1) * pn - pn1;
        pn1 = pn;
        pn = pm;
        if (n - 1 >= 1 && n - 1 <= nmax) out[(size_t)(n - 2) * stride] = d2(pm);
        if (fabs(pm.re) + fabs(pm.im) > 1e100) {
            pn = pn * 1e-100;
            pn1 = pn1 * 1e-100;
            for (int k = (n - 1 >= 1 ? n - 1 : 1); k <= nmax; ++k) {
                double2 &o = out[(size_t)(k - 1) * stride];
                o.x *= 1e-100;
                o.y *= 1e-100;
            }
        }
    }
    const cplx s = csin(z), c = ccos(z);
    const cplx psi1 = s * zinv - c;
    const cplx scale = (conjg(pn) * s + conjg(pn1) * psi1) * (1.0 / (abs2(pn) + abs2(pn1)));
    // read back in groups of 8 independent loads (see psi_chi_row)
    for (int n0 = 1; n0 <= nmax; n0 += 8) {
        double2 pr[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) pr[j] = out[(size_t)(min(n0 + j, nmax) - 1) * stride];
#pragma unroll
        for (int j = 0; j < 8; ++j)
            if (n0 + j <= nmax) out[(size_t)(n0 + j - 1) * stride] = d2(scale * cx(pr[j]));
    }
}

// Running efficiency sums of pymiecoated/mie_props.py:28-70, accumulated in
// the order coefficients are produced.
struct EffSums {
    static constexpr bool needs_inv_n = true;   // add_rcp takes 1/n
    double ext, sca, asy;
    cplx qb;
    cplx a1, b1;   // a_{n+1}, b_{n+1} of the previous (higher) order
    __device__ __forceinline__ void init() {
        ext = sca = asy = 0.0;
        qb = a1 = b1 = cx(0.0, 0.0);
    }
    // terms of order n given a_{n+1}, b_{n+1} (zero above nmax, mie_props.py:61-62)
    __device__ __forceinline__ void term(int n, cplx a, cplx b, cplx an1, cplx bn1) {
        const double dn = (double)n;
        const double cn = 2.0 * dn + 1.0;
        ext += cn * (a.re + b.re);
        sca += cn * (abs2(a) + abs2(b));
        const double sg = (n & 1) ? -cn : cn;   // (2n+1)(-1)^n
        qb = qb + (a - b) * sg;
        asy += dn * (dn + 2.0) / (dn + 1.0) * (a.re * an1.re + a.im * an1.im + b.re * bn1.re + b.im * bn1.im)
             + cn / (dn * (dn + 1.0)) * (a.re * b.re + a.im * b.im);
    }
    // order n, descending n = nmax..1
    __device__ __forceinline__ void add(int n, cplx a, cplx b) {
        term(n, a, b, a1, b1);
        a1 = a;
        b1 = b;
    }
    // the same with the reciprocals 1/n and 1/(n+1) supplied:
    // n (n+2)/(n+1) = (n+1) - 1/(n+1) and (2n+1)/(n (n+1)) = 1/n + 1/(n+1)
    __device__ __forceinline__ void add_rcp(int n, cplx a, cplx b, double inv_n, double inv_n1) {
        const double dn = (double)n;
        const double cn = 2.0 * dn + 1.0;
        ext += cn * (a.re + b.re);
        sca += cn * (abs2(a) + abs2(b));
        const double sg = (n & 1) ? -cn : cn;
        qb = qb + (a - b) * sg;
        asy += ((dn + 1.0) - inv_n1) * (a.re * a1.re + a.im * a1.im + b.re * b1.re + b.im * b1.im)
             + (inv_n + inv_n1) * (a.re * b.re + a.im * b.im);
        a1 = a;
        b1 = b;
    }
    // qext, qsca, qabs, qb, asy, qratio for outer size y
    __device__ __forceinline__ void finish(double y, double *e) const {
        const double y2 = y * y;
        const double qext = 2.0 * ext / y2;
        const double qsca = 2.0 * sca / y2;
        const double qbv = abs2(qb) / y2;
        e[0] = qext;
        e[1] = qsca;
        e[2] = qext - qsca;
        e[3] = qbv;
        e[4] = 4.0 / y2 * asy / qsca;
        e[5] = qbv / qsca;
    }
};

// a = N / (N - i M) with N = d psi_n - psi_{n-1}, M = d chi_n - chi_{n-1}:
// the quotient (d psi_n - psi_{n-1}) / (d xi_n - xi_{n-1}), xi = psi - i chi.
__device__ __forceinline__ cplx mie_ratio(cplx d, double psin, double chin, double psim, double chim)
{
    const cplx N = cx(d.re * psin - psim, d.im * psin);
    const cplx M = cx(d.re * chin - chim, d.im * chin);
    return N / cx(N.re + M.im, N.im - M.re);
}

// ---------------------------------------------------------------------------
// Homogeneous sphere, pymiecoated/mie_coeffs.py:83-130/132-180.
// D_n(z), z = sqrt(eps mu) x, by the reference's downward recurrence
// D_n = r - 1/(D_{n+1} + r), r = (n+1)/z, from D_nmx = 0 at
// nmx = round(max(nmax, |z|) + 16); a_n with da = D_n/m + n/x, b_n with
// db = D_n m + n/x, m = sqrt(eps/mu).  Coefficients are produced from n = nmax
// down to 1 and handed to emit(n, a_n, b_n); the efficiency sums ride along.
// row1: psi/chi of x for orders 1..nmax at row1[n-1]; it may alias the
// emitter's a_n output (row n is consumed before a_n is written).
// ---------------------------------------------------------------------------
// Medium constants of the homogeneous recurrences: z = zm x with
// zm = sqrt(eps mu) and the relative index m = sqrt(eps / mu)
// (pymiecoated/mie_coeffs.py:144-145), their reciprocals and |zm|.  They
// depend on the medium only, so a table computes them once per
// (wavelength, RH, component) unit.
struct HomogIndex {
    cplx zm, zminv, m, minv;
    double azm;
};

__device__ __forceinline__ HomogIndex homog_index(cplx eps, cplx mu)
{
    HomogIndex h;
    h.zm = csqrt(eps * mu);
    h.m = csqrt(eps / mu);
    h.zminv = cinv(h.zm);
    h.minv = cinv(h.m);
    h.azm = cabs(h.zm);
    return h;
}

// The recurrences of one instance given the medium constants and the size
// constants 1/x, sin x, cos x (a table computes those once per size row).
template <class Emit, class Sums>
__device__ __forceinline__ void homog_core(double x, double xinv, double sx, double cxv, const HomogIndex &h,
                                           const double2 *row1, int nmax, Emit &emit, Sums &es)
{
    const cplx m = h.m;
    const cplx minv = h.minv;
    const double az = h.azm * x;
    const int nmx = (int)rint(fmax((double)nmax, az) + 16.0);
    const cplx zinv = h.zminv * xinv;
    // Warm-up steps above nmax.  The reference runs nmx - 1 - nmax of them
    // from D = 0 (mie_coeffs.py:150, 168-170).  For n > |z| the recurrence
    // damps the start error by (|z| / (2n+1))^2 per step, so when
    // |z| < (nmax+1)/2 fewer steps reach the same converged D_nmax (damping
    // below 1e-17, plus two spare steps; the step count needs no FP64 log).
    int warm = nmx - 1 - nmax;
    if (az < 0.5 * (nmax + 1)) {
        const float q = 2.f * logf((2.f * (float)(nmax + 1) + 1.f) / (float)az);   // -ln(damping) per step
        const int need = (int)ceilf(39.2f / q) + 2;
        if (need < warm) warm = need;
    }
    cplx D = cx(0.0, 0.0);
    for (int k = nmax + warm; k > nmax; --k) {
        const cplx r = zinv * (double)(k + 1);
        D = r - cinv(D + r);
    }
    double2 pcn = row1[nmax - 1];
    es.init();
    // One reciprocal per order: at order k the denominators of a_k, b_k and
    // of the next D step (D_k + r_{k-1}) and k itself are inverted together,
    // 1/(A B C k), and the four reciprocals recovered by multiplication.
    cplx rk1 = zinv * (double)(nmax + 1);             // r_nmax = (nmax+1)/z
    cplx w = D + rk1;                                  // D_{nmax+1} + r_nmax
    double inv_w2 = 1.0 / abs2(w);                     // 1/|w|^2 for D_nmax
    double inv_n1 = 1.0 / (double)(nmax + 1);          // 1/(k+1)
    for (int k = nmax; k >= 1; --k) {
        const double dk = (double)k;
        const cplx r = rk1;                            // (k+1)/z
        D = cx(fma(-w.re, inv_w2, r.re), fma(w.im, inv_w2, r.im));   // D_k = r - 1/w
        const double2 pcm = (k > 1) ? row1[k - 2] : make_double2(sx, cxv);
        const double nx = dk * xinv;
        // da = D/m + k/x, db = D m + k/x
        const cplx da = cx(fma(D.re, minv.re, fma(-D.im, minv.im, nx)), fma(D.re, minv.im, D.im * minv.re));
        const cplx db = cx(fma(D.re, m.re, fma(-D.im, m.im, nx)), fma(D.re, m.im, D.im * m.re));
        const cplx Na = cx(da.re * pcn.x - pcm.x, da.im * pcn.x);
        const cplx Ma = cx(da.re * pcn.y - pcm.y, da.im * pcn.y);
        const cplx Nb = cx(db.re * pcn.x - pcm.x, db.im * pcn.x);
        const cplx Mb = cx(db.re * pcn.y - pcm.y, db.im * pcn.y);
        const cplx qa = cx(Na.re + Ma.im, Na.im - Ma.re);   // N - i M
        const cplx qbv = cx(Nb.re + Mb.im, Nb.im - Mb.re);
        const double A = abs2(qa), B = abs2(qbv);
        rk1 = zinv * dk;                                   // r_{k-1} = k/z
        w = D + rk1;                                       // D_k + r_{k-1}
        const double C = (k > 1) ? abs2(w) : 1.0;
        const double AB = A * B, ABC = AB * C;
        double t, inv_n = 0.0;                             // 1/(A B C), 1/k
        if (Sums::needs_inv_n) {
            const double inv = 1.0 / (ABC * dk);
            inv_n = ABC * inv;
            t = dk * inv;
        } else {
            t = 1.0 / ABC;
        }
        inv_w2 = AB * t;                                   // 1/C
        const double u = C * t;                            // 1/(A B)
        const double ia = B * u, ib = A * u;               // 1/A, 1/B
        const cplx a = cx((Na.re * qa.re + Na.im * qa.im) * ia, (Na.im * qa.re - Na.re * qa.im) * ia);
        const cplx b = cx((Nb.re * qbv.re + Nb.im * qbv.im) * ib, (Nb.im * qbv.re - Nb.re * qbv.im) * ib);
        emit(k, a, b);
        es.add_rcp(k, a, b, inv_n, inv_n1);
        inv_n1 = inv_n;
        pcn = pcm;
    }
}

// One instance from (x, eps, mu) alone.
template <class Emit, class Sums>
__device__ __forceinline__ void homog_instance(double x, cplx eps, cplx mu, const double2 *row1, int nmax,
                                               Emit &emit, Sums &es)
{
    const HomogIndex h = homog_index(eps, mu);
    double sx, cxv;
    sincos(x, &sx, &cxv);
    homog_core(x, 1.0 / x, sx, cxv, h, row1, nmax, emit, es);
}

// ---------------------------------------------------------------------------
// Coated sphere, pymiecoated/mie_coeffs.py:183-251.
// D_n at u = m1 x, v = m2 x, w = m2 y from one start
// nmax = round(max(nmax, max(|m1 y|, |m2 y|)) + 16) (the reference's), parked
// in dscr[5 (n-1) + {0,1,2}] for n <= nmax; psi_n(v), psi_n(w) by Miller's
// algorithm in dscr[5 (n-1) + {3,4}]; then upward: chi_n(v), chi_n(w) by the
// upward recurrence from cos / -sin (psi and chi are the functions the
// reference takes from scipy jv/yv of complex argument), the reference's ratio chain
// (uu, vv, fv, ku1, kv1, pt, prat, ku2, kv2 -> dns, gns) and a_n, b_n at y.
// Coefficients are emitted n = 1..nmax (ascending).  rowy1: psi/chi of y for
// orders 1..nmax at rowy1[n-1]; it may alias the emitter's a_n output.
// ---------------------------------------------------------------------------
//
// DFD (the mixed table path): the three downward D_n recurrences in
// double-float pairs (df.cuh, about 2^-46) instead of FP64, from the same
// start; the values are widened to FP64 for the ratio chain, which stays in
// FP64 with everything after it.  On GB300 the FP64 pipe issues a small
// fraction of the FP32 rate, and these recurrences (three arguments, up to
// max(|m1 y|, |m2 y|) + 16 steps each) were about half of the FP64 work of a
// coated instance.
template <class Emit, bool DFD = false>
__device__ __forceinline__ void coated_instance(double x, double y, cplx eps1, cplx eps2,
                                                const double2 *rowy1, int nmax,
                                                double2 *__restrict__ dscr, Emit &emit, EffSums &es)
{
    const cplx m1 = csqrt(eps1);
    const cplx m2 = csqrt(eps2);
    const cplx m = m2 / m1;
    const cplx minv = m1 / m2;
    const cplx u = m1 * x, v = m2 * x, w = m2 * y;
    const double mx = fmax(cabs(m1 * y), cabs(w));
    const int nmx = (int)rint(fmax((double)nmax, mx) + 16.0);
    const cplx uinv = cinv(u), vinv = cinv(v), winv = cinv(w);
    if (DFD) {
        const cdf zi[3] = {cdf{df_from_f64(uinv.re), df_from_f64(uinv.im)},
                           cdf{df_from_f64(vinv.re), df_from_f64(vinv.im)},
                           cdf{df_from_f64(winv.re), df_from_f64(winv.im)}};
        cdf D[3];
#pragma unroll
        for (int j = 0; j < 3; ++j) D[j] = cdf{df{0.f, 0.f}, df{0.f, 0.f}};
        for (int k = nmx - 1; k >= 1; --k) {
            const float kp = (float)(k + 1);
#pragma unroll
            for (int j = 0; j < 3; ++j) {
                const cdf r = cdf_mul_f(zi[j], kp);   // (k+1)/z
                const cdf wv = cdf_add(D[j], r);
                const df iw = df_rcp(df_fma(wv.re, wv.re, df_mul(wv.im, wv.im)));
                D[j] = cdf{df_fma(df_neg(wv.re), iw, r.re), df_fma(wv.im, iw, r.im)};   // r - 1/w
                if (k <= nmax)
                    dscr[5 * (k - 1) + j] = make_double2((double)D[j].re.hi + (double)D[j].re.lo,
                                                         (double)D[j].im.hi + (double)D[j].im.lo);
            }
        }
    } else {
        cplx Du = cx(0, 0), Dv = cx(0, 0), Dw = cx(0, 0);
        for (int k = nmx - 1; k >= 1; --k) {
            const double kp = (double)(k + 1);
            const cplx ru = uinv * kp, rv = vinv * kp, rw = winv * kp;
            Du = ru - cinv(Du + ru);
            Dv = rv - cinv(Dv + rv);
            Dw = rw - cinv(Dw + rw);
            if (k <= nmax) {
                dscr[5 * (k - 1) + 0] = d2(Du);
                dscr[5 * (k - 1) + 1] = d2(Dv);
                dscr[5 * (k - 1) + 2] = d2(Dw);
            }
        }
    }
    psi_row_complex(v, nmax, dscr + 3, 5);
    psi_row_complex(w, nmax, dscr + 4, 5);
    cplx chv = ccos(v), chw = ccos(w);
    cplx chvm = -csin(v), chwm = -csin(w);
    const double yinv = 1.0 / y;
    // The asymmetry term of order n needs a_{n+1}: coefficients come out
    // ascending here, so each order is summed one step late.
    es.init();
    cplx ap = cx(0, 0), bp = cx(0, 0);
    double sy, cy;
    sincos(y, &sy, &cy);
    double2 pcm = make_double2(sy, cy);
    for (int k = 1; k <= nmax; ++k) {
        const cplx dU = cx(dscr[5 * (k - 1) + 0]);
        const cplx dV = cx(dscr[5 * (k - 1) + 1]);
        const cplx dW = cx(dscr[5 * (k - 1) + 2]);
        const cplx pv = cx(dscr[5 * (k - 1) + 3]);
        const cplx pw = cx(dscr[5 * (k - 1) + 4]);
        const double dk = (double)k;
        const cplx chvn = vinv * (2.0 * dk - 1.0) * chv - chvm;
        chvm = chv;
        chv = chvn;
        const cplx chwn = winv * (2.0 * dk - 1.0) * chw - chwm;
        chwm = chw;
        chw = chwn;
        const cplx uu = m * dU - dV;
        const cplx vv = dU * minv - dV;
        const cplx fv = pv / chv;
        const cplx pwinv = cinv(pw);
        const cplx ku1 = uu * fv * pwinv;
        const cplx kv1 = vv * fv * pwinv;
        const cplx pt = pw - chw * fv;
        const cplx prat = pw / pv / chv;
        const cplx ku2 = uu * pt + prat;
        const cplx kv2 = vv * pt + prat;
        const cplx dns = ku1 / ku2 + dW;
        const cplx gns = kv1 / kv2 + dW;
        const double nr = dk * yinv;
        const double2 pcn = rowy1[k - 1];
        const cplx a = mie_ratio(dns / m2 + nr, pcn.x, pcn.y, pcm.x, pcm.y);
        const cplx b = mie_ratio(m2 * gns + nr, pcn.x, pcn.y, pcm.x, pcm.y);
        emit(k, a, b);
        if (k > 1) es.term(k - 1, ap, bp, a, b);
        ap = a;
        bp = b;
        pcm = pcn;
    }
    es.term(nmax, ap, bp, cx(0, 0), cx(0, 0));
}
