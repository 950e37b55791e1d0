// Mixed-precision table path: tensor-core (tcgen05) angular contraction with
// the Mueller elements and the size-distribution integration fused into the
// epilogue.
//
// The recurrences keep FP64 where stability needs it (k_tab_coeffs_mixed:
// D_n, psi/chi rows, the cancelling real parts of the a_n/b_n numerators and
// denominators); the ratio and the efficiency sums are FP32.  The
// coefficients leave it as FP32
//   c_n = a_n + b_n,  d_n = a_n - b_n   (float4 per order)
// with a per-instance exponent e_i = floor(log2 max |c|, |d|).  The two
// contractions
//   S+ = S1 + S2 = sum_n c_n (pi~_n + tau~_n),   S- = S1 - S2 = sum_n d_n (pi~_n - tau~_n)
// are GEMMs [instances x orders] x [orders x angles]: rows are (instance,
// Re/Im) pairs, 64 instances = M 128 per tile; columns are angles in blocks of
// 64 (N).  Each operand is split into FP16 hi + lo halves (values
// scaled by 2^(13 - e_i) so the row maximum sits just below 2^14), and
//   C P ~ C_hi P_hi + C_hi P_lo + C_lo P_hi
// is accumulated in FP32 in tensor memory: three tcgen05.mma per product and
// K step of 16 orders, six per step for S+ and S- (in windows of 48 orders,
// cross products first, see below).  The epilogue reads S+/S-
// rows from TMEM (tcgen05.ld), pairs Re/Im lanes, forms s11, s12, s33, s34
// and reduces them over the tile's 64 sizes with the PSD weights of every
// bin (the weights absorb 2^(2(e_i - E)) with E the unit's largest
// exponent), accumulating per unit in FP64.  Per-size phase matrices never
// reach global memory.
#include "common.cuh"
#include "mie_device.cuh"
#include "table_internal.cuh"
#include "tc.cuh"

#define TC_INST 64        // sizes per tile (M = 128 rows: Re, Im)
#define TC_NBLK 64        // angles per column block (N)
#define SHIFT_BITS 13

// ---------------------------------------------------------------------------
// Mixed-precision coefficients: FP32 (c, d) + exponent
// ---------------------------------------------------------------------------
// 1/c (c > 0) in FP64: the PTX approximate reciprocal (rcp.approx.ftz.f64)
// as the seed and one Newton-Raphson step (e = 1 - c y, y <- y + y e: the
// relative error squares), far below the FP32 coefficients this path emits.
// Emulated for x up to 650 with a 2^-23 seed: coefficients within 2.2e-7 of
// the instance maximum, the same as with the exact reciprocal, while the
// bare seed gives 1.3e-4.  No range test: the approximate reciprocal covers
// the normal FP64 range, and c = |D + r|^2 > 0 here (a zero would be a
// breakdown of the recurrence itself); FP64 comparisons would occupy the
// FP64 pipe this kernel is bound by.
__device__ __forceinline__ double rcp_newton(double c)
{
    double y;
    asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(c));
    return fma(y, fma(-c, y, 1.0), y);
}

// FP64 -> FP32 by integer operations on the bit pattern (exponent rebias,
// mantissa truncated to 23 bits: relative error below 2^-23; underflow gives
// a signed zero, overflow a signed infinity).  On GB300 the FP64 pipe is
// this kernel's bound and a conversion instruction occupies it, while the
// integer pipe is idle.
__device__ __forceinline__ float f64_to_f32_bits(double v)
{
    const unsigned hi = (unsigned)__double2hiint(v), lo = (unsigned)__double2loint(v);
    const unsigned sign = hi & 0x80000000u;
    const int ef = (int)((hi >> 20) & 0x7FFu) - 1023 + 127;
    const unsigned mant = ((hi & 0xFFFFFu) << 3) | (lo >> 29);
    if (ef <= 0) return __uint_as_float(sign);
    if (ef >= 255) return __uint_as_float(sign | 0x7F800000u);
    return __uint_as_float(sign | ((unsigned)ef << 23) | mant);
}

// N / (N - i M) in FP32 for N = (nr, ni), M = (mr, mi), with both scaled by
// the denominator's largest component (no overflow of |q|^2 for any size).
__device__ __forceinline__ float2 mie_ratio_f32(float nr, float ni, float mr, float mi)
{
    float qr = nr + mi, qi = ni - mr;
    const float s = __frcp_rn(fmaxf(fabsf(qr), fabsf(qi)));
    qr *= s;
    qi *= s;
    nr *= s;
    ni *= s;
    const float inv = __frcp_rn(fmaf(qr, qr, qi * qi));
    return make_float2(fmaf(nr, qr, ni * qi) * inv, fmaf(ni, qr, -nr * qi) * inv);
}

__device__ __forceinline__ void kahan(float &sum, float &comp, float v)
{
    const float y = v - comp;
    const float t = sum + y;
    comp = (t - sum) - y;
    sum = t;
}

// The homogeneous recurrences of homog_core (pymiecoated/mie_coeffs.py:132-180)
// with FP64 kept where stability needs it:
//   * the downward D_n recurrence (its reciprocal by rcp_newton),
//   * the real parts of N = D~ psi_n - psi_{n-1} and M = D~ chi_n - chi_{n-1}
//     (D~ = D/m + n/x or D m + n/x), which cancel -- N for small x, both once
//     psi and chi oscillate (n < x);
// and the rest in FP32: D~ imaginary parts, the products N.im, M.im and the
// ratio a = N / (N - i M).  Coefficients go to emit(k, a, b) from k = nmax
// down to 1.  row1 / rowf: psi_n, chi_n of x (FP64 / FP32) at [n - 1].
// Emulated against the FP64 recurrences for x in [1e-3, 650] and the
// benchmark indices: within 2.2e-7 of each instance's largest coefficient.
template <class Emit>
__device__ __forceinline__ void homog_core_mixed(double x, double xinv, double sx, double cxv, const HomogIndex &h,
                                                 const double2 *__restrict__ row1, const float2 *__restrict__ rowf,
                                                 int nmax, Emit &emit)
{
    const cplx m = h.m, minv = h.minv;
    const float mfr = (float)m.re, mfi = (float)m.im, mifr = (float)minv.re, mifi = (float)minv.im;
    const double az = h.azm * x;
    const int nmx = (int)rint(fmax((double)nmax, az) + 16.0);
    const cplx zinv = h.zminv * xinv;
    // Warm-up steps above nmax.  When |z| < nmax + 1 every step lies where
    // the recurrence damps the start error by (|z| / (2n+1))^2 per step, so
    // the steps are counted for a damping of e^-23 (1e-10; the FP64 path
    // asks for 1e-17); emulated for x in [1e-3, 650]: the same coefficients
    // to 2.2e-7 with 24% fewer steps on the sulfate-like table.
    int warm = nmx - 1 - nmax;
    if (az < (double)(nmax + 1)) {
        const float q = 2.f * logf((2.f * (float)(nmax + 1) + 1.f) / (float)az);
        const int need = (int)ceilf(23.0f / q) + 2;
        if (need < warm) warm = need;
    }
    cplx D = cx(0.0, 0.0);
    // r_k = (k+1)/z and k/x step down by 1/z and 1/x (no integer conversion
    // per order; the accumulated rounding stays near 1e-13)
    cplx r = zinv * (double)(nmax + warm + 1);
    for (int k = nmax + warm; k > nmax; --k) {
        const cplx w = D + r;
        const double iw = rcp_newton(abs2(w));
        D = cx(fma(-w.re, iw, r.re), fma(w.im, iw, r.im));   // r - 1/w
        r = r - zinv;
    }
    cplx rk = r;                            // r_nmax = (nmax+1)/z
    cplx w = D + rk;                        // D_{nmax+1} + r_nmax
    double iw = rcp_newton(abs2(w));
    double2 pn = row1[nmax - 1];
    float2 pnf = rowf[nmax - 1];
    double nx = (double)nmax * xinv;        // k/x
    for (int k = nmax; k >= 1; --k) {
        D = cx(fma(-w.re, iw, rk.re), fma(w.im, iw, rk.im));   // D_k
        rk = rk - zinv;                                          // r_{k-1} = k/z
        if (k > 1) {
            w = D + rk;
            iw = rcp_newton(abs2(w));
        }
        const double2 pm = (k > 1) ? row1[k - 2] : make_double2(sx, cxv);
        const float2 pmf = (k > 1) ? rowf[k - 2] : make_float2((float)sx, (float)cxv);
        const double dar = fma(D.re, minv.re, fma(-D.im, minv.im, nx));   // Re(D/m) + k/x
        const double dbr = fma(D.re, m.re, fma(-D.im, m.im, nx));         // Re(D m) + k/x
        const float nar = f64_to_f32_bits(fma(dar, pn.x, -pm.x)), nbr = f64_to_f32_bits(fma(dbr, pn.x, -pm.x));
        const float mar = f64_to_f32_bits(fma(dar, pn.y, -pm.y)), mbr = f64_to_f32_bits(fma(dbr, pn.y, -pm.y));
        const float Dr = f64_to_f32_bits(D.re), Di = f64_to_f32_bits(D.im);
        const float dai = fmaf(Dr, mifi, Di * mifr), dbi = fmaf(Dr, mfi, Di * mfr);
        const float2 a = mie_ratio_f32(nar, dai * pnf.x, mar, dai * pnf.y);
        const float2 b = mie_ratio_f32(nbr, dbi * pnf.x, mbr, dbi * pnf.y);
        emit(k, a, b);
        pn = pm;
        pnf = pmf;
        nx -= xinv;
    }
}

// Emits FP32 (c, d) = (a + b, a - b) and accumulates the efficiency sums of
// pymiecoated/mie_props.py:28-70 from the FP32 a_n, b_n with Kahan
// compensation (the accumulated rounding stays at the FP32 unit roundoff
// whatever nmax is):
//   ext = sum (2n+1) Re(a + b),  sca = sum (2n+1)(|a|^2 + |b|^2),
//   asy = sum n(n+2)/(n+1) Re(a_n a*_{n+1} + b_n b*_{n+1}) + (2n+1)/(n(n+1)) Re(a_n b*_n),
//   qb  = sum (2n+1)(-1)^n (a_n - b_n).
struct EmitMixed {
    float4 *cf;
    float amax;
    float ext, sca, asy, qbr, qbi;
    float ext_c, sca_c, asy_c, qbr_c, qbi_c;   // Kahan compensations
    float2 pa, pb;                             // a, b of order n+1 (zero above nmax)
    float inv_n1;                              // 1/(n+1)
    __device__ __forceinline__ void operator()(int k, float2 a, float2 b) {
        const float4 q = make_float4(a.x + b.x, a.y + b.y, a.x - b.x, a.y - b.y);
        cf[k - 1] = q;
        amax = fmaxf(amax, fmaxf(fmaxf(fabsf(q.x), fabsf(q.y)), fmaxf(fabsf(q.z), fabsf(q.w))));
        const float fk = (float)k;
        const float cn = 2.f * fk + 1.f;
        const float inv_n = __frcp_rn(fk);
        kahan(ext, ext_c, cn * q.x);
        kahan(sca, sca_c, cn * (fmaf(a.x, a.x, a.y * a.y) + fmaf(b.x, b.x, b.y * b.y)));
        const float up = fmaf(a.x, pa.x, fmaf(a.y, pa.y, fmaf(b.x, pb.x, b.y * pb.y)));
        const float rab = fmaf(a.x, b.x, a.y * b.y);
        kahan(asy, asy_c, ((fk + 1.f) - inv_n1) * up + (inv_n + inv_n1) * rab);
        const float sg = (k & 1) ? -cn : cn;   // (2k+1)(-1)^k
        kahan(qbr, qbr_c, sg * q.z);
        kahan(qbi, qbi_c, sg * q.w);
        pa = a;
        pb = b;
        inv_n1 = inv_n;
    }
};

// Coated units of the mixed table: the FP64 coated recurrences (the
// Toon-Ackerman ratio chain of mie_coeffs.py:183-251) with FP64 efficiency
// sums; the coefficients leave as FP32 (c, d) like the homogeneous ones.
struct EmitCf {
    float4 *cf;
    float amax;
    __device__ __forceinline__ void operator()(int k, cplx a, cplx b) {
        const float4 q = make_float4((float)(a.re + b.re), (float)(a.im + b.im), (float)(a.re - b.re),
                                     (float)(a.im - b.im));
        cf[k - 1] = q;
        amax = fmaxf(amax, fmaxf(fmaxf(fabsf(q.x), fabsf(q.y)), fmaxf(fabsf(q.z), fabsf(q.w))));
    }
};

// A operand of the contraction, written once per (unit, 64-size tile,
// 16-order chunk) as a 16 KB block in the no-swizzle K-major shared-memory
// layout
//   [matrix C_hi C_lo D_hi D_lo][kg = order / 8 % 2][row / 8][row % 8][8 orders]
// (rows 2 i, 2 i + 1 = Re, Im of size i), so that the contraction loads it
// with one bulk copy per angle block.  split_rows writes the rows of one
// instance (size i of its unit): FP32 (c, d) orders 1..nmax -> FP16 hi/lo
// scaled by 2^(13 - e_i), rows 2 ia, 2 ia + 1 (ia = i % 64) of every chunk
// of the instance's tile, zero past nmax.  The coefficient kernels call it
// once an instance is done: its coefficients are still in L2, and the
// integer/FP32/LSU work hides under their FP64 recurrences.
__device__ __forceinline__ void split_rows(const TabView &v, int64_t unit, int i, int ex, int nmax,
                                           const float4 *__restrict__ cfi, const int *__restrict__ tile_cbase,
                                           const int64_t *__restrict__ unit_cbase, int ntiles,
                                           uint8_t *__restrict__ asplit)
{
    const int lam = (int)(unit / ((int64_t)v.n_rh * v.n_comp));
    const int *tcb = tile_cbase + (size_t)v.le(lam) * (ntiles + 1);
    const int tile = i >> 6, ia = i & 63;
    const int nc = tcb[tile + 1] - tcb[tile];
    uint8_t *dst = asplit + (size_t)(unit_cbase[unit] + tcb[tile]) * 16384;
    const float sc = ldexpf(1.0f, max(-126, min(126, SHIFT_BITS - ex)));
    const int r0 = 2 * ia, r1 = 2 * ia + 1;
    for (int j = 0; j < nc; ++j)
#pragma unroll
        for (int kg = 0; kg < 2; ++kg) {
            __half ch[4][8], cl[4][8];
#pragma unroll
            for (int jj = 0; jj < 8; ++jj) {
                const int k = 16 * j + 8 * kg + jj;
                float4 q = make_float4(0.f, 0.f, 0.f, 0.f);
                if (k < nmax) q = cfi[k];
                split_f16(q.x * sc, ch[0][jj], cl[0][jj]);
                split_f16(q.y * sc, ch[1][jj], cl[1][jj]);
                split_f16(q.z * sc, ch[2][jj], cl[2][jj]);
                split_f16(q.w * sc, ch[3][jj], cl[3][jj]);
            }
            const uint32_t o0 = (kg * 16 + (r0 >> 3)) * 128 + (r0 & 7) * 16;
            const uint32_t o1 = (kg * 16 + (r1 >> 3)) * 128 + (r1 & 7) * 16;
            uint8_t *blk = dst + (size_t)j * 16384;
            *(uint4 *)(blk + 0 * 4096 + o0) = *(uint4 *)ch[0];
            *(uint4 *)(blk + 0 * 4096 + o1) = *(uint4 *)ch[1];
            *(uint4 *)(blk + 1 * 4096 + o0) = *(uint4 *)cl[0];
            *(uint4 *)(blk + 1 * 4096 + o1) = *(uint4 *)cl[1];
            *(uint4 *)(blk + 2 * 4096 + o0) = *(uint4 *)ch[2];
            *(uint4 *)(blk + 2 * 4096 + o1) = *(uint4 *)ch[3];
            *(uint4 *)(blk + 3 * 4096 + o0) = *(uint4 *)cl[2];
            *(uint4 *)(blk + 3 * 4096 + o1) = *(uint4 *)cl[3];
        }
    // the last size of a partial tile also zeroes the rows of the sizes the
    // tile lacks (their PSD weights are zero, but 0 x NaN would not be)
    const int ntile = min(64, v.n_size - 64 * tile);
    if (ia == ntile - 1 && ntile < 64) {
        const uint4 z = make_uint4(0u, 0u, 0u, 0u);
        for (int j = 0; j < nc; ++j)
            for (int r = 2 * ntile; r < 128; ++r)
#pragma unroll
                for (int kg = 0; kg < 2; ++kg) {
                    const uint32_t o = (kg * 16 + (r >> 3)) * 128 + (r & 7) * 16;
                    uint8_t *blk = dst + (size_t)j * 16384;
#pragma unroll
                    for (int mtx = 0; mtx < 4; ++mtx) *(uint4 *)(blk + mtx * 4096 + o) = z;
                }
    }
}

__global__ void __launch_bounds__(128) k_tab_coeffs_mixed_coated(TabView v, int64_t n_inst, float4 *__restrict__ cf,
                                                                 int *__restrict__ eexp, int *__restrict__ eunit,
                                                                 int *flags, const int *__restrict__ tile_cbase,
                                                                 const int64_t *__restrict__ unit_cbase, int ntiles,
                                                                 uint8_t *__restrict__ asplit)
{
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n_inst) return;
    const int i = (int)(t % v.n_size);
    const int64_t unit = t / v.n_size;
    const int lam = (int)(unit / ((int64_t)v.n_rh * v.n_comp));
    const int le = v.le(lam);
    const int64_t row = (int64_t)le * v.n_size + i;
    const int64_t o = v.off[row];
    const int nmax = (int)(v.off[row + 1] - o);
    const int64_t c = v.unit_base[unit] + (o - v.off[(int64_t)le * v.n_size]);
    const double x = v.xg[row];
    EmitCf emit{cf + c, 0.f};
    EffSums es;
    coated_table_instance(v, unit, c, o, nmax, x, emit, es, flags);
    double e[6];
    es.finish(x, e);
    double *o4 = v.eff4 + t * 4;
    o4[0] = e[0];
    o4[1] = e[1];
    o4[2] = e[3];
    o4[3] = e[4];
    const int ex = emit.amax > 0.f ? ilogbf(emit.amax) : -1000;
    eexp[t] = ex;
    atomicMax(eunit + unit, ex);
    split_rows(v, unit, i, ex, nmax, cf + c, tile_cbase, unit_cbase, ntiles, asplit);
}

__global__ void __launch_bounds__(256) k_tab_coeffs_mixed(TabView v, int64_t n_inst, float4 *__restrict__ cf,
                                                          int *__restrict__ eexp, int *__restrict__ eunit,
                                                          int *flags, const int *__restrict__ tile_cbase,
                                                          const int64_t *__restrict__ unit_cbase, int ntiles,
                                                          uint8_t *__restrict__ asplit)
{
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n_inst) return;
    const int i = (int)(t % v.n_size);
    const int64_t unit = t / v.n_size;
    const int lam = (int)(unit / ((int64_t)v.n_rh * v.n_comp));
    const int le = v.le(lam);
    const int64_t row = (int64_t)le * v.n_size + i;
    const int64_t o = v.off[row];
    const int nmax = (int)(v.off[row + 1] - o);
    const int64_t c = v.unit_base[unit] + (o - v.off[(int64_t)le * v.n_size]);
    const double x = v.xg[row];
    const double4 rc = v.rowc[row];
    const HomogIndex h = v.hidx[unit];
    EmitMixed emit;
    emit.cf = cf + c;
    emit.amax = 0.f;
    emit.ext = emit.sca = emit.asy = emit.qbr = emit.qbi = 0.f;
    emit.ext_c = emit.sca_c = emit.asy_c = emit.qbr_c = emit.qbi_c = 0.f;
    emit.pa = emit.pb = make_float2(0.f, 0.f);
    emit.inv_n1 = __frcp_rn((float)(nmax + 1));
    homog_core_mixed(x, rc.z, rc.x, rc.y, h, v.pc + o, v.pcf + o, nmax, emit);
    const double iy2 = rc.z * rc.z;   // 1 / x^2
    const double qext = 2.0 * ((double)emit.ext - (double)emit.ext_c) * iy2;
    const double sca = (double)emit.sca - (double)emit.sca_c;
    const double qsca = 2.0 * sca * iy2;
    const double qr = (double)emit.qbr - (double)emit.qbr_c, qi = (double)emit.qbi - (double)emit.qbi_c;
    double *o4 = v.eff4 + t * 4;
    o4[0] = qext;
    o4[1] = qsca;
    o4[2] = (qr * qr + qi * qi) * iy2;
    o4[3] = 2.0 * ((double)emit.asy - (double)emit.asy_c) / sca;   // 4/x^2 asy / qsca
    const int ex = emit.amax > 0.f ? ilogbf(emit.amax) : -1000;
    eexp[t] = ex;
    atomicMax(eunit + unit, ex);
    split_rows(v, unit, i, ex, nmax, cf + c, tile_cbase, unit_cbase, ntiles, asplit);
}

// FP32 copy of the psi/chi rows for the FP32 parts of the mixed recurrences.
__global__ void k_f64x2_to_f32x2(int64_t n, const double2 *__restrict__ src, float2 *__restrict__ dst)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        const double2 v = src[i];
        dst[i] = make_float2((float)v.x, (float)v.y);
    }
}

__global__ void k_fill_int(int n, int *p, int val)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) p[i] = val;
}

// ---------------------------------------------------------------------------
// B operands: (p, q) = (pi~ + tau~, pi~ - tau~) split into FP16 hi/lo, in the
// no-swizzle K-major canonical layout [k/8][angle/8][8 angles][8 orders].
// Matrices 0..3: P_hi, P_lo, Q_hi, Q_lo, each n_pad x k_pad halves.
// ---------------------------------------------------------------------------
__global__ void k_tab_bt_f16(int nang, int n_pad, int k_pad, int nmax, const double *__restrict__ cost,
                             __half *__restrict__ bt)
{
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= n_pad) return;
    const size_t mat = (size_t)n_pad * k_pad;
    const double u = a < nang ? cost[a] : 0.0;
    double pm2 = 0.0, pm1 = 0.0;
    for (int n = 1; n <= k_pad; ++n) {
        float p = 0.f, q = 0.f;
        if (a < nang && n <= nmax) {
            double pv, tv;
            if (n == 1) {
                pv = 1.0;
                tv = u;
            } else if (n == 2) {
                pv = 3.0 * u;
                tv = 6.0 * u * u - 3.0;
            } else {
                const double dn = (double)(n - 1);
                pv = (2.0 * dn + 1.0) / dn * pm1 * u - (dn + 1.0) / dn * pm2;
                tv = (dn + 1.0) * u * pv - (dn + 2.0) * pm1;
            }
            pm2 = pm1;
            pm1 = pv;
            const double s = (2.0 * n + 1.0) / ((double)n * (double)(n + 1));
            p = (float)(pv * s + tv * s);
            q = (float)(pv * s - tv * s);
        }
        const int k = n - 1;
        const size_t off = ((size_t)(k >> 3) * (n_pad >> 3) + (a >> 3)) * 64 + (a & 7) * 8 + (k & 7);
        __half h, l;
        split_f16(p, h, l);
        bt[off] = h;
        bt[mat + off] = l;
        split_f16(q, h, l);
        bt[2 * mat + off] = h;
        bt[3 * mat + off] = l;
    }
}

// ---------------------------------------------------------------------------
// The tensor-core contraction with the fused epilogue.
//
// Accuracy of the FP32 accumulation.  Measured on GB300 with a two-MMA probe
// (kind::f16, FP32 accumulator): inside one MMA the 16 products and the
// accumulator are aligned to the largest of them, every addend keeps only
// the bits down to a quarter of that value's FP32 ulp (0.5 survives next to
// 2^24, 0.25 does not), and the sum is truncated toward zero.  A long chain
// of MMAs into one accumulator therefore loses a fraction of an ulp per
// product, always in the same direction: at forward angles, where all terms
// of S+ add coherently, x = 628 gave 1.4e-6 of P11.  Here every tile's
// orders are split into windows of g.win (<= TC_NS) 16-order chunks; each window
// starts a fresh accumulator, adds the two cross products of its orders
// (C_hi P_lo, C_lo P_hi, 2^-11 of the result) while the accumulator is small
// and then the C_hi P_hi products, and the epilogue adds the windows in FP32
// registers with round-to-nearest.  Emulating the measured rule puts the
// bulk P11 error at x = 628 near 2.6e-7 this way.
//
// Pipeline (one CTA per SM, persistent, 10 warps):
//   warps 0-7   epilogue: TMEM -> window sums -> Mueller -> PSD-weighted sums
//   warp 8      MMA issue (one thread)
//   warp 9      producer (one thread): bulk copies of the split A operand
//               (split_rows) and of B orders > 16 into a TC_NS-stage
//               shared-memory ring
// Angles go in blocks of 64 (MMA N = 64); TMEM holds TC_NSETS accumulator
// sets (S+ 64 columns | S- 64 columns), so the MMAs run up to four windows
// ahead of the epilogue.  The B chunk of orders 1..16 stays resident for up
// to TC_B0_SLOTS angle blocks (loaded once: it is the same for every unit;
// 84% of the sulfate-like table's 64-size tiles need no other order); with
// more blocks one slot is reloaded at every block change.  mbarriers: stage
// full/empty, resident-B full/empty, accumulator-set full/empty.  Every wait
// is bounded and also ends when another role has raised the block's abort
// flag; role-wide decisions are taken by one thread and shared through a
// named barrier, so each role leaves its loops uniformly.
// ---------------------------------------------------------------------------
struct TcArgs {
    TabView v;
    const float4 *cf;
    const int *eexp;
    const int *eunit;
    const __half *bt;
    int n_pad, k_pad;
    const int *unit_order;
    const uint8_t *asplit;       // split A operand (split_rows)
    const int *tile_cbase;       // [n_le][ntiles + 1]
    const int64_t *unit_cbase;   // [n_units]
    int ntiles;
    int win;                     // accumulation window (16-order chunks, <= TC_NS)
    int *flags;
};

#define TC_KC16 16                                     // orders per chunk (one MMA K step)
#define TC_NS 4                                        // ring stages
#define TC_WIN_MAX TC_NS                               // longest accumulation window (chunks)
#define TC_NSETS 4                                     // TMEM accumulator sets of 128 columns
#define TC_B0_SLOTS 4                                  // resident B chunks (angle blocks)
#define TC_A16_MAT (TC_KC16 * 128 * 2)                 // one A matrix of a chunk: 4 KB
#define TC_A16_BYTES (4 * TC_A16_MAT)                  // C_hi C_lo D_hi D_lo: 16 KB
#define TC_B16_MAT (TC_KC16 * TC_NBLK * 2)             // one B matrix of a chunk: 2 KB
#define TC_B16_BYTES (4 * TC_B16_MAT)                  // P_hi P_lo Q_hi Q_lo: 8 KB
#define TC_STAGE_BYTES (TC_A16_BYTES + TC_B16_BYTES)   // 24 KB
#define TC_STAGE_PITCH 66                              // 64 columns + 2: conflict-free pair writes
#define TC_STAGE_FLOATS (4 * TC_INST * TC_STAGE_PITCH) // Mueller staging [k][size][col]: 66 KB
#define TC_EPI_THREADS 256
#define TC_THREADS (TC_EPI_THREADS + 64)             // + the MMA warp and the producer warp
#define TC_SMEM_BYTES                                                                                  \
    (TC_B0_SLOTS * TC_B16_BYTES + TC_NS * TC_STAGE_BYTES + TC_STAGE_FLOATS * 4 + 8 * TC_INST * 4 + 256)
#define TC_BAR_EPI 1                                   // named barrier id of the epilogue warps
#define TC_SLEEP_NS 32                                 // back-off of the MMA and producer waits

static_assert(TC_NSETS * 128 <= 512, "TMEM columns");

// k-th unit of CTA `cta` among G CTAs: units in decreasing-work order,
// dealt in a snake (c, then G-1-c) so that every CTA gets a similar mix.
__device__ __forceinline__ int64_t tc_unit_index(int k, int cta, int G)
{
    return (int64_t)k * G + ((k & 1) ? (G - 1 - cta) : cta);
}

// Chunk j (orders 16 j + 1 .. 16 j + 16) of angle block blk of the four B
// matrices, global [m][k/8][angle/8][8][8] -> shared [m][kg][ng][8][8]: per
// (m, kg) one contiguous run of 8 core matrices (1 KB).  One thread; the
// caller has armed `bar` with the bytes (mbar_arrive_expect_tx).
__device__ __forceinline__ void tc_copy_b16(const TcArgs &g, uint8_t *dst, int j, int blk, uint64_t *bar)
{
    const int ngt = g.n_pad / 8, nng = TC_NBLK / 8;
    const size_t mat = (size_t)g.n_pad * g.k_pad;
#pragma unroll
    for (int m = 0; m < 4; ++m)
#pragma unroll
        for (int kg = 0; kg < 2; ++kg) {
            const __half *src = g.bt + m * mat + ((size_t)(2 * j + kg) * ngt + (size_t)blk * nng) * 64;
            bulk_g2s(dst + m * TC_B16_MAT + kg * nng * 128, src, nng * 128, bar);
        }
}

template <int NB>
__global__ void __launch_bounds__(TC_THREADS, 1) k_tab_s12_tc(TcArgs g)
{
    extern __shared__ __align__(1024) uint8_t smem[];
    uint8_t *sB0 = smem;                                            // resident B chunks, orders 1..16
    uint8_t *sStage = sB0 + TC_B0_SLOTS * TC_B16_BYTES;             // TC_NS x (A 16 KB | B 8 KB)
    float *stage = (float *)(sStage + TC_NS * TC_STAGE_BYTES);     // Mueller staging [4][64][66]
    float *sw = stage + TC_STAGE_FLOATS;                            // [64 sizes][8 bins]
    uint64_t *bars = (uint64_t *)(sw + 8 * TC_INST);
    uint64_t *full = bars, *empty = bars + TC_NS;
    uint64_t *b0_full = bars + 2 * TC_NS, *b0_empty = b0_full + 1;
    uint64_t *acc_full = b0_full + 2, *acc_empty = acc_full + TC_NSETS, *drain = acc_empty + TC_NSETS;
    uint32_t *s_tmem = (uint32_t *)(drain + 1);
    volatile int *s_abort = (volatile int *)(s_tmem + 1);
    volatile int *s_epi_go = s_abort + 1;    // [2] epilogue: 1 = accumulator set ready, 0 = stop

    const TabView &v = g.v;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int nblocks = g.n_pad / TC_NBLK;
    const bool reload = nblocks > TC_B0_SLOTS;   // one resident slot, reloaded per block
    if (warp == 0) tmem_alloc(s_tmem, 512);
    if (tid == 0) {
        for (int i = 0; i < TC_NS; ++i) {
            mbar_init(full + i, 1);    // the producer's arrival with the copies' bytes
            mbar_init(empty + i, 1);   // tcgen05.commit
        }
        mbar_init(b0_full, 1);
        mbar_init(b0_empty, 1);
        for (int i = 0; i < TC_NSETS; ++i) {
            mbar_init(acc_full + i, 1);
            mbar_init(acc_empty + i, TC_EPI_THREADS / 32);
        }
        mbar_init(drain, 1);
        fence_mbar_init();
        *s_abort = 0;
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *s_tmem;
    const int64_t n_units = (int64_t)v.n_lambda * v.n_rh * v.n_comp;
    const int G = gridDim.x, cta = blockIdx.x;

    if (warp == 8) {
        // ================= MMA issue =================
        if (lane == 0) {
            const uint32_t idesc = idesc_f16_f32(128, TC_NBLK);
            uint32_t it = 0, item = 0, b0_loads = 0;
            int prev_blk = -1;
            bool ok = true;
            if (!reload) {   // every block's resident chunk, loaded once
                ok = mbar_wait_or_abort(b0_full, 0, s_abort, TC_SLEEP_NS);
                b0_loads = 1;
            }
            for (int k = 0; ok; ++k) {
                const int64_t uidx = tc_unit_index(k, cta, G);
                if (uidx >= n_units) break;
                const int64_t unit = g.unit_order[uidx];
                const int lam = (int)(unit / ((int64_t)v.n_rh * v.n_comp));
                const int64_t *off = v.off + (int64_t)v.le(lam) * v.n_size;
                for (int blk = 0; blk < nblocks && ok; ++blk) {
                    if (reload && blk != prev_blk) {   // the producers reload the resident slot
                        if (prev_blk >= 0) mma_commit(b0_empty);
                        if (!mbar_wait_or_abort(b0_full, b0_loads & 1u, s_abort, TC_SLEEP_NS)) {
                            ok = false;
                            break;
                        }
                        ++b0_loads;
                        prev_blk = blk;
                    }
                    const uint32_t aB0 = smem_u32(sB0 + (reload ? 0 : blk) * TC_B16_BYTES);
                    for (int t0 = 0; t0 < v.n_size && ok; t0 += TC_INST) {
                        const int ntile = min(TC_INST, v.n_size - t0);
                        const int kt = (int)(off[t0 + ntile] - off[t0 + ntile - 1]);
                        const int nc = (kt + TC_KC16 - 1) / TC_KC16;
                        for (int w0 = 0; w0 < nc && ok; w0 += g.win) {
                            const int nj = min(g.win, nc - w0);
                            const uint32_t set = item % TC_NSETS, use = item / TC_NSETS;
                            if (use > 0 && !mbar_wait_or_abort(acc_empty + set, (use - 1) & 1u, s_abort, TC_SLEEP_NS)) {
                                ok = false;
                                break;
                            }
                            for (int j = 0; j < nj && ok; ++j) {
                                const uint32_t c = it + j;
                                ok = mbar_wait_or_abort(full + c % TC_NS, (c / TC_NS) & 1u, s_abort, TC_SLEEP_NS);
                            }
                            if (!ok) break;
                            tc_fence_after();
                            const uint32_t d = tmem + set * 128;   // S+ at d, S- at d + 64
                            for (int pass = 0; pass < 2; ++pass) {
                                for (int j = 0; j < nj; ++j) {
                                    const uint32_t c = it + j;
                                    const uint32_t aA = smem_u32(sStage + (c % TC_NS) * TC_STAGE_BYTES);
                                    const uint32_t aB = (w0 + j) == 0 ? aB0 : aA + TC_A16_BYTES;
                                    // A: LBO (K step of 8 orders) = 16 core matrices; B: 8
                                    const uint64_t a_chi = smem_desc(aA + 0 * TC_A16_MAT, 16 * 128, 128);
                                    const uint64_t a_dhi = smem_desc(aA + 2 * TC_A16_MAT, 16 * 128, 128);
                                    const uint64_t b_phi = smem_desc(aB + 0 * TC_B16_MAT, (TC_NBLK / 8) * 128, 128);
                                    const uint64_t b_qhi = smem_desc(aB + 2 * TC_B16_MAT, (TC_NBLK / 8) * 128, 128);
                                    if (pass == 0) {   // cross products: small accumulator
                                        const uint64_t a_clo = smem_desc(aA + 1 * TC_A16_MAT, 16 * 128, 128);
                                        const uint64_t a_dlo = smem_desc(aA + 3 * TC_A16_MAT, 16 * 128, 128);
                                        const uint64_t b_plo =
                                            smem_desc(aB + 1 * TC_B16_MAT, (TC_NBLK / 8) * 128, 128);
                                        const uint64_t b_qlo =
                                            smem_desc(aB + 3 * TC_B16_MAT, (TC_NBLK / 8) * 128, 128);
                                        mma_f16(d, a_chi, b_plo, idesc, j == 0 ? 0u : 1u);
                                        mma_f16(d, a_clo, b_phi, idesc, 1u);
                                        mma_f16(d + 64, a_dhi, b_qlo, idesc, j == 0 ? 0u : 1u);
                                        mma_f16(d + 64, a_dlo, b_qhi, idesc, 1u);
                                    } else {
                                        mma_f16(d, a_chi, b_phi, idesc, 1u);
                                        mma_f16(d + 64, a_dhi, b_qhi, idesc, 1u);
                                        mma_commit(empty + c % TC_NS);   // stage free when its MMAs are done
                                    }
                                }
                            }
                            it += nj;
                            mma_commit(acc_full + set);
                            ++item;
                        }
                    }
                }
            }
            if (!ok) {
                *s_abort = 1;
                atomicOr(g.flags, GBMIE_FLAG_TIMEOUT);
            }
            // every issued MMA has finished before TMEM is released
            mma_commit(drain);
            if (!mbar_wait(drain, 0)) atomicOr(g.flags, GBMIE_FLAG_TIMEOUT);
        }
        __syncwarp();
    } else if (warp == 9) {
        // ================= producer: bulk copies (one thread) =================
        if (lane == 0) {
            uint32_t it = 0, b0_loads = 0;
            int prev_blk = -1;
            uint64_t *last_tx = nullptr;   // barrier of the last bulk copy, and its phase
            uint32_t last_tx_phase = 0;
            bool ok = true;
            if (!reload) {
                mbar_arrive_expect_tx(b0_full, (uint32_t)(nblocks * TC_B16_BYTES));
                for (int b = 0; b < nblocks; ++b) tc_copy_b16(g, sB0 + b * TC_B16_BYTES, 0, b, b0_full);
                last_tx = b0_full;
                last_tx_phase = 0;
            }
            for (int k = 0; ok; ++k) {
                const int64_t uidx = tc_unit_index(k, cta, G);
                if (uidx >= n_units) break;
                const int64_t unit = g.unit_order[uidx];
                const int lam = (int)(unit / ((int64_t)v.n_rh * v.n_comp));
                const int *tcb = g.tile_cbase + (size_t)v.le(lam) * (g.ntiles + 1);
                const uint8_t *ua = g.asplit + (size_t)g.unit_cbase[unit] * TC_A16_BYTES;
                for (int blk = 0; blk < nblocks && ok; ++blk) {
                    if (reload && blk != prev_blk) {
                        if (prev_blk >= 0 && !mbar_wait_or_abort(b0_empty, (b0_loads - 1) & 1u, s_abort, TC_SLEEP_NS)) {
                            ok = false;
                            break;
                        }
                        mbar_arrive_expect_tx(b0_full, TC_B16_BYTES);
                        tc_copy_b16(g, sB0, 0, blk, b0_full);
                        last_tx = b0_full;
                        last_tx_phase = b0_loads & 1u;
                        ++b0_loads;
                        prev_blk = blk;
                    }
                    for (int tile = 0; tile < g.ntiles && ok; ++tile) {
                        const int nc = tcb[tile + 1] - tcb[tile];
                        for (int j = 0; j < nc; ++j) {
                            const uint32_t c = it++;
                            const int st = (int)(c % TC_NS);
                            uint8_t *sA = sStage + st * TC_STAGE_BYTES;
                            if (c >= TC_NS && !mbar_wait_or_abort(empty + st, (c / TC_NS - 1) & 1u, s_abort, TC_SLEEP_NS)) {
                                ok = false;
                                break;
                            }
                            mbar_arrive_expect_tx(full + st, TC_A16_BYTES + (j > 0 ? TC_B16_BYTES : 0));
                            bulk_g2s(sA, ua + (size_t)(tcb[tile] + j) * TC_A16_BYTES, TC_A16_BYTES, full + st);
                            if (j > 0) tc_copy_b16(g, sA + TC_A16_BYTES, j, blk, full + st);
                            last_tx = full + st;
                            last_tx_phase = (c / TC_NS) & 1u;
                        }
                    }
                }
            }
            if (!ok || *s_abort) {
                *s_abort = 1;
                atomicOr(g.flags, GBMIE_FLAG_TIMEOUT);
                // a bulk copy still in flight must land before shared memory is released
                if (last_tx) mbar_wait(last_tx, last_tx_phase, 1u << 20);
            }
        }
        __syncwarp();
    } else {
        // ================= epilogue (warps 0-7) =================
        // One flat sequence of tiles s = (unit k, angle block, 64-size tile);
        // the PSD weights of tile s + 1 are fetched into registers while tile
        // s is processed and land in shared memory after its last barrier.
        uint32_t item = 0;
        bool ok = true;
        const int q = warp & 3, half = warp >> 2;
        const int il = 16 * q + (lane >> 1);
        const bool odd = lane & 1;
        const int kk = warp >> 1, cg = warp & 1, hh = lane >> 4, cp = lane & 15;
        const int ntl = g.ntiles;
        // per-unit constants of this CTA's kq-th unit (valid = false past its last unit)
        struct UnitC {
            bool valid;
            int comp, lr, lam, E;
            const float *Wb;
            const int *ex;
            const int64_t *off;
        };
        auto unit_c = [&](int kq) -> UnitC {
            UnitC u;
            const int64_t uidx = tc_unit_index(kq, cta, G);
            u.valid = uidx < n_units;
            if (!u.valid) return u;
            const int unit = g.unit_order[uidx];
            u.comp = unit % v.n_comp;
            u.lr = unit / v.n_comp;
            u.lam = u.lr / v.n_rh;
            const int rhi = u.lr - u.lam * v.n_rh;
            u.Wb = v.Wf + v.wlam(u.lam) + ((size_t)rhi * v.n_bin * v.n_comp + u.comp) * v.n_size;
            u.ex = g.eexp + (size_t)unit * v.n_size;
            u.E = g.eunit[unit];
            u.off = v.off + (int64_t)v.le(u.lam) * v.n_size;
            return u;
        };
        // PSD weights of a tile scaled by 2^(2 (e_i - E)) (E is the unit's largest
        // exponent, so the power is <= 1; below 2^-126 the weight is dropped) for
        // this thread's two entries idx = tid, tid + 256 of [64 sizes][8 bins]
        auto fetch_w = [&](const UnitC &u, int tile, float &w0, float &w1) {
            const int t0 = tile * TC_INST, ntile = min(TC_INST, v.n_size - t0);
            float w[2];
#pragma unroll
            for (int h2 = 0; h2 < 2; ++h2) {
                const int idx = tid + h2 * TC_EPI_THREADS, b = idx & 7, i = idx >> 3;
                w[h2] = 0.f;
                if (i < ntile && b < v.n_bin && b < NB) {
                    const int e = 2 * (u.ex[t0 + i] - u.E);
                    const float p2 = e < -126 ? 0.f : __int_as_float((e + 127) << 23);
                    w[h2] = u.Wb[(size_t)b * v.n_comp * v.n_size + t0 + i] * p2;
                }
            }
            w0 = w[0];
            w1 = w[1];
        };
        float wn0 = 0.f, wn1 = 0.f;
        UnitC cu = unit_c(0);
        if (cu.valid) {
            fetch_w(cu, 0, wn0, wn1);
            sw[tid] = wn0;
            sw[tid + TC_EPI_THREADS] = wn1;
        }
        float uh[2][NB], ul[2][NB];   // per-(unit, block) sums, unevaluated FP32 pairs (two-sum)
        int kq = 0, blk = 0, tile = 0;   // the tile sequence: units, angle blocks, 64-size tiles
        while (ok && cu.valid) {
            const int comp = cu.comp, lr = cu.lr;
            const int64_t *off = cu.off;
            const int t0 = tile * TC_INST, ntile = min(TC_INST, v.n_size - t0);
            const int kt = (int)(off[t0 + ntile] - off[t0 + ntile - 1]);
            const int nwin = ((kt + TC_KC16 - 1) / TC_KC16 + g.win - 1) / g.win;
            if (tile == 0) {
#pragma unroll
                for (int c = 0; c < 2; ++c)
#pragma unroll
                    for (int b = 0; b < NB; ++b) uh[c][b] = ul[c][b] = 0.f;
            }
            int nk = kq, nb = blk, nt = tile + 1;   // the next tile
            if (nt == ntl) {
                nt = 0;
                if (++nb == nblocks) {
                    nb = 0;
                    ++nk;
                }
            }
            const UnitC nu = nk == kq ? cu : unit_c(nk);
            const bool have_next = nu.valid;
            if (have_next) fetch_w(nu, nt, wn0, wn1);   // in flight during this tile
            // window sums of S+ and S- (Re/Im of this lane's row, 32 columns)
            float rp[32], rm[32];
            for (int w = 0; w < nwin; ++w) {
                const uint32_t set = item % TC_NSETS, use = item / TC_NSETS;
                if (tid == 0) s_epi_go[item & 1] = mbar_wait_or_abort(acc_full + set, use & 1u, s_abort) ? 1 : 0;
                named_bar_sync(TC_BAR_EPI, TC_EPI_THREADS);
                if (!s_epi_go[item & 1]) {
                    ok = false;
                    break;
                }
                tc_fence_after();
                const uint32_t ta = tmem + ((uint32_t)(32 * q) << 16) + set * 128 + 32 * half;
                if (w == 0) {
                    tmem_ld32(ta, rp);
                    tmem_ld32(ta + 64, rm);
                } else {
                    float t[32];
                    tmem_ld32(ta, t);
#pragma unroll
                    for (int i = 0; i < 32; ++i) rp[i] += t[i];
                    tmem_ld32(ta + 64, t);
#pragma unroll
                    for (int i = 0; i < 32; ++i) rm[i] += t[i];
                }
                tc_fence_before();
                __syncwarp();
                if (lane == 0) mbar_arrive(acc_empty + set);
                ++item;
            }
            if (!ok) break;
            // Mueller phase: warp (q = TMEM lane quarter, half = warp / 4) holds
            // rows 32 q .. + 31 (sizes 16 q .. + 15, Re/Im lane pairs) for 32
            // columns; the even lane forms column 2p and the odd lane 2p + 1.
            float *strow = stage + il * TC_STAGE_PITCH + 32 * half + (odd ? 1 : 0);
#pragma unroll
            for (int pj = 0; pj < 16; ++pj) {
                const int j0 = 2 * pj, j1 = 2 * pj + 1;
                const float xp = __shfl_xor_sync(0xffffffffu, odd ? rp[j0] : rp[j1], 1);
                const float xm = __shfl_xor_sync(0xffffffffu, odd ? rm[j0] : rm[j1], 1);
                const float pr = odd ? xp : rp[j0], pi = odd ? rp[j1] : xp;
                const float mr = odd ? xm : rm[j0], mi = odd ? rm[j1] : xm;
                const float A2 = pr * pr + pi * pi, B2 = mr * mr + mi * mi;
                float *st = strow + j0;
                st[0 * TC_INST * TC_STAGE_PITCH] = 0.25f * (A2 + B2);
                st[1 * TC_INST * TC_STAGE_PITCH] = -0.5f * (pr * mr + pi * mi);
                st[2 * TC_INST * TC_STAGE_PITCH] = 0.25f * (A2 - B2);
                st[3 * TC_INST * TC_STAGE_PITCH] = -0.5f * (mr * pi - mi * pr);
            }
            named_bar_sync(TC_BAR_EPI, TC_EPI_THREADS);
            // Reduction phase: warp w sums element kk = w / 2 over columns
            // 32 (w % 2) + 2 cp + {0, 1} (cp = lane % 16) and sizes 32 h .. + 31
            // (h = lane / 16) for every bin; the two halves meet by a shuffle.
            {
                float acc[2][NB];
#pragma unroll
                for (int c = 0; c < 2; ++c)
#pragma unroll
                    for (int b = 0; b < NB; ++b) acc[c][b] = 0.f;
                const float *src = stage + (kk * TC_INST + 32 * hh) * TC_STAGE_PITCH + 32 * cg + 2 * cp;
                const float *wsrc = sw + 32 * hh * 8;
#pragma unroll 4
                for (int i = 0; i < 32; ++i) {
                    const float2 sv = *(const float2 *)(src + i * TC_STAGE_PITCH);
                    const float4 w0 = *(const float4 *)(wsrc + 8 * i);
                    float wv[8] = {w0.x, w0.y, w0.z, w0.w, 0.f, 0.f, 0.f, 0.f};
                    if (NB > 4) {
                        const float4 w1 = *(const float4 *)(wsrc + 8 * i + 4);
                        wv[4] = w1.x;
                        wv[5] = w1.y;
                        wv[6] = w1.z;
                        wv[7] = w1.w;
                    }
#pragma unroll
                    for (int b = 0; b < NB; ++b) {
                        acc[0][b] = fmaf(wv[b], sv.x, acc[0][b]);
                        acc[1][b] = fmaf(wv[b], sv.y, acc[1][b]);
                    }
                }
#pragma unroll
                for (int c = 0; c < 2; ++c)
#pragma unroll
                    for (int b = 0; b < NB; ++b) {
                        const float a = acc[c][b] + __shfl_xor_sync(0xffffffffu, acc[c][b], 16);
                        // two-sum: (uh + ul) += a exactly-rounded
                        const float sum = uh[c][b] + a;
                        const float bp = sum - uh[c][b];
                        ul[c][b] += (uh[c][b] - (sum - bp)) + (a - bp);
                        uh[c][b] = sum;
                    }
            }
            named_bar_sync(TC_BAR_EPI, TC_EPI_THREADS);
            // every reader of sw and stage has passed the barrier: the next tile's weights go in
            if (have_next) {
                sw[tid] = wn0;
                sw[tid + TC_EPI_THREADS] = wn1;
            }
            if (tile == ntl - 1 && hh == 0) {
                // unit results of this angle block: lanes of the first size half
                // hold the combined sums of (element kk, two columns)
                const double f2 = ldexp(1.0, 2 * (cu.E - SHIFT_BITS));
#pragma unroll
                for (int c = 0; c < 2; ++c) {
                    const int col = blk * TC_NBLK + 32 * cg + 2 * cp + c;
                    if (col < v.n_ang) {
#pragma unroll
                        for (int b = 0; b < NB; ++b) {
                            if (b < v.n_bin) {
                                const double f = v.frac[(size_t)b * v.n_comp + comp];
                                atomicAdd(v.pacc + (((size_t)lr * v.n_bin + b) * 4 + kk) * v.n_ang + col,
                                          f * ((double)uh[c][b] + (double)ul[c][b]) * f2);
                            }
                        }
                    }
                }
            }
            kq = nk;
            blk = nb;
            tile = nt;
            cu = nu;
        }
        if (!ok && tid == 0) {
            *s_abort = 1;
            atomicOr(g.flags, GBMIE_FLAG_TIMEOUT);
        }
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 0) tmem_dealloc(tmem, 512);
}

// ---------------------------------------------------------------------------
// host launchers (called from gbmie_table_run)
// ---------------------------------------------------------------------------
int launch_table_mixed(gbmie_ctx *ctx, gbmie_table_plan *p, TabView &v, char *scr)
{
    const gbmie_table_desc &d = p->d;
    cudaStream_t st = ctx->stream;
    float4 *cf = (float4 *)(scr + p->o_cf);
    int *eexp = (int *)(scr + p->o_eexp);
    int *eunit = (int *)(scr + p->o_eunit);
    ctx_pre_launch(ctx);
    k_f64x2_to_f32x2<<<(unsigned)ceil_div64(p->pc_total, 256), 256, 0, st>>>(p->pc_total, v.pc, v.pcf);
    GBMIE_TRY(ctx_check_launch(ctx, "k_f64x2_to_f32x2"));
    ctx_pre_launch(ctx);
    k_fill_int<<<(unsigned)ceil_div64(p->n_units, 256), 256, 0, st>>>((int)p->n_units, eunit, -100000);
    GBMIE_TRY(ctx_check_launch(ctx, "k_fill_int"));
    ctx_pre_launch(ctx);
    uint8_t *asplit = (uint8_t *)(scr + p->o_asplit);
    if (d.m_core) {
        k_tab_coeffs_mixed_coated<<<(unsigned)ceil_div64(p->n_inst, 128), 128, 0, st>>>(
            v, p->n_inst, cf, eexp, eunit, ctx->d_flags, p->tile_cbase, p->unit_cbase, p->ntiles, asplit);
        GBMIE_TRY(ctx_check_launch(ctx, "k_tab_coeffs_mixed_coated"));
    } else {
        k_tab_coeffs_mixed<<<(unsigned)ceil_div64(p->n_inst, p->coef_block), p->coef_block, 0, st>>>(
            v, p->n_inst, cf, eexp, eunit, ctx->d_flags, p->tile_cbase, p->unit_cbase, p->ntiles, asplit);
        GBMIE_TRY(ctx_check_launch(ctx, "k_tab_coeffs_mixed"));
    }
    TcArgs a;
    a.v = v;
    a.cf = cf;
    a.eexp = eexp;
    a.eunit = eunit;
    a.bt = p->bt;
    a.n_pad = p->n_pad_total;
    a.k_pad = p->k_pad;
    a.unit_order = p->unit_order;
    a.asplit = asplit;
    a.tile_cbase = p->tile_cbase;
    a.unit_cbase = p->unit_cbase;
    a.ntiles = p->ntiles;
    a.win = p->tc_win < 1 ? 1 : (p->tc_win > TC_WIN_MAX ? TC_WIN_MAX : p->tc_win);
    a.flags = ctx->d_flags;
    int nsm = 0;
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, ctx->device);
    const int grid = (int)(p->n_units < nsm ? p->n_units : nsm);
    const size_t smem = TC_SMEM_BYTES;
    cudaError_t e = cudaSuccess;
    ctx_pre_launch(ctx);
#define TC_LAUNCH(NBV)                                                                                   \
    case NBV:                                                                                            \
        e = cudaFuncSetAttribute(k_tab_s12_tc<NBV>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem); \
        k_tab_s12_tc<NBV><<<grid, TC_THREADS, smem, st>>>(a);                                            \
        break;
    switch (d.n_bin) {
        TC_LAUNCH(1) TC_LAUNCH(2) TC_LAUNCH(3) TC_LAUNCH(4) TC_LAUNCH(5) TC_LAUNCH(6) TC_LAUNCH(7)
        default:
        TC_LAUNCH(8)
    }
#undef TC_LAUNCH
    GBMIE_TRY(ctx_cuda(ctx, e, "k_tab_s12_tc smem attribute"));
    return ctx_check_launch(ctx, "k_tab_s12_tc");
}

size_t table_mixed_smem_bytes() { return TC_SMEM_BYTES; }

// The B operands depend only on the angles and the largest nmax: built once
// per plan into plan-owned memory (plan creation synchronises afterwards).
int build_table_bt(gbmie_ctx *ctx, gbmie_table_plan *p)
{
    const size_t bytes = 4 * 2 * (size_t)p->n_pad_total * p->k_pad;
    GBMIE_TRY(ctx_cuda(ctx, cudaMalloc(&p->bt, bytes), "B operand tables"));
    ctx_pre_launch(ctx);
    k_tab_bt_f16<<<(p->n_pad_total + 127) / 128, 128, 0, ctx->stream>>>(p->d.n_ang, p->n_pad_total, p->k_pad,
                                                                         p->nmax_max, p->d.cos_theta, p->bt);
    return ctx_check_launch(ctx, "k_tab_bt_f16");
}

// Autotuning of the mixed path on the plan's own data (after one full run
// has filled its buffers): the block size of k_tab_coeffs_mixed (64, 128,
// 256) and the contraction's accumulation window (2, 3 or 4 chunks of 16
// orders; every window keeps the measured accumulation error near 2e-7 of
// P11), each the fastest of two timed launches.  Leaves pacc holding
// partial sums: the caller runs the table again.
int tune_table_mixed(gbmie_ctx *ctx, gbmie_table_plan *p, TabView &v, char *scr, cudaEvent_t e0, cudaEvent_t e1)
{
    cudaStream_t st = ctx->stream;
    float4 *cf = (float4 *)(scr + p->o_cf);
    int *eexp = (int *)(scr + p->o_eexp);
    int *eunit = (int *)(scr + p->o_eunit);
    float best = 3.4e38f;
    int pick = p->coef_block;
    if (!p->d.m_core) {
        const int blocks[3] = {64, 128, 256};
        for (int c = 0; c < 3; ++c)
            for (int rep = 0; rep < 2; ++rep) {
                const int bs = blocks[c];
                cudaEventRecord(e0, st);
                k_tab_coeffs_mixed<<<(unsigned)ceil_div64(p->n_inst, bs), bs, 0, st>>>(
                    v, p->n_inst, cf, eexp, eunit, ctx->d_flags, p->tile_cbase, p->unit_cbase, p->ntiles,
                    (uint8_t *)(scr + p->o_asplit));
                cudaEventRecord(e1, st);
                GBMIE_TRY(ctx_cuda(ctx, cudaEventSynchronize(e1), "tune coefficients"));
                float ms = 0.f;
                cudaEventElapsedTime(&ms, e0, e1);
                if (ms < best) {
                    best = ms;
                    pick = bs;
                }
            }
        p->coef_block = pick;
    }
    best = 3.4e38f;
    int wpick = p->tc_win;
    for (int w = 2; w <= TC_WIN_MAX; ++w)
        for (int rep = 0; rep < 2; ++rep) {
            p->tc_win = w;
            const int save = ctx->timing;
            ctx->timing = 0;
            cudaEventRecord(e0, st);
            const int rc = launch_table_mixed(ctx, p, v, scr);
            cudaEventRecord(e1, st);
            ctx->timing = save;
            GBMIE_TRY(rc);
            GBMIE_TRY(ctx_cuda(ctx, cudaEventSynchronize(e1), "tune contraction"));
            float ms = 0.f;
            cudaEventElapsedTime(&ms, e0, e1);
            if (ms < best) {
                best = ms;
                wpick = w;
            }
        }
    p->tc_win = wpick;
    return GBMIE_OK;
}

