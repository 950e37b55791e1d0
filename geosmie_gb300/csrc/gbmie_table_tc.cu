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
// are GEMMs [angles x orders] x [orders x instances]: rows (MMA M) are
// angles in blocks of 128, columns (N) the (instance, Re/Im) pairs of half a
// 64-size tile.  Each operand is split into FP16 hi + lo halves (coefficients
// scaled by 2^(13 - e_i) so the instance's maximum sits just below 2^14), and
//   P C ~ P_hi C_hi + P_hi C_lo + P_lo C_hi
// is accumulated in FP32 in tensor memory: three tcgen05.mma per product and
// K step of 16 orders, six per step for S+ and S- (in windows of up to 64
// orders, cross products first, see below).  The epilogue reads S+/S- from
// TMEM (tcgen05.ld; one angle per thread), forms s11, s12, s33, s34 and sums
// them over the tile's sizes with the PSD weights of every bin (the weights
// absorb 2^(2(e_i - E)) with E the unit's largest exponent), accumulating
// per unit in FP64.  Per-size phase matrices never reach global memory.
#include "common.cuh"
#include "df.cuh"
#include "mie_device.cuh"
#include "table_internal.cuh"
#include "tc.cuh"

#define TC_KC16 16                      // orders per chunk (one MMA K step)
#define TC_INST 64                      // sizes per tile
#define TC_HALF 32                      // sizes per half tile (MMA N = 64: Re, Im)
#define TC_ABLK 128                     // angles per block (MMA M)
#define TC_MAT_A (16 * TC_ABLK * 2)     // one angle-function matrix of a 16-order chunk: 4 KB
// one coefficient matrix of a tile's chunk: 128 rows (64 sizes x Re, Im) x
// 16 orders, FP16, K-major core matrices [kg = order / 8 % 2][row / 8][row %
// 8][8 orders]: 4 KB.  A whole-tile MMA reads it with N = 128, a half-tile
// MMA its rows 64 h .. 64 h + 63 (1 KB further on per h) with N = 64; both
// step 2 KB between the two 8-order groups
#define TC_MAT_B (16 * 2 * TC_INST * 2)
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

// x 2^k as FP64 by integer operations on the bit pattern (exact: the FP64
// exponent range holds every FP32 value times the powers of two used here;
// zeros and FP32 subnormals give zero).  FP64 arithmetic and conversions
// occupy GB300's narrow FP64 pipe; these are integer instructions.
__device__ __forceinline__ double f32_to_f64_pow2(float x, int k)
{
    const unsigned u = __float_as_uint(x);
    const unsigned e = (u >> 23) & 0xFFu;
    if (e == 0u) return 0.0;
    const unsigned hi = (u & 0x80000000u) | ((e + 896u + (unsigned)k) << 20) | ((u & 0x7FFFFFu) >> 3);
    return __hiloint2double((int)hi, (int)(u << 29));
}

// pair -> FP64 (one FP64 addition)
__device__ __forceinline__ double df_to_f64(df a) { return f32_to_f64_pow2(a.hi, 0) + f32_to_f64_pow2(a.lo, 0); }

// N / (N - i M) in FP32 for N = (nr, ni), M = (mr, mi), with both scaled by
// the denominator's largest component (no overflow of |q|^2 for any size);
// dsq = 1 / |N - i M|^2 (capped at the FP32 maximum, so that 0 x dsq = 0).
__device__ __forceinline__ float2 mie_ratio_f32(float nr, float ni, float mr, float mi, float &dsq)
{
    float qr = nr + mi, qi = ni - mr;
    const float s = __frcp_rn(fmaxf(fabsf(qr), fabsf(qi)));
    qr *= s;
    qi *= s;
    nr *= s;
    ni *= s;
    const float inv = __frcp_rn(fmaf(qr, qr, qi * qi));
    dsq = fminf(s * (s * inv), 3.4028235e38f);
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
// with double-float pairs (df.cuh, ~2^-46) where stability needs more than
// FP32:
//   * the downward D_n recurrence (r_k = (k+1)/z formed per step, the
//     reciprocal by df_rcp),
//   * the real parts of N = D~ psi_n - psi_{n-1} and M = D~ chi_n - chi_{n-1}
//     (D~ = D/m + n/x or D m + n/x), which cancel -- N for small x, both once
//     psi and chi oscillate (n < x);
// and the rest in FP32: D~ imaginary parts, the products N.im, M.im and the
// ratio a = N / (N - i M).  Coefficients go to emit(k, a, b, t) from k = nmax
// down to 1.  rowd: psi_n, chi_n of x as pairs (psi hi, lo, chi hi, lo) at
// [(n - 1) rs].  GB300's FP64 pipe issues a small fraction of the FP32 rate, so
// the pairs (a few FP32 operations per FP64 one) run these recurrences
// several times faster than FP64 did; the precision they keep (2^-46 against
// 2^-53) is far below the FP32 coefficients this path emits: the largest
// cancellation, N at the smallest sizes (O(x^2), x >= 1e-3), costs 20 bits.
//
// t is the order's absorption without cancellation.  With r = M / N,
// a = 1 / (1 - i r) and Re a - |a|^2 = Im(r) |a|^2; Im(M N*) = Im(D~) W with
// W = psi_n chi_{n-1} - chi_n psi_{n-1} = -1 (the Riccati-Bessel Wronskian in
// pymiecoated's sign, chi = -x y_n), so
//   Re a - |a|^2 = -Im(D~) / |N - i M|^2
// and t = Im(D~_a) / |N_a - i M_a|^2 + Im(D~_b) / |N_b - i M_b|^2, the two of
// the same sign for a passive particle.  Re a - |a|^2 formed from the
// coefficients themselves cancels: Re a and |a|^2 agree to 1 - 1e-8 for the
// sulfate-like indices (Im m ~ 1e-8), far past FP32.
//
// hd: the unit's constants as pairs (k_mixed_consts): m, 1/m, x/z, (|z|/x);
// r0 = (sin x, cos x) = (psi_0, chi_0) and xi = 1/x as pairs, xf = x.
//
// DN64 (a measurement variant, gbmie_table_plan_set_dn_fp64): the downward
// D_n recurrence in FP64 from the reference's start, zero at
// nmx = round(max(nmax, |m x|) + 16) (mie_coeffs.py:101,119-121), with
// z = m x formed in FP64 from m64 and x64; D_k is then rounded to pairs for
// the numerators, which are as above.
template <bool DN64, class Emit>
__device__ __forceinline__ void homog_core_mixed(const float4 *__restrict__ hd, float4 r0, df xi, float xf,
                                                 const float4 *__restrict__ rowd, int rs, int nmax, Emit &emit,
                                                 double2 m64 = make_double2(0.0, 0.0), double x64 = 0.0)
{
    const float4 hm = hd[0], hmi = hd[1], hz = hd[2];
    const float azm = hd[3].x;
    const df m_re = df{hm.x, hm.y}, m_im = df{hm.z, hm.w};
    const df mi_re = df{hmi.x, hmi.y}, mi_im = df{hmi.z, hmi.w};
    const float mfr = m_re.hi, mfi = m_im.hi, mifr = mi_re.hi, mifi = mi_im.hi;
    const float az = azm * xf;
    const int nmx = (int)rintf(fmaxf((float)nmax, az) + 16.0f);
    const cdf zinv = cdf{df_mul(df{hz.x, hz.y}, xi), df_mul(df{hz.z, hz.w}, xi)};   // 1/z
    // Warm-up steps above nmax.  When |z| < nmax + 1 every step lies where
    // the recurrence damps the start error by (|z| / (2n+1))^2 per step, so
    // the steps are counted for a damping of e^-23 (1e-10; the FP64 path
    // asks for 1e-17); emulated for x in [1e-3, 650]: the same coefficients
    // to 2.2e-7 with 24% fewer steps on the sulfate-like table.
    int warm = nmx - 1 - nmax;
    if (!DN64 && az < (float)(nmax + 1)) {
        const float q = 2.f * logf((2.f * (float)(nmax + 1) + 1.f) / az);
        const int need = (int)ceilf(23.0f / q) + 2;
        if (need < warm) warm = need;
    }
    cdf D = cdf{df{0.f, 0.f}, df{0.f, 0.f}};
    cdf rk, w;
    df iw;
    cplx D64 = cx(0.0, 0.0), zi64 = cx(0.0, 0.0);
    if (DN64) {
        const cplx z64 = cx(m64.x * x64, m64.y * x64);
        const int nmx64 = (int)rint(fmax((double)nmax, cabs(z64)) + 16.0);
        zi64 = 1.0 / z64;
        for (int k = nmx64 - 1; k > nmax; --k) {
            const cplx r = zi64 * (double)(k + 1);
            D64 = r - cinv(D64 + r);
        }
    } else {
        for (int k = nmax + warm; k > nmax; --k) {
            const cdf r = cdf_mul_f(zinv, (float)(k + 1));   // (k+1)/z
            const cdf w1 = cdf_add(D, r);
            const df iw1 = df_rcp(df_fma(w1.re, w1.re, df_mul(w1.im, w1.im)));
            D = cdf{df_fma(df_neg(w1.re), iw1, r.re), df_fma(w1.im, iw1, r.im)};   // r - 1/w
        }
        rk = cdf_mul_f(zinv, (float)(nmax + 1));   // r_nmax = (nmax+1)/z
        w = cdf_add(D, rk);                         // D_{nmax+1} + r_nmax
        iw = df_rcp(df_fma(w.re, w.re, df_mul(w.im, w.im)));
    }
    // psi_k, chi_k (pn) and psi_{k-1}, chi_{k-1} (pm); the row entry of the
    // next order is loaded one order ahead (its latency overlaps an order's
    // arithmetic)
    float4 pn = rowd[(nmax - 1) * rs];
    float4 pm = nmax > 1 ? rowd[(nmax - 2) * rs] : r0;
    for (int k = nmax; k >= 1; --k) {
        const float4 pnext = k > 2 ? rowd[(k - 3) * rs] : r0;
        if (DN64) {
            const cplx r = zi64 * (double)(k + 1);
            D64 = r - cinv(D64 + r);   // D_k
            D = cdf{df_from_f64(D64.re), df_from_f64(D64.im)};
        } else {
            D = cdf{df_fma(df_neg(w.re), iw, rk.re), df_fma(w.im, iw, rk.im)};   // D_k
            if (k > 1) {
                rk = cdf_mul_f(zinv, (float)k);   // r_{k-1} = k/z
                w = cdf_add(D, rk);
                iw = df_rcp(df_fma(w.re, w.re, df_mul(w.im, w.im)));
            }
        }
        const df nx = df_mul_f(xi, (float)k);   // k/x
        const df dar = df_fma(D.re, mi_re, df_fma(df_neg(D.im), mi_im, nx));   // Re(D/m) + k/x
        const df dbr = df_fma(D.re, m_re, df_fma(df_neg(D.im), m_im, nx));     // Re(D m) + k/x
        const df psn = df{pn.x, pn.y}, chn = df{pn.z, pn.w};
        const df psm = df{-pm.x, -pm.y}, chm = df{-pm.z, -pm.w};
        const float nar = df_fma(dar, psn, psm).hi, nbr = df_fma(dbr, psn, psm).hi;
        const float mar = df_fma(dar, chn, chm).hi, mbr = df_fma(dbr, chn, chm).hi;
        const float Dr = D.re.hi, Di = D.im.hi;
        const float dai = fmaf(Dr, mifi, Di * mifr), dbi = fmaf(Dr, mfi, Di * mfr);
        float ida, idb;   // 1 / |N - i M|^2 of a and b
        const float2 a = mie_ratio_f32(nar, dai * pn.x, mar, dai * pn.z, ida);
        const float2 b = mie_ratio_f32(nbr, dbi * pn.x, mbr, dbi * pn.z, idb);
        emit(k, a, b, fmaf(dai, ida, dbi * idb));
        pn = pm;
        pm = pnext;
    }
}

// Emits FP32 (c, d) = (a + b, a - b) and accumulates the efficiency sums of
// pymiecoated/mie_props.py:28-70 from the FP32 a_n, b_n with Kahan
// compensation (the accumulated rounding stays at the FP32 unit roundoff
// whatever nmax is):
//   sca = sum (2n+1)(|a|^2 + |b|^2),
//   abs = sum (2n+1) t_n  (t_n of homog_core_mixed: -(Re(a + b) - |a|^2 - |b|^2)),
//   asy = sum n(n+2)/(n+1) Re(a_n a*_{n+1} + b_n b*_{n+1}) + (2n+1)/(n(n+1)) Re(a_n b*_n),
//   qb  = sum (2n+1)(-1)^n (a_n - b_n).
// The reference's ext = sum (2n+1) Re(a + b) is formed as sca - abs: both
// terms keep their relative precision, so qext, qsca and qabs = qext - qsca
// all do, however weak or strong the absorption.
struct EmitMixed {
    float4 *cf;    // order k at cf[(k - 1) * cs]
    int cs;
    float amax;
    float ab, sca, asy, qbr, qbi;
    float ab_c, sca_c, asy_c, qbr_c, qbi_c;   // Kahan compensations
    float2 pa, pb;                             // a, b of order n+1 (zero above nmax)
    float inv_n1;                              // 1/(n+1)
    __device__ __forceinline__ void operator()(int k, float2 a, float2 b, float t) {
        const float4 q = make_float4(a.x + b.x, a.y + b.y, a.x - b.x, a.y - b.y);
        cf[(k - 1) * cs] = q;
        amax = fmaxf(amax, fmaxf(fmaxf(fabsf(q.x), fabsf(q.y)), fmaxf(fabsf(q.z), fabsf(q.w))));
        const float fk = (float)k;
        const float cn = 2.f * fk + 1.f;
        const float inv_n = __frcp_rn(fk);
        kahan(ab, ab_c, cn * t);
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

// Coated units of the mixed table: the coated recurrences of
// mie_coeffs.py:183-251 with the Toon-Ackerman ratio chain, the psi/chi rows
// and the efficiency sums in FP64 and the three D_n recurrences in
// double-float; the coefficients leave as FP32 (c, d) like the homogeneous
// ones.
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

// Coefficient operand of the contraction (MMA B), written once per (unit,
// 64-size tile, 16-order chunk) as a 16 KB block in the no-swizzle K-major
// shared-memory layout
//   [matrix C_hi C_lo D_hi D_lo][kg = order / 8 % 2][row / 8][row % 8][8 orders]
// (rows 2 i, 2 i + 1 = Re, Im of size i of the tile), so that the contraction
// loads a tile's chunk with one 16 KB bulk copy and multiplies the whole tile
// or either half of it.  split_rows writes the rows of
// one instance (size i of its unit): FP32 (c, d) orders 1..nmax -> FP16
// hi/lo scaled by 2^(13 - e_i), in every chunk of the instance's tile, zero
// past nmax.  The coefficient kernels call it
// once an instance is done: its coefficients are still in L2.  The chunk
// bases of the tile (SplitIdx) are loaded when the instance starts, so their
// latency overlaps the recurrences.
struct SplitIdx {
    int cb0, cb1;    // tile_cbase[tile], [tile + 1] of the instance's grid
    long long ucb;   // unit_cbase[unit]
};
__device__ __forceinline__ SplitIdx split_idx(const TabView &v, int64_t unit, int i,
                                              const int *__restrict__ tile_cbase,
                                              const int64_t *__restrict__ unit_cbase, int ntiles)
{
    const int lam = (int)(unit / ((int64_t)v.n_rh * v.n_comp));
    const int *tcb = tile_cbase + (size_t)v.le(lam) * (ntiles + 1) + (i >> 6);
    SplitIdx s;
    s.cb0 = ldg_pin_s32(tcb);
    s.cb1 = ldg_pin_s32(tcb + 1);
    s.ucb = ldg_pin_s64(unit_cbase + unit);
    return s;
}
// cfi[k * cstride]: order k + 1 (global memory, stride 1, or this thread's
// column of the block's shared staging, stride blockDim)
__device__ __forceinline__ void split_rows(const TabView &v, int i, int ex, int nmax, const float4 *cfi, int cstride,
                                           const SplitIdx &si, uint8_t *__restrict__ asplit)
{
    const int tile = i >> 6, ia = i & 63;
    const int nc = si.cb1 - si.cb0;
    uint8_t *dst = asplit + (size_t)(si.ucb + si.cb0) * 16384;
    const float sc = ldexpf(1.0f, max(-126, min(126, SHIFT_BITS - ex)));
    const int r0 = 2 * ia;
    for (int j = 0; j < nc; ++j)
#pragma unroll
        for (int kg = 0; kg < 2; ++kg) {
            __half ch[4][8], cl[4][8];
#pragma unroll
            for (int jj = 0; jj < 8; ++jj) {
                const int k = 16 * j + 8 * kg + jj;
                float4 q = make_float4(0.f, 0.f, 0.f, 0.f);
                if (k < nmax) q = cfi[k * cstride];
                split_f16(q.x * sc, ch[0][jj], cl[0][jj]);
                split_f16(q.y * sc, ch[1][jj], cl[1][jj]);
                split_f16(q.z * sc, ch[2][jj], cl[2][jj]);
                split_f16(q.w * sc, ch[3][jj], cl[3][jj]);
            }
            // rows r0 (Re) and r1 = r0 + 1 (Im) of a matrix are 32 contiguous,
            // 32-byte aligned bytes (r0 even): one 256-bit store each
            const uint32_t o0 = kg * 2048 + (r0 >> 3) * 128 + (r0 & 7) * 16;
            uint8_t *blk = dst + (size_t)j * 16384;
            st_global_32b(blk + 0 * TC_MAT_B + o0, *(uint4 *)ch[0], *(uint4 *)ch[1]);
            st_global_32b(blk + 1 * TC_MAT_B + o0, *(uint4 *)cl[0], *(uint4 *)cl[1]);
            st_global_32b(blk + 2 * TC_MAT_B + o0, *(uint4 *)ch[2], *(uint4 *)ch[3]);
            st_global_32b(blk + 3 * TC_MAT_B + o0, *(uint4 *)cl[2], *(uint4 *)cl[3]);
        }
    // the sizes of a partial tile also zero the rows of the sizes the tile
    // lacks (their PSD weights are zero, but 0 x NaN would not be): a
    // whole-tile MMA reads all 128 rows.  Size ia takes the absent sizes ia +
    // ntile, ia + 2 ntile, ... (one 32-byte store per row pair, as above)
    const int ntile = min(64, v.n_size - 64 * tile);
    if (ntile < 64) {
        const uint4 z = make_uint4(0u, 0u, 0u, 0u);
        for (int a = ia + ntile; a < 64; a += ntile) {
            const int r = 2 * a;
            for (int j = 0; j < nc; ++j)
#pragma unroll
                for (int kg = 0; kg < 2; ++kg) {
                    const uint32_t o = kg * 2048 + (r >> 3) * 128 + (r & 7) * 16;
                    uint8_t *blk = dst + (size_t)j * 16384;
#pragma unroll
                    for (int mtx = 0; mtx < 4; ++mtx) st_global_32b(blk + mtx * TC_MAT_B + o, z, z);
                }
        }
    }
}

// Persistent like k_tab_coeffs_mixed: warps take (unit, 32-size group)
// tasks, heavy groups first, from the plan's task list.
__global__ void __launch_bounds__(128) k_tab_coeffs_mixed_coated(TabView v, const int2 *__restrict__ tasks,
                                                                 int ntasks, int *__restrict__ next,
                                                                 float4 *__restrict__ cf, int *__restrict__ eexp,
                                                                 int *__restrict__ eunit, int *flags,
                                                                 const int *__restrict__ tile_cbase,
                                                                 const int64_t *__restrict__ unit_cbase, int ntiles,
                                                                 uint8_t *__restrict__ asplit)
{
    const int lane = threadIdx.x & 31;
    for (;;) {
        int tk_i = 0;
        if (lane == 0) tk_i = atomicAdd(next, 1);
        tk_i = __shfl_sync(0xffffffffu, tk_i, 0);
        if (tk_i >= ntasks) break;
        const int2 tk = tasks[tk_i];   // (unit, group)
        const int i = 32 * tk.y + lane;
        const int64_t unit = tk.x;
        if (i < v.n_size) {
            const int64_t t = unit * v.n_size + i;
            const int lam = (int)(unit / ((int64_t)v.n_rh * v.n_comp));
            const int le = v.le(lam);
            const int64_t row = (int64_t)le * v.n_size + i;
            const int64_t o = v.off[row];
            const int nmax = (int)(v.off[row + 1] - o);
            const int64_t c = v.unit_base[unit] + (o - v.off[(int64_t)le * v.n_size]);
            const double x = v.xg[row];
            EmitCf emit{cf + c, 0.f};
            EffSums es;
            coated_table_instance<EmitCf, true>(v, unit, c, o, nmax, x, emit, es, flags);
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
            split_rows(v, i, ex, nmax, cf + c, 1, split_idx(v, unit, i, tile_cbase, unit_cbase, ntiles), asplit);
        }
        __syncwarp();
    }
}

// One thread per instance; the threads of a unit are padded to whole warps
// (n_pad = 32 ngrp per unit) so that a warp is one group of 32 sizes and its
// row loads and coefficient stores are one contiguous segment per order.
// One instance (unit, size i) of the mixed coefficients: the recurrences,
// the efficiencies, the instance's exponent and its rows of the
// contraction's split operand.  stage: this thread's column of the block's
// shared staging (stride stage_stride); an instance of one 16-order chunk
// keeps its coefficients there until split_rows reads them (no global round
// trip), longer ones go through cf.
template <bool DN64>
__device__ __forceinline__ void coeffs_mixed_instance(const TabView &v, int64_t unit, int i, float4 *__restrict__ cf,
                                                      float4 *stage, int stage_stride, int *__restrict__ eexp,
                                                      int *__restrict__ eunit, const int *__restrict__ tile_cbase,
                                                      const int64_t *__restrict__ unit_cbase, int ntiles,
                                                      uint8_t *__restrict__ asplit)
{
    const int64_t t = unit * v.n_size + i;   // the instance
    const int lam = (int)(unit / ((int64_t)v.n_rh * v.n_comp));
    const int le = v.le(lam);
    const int64_t row = (int64_t)le * v.n_size + i;
    const int64_t o = v.off[row];
    const int nmax = (int)(v.off[row + 1] - o);
    const int64_t gb = v.grel[(int64_t)le * (v.ngrp + 1) + (i >> 5)] + (i & 31);   // order 1 within the block
    const float4 rc0 = v.rowcd[2 * row], rc1 = v.rowcd[2 * row + 1];
    const df xi = df{rc1.x, rc1.y};
    const bool staged = nmax <= TC_KC16;
    EmitMixed emit;
    emit.cf = staged ? stage : cf + v.gunit[unit] + gb;
    emit.cs = staged ? stage_stride : 32;
    emit.amax = 0.f;
    emit.ab = emit.sca = emit.asy = emit.qbr = emit.qbi = 0.f;
    emit.ab_c = emit.sca_c = emit.asy_c = emit.qbr_c = emit.qbi_c = 0.f;
    emit.pa = emit.pb = make_float2(0.f, 0.f);
    emit.inv_n1 = __frcp_rn((float)(nmax + 1));
    const float4 *rowd = v.pcd + v.grow[le] + gb;
    if (DN64) homog_core_mixed<true>(v.hdf + 4 * unit, rc0, xi, rc1.z, rowd, 32, nmax, emit, v.m[unit], v.xg[row]);
    else homog_core_mixed<false>(v.hdf + 4 * unit, rc0, xi, rc1.z, rowd, 32, nmax, emit);
    // efficiencies from the compensated sums (value = sum - compensation), in
    // pairs; one FP64 addition per output
    const df iy2 = df_mul(xi, xi);   // 1 / x^2
    const df sca = df_two_sum(emit.sca, -emit.sca_c);
    const df sca2 = df_mul(sca, iy2);
    const df qsca = df{2.f * sca2.hi, 2.f * sca2.lo};
    const df ab2 = df_mul(df_two_sum(emit.ab, -emit.ab_c), iy2);
    const df qext = df_sub(qsca, df{2.f * ab2.hi, 2.f * ab2.lo});
    const df qr = df_two_sum(emit.qbr, -emit.qbr_c), qi = df_two_sum(emit.qbi, -emit.qbi_c);
    const df qbv = df_mul(df_fma(qr, qr, df_mul(qi, qi)), iy2);
    const df asy = df_mul(df_two_sum(emit.asy, -emit.asy_c), df_rcp(sca));   // 4/x^2 asy / qsca, halved
    double *o4 = v.eff4 + t * 4;
    o4[0] = df_to_f64(qext);
    o4[1] = df_to_f64(qsca);
    o4[2] = df_to_f64(qbv);
    o4[3] = df_to_f64(df{2.f * asy.hi, 2.f * asy.lo});
    const int ex = emit.amax > 0.f ? ilogbf(emit.amax) : -1000;
    eexp[t] = ex;
    atomicMax(eunit + unit, ex);
    split_rows(v, i, ex, nmax, emit.cf, emit.cs, split_idx(v, unit, i, tile_cbase, unit_cbase, ntiles), asplit);
}

// Persistent: a grid that fills the GPU once (blocks resident per SM x SMs);
// every warp takes tasks -- one group of 32 sizes of one unit, a lane per
// size -- from a global counter until none is left.  The task list (plan
// time) orders the groups by decreasing largest nmax (heavy tasks first, so
// that the last ones to run are light) and no warp waits for its block's
// other warps, so that the SMs stay filled to the end: with a thread per
// instance and one block per 64 or 128 sizes, blocks held their slots until
// their slowest warp finished and the SMs ran at about 12 of the 20 warps
// their registers allow.
template <bool DN64>
__global__ void __launch_bounds__(256) k_tab_coeffs_mixed(TabView v, const int2 *__restrict__ tasks, int ntasks,
                                                          int *__restrict__ next, float4 *__restrict__ cf,
                                                          int *__restrict__ eexp, int *__restrict__ eunit,
                                                          const int *__restrict__ tile_cbase,
                                                          const int64_t *__restrict__ unit_cbase, int ntiles,
                                                          uint8_t *__restrict__ asplit)
{
    extern __shared__ float4 cf_stage[];
    const int lane = threadIdx.x & 31;
    for (;;) {
        int t = 0;
        if (lane == 0) t = atomicAdd(next, 1);
        t = __shfl_sync(0xffffffffu, t, 0);
        if (t >= ntasks) break;
        const int2 tk = tasks[t];   // (unit, group)
        const int i = 32 * tk.y + lane;
        if (i < v.n_size)
            coeffs_mixed_instance<DN64>(v, tk.x, i, cf, cf_stage + threadIdx.x, (int)blockDim.x, eexp, eunit,
                                        tile_cbase, unit_cbase, ntiles, asplit);
        __syncwarp();
    }
}

// blocks of k_tab_coeffs_mixed resident per SM at `block` threads, times the SMs
static int coef_grid(gbmie_ctx *ctx, bool dn64, int block, int *grid)
{
    int nb = 0, nsm = 0;
    GBMIE_TRY(ctx_cuda(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                                &nb, dn64 ? k_tab_coeffs_mixed<true> : k_tab_coeffs_mixed<false>, block,
                                TC_KC16 * sizeof(float4) * (size_t)block),
                       "coefficient occupancy"));
    GBMIE_TRY(ctx_cuda(ctx, cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, ctx->device), "SM count"));
    *grid = (nb > 0 ? nb : 1) * nsm;
    return GBMIE_OK;
}

// Per-unit and per-row constants of the mixed recurrences as FP32 pairs:
// hdf[4 u] = m, 1/m, x/z (1/z = (x/z)(1/x)), (|z|/x); rowcd[2 j] = (sin x, cos x),
// (1/x, x).
__global__ void k_mixed_consts(int64_t n_units, const HomogIndex *__restrict__ hidx, float4 *__restrict__ hdf,
                               int64_t nrows, const double4 *__restrict__ rowc, const double *__restrict__ xg,
                               float4 *__restrict__ rowcd)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n_units) {
        const HomogIndex h = hidx[i];
        const df a = df_from_f64(h.m.re), b = df_from_f64(h.m.im);
        const df c = df_from_f64(h.minv.re), d = df_from_f64(h.minv.im);
        const df e = df_from_f64(h.zminv.re), f = df_from_f64(h.zminv.im);
        hdf[4 * i] = make_float4(a.hi, a.lo, b.hi, b.lo);
        hdf[4 * i + 1] = make_float4(c.hi, c.lo, d.hi, d.lo);
        hdf[4 * i + 2] = make_float4(e.hi, e.lo, f.hi, f.lo);
        hdf[4 * i + 3] = make_float4((float)h.azm, 0.f, 0.f, 0.f);
    }
    if (i < nrows) {
        const double4 rc = rowc[i];
        const df s = df_from_f64(rc.x), c = df_from_f64(rc.y), xi = df_from_f64(rc.z);
        rowcd[2 * i] = make_float4(s.hi, s.lo, c.hi, c.lo);
        rowcd[2 * i + 1] = make_float4(xi.hi, xi.lo, (float)xg[i], 0.f);
    }
}

__global__ void k_fill_int(int n, int *p, int val)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) p[i] = val;
}

// ---------------------------------------------------------------------------
// Angle-function operand (MMA A): (p, q) = (pi~ + tau~, pi~ - tau~) split
// into FP16 hi/lo, one 16 KB block per (128-angle block, 16-order chunk) in
// the no-swizzle K-major shared-memory layout
//   [matrix P_hi P_lo Q_hi Q_lo][kg = order / 8 % 2][angle / 8 (16)][angle % 8][8 orders]
// ---------------------------------------------------------------------------
__global__ void k_tab_bt_f16(int nang, int n_pad, int k_pad, int nmax, const double *__restrict__ cost,
                             __half *__restrict__ bt)
{
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= n_pad) return;
    const int nkc = k_pad / 16;
    const int ab = a / TC_ABLK, ag = (a % TC_ABLK) >> 3, a8 = a & 7;
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
        const size_t mat = TC_MAT_A / 2;   // halves per matrix
        const size_t off = (size_t)(ab * nkc + (k >> 4)) * 4 * mat + (((k >> 3) & 1) * 16 + ag) * 64 + a8 * 8 + (k & 7);
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
// orders are split into windows of g.win (<= TC_WIN_MAX) 16-order chunks; each window
// starts a fresh accumulator, adds the two cross products of its orders
// (P_hi C_lo, P_lo C_hi, 2^-11 of the result) while the accumulator is small
// and then the P_hi C_hi products, and the epilogue adds the windows in FP32
// registers with round-to-nearest.  Emulating the measured rule puts the
// bulk P11 error at x = 628 near 2.6e-7 this way.
//
// Orientation: angles are the MMA's M (128 per block, TMEM lanes), the
// (size, Re/Im) rows of a 64-size tile its N (128 columns), or of half a
// tile (64 columns) when the tile's orders span several accumulation
// windows.  Each epilogue thread owns one angle and 16 sizes of each half
// tile, so the Mueller elements and their PSD-weighted sums over sizes stay
// in its registers: no shared-memory staging, no shuffles and no barrier
// among the epilogue warps.
//
// Pipeline (one CTA per SM, persistent, 12 warps):
//   warps 0-7   epilogue: warp w reads TMEM lanes 32 (w % 4) .. + 31 (its
//               angles) and columns of sizes 16 (w / 4) .. + 15 of each half
//               tile; window sums -> Mueller -> PSD-weighted sums
//   warps 8, 10 MMA issue (one thread each; items alternate between them)
//   warp 9      producer (one thread): bulk copies of the coefficient chunks
//               of a tile (split_rows) and of the angle functions of orders
//               > 16 into a TC_NS(NB)-stage shared-memory ring
//   warp 11     weights: per tile the chunk count, the unit's constants and
//               the PSD weights, scaled and paired for the epilogue's packed
//               FMAs, into a TC_NW-slot shared-memory ring (the epilogue
//               warps make no global loads)
// Work items are (unit, angle block, 64-size tile) when the tile's orders
// fit one accumulation window (S+ and S- of its 64 sizes fill both of an
// issuer's accumulator sets), else (unit, angle block, tile, half tile) with
// one set per window; a half tile without sizes (the last tile of a grid) is
// skipped by every role.  Whole-tile items halve the windows, MMA
// instructions and hand-offs per size, which is what the contraction's time
// follows.  TMEM holds TC_NSETS accumulator sets of 128 columns, so the MMAs
// run up to two whole-tile or four half-tile windows ahead of the epilogue.
// The angle-function chunk of orders 1..16 stays resident for up to
// TC_B0_SLOTS angle blocks (loaded once: it is the same for every unit; 84%
// of the sulfate-like table's tiles need no other order); with more blocks
// one slot is reloaded at every (unit, block) change.  mbarriers: stage
// full/empty, resident full/empty, accumulator-set full/empty, weight slot
// full/empty.  Every wait is bounded and also ends when another role has
// raised the block's abort flag; the epilogue warps decide per warp (lane 0
// waits, the warp follows its answer).
// ---------------------------------------------------------------------------
struct TcArgs {
    TabView v;
    const float4 *cf;
    const int *eexp;
    const int *eunit;
    const __half *bt;
    int n_pad, k_pad;
    const int *unit_order;
    const uint8_t *asplit;       // coefficient operand (split_rows)
    const int *tile_cbase;       // [n_le][ntiles + 1]
    const int64_t *unit_cbase;   // [n_units]
    int ntiles;
    int win;                     // accumulation window (16-order chunks, <= TC_WIN_MAX)
    uint32_t wait_limit;         // tries of every pipeline wait (gbmie_table_plan_set_wait_limit)
    int ntr, tpr;                // tile ranges per (unit, angle block) and tiles per range
    int *flags;
};

// ring stages of a tile's chunk (coefficients of 64 sizes, angle functions
// of orders > 16): the copies of a stage's next chunk wait for its MMAs, so
// the ring's depth bounds the chunks in flight.  Sulfate-like table (5
// bins), the same GB300 in one run: 4 stages 2.79-2.80 ms (table 4.43 ms,
// e2e 905-916M instance-evals/s), 5 stages 2.73 ms (table 4.36 ms, e2e 926M);
// tables of more bins keep 4 (their running sums and weights leave no room
// for a fifth)
#define TC_NS(NB) ((NB) <= 5 ? 5 : 4)
// longest accumulation window (chunks): the windows the accuracy of the FP32
// accumulation was checked with (2-4 keep it near 2e-7); a window's chunks
// sit in the ring together
#define TC_WIN_MAX 4
static_assert(TC_WIN_MAX <= TC_NS(8), "a window's chunks must fit the ring");
#define TC_NSETS 4                                     // TMEM accumulator sets of 128 columns
// resident angle-function chunks (angle blocks; tables of more than 256
// angles reload one slot per (unit, block))
#define TC_B0_SLOTS(NB) 2
#define TC_A_BYTES (4 * TC_MAT_A)                      // P_hi P_lo Q_hi Q_lo of a chunk: 16 KB
#define TC_B_BYTES (4 * TC_MAT_B)                      // C_hi C_lo D_hi D_lo of a tile's chunk: 16 KB
#define TC_STAGE_BYTES (TC_B_BYTES + TC_A_BYTES)       // 32 KB
#define TC_EPI_WARPS 8
#define TC_EPI_THREADS (32 * TC_EPI_WARPS)
#define TC_THREADS (TC_EPI_THREADS + 128)              // + two MMA warps, the producer and the weights warp
// register bound of 12 warps: three warps on an SM sub-partition fit its
// 16K registers at 168 each
#define TC_REG_BOUND_THREADS 384
// weight-ring slots (items); with half-tile items only, measured on the
// sulfate-like table with 2, 4, 6, 8 and 10 slots: 3.23, 3.10, 3.03, 3.06,
// 3.09 ms; with whole-tile items 4 and 6 slots measure the same (2.86 ms)
#define TC_NW 4
// mbarriers (2 TC_NS + 2 + 2 TC_NSETS + 1 + 2 TC_NW), the TMEM address, the
// abort flag and the stages' chunk tags
#define TC_CTRL_BYTES 512
#define TC_NP(NB) (((NB) + 1) / 2)                     // float4 weight entries per size: two bins each
#define TC_WSLOT_FLOATS(NB) (16 + TC_INST * 4 * TC_NP(NB))   // header + 64 sizes x bin pairs x (w, w, w', w')
#define TC_SUM_FLOATS(NB) (4 * (NB) * TC_EPI_THREADS)  // running sums [bin][thread] of (E0 pair, E1 pair)
#define TC_SMEM_BYTES(NB)                                                                                  \
    (TC_B0_SLOTS(NB) * TC_A_BYTES + TC_NS(NB) * TC_STAGE_BYTES + TC_NW * TC_WSLOT_FLOATS(NB) * 4 +             \
     TC_SUM_FLOATS(NB) * 4 + TC_CTRL_BYTES)
#define TC_NO_EX (-0x40000000)                         // no size: its weights are dropped
#define TC_SLEEP_NS 32                                 // back-off of the MMA and producer waits
// back-off of the epilogue warps' waits (their lane 0 polls the weight slot
// and the accumulator set): a polling warp takes issue slots from the
// single-thread roles on its sub-partition.  Sulfate-like table, contraction
// 3.04 ms without back-off, 2.98 / 2.97 / 2.97 ms with 32 / 128 / 512 ns; a
// try_wait suspend-time hint of 1 us instead: 3.13 ms; back-off in the
// issuers' waits as well: 2.99-3.01 ms
#define TC_EPI_SLEEP_NS 128

static_assert(TC_NSETS * 128 <= 512, "TMEM columns");
static_assert(8 * (2 * TC_NS(1) + 2 + 2 * TC_NSETS + 1 + 2 * TC_NW) + 4 + 8 + 4 * TC_NS(1) <= TC_CTRL_BYTES, "control block");
static_assert(TC_SMEM_BYTES(1) <= 227 * 1024 && TC_SMEM_BYTES(2) <= 227 * 1024 && TC_SMEM_BYTES(3) <= 227 * 1024 &&
                  TC_SMEM_BYTES(4) <= 227 * 1024 && TC_SMEM_BYTES(5) <= 227 * 1024 && TC_SMEM_BYTES(6) <= 227 * 1024 &&
                  TC_SMEM_BYTES(7) <= 227 * 1024 && TC_SMEM_BYTES(8) <= 227 * 1024,
              "shared memory");

// k-th unit of CTA `cta` among G CTAs: units in decreasing-work order,
// dealt in a snake (c, then G-1-c) so that every CTA gets a similar mix.
__device__ __forceinline__ int64_t tc_unit_index(int k, int cta, int G)
{
    return (int64_t)k * G + ((k & 1) ? (G - 1 - cta) : cta);
}

// Work items of the contraction: (unit, angle block, range of tpr tiles),
// units in decreasing-work order (unit_order), the k-th of CTA cta dealt as
// above.  A (unit, block) split over several items, possibly on several
// CTAs, is summed by the FP64 additions of the items' partial sums, so that
// tables with few units (a single wavelength, or 20) still fill every SM.
struct TcWork {
    int64_t unit;
    int ab, t0, t1;
    bool valid;
};
__device__ __forceinline__ TcWork tc_work(const TcArgs &g, int k, int cta, int G, int nblocks, int ntl,
                                          int64_t n_units)
{
    TcWork w;
    const int64_t per = (int64_t)nblocks * g.ntr;
    const int64_t widx = tc_unit_index(k, cta, G);
    w.valid = widx < n_units * per;
    if (!w.valid) {
        w.unit = 0;
        w.ab = w.t0 = w.t1 = 0;
        return w;
    }
    const int64_t r = widx / per;
    const int rem = (int)(widx - r * per);
    w.ab = rem / g.ntr;
    w.t0 = (rem - w.ab * g.ntr) * g.tpr;
    w.t1 = min(ntl, w.t0 + g.tpr);
    w.unit = g.unit_order[r];
    return w;
}

template <int NB>
__global__ void __launch_bounds__(TC_REG_BOUND_THREADS, 1) k_tab_s12_tc(TcArgs g)
{
    extern __shared__ __align__(1024) uint8_t smem[];
    constexpr int NS = TC_NS(NB);                                   // ring stages
    uint8_t *sB0 = smem;                                            // resident angle chunks, orders 1..16
    uint8_t *sStage = sB0 + TC_B0_SLOTS(NB) * TC_A_BYTES;           // NS x (coeff 16 KB | angles 16 KB)
    float *sW = (float *)(sStage + NS * TC_STAGE_BYTES);         // weight ring [TC_NW][TC_WSLOT_FLOATS(NB)]
    float *sSum = sW + TC_NW * TC_WSLOT_FLOATS(NB);                 // per-(unit, block) running sums
    uint64_t *bars = (uint64_t *)(sSum + TC_SUM_FLOATS(NB));
    uint64_t *full = bars, *empty = bars + NS;
    uint64_t *b0_full = bars + 2 * NS, *b0_empty = b0_full + 1;
    uint64_t *acc_full = b0_full + 2, *acc_empty = acc_full + TC_NSETS, *drain = acc_empty + TC_NSETS;
    uint64_t *w_full = drain + 1, *w_empty = w_full + TC_NW;
    uint32_t *s_tmem = (uint32_t *)(w_empty + TC_NW);
    volatile int *s_abort = (volatile int *)(s_tmem + 1);
    // s_chunk[st]: the chunk the producer is loading into stage st.  An issuer
    // skips the other issuer's chunks, so it can wait on a stage two phases
    // ahead of the producer, where the barrier's parity alone would also match
    // the older phase; it trusts the parity only once s_chunk holds its chunk
    // (the producer writes it after the stage's previous chunk was consumed,
    // so the stage's pending phase is then exactly that chunk's).
    volatile int *s_chunk = s_abort + 2;

    const TabView &v = g.v;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int nblocks = g.n_pad / TC_ABLK;
    const int nkc = g.k_pad / TC_KC16;
    const int ntl = g.ntiles;
    const bool reload = nblocks > TC_B0_SLOTS(NB);   // one resident slot, reloaded per (unit, block)
    if (warp == 0) tmem_alloc(s_tmem, 512);
    if (tid == 0) {
        for (int i = 0; i < NS; ++i) {
            mbar_init(full + i, 1);    // the producer's arrival with the copies' bytes
            mbar_init(empty + i, 1);   // tcgen05.commit
        }
        mbar_init(b0_full, 1);
        mbar_init(b0_empty, 2);   // both issuers leave the block
        for (int i = 0; i < TC_NSETS; ++i) {
            mbar_init(acc_full + i, 1);
            mbar_init(acc_empty + i, TC_EPI_WARPS);
        }
        mbar_init(drain, 2);
        for (int i = 0; i < TC_NW; ++i) {
            mbar_init(w_full + i, 1);                 // the weights warp's lane 0
            mbar_init(w_empty + i, TC_EPI_WARPS);     // every epilogue warp, after its compute
        }
        fence_mbar_init();
        *s_abort = 0;
        for (int i = 0; i < NS; ++i) s_chunk[i] = -1;
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *s_tmem;
    const int64_t n_units = (int64_t)v.n_lambda * v.n_rh * v.n_comp;
    const int G = gridDim.x, cta = blockIdx.x;

    if (warp == 8 || warp == 10) {
        // ================= MMA issue: two issuers, alternate items =================
        // Issuer p (warp 8: p = 0, warp 10: p = 1) takes the items of parity p
        // and the accumulator sets 2p, 2p + 1; both walk every item to keep
        // the ring's chunk count.  One issuing thread alone could not keep up:
        // the issue of one small MMA and its bookkeeping took several times
        // the tensor core's time for it.
        const uint32_t p = warp == 10 ? 1u : 0u;
        if (lane == 0) {
            // whole-tile items N = 128 (64 sizes x Re, Im), half-tile items N = 64
            const uint32_t idesc_t = idesc_f16_f32(TC_ABLK, 2 * TC_INST), idesc_h = idesc_f16_f32(TC_ABLK, 2 * TC_HALF);
            // no-swizzle K-major descriptors without the start address: A (angles)
            // LBO = 16 core matrices (K step of 8 orders), B (coefficients) 16; SBO 128 B
            constexpr uint64_t DESC_A = ((uint64_t)((16 * 128) >> 4) << 16) | ((uint64_t)(128 >> 4) << 32) | (1ull << 46);
            constexpr uint64_t DESC_B = ((uint64_t)((16 * 128) >> 4) << 16) | ((uint64_t)(128 >> 4) << 32) | (1ull << 46);
            const uint32_t sStage0 = smem_u32(sStage);
            uint32_t it = 0, ii = 0, wc = 0, b0_loads = 0;   // chunks, items, own windows
            bool ok = true, have_b0 = false;
            if (!reload) {   // every block's resident chunk, loaded once
                ok = mbar_wait_or_abort(b0_full, 0, s_abort, 0, g.wait_limit);
                b0_loads = 1;
            }
            for (int k = 0; ok; ++k) {
                const TcWork wk = tc_work(g, k, cta, G, nblocks, ntl, n_units);
                if (!wk.valid) break;
                const int64_t unit = wk.unit;
                const int lam = (int)(unit / ((int64_t)v.n_rh * v.n_comp));
                const int64_t *off = v.off + (int64_t)v.le(lam) * v.n_size;
                {
                    const int ab = wk.ab;
                    if (reload) {   // the producer reloads the resident slot
                        if (have_b0) mma_commit(b0_empty);
                        if (!mbar_wait_or_abort(b0_full, b0_loads & 1u, s_abort, TC_SLEEP_NS, g.wait_limit)) {
                            ok = false;
                            break;
                        }
                        ++b0_loads;
                        have_b0 = true;
                    }
                    const uint32_t aB0 = smem_u32(sB0 + (reload ? 0 : ab) * TC_A_BYTES);
                    // nmax of a tile's last size, loaded one tile ahead
                    auto last_of = [&](int t) { return min(TC_INST * (t + 1), v.n_size); };
                    long long o1 = ldg_pin_s64(off + last_of(wk.t0)), o0 = ldg_pin_s64(off + last_of(wk.t0) - 1);
                    for (int tile = wk.t0; tile < wk.t1 && ok; ++tile) {
                        const int t0 = tile * TC_INST, ntile = min(TC_INST, v.n_size - t0);
                        const int kt = (int)(o1 - o0);
                        if (tile + 1 < wk.t1) {
                            o1 = ldg_pin_s64(off + last_of(tile + 1));
                            o0 = ldg_pin_s64(off + last_of(tile + 1) - 1);
                        }
                        const int nc = (kt + TC_KC16 - 1) / TC_KC16;
                        // a tile whose chunks fit one window is one item (N = 128,
                        // its S+ and S- in both of the issuer's accumulator sets);
                        // otherwise each half tile with sizes is one (N = 64, one
                        // set per window)
                        const bool whole = nc <= g.win;
                        const int nitem = whole ? 1 : (ntile > TC_HALF ? 2 : 1);
                        for (int h = 0; h < nitem && ok; ++h, ++ii) {
                            if ((ii & 1u) != p) {   // the other issuer's item
                                it += nc;
                                continue;
                            }
                            const uint32_t bh = whole ? 0u : (uint32_t)h * (1024 >> 4);   // half tile: rows 64 h..
                            const uint32_t idesc = whole ? idesc_t : idesc_h;
                            for (int w0 = 0; w0 < nc && ok; w0 += g.win) {
                                const int nj = min(g.win, nc - w0);
                                // accumulator sets: one per window, both for a whole tile
                                const int nset = whole ? 2 : 1;
                                uint32_t set[2];
                                for (int q = 0; q < nset && ok; ++q) {
                                    const uint32_t x = wc + q;
                                    set[q] = 2 * p + (x & 1u);
                                    const uint32_t use = x >> 1;
                                    if (use > 0 &&
                                        !mbar_wait_or_abort(acc_empty + set[q], (use - 1) & 1u, s_abort, 0, g.wait_limit))
                                        ok = false;
                                }
                                if (!ok) break;
                                for (int j = 0; j < nj && ok; ++j) {
                                    const uint32_t c = it + j, st = c % NS, par = (c / NS) & 1u;
                                    ok = false;
                                    for (uint32_t tr = 0; tr < g.wait_limit; ++tr) {
                                        if (s_chunk[st] == (int)c) {
                                            if (mbar_try(full + st, par)) {
                                                ok = true;
                                                break;
                                            }
                                        } else {
                                            __nanosleep(TC_SLEEP_NS);   // the producer has not reached c
                                        }
                                        if ((tr & 255u) == 255u && *s_abort) break;
                                    }
                                }
                                if (!ok) break;
                                tc_fence_after();
                                // S+ and S- columns: a half-tile window's set holds S+ at
                                // 0 and S- at 64; a whole tile's S+ fills one set, S- the other
                                const uint32_t dp = tmem + set[0] * 128;
                                const uint32_t dm = whole ? tmem + set[1] * 128 : dp + 64;
                                for (int pass = 0; pass < 2; ++pass) {
                                    for (int j = 0; j < nj; ++j) {
                                        const uint32_t c = it + j;
                                        const uint32_t sB = sStage0 + (c % NS) * TC_STAGE_BYTES;
                                        const uint32_t sA = (w0 + j) == 0 ? aB0 : sB + TC_B_BYTES;
                                        // descriptors: constant LBO/SBO fields + start address / 16;
                                        // matrix m of an operand starts m x its matrix size later
                                        const uint64_t a0 = DESC_A | (sA >> 4), b0 = (DESC_B | (sB >> 4)) + bh;
                                        constexpr uint64_t MA = TC_MAT_A >> 4, MB = TC_MAT_B >> 4;
                                        if (pass == 0) {   // cross products: small accumulator
                                            mma_f16(dp, a0, b0 + MB, idesc, j == 0 ? 0u : 1u);
                                            mma_f16(dp, a0 + MA, b0, idesc, 1u);
                                            mma_f16(dm, a0 + 2 * MA, b0 + 3 * MB, idesc, j == 0 ? 0u : 1u);
                                            mma_f16(dm, a0 + 3 * MA, b0 + 2 * MB, idesc, 1u);
                                        } else {
                                            mma_f16(dp, a0, b0, idesc, 1u);
                                            mma_f16(dm, a0 + 2 * MA, b0 + 2 * MB, idesc, 1u);
                                            mma_commit(empty + c % NS);   // stage free when its MMAs are done
                                        }
                                    }
                                }
                                it += nj;
                                for (int q = 0; q < nset; ++q) mma_commit(acc_full + set[q]);
                                wc += nset;
                            }
                        }
                    }
                }
            }
            if (!ok) {
                *s_abort = 1;
                atomicOr(g.flags, GBMIE_FLAG_TIMEOUT);
            }
            // every issued MMA (both issuers) has finished before TMEM is released
            mma_commit(drain);
            if (!mbar_wait(drain, 0)) atomicOr(g.flags, GBMIE_FLAG_TIMEOUT);
        }
        __syncwarp();
    } else if (warp == 9) {
        // ================= producer: bulk copies (one thread) =================
        if (lane == 0) {
            uint32_t it = 0, b0_loads = 0;
            // the phase of the latest bulk copy into each ring stage (bit
            // NS + st: stage st has one) and into the resident slot, so
            // that an abort can wait for every copy still in flight
            uint32_t st_phase = 0, tx_used = 0, b0_phase = 0;
            bool ok = true;
            if (!reload) {
                mbar_arrive_expect_tx(b0_full, (uint32_t)(nblocks * TC_A_BYTES));
                for (int b = 0; b < nblocks; ++b)
                    bulk_g2s(sB0 + b * TC_A_BYTES, (const uint8_t *)g.bt + (size_t)b * nkc * TC_A_BYTES, TC_A_BYTES,
                             b0_full);
                tx_used |= 1u << (2 * NS);
                b0_phase = 0;
            }
            for (int k = 0; ok; ++k) {
                const TcWork wk = tc_work(g, k, cta, G, nblocks, ntl, n_units);
                if (!wk.valid) break;
                const int64_t unit = wk.unit;
                const int lam = (int)(unit / ((int64_t)v.n_rh * v.n_comp));
                const int *tcb = g.tile_cbase + (size_t)v.le(lam) * (ntl + 1);
                const uint8_t *ua = g.asplit + (size_t)g.unit_cbase[unit] * TC_B_BYTES;
                const int comp = (int)(unit % v.n_comp), rhi = (int)((unit / v.n_comp) % v.n_rh);
                const float *uW = v.Wf + v.wlam(lam) + ((size_t)rhi * v.n_bin * v.n_comp + comp) * v.n_size;
                const int *uex = g.eexp + (size_t)unit * v.n_size;
                {
                    const int ab = wk.ab;
                    const uint8_t *gA = (const uint8_t *)g.bt + (size_t)ab * nkc * TC_A_BYTES;
                    if (reload) {
                        if (b0_loads > 0 &&
                            !mbar_wait_or_abort(b0_empty, (b0_loads - 1) & 1u, s_abort, TC_SLEEP_NS, g.wait_limit)) {
                            ok = false;
                            break;
                        }
                        mbar_arrive_expect_tx(b0_full, TC_A_BYTES);
                        bulk_g2s(sB0, gA, TC_A_BYTES, b0_full);
                        tx_used |= 1u << (2 * NS);
                        b0_phase = b0_loads & 1u;
                        ++b0_loads;
                    }
                    // chunk bases tcb[tile], tcb[tile + 1], loaded one tile ahead
                    int cb0 = ldg_pin_s32(tcb + wk.t0), cb1 = ldg_pin_s32(tcb + wk.t0 + 1);
                    for (int tile = wk.t0; tile < wk.t1 && ok; ++tile) {
                        const int ntile = min(TC_INST, v.n_size - tile * TC_INST);
                        const int base = cb0, nc = cb1 - cb0;
                        if (tile + 1 < wk.t1) {
                            cb0 = cb1;
                            cb1 = ldg_pin_s32(tcb + tile + 2);
                        }
                        // the coefficient chunks of the next tile into L2, and the
                        // PSD weights and exponents of the tile after it (the
                        // weights warp reads them a few items ahead; they were
                        // evicted by the coefficient operand)
                        if (tile + 1 < wk.t1)
                            bulk_prefetch_l2(ua + (size_t)cb0 * TC_B_BYTES, (uint32_t)(cb1 - cb0) * TC_B_BYTES);
                        if (tile + 2 < wk.t1) {
                            const int tp = tile + 2;
                            const int t0 = tp * TC_INST, nt = min(TC_INST, v.n_size - t0);
                            auto pf = [&](const void *p, size_t bytes) {
                                const uintptr_t a0 = (uintptr_t)p & ~(uintptr_t)15, a1 = ((uintptr_t)p + bytes) & ~(uintptr_t)15;
                                if (a1 > a0) bulk_prefetch_l2((const void *)a0, (uint32_t)(a1 - a0));
                            };
                            pf(uex + t0, sizeof(int) * nt);
                            for (int b = 0; b < v.n_bin && b < NB; ++b)
                                pf(uW + (size_t)b * v.n_comp * v.n_size + t0, sizeof(float) * nt);
                        }
                        // the tile's items (one, or one per half tile with sizes:
                        // the issuers' rule), each reading every chunk of the tile
                        const int nitem = nc <= g.win ? 1 : (ntile > TC_HALF ? 2 : 1);
                        for (int h = 0; h < nitem && ok; ++h) {
                            for (int j = 0; j < nc; ++j) {
                                const uint32_t c = it++;
                                const int st = (int)(c % NS);
                                uint8_t *sS = sStage + st * TC_STAGE_BYTES;
                                if (c >= NS &&
                                    !mbar_wait_or_abort(empty + st, (c / NS - 1) & 1u, s_abort, TC_SLEEP_NS, g.wait_limit)) {
                                    ok = false;
                                    break;
                                }
                                s_chunk[st] = (int)c;
                                mbar_arrive_expect_tx(full + st, TC_B_BYTES + (j > 0 ? TC_A_BYTES : 0));
                                bulk_g2s(sS, ua + (size_t)(base + j) * TC_B_BYTES, TC_B_BYTES, full + st);
                                if (j > 0) bulk_g2s(sS + TC_B_BYTES, gA + (size_t)j * TC_A_BYTES, TC_A_BYTES, full + st);
                                tx_used |= 1u << (NS + st);
                                st_phase = (st_phase & ~(1u << st)) | (((c / NS) & 1u) << st);
                            }
                        }
                    }
                }
            }
            if (!ok) {
                *s_abort = 1;
                atomicOr(g.flags, GBMIE_FLAG_TIMEOUT);
            }
            // every bulk copy must land before shared memory is released, also
            // when another role gave up and left copies unconsumed: wait for
            // the latest phase of every stage that received one (an earlier
            // phase of a stage completed before its next copy was issued); in
            // a run without timeouts these have all completed already
            for (int st = 0; st < NS; ++st)
                if ((tx_used >> (NS + st)) & 1u && !mbar_wait(full + st, (st_phase >> st) & 1u, 1u << 20))
                    atomicOr(g.flags, GBMIE_FLAG_TIMEOUT);
            if ((tx_used >> (2 * NS)) & 1u && !mbar_wait(b0_full, b0_phase, 1u << 20))
                atomicOr(g.flags, GBMIE_FLAG_TIMEOUT);
        }
        __syncwarp();
    } else if (warp == 11) {
        // ================= item info and PSD weights (one warp) =================
        // Item i (the epilogue's order) gets weight-ring slot i % TC_NW: a
        // header (the item's accumulation-window count, the unit's largest
        // exponent E, its (wavelength, RH) index and component; whether the
        // item is a whole tile, else which half) and, per size s of the tile
        // (lanes s and s - 32), the bins' weights as pairs (w_b 2^(2 (e_s - E)),
        // the same): the scaled, duplicated form the epilogue's packed FMAs read
        // (E is the unit's largest exponent, so the power is <= 1; below 2^-126
        // the weight is dropped).  The warp steps over tiles: the loads of tile
        // t + 1 are issued before the waits for tile t's slots (one, or one per
        // half tile), so their latency overlaps them, and no load waits for
        // another's value.
        struct UnitW {
            bool valid;
            int comp, lr, E, t0, t1;
            const float *Wb;
            const int *ex;
            const int *tcb;
        };
        auto unit_w = [&](int k) -> UnitW {
            UnitW u;
            const TcWork wk = tc_work(g, k, cta, G, nblocks, ntl, n_units);
            u.valid = wk.valid;
            if (!u.valid) return u;
            const int unit = (int)wk.unit;
            u.t0 = wk.t0;
            u.t1 = wk.t1;
            u.comp = unit % v.n_comp;
            u.lr = unit / v.n_comp;
            const int lam = u.lr / v.n_rh;
            const int rhi = u.lr - lam * v.n_rh;
            u.Wb = v.Wf + v.wlam(lam) + ((size_t)rhi * v.n_bin * v.n_comp + u.comp) * v.n_size;
            u.ex = g.eexp + (size_t)unit * v.n_size;
            u.E = g.eunit[unit];
            u.tcb = g.tile_cbase + (size_t)v.le(lam) * (ntl + 1);
            return u;
        };
        struct WTile {
            int cb0, cb1, ex[2];   // chunk bases of the tile; sizes lane, 32 + lane: exponents (TC_NO_EX: none)
            float w[2][NB];
        };
        auto load_tile = [&](const UnitW &u, int tile, WTile &it) {
            it.cb0 = ldg_pin_s32(u.tcb + tile);
            it.cb1 = ldg_pin_s32(u.tcb + tile + 1);
#pragma unroll
            for (int hh = 0; hh < 2; ++hh) {
                const int si = tile * TC_INST + TC_HALF * hh + lane;
                it.ex[hh] = TC_NO_EX;
#pragma unroll
                for (int b = 0; b < NB; ++b) it.w[hh][b] = 0.f;
                if (si < v.n_size) {
                    it.ex[hh] = ldg_pin_s32(u.ex + si);
#pragma unroll
                    for (int b = 0; b < NB; ++b)
                        if (b < v.n_bin) it.w[hh][b] = ldg_pin_f32(u.Wb + (size_t)b * v.n_comp * v.n_size + si);
                }
            }
        };
        bool ok = true;
        uint32_t iw = 0;
        int kq = 0;
        UnitW u = unit_w(0);
        int tile = u.valid ? u.t0 : 0;
        // One step: issue the loads of the next tile into nxt, then for each
        // item of the current tile wait for its slot and store it from cur.
        // Steps alternate the roles of the two buffers (no register copies: a
        // copy would wait for the loads it copies).
        auto step = [&](const WTile &cur, WTile &nxt) {
            int nk = kq, nt = tile + 1;
            if (nt == u.t1) ++nk;   // the next work item
            const UnitW un = nk == kq ? u : unit_w(nk);
            if (nk != kq && un.valid) nt = un.t0;
            if (un.valid) load_tile(un, nt, nxt);
            // the tile's items: the issuers' rule
            const int nc = cur.cb1 - cur.cb0;
            const int ntile = min(TC_INST, v.n_size - tile * TC_INST);
            const bool whole = nc <= g.win;
            const int nitem = whole ? 1 : (ntile > TC_HALF ? 2 : 1);
            float4 wq[2][TC_NP(NB)];
#pragma unroll
            for (int hh = 0; hh < 2; ++hh) {
                const int e = cur.ex[hh] == TC_NO_EX ? -100000 : 2 * (cur.ex[hh] - u.E);
                const float p2 = e < -126 ? 0.f : __int_as_float((e + 127) << 23);
#pragma unroll
                for (int pp = 0; pp < TC_NP(NB); ++pp) {
                    const float w0 = 2 * pp < NB ? cur.w[hh][2 * pp] * p2 : 0.f;
                    const float w1 = 2 * pp + 1 < NB ? cur.w[hh][2 * pp + 1] * p2 : 0.f;
                    wq[hh][pp] = make_float4(w0, w0, w1, w1);
                }
            }
            for (int hi = 0; hi < nitem; ++hi) {
                const uint32_t slot = iw % TC_NW;
                int go = 1;
                if (lane == 0 && iw >= TC_NW)
                    go = mbar_wait_or_abort(w_empty + slot, (iw / TC_NW - 1) & 1u, s_abort, TC_SLEEP_NS, g.wait_limit) ? 1
                                                                                                                      : 0;
                go = __shfl_sync(0xffffffffu, go, 0);
                if (!go) {
                    ok = false;
                    return;
                }
                float *ws = sW + slot * TC_WSLOT_FLOATS(NB);
#pragma unroll
                for (int hh = 0; hh < 2; ++hh) {
                    float4 *dst = (float4 *)(ws + 16 + 4 * TC_NP(NB) * (TC_HALF * hh + lane));
#pragma unroll
                    for (int pp = 0; pp < TC_NP(NB); ++pp) dst[pp] = wq[hh][pp];
                }
                if (lane == 0) {
                    *(int4 *)ws = make_int4(whole ? 1 : (nc + g.win - 1) / g.win, u.E, u.lr, u.comp);
                    *(int4 *)(ws + 4) = make_int4(whole ? 1 : 0, hi, 0, 0);
                }
                __syncwarp();
                if (lane == 0) mbar_arrive(w_full + slot);
                ++iw;
            }
            u = un;
            kq = nk;
            tile = nt;
        };
        WTile ia, ib;
        if (u.valid) load_tile(u, u.t0, ia);
        while (ok && u.valid) {
            step(ia, ib);
            if (!ok || !u.valid) break;
            step(ib, ia);
        }
        if (!ok && lane == 0) {
            *s_abort = 1;
            atomicOr(g.flags, GBMIE_FLAG_TIMEOUT);
        }
    } else {
        // ================= epilogue (warps 0-7) =================
        // Items in the MMA's order; each item's chunk count, unit constants
        // and scaled PSD weights come from the weights warp's ring.
        // Per size the thread forms E0 = (|S+|^2, |S-|^2) and
        // E1 = (Re S+ S-*, Im S- S+*) and adds w_b E0, w_b E1 with packed FP32
        // pair FMAs; the constant factors of the Mueller elements
        //   s11 = (|S+|^2 + |S-|^2)/4, s12 = -Re(S+ S-*)/2,
        //   s33 = (|S+|^2 - |S-|^2)/4, s34 = -Im(S- S+*)/2
        // are applied to the unit's sums.
        const int q = warp & 3, wh = warp >> 2;
        constexpr int NP = TC_NP(NB);   // 16-byte weight loads per size: two bins each
        bool ok = true;
        uint32_t wce[2] = {0u, 0u}, ie = 0;   // accumulator sets read per issuer; items
        int kq = 0;
        TcWork cw = tc_work(g, 0, cta, G, nblocks, ntl, n_units);
        int tile = cw.t0;
        // Sums over sizes: acc[e][b] (registers) collects a tile's w_b E_e
        // (packed pairs); at the tile's end the running sum H (this thread's
        // column of sSum: [bin][thread] of (E0 pair, E1 pair), 16 bytes per
        // access) takes H + acc by an exact two-sum whose rounding error
        // stays in acc as the next tile's start (block-wise compensated
        // summation), so the per-(unit, block) sum H + acc keeps FP32
        // relative precision whatever the size count.  A thread's sizes are
        // 16 wh .. 16 wh + 15 of each half tile, in half-tile order, whether
        // the tile comes as one item or as two.
        f32x2 acc[2][NB];
        ulonglong2 *sh = (ulonglong2 *)sSum + tid;
#pragma unroll
        for (int b = 0; b < NB; ++b) {
            acc[0][b] = acc[1][b] = 0ull;
            sh[b * TC_EPI_THREADS] = make_ulonglong2(0ull, 0ull);
        }
        // lane 0 waits, the warp follows its answer
        auto warp_wait = [&](uint64_t *bar, uint32_t parity) -> bool {
            int go = 1;
            if (lane == 0) go = mbar_wait_or_abort(bar, parity, s_abort, TC_EPI_SLEEP_NS, g.wait_limit) ? 1 : 0;
            return __shfl_sync(0xffffffffu, go, 0) != 0;
        };
        while (ok && cw.valid) {
            const int ntile = min(TC_INST, v.n_size - tile * TC_INST);
            const int ab = cw.ab;
            const bool active = TC_ABLK * ab + 32 * q < v.n_ang;   // this warp has angles in the block
            // the item's slot of the weight ring
            const uint32_t wsl = ie % TC_NW;
            if (!warp_wait(w_full + wsl, (ie / TC_NW) & 1u)) {
                ok = false;
                break;
            }
            const float *ws = sW + wsl * TC_WSLOT_FLOATS(NB);
            const int4 hdr = *(const int4 *)ws;         // windows, E, (wavelength, RH) index, component
            const int4 hd2 = *(const int4 *)(ws + 4);   // whole tile, else the half
            const bool whole = hd2.x != 0;
            const int hcur = hd2.y;
            // the next item; tend: this item ends its tile, wend: the work item
            int nk = kq, nt = tile;
            const bool tend = whole || hcur == 1 || TC_HALF * (hcur + 1) >= ntile;
            bool wend = false;
            if (tend && ++nt == cw.t1) {
                wend = true;
                ++nk;
            }
            const uint32_t ip = ie & 1u;   // the item's issuer
            const uint32_t lanes = tmem + ((uint32_t)(32 * q) << 16);
            // passes of 16 sizes: a whole tile's two halves (one window: S+ of the
            // 64 sizes in one accumulator set, S- in the issuer's other), or the
            // half tile's windows
            const uint32_t wi0 = ip ? wce[1] : wce[0];
            const uint32_t sp = 2 * ip + (wi0 & 1u), sm = 2 * ip + ((wi0 + 1) & 1u);
            const int npass = whole ? 2 : 1;
#pragma unroll 1
            for (int hh = 0; hh < npass; ++hh) {
                float rp[32], rm[32];
                bool use, pend = false, rel = false;
                int half;
                if (whole) {
                    if (hh == 0) {
                        if (!warp_wait(acc_full + sp, (wi0 >> 1) & 1u) ||
                            !warp_wait(acc_full + sm, ((wi0 + 1) >> 1) & 1u)) {
                            ok = false;
                            break;
                        }
                        tc_fence_after();
                    }
                    half = hh;
                    use = active && TC_HALF * hh < ntile;
                    if (use) {
                        // sizes 0-7 of the pass now, 8-15 in flight while 0-7 are summed
                        const uint32_t col = 64 * hh + 32 * wh;
                        tmem_ld8x2(lanes + sp * 128 + col, lanes + sm * 128 + col, rp, rm);
                        tmem_ld8x2(lanes + sp * 128 + col + 8, lanes + sm * 128 + col + 8, rp + 8, rm + 8);
                        tmem_ld16x2_nowait(lanes + sp * 128 + col + 16, lanes + sm * 128 + col + 16, rp + 16, rm + 16);
                        pend = true;
                    }
                    if (hh == 1 && !use) {   // both sets read
                        tc_fence_before();
                        __syncwarp();
                        if (lane == 0) {
                            mbar_arrive(acc_empty + sp);
                            mbar_arrive(acc_empty + sm);
                        }
                    }
                    if (hh == 1) {
                        if (ip) wce[1] += 2;
                        else wce[0] += 2;
                    }
                    // a whole tile's sets are released once the last pass's
                    // in-flight half has landed (in the sums below)
                    rel = hh == 1 && use;
                } else {
                    // window sums of S+ and S- (this lane's angle, 16 sizes x
                    // Re/Im); later windows are added in pieces of 4 sizes (fewer
                    // live registers)
                    const int nwin = hdr.x;
                    for (int w = 0; w < nwin; ++w) {
                        const uint32_t wi = ip ? wce[1] : wce[0];
                        const uint32_t set = 2 * ip + (wi & 1u), su = wi >> 1;
                        if (!warp_wait(acc_full + set, su & 1u)) {
                            ok = false;
                            break;
                        }
                        tc_fence_after();
                        if (active) {
                            const uint32_t ta = lanes + set * 128 + 32 * wh;
                            if (w == 0) {
                                tmem_ld32x2(ta, ta + 64, rp, rm);
                            } else {
#pragma unroll
                                for (int hf = 0; hf < 4; ++hf) {
                                    float t[8], u[8];
                                    tmem_ld8x2(ta + 8 * hf, ta + 64 + 8 * hf, t, u);
#pragma unroll
                                    for (int i = 0; i < 8; ++i) {
                                        rp[8 * hf + i] += t[i];
                                        rm[8 * hf + i] += u[i];
                                    }
                                }
                            }
                        }
                        tc_fence_before();
                        __syncwarp();
                        if (lane == 0) mbar_arrive(acc_empty + set);
                        if (ip) ++wce[1];
                        else ++wce[0];
                    }
                    half = hcur;
                    use = active && nwin > 0;
                }
                if (!ok) break;
                if (use) {
                    const float *wb = ws + 16 + 4 * NP * (TC_HALF * half + 16 * wh);   // this thread's 16 sizes
                    // per group of 8 sizes: the pairs first (independent work for the
                    // scheduler), then the weighted sums; rp/rm die as E0/E1 are formed
#pragma unroll
                    for (int sg = 0; sg < 16; sg += 8) {
                        if (sg == 8 && pend) {
                            tmem_wait_tie(rp + 16, rm + 16);
                            if (rel) {   // both sets read
                                tc_fence_before();
                                __syncwarp();
                                if (lane == 0) {
                                    mbar_arrive(acc_empty + sp);
                                    mbar_arrive(acc_empty + sm);
                                }
                            }
                        }
                        f32x2 E0[8], E1[8];
#pragma unroll
                        for (int s = 0; s < 8; ++s) {
                            const float pr = rp[2 * (sg + s)], pi = rp[2 * (sg + s) + 1], mr = rm[2 * (sg + s)],
                                        mi = rm[2 * (sg + s) + 1];
                            E0[s] = f2_pack(fmaf(pr, pr, pi * pi), fmaf(mr, mr, mi * mi));
                            E1[s] = f2_pack(fmaf(pr, mr, pi * mi), fmaf(mr, pi, -(mi * pr)));
                        }
#pragma unroll
                        for (int s = 0; s < 8; ++s) {
                            const f32x2 e0 = E0[s], e1 = E1[s];
                            const ulonglong2 *wp = (const ulonglong2 *)(wb + 4 * NP * (sg + s));
#pragma unroll
                            for (int p = 0; p < NP; ++p) {
                                const ulonglong2 w2 = wp[p];   // (w_2p, w_2p), (w_2p+1, w_2p+1)
                                acc[0][2 * p] = f2_fma(w2.x, e0, acc[0][2 * p]);
                                acc[1][2 * p] = f2_fma(w2.x, e1, acc[1][2 * p]);
                                if (2 * p + 1 < NB) {
                                    acc[0][2 * p + 1] = f2_fma(w2.y, e0, acc[0][2 * p + 1]);
                                    acc[1][2 * p + 1] = f2_fma(w2.y, e1, acc[1][2 * p + 1]);
                                }
                            }
                        }
                    }
                }
            }
            if (!ok) break;
            // the slot is read (every warp, active or not, waited for it first)
            __syncwarp();
            if (lane == 0) mbar_arrive(w_empty + wsl);
            if (tend) {
                // end of a tile: H += acc exactly rounded, the error stays in acc
                auto two_sum = [](f32x2 &hi, f32x2 &a) {
                    const f32x2 sum = f2_add(hi, a);
                    const f32x2 bp = f2_sub(sum, hi);
                    a = f2_add(f2_sub(hi, f2_sub(sum, bp)), f2_sub(a, bp));
                    hi = sum;
                };
#pragma unroll
                for (int b = 0; b < NB; ++b) {
                    ulonglong2 Hb = sh[b * TC_EPI_THREADS];
                    two_sum(Hb.x, acc[0][b]);
                    two_sum(Hb.y, acc[1][b]);
                    sh[b * TC_EPI_THREADS] = Hb;
                }
                if (wend) {
                    // end of the work item: this thread's share of the (unit, block)'s
                    // sums.  Each sum is the unevaluated pair H + acc; the Mueller
                    // combinations are formed on the pairs in FP32 (two-sum for
                    // E0a +- E0b), both parts are scaled by 2^(2 (E - 13)) exactly
                    // in the integer domain and their FP64 sum is stored in the
                    // partial-sum slot of (tile range, size half) of the unit.
                    const int ang = TC_ABLK * ab + 32 * q + lane;
                    if (ang < v.n_ang) {
                        double *part = v.part + ((size_t)cw.unit * v.n_slots + 2 * (cw.t0 / g.tpr) + wh) *
                                                    v.n_bin * 4 * v.n_ang;
                        const int k2 = 2 * (hdr.y - SHIFT_BITS);
#pragma unroll
                        for (int b = 0; b < NB; ++b) {
                            if (b < v.n_bin) {
                                const double fr = v.frac[(size_t)b * v.n_comp + hdr.w];
                                const ulonglong2 Hb = sh[b * TC_EPI_THREADS];
                                float h0, h1, h2, h3, l0, l1, l2, l3;
                                f2_unpack(Hb.x, h0, h1);
                                f2_unpack(Hb.y, h2, h3);
                                f2_unpack(acc[0][b], l0, l1);
                                f2_unpack(acc[1][b], l2, l3);
                                float mh[4], ml[4];
                                {
                                    const float sp = h0 + h1, bp = sp - h0;
                                    const float ep = (h0 - (sp - bp)) + (h1 - bp);
                                    const float sm = h0 - h1, bm = sm - h0;
                                    const float em = (h0 - (sm - bm)) + (-h1 - bm);
                                    mh[0] = 0.25f * sp;
                                    ml[0] = 0.25f * (ep + (l0 + l1));
                                    mh[2] = 0.25f * sm;
                                    ml[2] = 0.25f * (em + (l0 - l1));
                                    mh[1] = -0.5f * h2;
                                    ml[1] = -0.5f * l2;
                                    mh[3] = -0.5f * h3;
                                    ml[3] = -0.5f * l3;
                                }
                                const bool unit_frac = __double_as_longlong(fr) == 0x3FF0000000000000ll;
#pragma unroll
                                for (int k = 0; k < 4; ++k) {
                                    double a = f32_to_f64_pow2(mh[k], k2), c = f32_to_f64_pow2(ml[k], k2);
                                    if (!unit_frac) {
                                        a *= fr;
                                        c *= fr;
                                    }
                                    part[((size_t)b * 4 + k) * v.n_ang + ang] = a + c;
                                }
                            }
                        }
                    }
#pragma unroll
                    for (int b = 0; b < NB; ++b) {
                        acc[0][b] = acc[1][b] = 0ull;
                        sh[b * TC_EPI_THREADS] = make_ulonglong2(0ull, 0ull);
                    }
                }
            }
            if (nk != kq) {
                kq = nk;
                cw = tc_work(g, kq, cta, G, nblocks, ntl, n_units);
                nt = cw.t0;
            }
            tile = nt;
            ++ie;
        }
        if (!ok && lane == 0) {
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
// shared staging of k_tab_coeffs_mixed: 16 orders x float4 per thread
static size_t coef_stage_bytes(int block) { return (size_t)TC_KC16 * sizeof(float4) * (size_t)block; }
// the attribute is set once per device, on the first (uncaptured) run: a
// table run may be recorded into a CUDA graph later
static int coef_stage_attr(gbmie_ctx *ctx)
{
    static volatile bool done[64];
    const int dev = ctx->device;
    if (dev >= 0 && dev < 64 && done[dev]) return GBMIE_OK;
    int st = ctx_cuda(ctx, cudaFuncSetAttribute(k_tab_coeffs_mixed<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                (int)coef_stage_bytes(256)),
                      "k_tab_coeffs_mixed shared memory");
    if (st == GBMIE_OK)
        st = ctx_cuda(ctx, cudaFuncSetAttribute(k_tab_coeffs_mixed<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                (int)coef_stage_bytes(256)),
                      "k_tab_coeffs_mixed shared memory");
    if (st == GBMIE_OK && dev >= 0 && dev < 64) done[dev] = true;
    return st;
}

int launch_table_mixed(gbmie_ctx *ctx, gbmie_table_plan *p, TabView &v, char *scr)
{
    const gbmie_table_desc &d = p->d;
    cudaStream_t st = ctx->stream;
    float4 *cf = (float4 *)(scr + p->o_cf);
    int *eexp = (int *)(scr + p->o_eexp);
    int *eunit = (int *)(scr + p->o_eunit);
    {
        const int64_t nrows = (int64_t)p->n_le * v.n_size;
        const int64_t nc = nrows > p->n_units ? nrows : p->n_units;
        ctx_pre_launch(ctx);
        k_mixed_consts<<<(unsigned)ceil_div64(nc, 256), 256, 0, st>>>(p->n_units, v.hidx, v.hdf, nrows, v.rowc, v.xg,
                                                                      v.rowcd);
        GBMIE_TRY(ctx_check_launch(ctx, "k_mixed_consts"));
    }
    ctx_pre_launch(ctx);
    k_fill_int<<<(unsigned)ceil_div64(p->n_units, 256), 256, 0, st>>>((int)p->n_units, eunit, -100000);
    GBMIE_TRY(ctx_check_launch(ctx, "k_fill_int"));
    ctx_pre_launch(ctx);
    uint8_t *asplit = (uint8_t *)(scr + p->o_asplit);
    if (d.m_core) {
        int nb = 0, nsm = 0;
        GBMIE_TRY(ctx_cuda(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_tab_coeffs_mixed_coated, 128, 0),
                           "coated occupancy"));
        GBMIE_TRY(ctx_cuda(ctx, cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, ctx->device), "SM count"));
        int *next = (int *)(scr + p->o_cnext);
        GBMIE_TRY(ctx_cuda(ctx, cudaMemsetAsync(next, 0, sizeof(int), st), "task counter"));
        ctx_pre_launch(ctx);
        k_tab_coeffs_mixed_coated<<<(nb > 0 ? nb : 1) * nsm, 128, 0, st>>>(
            v, p->ctasks, p->n_ctasks, next, cf, eexp, eunit, ctx->d_flags, p->tile_cbase, p->unit_cbase, p->ntiles,
            asplit);
        GBMIE_TRY(ctx_check_launch(ctx, "k_tab_coeffs_mixed_coated"));
    } else {
        GBMIE_TRY(coef_stage_attr(ctx));
        auto kern = p->dn_fp64 ? k_tab_coeffs_mixed<true> : k_tab_coeffs_mixed<false>;
        int grid = 0;
        GBMIE_TRY(coef_grid(ctx, p->dn_fp64, p->coef_block, &grid));
        int *next = (int *)(scr + p->o_cnext);
        GBMIE_TRY(ctx_cuda(ctx, cudaMemsetAsync(next, 0, sizeof(int), st), "task counter"));
        ctx_pre_launch(ctx);
        kern<<<grid, p->coef_block, coef_stage_bytes(p->coef_block), st>>>(
            v, p->ctasks, p->n_ctasks, next, cf, eexp, eunit, p->tile_cbase, p->unit_cbase, p->ntiles, asplit);
        GBMIE_TRY(ctx_check_launch(ctx, p->dn_fp64 ? "k_tab_coeffs_mixed_dn64" : "k_tab_coeffs_mixed"));
    }
    GBMIE_TRY(ctx_cuda(ctx, cudaStreamWaitEvent(st, ctx->ev_join, 0), "join"));   // the PSD weights
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
    a.wait_limit = p->wait_limit;
    a.flags = ctx->d_flags;
    int nsm = 0;
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, ctx->device);
    // work items: (unit, angle block) pairs, each split into tile ranges when
    // there are fewer than four pairs per SM (tables of few wavelengths); the
    // plan fixed the split with its partial-sum slots (two per range)
    const int nblocks = p->n_pad_total / TC_ABLK;
    const int64_t pairs = p->n_units * (int64_t)nblocks;
    a.tpr = p->tc_tpr;
    a.ntr = p->tc_ntr;
    if (2 * a.ntr > p->n_slots)
        return ctx_fail(ctx, GBMIE_ERR_INVALID, "k_tab_s12_tc: %d partial-sum slots needed, %d held", 2 * a.ntr,
                        p->n_slots);
    p->slots_used = 2 * a.ntr;
    const int64_t nwork = pairs * a.ntr;
    const int grid = (int)(nwork < nsm ? nwork : nsm);
    cudaError_t e = cudaSuccess;
    ctx_pre_launch(ctx);
#define TC_LAUNCH(NBV)                                                                                   \
    case NBV:                                                                                            \
        e = cudaFuncSetAttribute(k_tab_s12_tc<NBV>, cudaFuncAttributeMaxDynamicSharedMemorySize,              \
                                 (int)TC_SMEM_BYTES(NBV));                                               \
        k_tab_s12_tc<NBV><<<grid, TC_THREADS, TC_SMEM_BYTES(NBV), st>>>(a);                              \
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

size_t table_mixed_smem_bytes() { return TC_SMEM_BYTES(8); }
int table_tc_win_max() { return TC_WIN_MAX; }

// The B operands depend only on the angles and the largest nmax: built once
// per plan into plan-owned memory (plan creation synchronises afterwards).
int build_table_bt(gbmie_ctx *ctx, gbmie_table_plan *p)
{
    GBMIE_TRY(coef_stage_attr(ctx));   // at plan time: never inside a graph capture
    const size_t bytes = 4 * 2 * (size_t)p->n_pad_total * p->k_pad;
    void *mem = nullptr;
    int fresh = 0;
    GBMIE_TRY(ctx_angle_op_get(ctx, p->hcos, p->d.n_ang, p->n_pad_total, p->k_pad, p->nmax_max, bytes, &mem,
                               &p->bt_entry, &fresh));
    p->bt = (__half *)mem;
    if (!fresh) return GBMIE_OK;   // the same angles and orders: the cached operand
    ctx_pre_launch(ctx);
    k_tab_bt_f16<<<(p->n_pad_total + 127) / 128, 128, 0, ctx->stream>>>(p->d.n_ang, p->n_pad_total, p->k_pad,
                                                                         p->nmax_max, p->d.cos_theta, p->bt);
    const int st = ctx_check_launch(ctx, "k_tab_bt_f16");
    if (st != GBMIE_OK && p->bt_entry >= 0) ctx->angle_ops[p->bt_entry].n_ang = -1;   // never matched again
    return st;
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
                auto kern = p->dn_fp64 ? k_tab_coeffs_mixed<true> : k_tab_coeffs_mixed<false>;
                int grid = 0;
                GBMIE_TRY(coef_grid(ctx, p->dn_fp64, bs, &grid));
                int *next = (int *)(scr + p->o_cnext);
                GBMIE_TRY(ctx_cuda(ctx, cudaMemsetAsync(next, 0, sizeof(int), st), "task counter"));
                cudaEventRecord(e0, st);
                kern<<<grid, bs, coef_stage_bytes(bs), st>>>(v, p->ctasks, p->n_ctasks, next, cf, eexp, eunit,
                                                               p->tile_cbase, p->unit_cbase, p->ntiles,
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

