// Table generation: the (bin x wavelength x RH) sweep of
// geosmie/dointegration.py:786-1031 on the GPU, FP64 ("plain") form.
//
// Work decomposition
//   instance  = (wavelength, RH, component, size)           Mie evaluation
//   unit      = (wavelength, RH, component)                 shares m
//   entry     = (bin, wavelength, RH)                       one table row
// Size grids: GBMIE_GRID_X (one x grid for all wavelengths, the reference's
// layout) or GBMIE_GRID_RADIUS (x = 2 pi r / lambda).  The "x-grid set" le
// is 0 for GRID_X and the wavelength for GRID_RADIUS.
//
// Device data (context scratch, carved by the plan):
//   pc     psi_n/chi_n rows of every (le, size), orders 1..nmax, CSR by off
//   an,bn  coefficients of every instance, unit_base[unit] + off[le, i]
//   eff4   (qext, qsca, qb, asy) per instance
//   W      PSD weights [wl][rh][bin][comp][size]; sums [..][4] (num, S r^2 w,
//          S r^3 w, S r^4 w); reff0 [wl][bin][comp]
//   pacc   number-weighted Mueller sums [wl][rh][bin][4][ang]
//          (s11, s12, s33, s34; s22 = s11 and s44 = s33 by construction,
//          dointegration.py:1044-1050)
#include "common.cuh"
#include "mie_device.cuh"
#include "gsf.cuh"

#include "table_internal.cuh"

#include <string.h>

// ---------------------------------------------------------------------------
// plan kernels
// ---------------------------------------------------------------------------
__global__ void k_tab_make_x(int n_le, int n_size, int grid_kind, const double *__restrict__ grid,
                             const double *__restrict__ lambda, double *__restrict__ xg, int *flags)
{
    const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= (int64_t)n_le * n_size) return;
    const int le = (int)(j / n_size), i = (int)(j % n_size);
    const double g = grid[i];
    const double x = grid_kind == GBMIE_GRID_X ? g : TWO_PI * g / lambda[le];
    if (!(x > 0.0) || !isfinite(x)) atomicOr(flags, GBMIE_FLAG_INVALID);
    xg[j] = x;
}

// ---------------------------------------------------------------------------
// run kernels
// ---------------------------------------------------------------------------
// psi/chi rows per (wavelength block, size) in FP64 (CSR, pc) or, for
// homogeneous mixed plans (pairs = 1), as FP32 pairs only, in the order-major
// groups of 32 sizes the mixed recurrences read (TabView::pcd; the pair
// slots also hold the unnormalised psi values meanwhile, so that a warp's
// stores and loads of an order are one segment).
__global__ void __launch_bounds__(128) k_tab_psi_chi(int64_t nrows, const double *__restrict__ xg,
                                                     const int64_t *__restrict__ off, double2 *__restrict__ pc,
                                                     double4 *__restrict__ rowc, TabView v, int pairs)
{
    const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= nrows) return;
    const int64_t o = off[j];
    const double x = xg[j];
    float4 *pr = nullptr;
    if (pairs) {
        const int le = (int)(j / v.n_size), i = (int)(j - (int64_t)le * v.n_size);
        pr = v.pcd + v.grow[le] + v.grel[(int64_t)le * (v.ngrp + 1) + (i >> 5)] + (i & 31);
    }
    psi_chi_row(x, (int)(off[j + 1] - o), pairs ? nullptr : pc + o, pr, 32);
    double s, c;
    sincos(x, &s, &c);
    rowc[j] = make_double4(s, c, 1.0 / x, 0.0);
}

// Medium constants per (lam, rh, comp) unit (eps = m^2, mu = 1 as the
// reference's Mie(m=...) sets them); a non-finite index raises the invalid flag.
__global__ void k_tab_index(int64_t n_units, const double2 *__restrict__ m, HomogIndex *__restrict__ hidx,
                            int *flags)
{
    const int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (u >= n_units) return;
    const cplx mu = cx(m[u]);
    if (!isfinite(mu.re) || !isfinite(mu.im)) atomicOr(flags, GBMIE_FLAG_INVALID);
    hidx[u] = homog_index(mu * mu, cx(1.0, 0.0));
}

// PSD weights of (lam, rh, bin, comp): lognormal dN/dx x dgrid or r^-4 x
// dgrid, normalised (dointegration.py:546-583, 626-662), or the caller's
// weights; plus the radius moments and the dry effective radius.
__global__ void __launch_bounds__(256) k_tab_weights(TabView v, const double *__restrict__ wgiven)
{
    const int blk = blockIdx.x;   // ((lam * n_rh + rh) * n_bin + bin) * n_comp + comp, lam = 0 if shared
    const int comp = blk % v.n_comp;
    const int bin = (blk / v.n_comp) % v.n_bin;
    const int rh = (blk / (v.n_comp * v.n_bin)) % v.n_rh;
    const int lam = blk / (v.n_comp * v.n_bin * v.n_rh);
    const int n = v.n_size;
    double *W = v.W + (size_t)blk * n;   // caller-supplied weights: never wavelength-shared
    const double *xs = v.xg + (size_t)v.le(lam) * n;
    const double *pp = v.psd_param + ((size_t)bin * v.n_comp + comp) * 4;
    const double lamv = v.lambda[lam];
    const double xconv = TWO_PI / lamv;
    double tot[1] = {0.0};
    if (v.psd_kind == GBMIE_PSD_WEIGHTS) {
        const double *src = wgiven + (size_t)blk * n;
        for (int i = threadIdx.x; i < n; i += blockDim.x) W[i] = src[i];
        tot[0] = 1.0;
    } else if (v.psd_kind == GBMIE_PSD_LOGNORM) {
        const double gfp = v.gf_psd[rh];
        const double xmode = pp[0] * gfp * xconv, xmin = pp[1] * xconv, xmax = pp[2] * gfp * xconv;
        const double lns = log(pp[3]);
        const double c0 = 1.0 / (sqrt(TWO_PI) * lns), c1 = 1.0 / (2.0 * lns * lns);
        for (int i = threadIdx.x; i < n; i += blockDim.x) {
            const double x = xs[i];
            double w = 0.0;
            if (x < xmax && x > xmin) {
                const double l = log(x / xmode);
                w = c0 / x * exp(-(l * l) * c1) * v.dgrid[i];
            }
            W[i] = w;
            tot[0] += w;
        }
        block_sum<1>(tot);
    } else {   // GBMIE_PSD_POWER4
        for (int i = threadIdx.x; i < n; i += blockDim.x) {
            const double r = v.radius(lam, i);
            double w = 0.0;
            if (!(r < pp[0]) && !(r > pp[1])) w = 1.0 / (r * r * r * r) * v.dgrid[i];
            W[i] = w;
            tot[0] += w;
        }
        block_sum<1>(tot);
    }
    const double inv = (v.psd_kind == GBMIE_PSD_WEIGHTS || tot[0] == 0.0) ? 1.0 : 1.0 / tot[0];
    double s[4] = {0.0, 0.0, 0.0, 0.0};
    float *Wf = v.Wf ? v.Wf + (size_t)blk * n : nullptr;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const double w = W[i] * inv;
        if (v.psd_kind != GBMIE_PSD_WEIGHTS) W[i] = w;
        if (Wf) Wf[i] = (float)w;
        const double r = v.radius(lam, i);
        const double r2 = r * r * w;
        s[0] += w;
        s[1] += r2;
        s[2] += r2 * r;
        s[3] += r2 * r * r;
    }
    block_sum<4>(s);
    if (threadIdx.x == 0) {
        double *o = v.sums + (size_t)blk * 4;
        o[0] = s[0];
        o[1] = s[1];
        o[2] = s[2];
        o[3] = s[3];
        if (rh == v.rh0) v.reff0[((size_t)lam * v.n_bin + bin) * v.n_comp + comp] = s[3] / s[2];
    }
}

// Coefficients + per-instance efficiencies, one thread per instance.
struct EmitTab {
    double2 *an, *bn;
    __device__ __forceinline__ void operator()(int k, cplx a, cplx b) const {
        an[k - 1] = d2(a);
        bn[k - 1] = d2(b);
    }
};

__global__ void __launch_bounds__(128) k_tab_coeffs(TabView v, int64_t n_inst, int *flags)
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
    EmitTab emit{v.an + c, v.bn + c};
    EffSums es;
    homog_core(x, rc.z, rc.x, rc.y, v.hidx[unit], v.pc + o, nmax, emit, es);
    double e[6];
    es.finish(x, e);
    double *o4 = v.eff4 + t * 4;
    o4[0] = e[0];
    o4[1] = e[1];
    o4[2] = e[3];
    o4[3] = e[4];
}

__global__ void __launch_bounds__(128) k_tab_coeffs_coated(TabView v, int64_t n_inst, int *flags)
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
    EmitTab emit{v.an + c, v.bn + c};
    EffSums es;
    coated_table_instance(v, unit, c, o, nmax, v.xg[row], emit, es, flags);
    double e[6];
    es.finish(v.xg[row], e);
    double *o4 = v.eff4 + t * 4;
    o4[0] = e[0];
    o4[1] = e[1];
    o4[2] = e[3];
    o4[3] = e[4];
}

// Fused S+/S- sums, Mueller elements and number-weighted size integration
// (rawMie + calculateScatVals + the phase part of integratePSD,
// dointegration.py:1044-1050, 1160-1166).  Block = (unit, chunk of sizes);
// threads over angles; the chunk's coefficients (contiguous in memory)
// streamed through shared memory as (a+b, a-b).
#define TAB_CAP 2048
template <int NB>
__global__ void __launch_bounds__(256) k_tab_s12_plain(TabView v, int chunk, int nchunk, const int2 *__restrict__ brange,
                                                       int slot0)
{
    __shared__ double2 cd[TAB_CAP][2];
    const int64_t unit = blockIdx.x / nchunk;
    const int ch = blockIdx.x % nchunk;
    const int comp = (int)(unit % v.n_comp);
    const int64_t lr = unit / v.n_comp;   // lam * n_rh + rh
    const int lam = (int)(lr / v.n_rh);
    const int le = v.le(lam);
    const int2 rg = brange[le];           // this launch's nmax bucket on this x grid
    const int i0 = rg.x + ch * chunk, i1 = min(rg.y, i0 + chunk);
    const int nang = v.n_ang;
    // this block's partial-sum plane: slot slot0 + ch of the unit
    double *part = v.part + ((size_t)unit * v.n_slots + slot0 + ch) * v.n_bin * 4 * nang;
    if (i0 >= i1) {   // no sizes of this unit in the chunk: its plane is zero
        for (int e = threadIdx.x; e < v.n_bin * 4 * nang; e += blockDim.x) part[e] = 0.0;
        return;
    }
    const int64_t *off = v.off + (int64_t)le * v.n_size;   // off[i] for this x grid
    const int64_t cbase = v.unit_base[unit] - off[0];
    const double2 *A = v.an + cbase, *B = v.bn + cbase;
    const int64_t wstride = v.n_size;
    const double *Wb = v.W + v.wlam(lam) + ((size_t)(lr % v.n_rh) * v.n_bin * v.n_comp + comp) * wstride;
    for (int a0 = 0; a0 < nang; a0 += blockDim.x) {
        const int a = a0 + threadIdx.x;
        const bool act = a < nang;
        double acc[NB][4];
#pragma unroll
        for (int b = 0; b < NB; ++b) acc[b][0] = acc[b][1] = acc[b][2] = acc[b][3] = 0.0;
        double sp_r = 0, sp_i = 0, sm_r = 0, sm_i = 0;
        int j = i0;                // current size
        int64_t pos = off[i0];     // next unconsumed coefficient (CSR position)
        const int64_t pend = off[i1];
        while (pos < pend) {
            const int64_t cnt = min((int64_t)TAB_CAP, pend - pos);
            __syncthreads();
            for (int k = threadIdx.x; k < cnt; k += blockDim.x) {
                const double2 av = A[pos + k], bv = B[pos + k];
                cd[k][0] = make_double2(av.x + bv.x, av.y + bv.y);
                cd[k][1] = make_double2(av.x - bv.x, av.y - bv.y);
            }
            __syncthreads();
            int64_t p = pos;
            const int64_t pe = pos + cnt;
            while (p < pe) {
                const int64_t jb = off[j], je = off[j + 1];
                const int64_t stop = min(je, pe);
                if (act) {
                    const double2 *col = v.pq + (int64_t)(p - jb) * nang + a;
                    for (int64_t q = p; q < stop; ++q) {
                        const double2 t = *col;
                        col += nang;
                        const double2 c = cd[q - pos][0], d = cd[q - pos][1];
                        sp_r = fma(c.x, t.x, sp_r);
                        sp_i = fma(c.y, t.x, sp_i);
                        sm_r = fma(d.x, t.y, sm_r);
                        sm_i = fma(d.y, t.y, sm_i);
                    }
                }
                p = stop;
                if (stop == je) {   // size j complete
                    if (act) {
                        const double A2 = sp_r * sp_r + sp_i * sp_i, B2 = sm_r * sm_r + sm_i * sm_i;
                        const double s11 = 0.25 * (A2 + B2);
                        const double s12 = -0.5 * (sp_r * sm_r + sp_i * sm_i);
                        const double s33 = 0.25 * (A2 - B2);
                        const double s34 = -0.5 * (sm_r * sp_i - sm_i * sp_r);
#pragma unroll
                        for (int b = 0; b < NB; ++b) {
                            if (b < v.n_bin) {
                                const double w = Wb[(size_t)b * v.n_comp * wstride + j];
                                acc[b][0] = fma(w, s11, acc[b][0]);
                                acc[b][1] = fma(w, s12, acc[b][1]);
                                acc[b][2] = fma(w, s33, acc[b][2]);
                                acc[b][3] = fma(w, s34, acc[b][3]);
                            }
                        }
                    }
                    sp_r = sp_i = sm_r = sm_i = 0.0;
                    ++j;
                }
            }
            pos = pe;
        }
        if (act) {
#pragma unroll
            for (int b = 0; b < NB; ++b) {
                if (b < v.n_bin) {
                    const double f = v.frac[(size_t)b * v.n_comp + comp];
                    double *dst = part + (size_t)b * 4 * nang + a;
                    dst[0] = f * acc[b][0];
                    dst[nang] = f * acc[b][1];
                    dst[2 * nang] = f * acc[b][2];
                    dst[3 * nang] = f * acc[b][3];
                }
            }
        }
    }
}

// Scalar integration of integratePSD ('dumix', dointegration.py:1064-1209),
// one block per (lam, rh) covering every bin: the per-size features
//   A, qext A, qsca A, qabs A, qb A, g A qsca, csca A qsca, cext A qsca, A qsca
// (the weight becomes A qsca from 'g' on, the reference's aliasing) are
// formed once and weighted with each bin's PSD.  Plain: FP64 sums.  Mixed:
// FP32 with Kahan compensation.  sraw: qext qsca qabs qb g csca cext bsca
// bext bbck; nlraw: mass volume area rEff rMass (before division by mass0).
template <typename T>
struct KSum {
    T s, c;
    __device__ __forceinline__ void zero() { s = c = (T)0; }
    __device__ __forceinline__ void add(T v) {
        if (sizeof(T) == 8) {
            s += v;
        } else {   // Kahan
            const T y = v - c;
            const T t = s + y;
            c = (t - s) - y;
            s = t;
        }
    }
    __device__ __forceinline__ double val() const { return (double)s - (double)c; }
};

// (launch bounds match the launches: 64 threads for the FP32 sums of the
// mixed path, 256 for the FP64 sums; one block per SM is enough for the
// register bound, which lets the sums and the prefetched next size stay in
// registers: 0.25 -> 0.17 ms on the sulfate-like table)
template <int NB, typename T>
__global__ void __launch_bounds__(sizeof(T) == 4 ? 64 : 256, 1) k_tab_scalars(TabView v)
{
    __shared__ double sR[NB][15];
    __shared__ double sRed[8][NB * 9];
    __shared__ double sS[NB * 9];
    const int64_t lr = blockIdx.x;   // lam * n_rh + rh
    const int rh = (int)(lr % v.n_rh), lam = (int)(lr / v.n_rh);
    for (int t = threadIdx.x; t < NB * 15; t += blockDim.x) sR[t / 15][t % 15] = 0.0;   // any block size
    // radii are scaled by a power of two that brings the largest to [1, 2):
    // exact, and A^2 qsca of nanometre particles stays inside the FP32 range
    const double rscale = ldexp(1.0, -ilogb(v.radius(lam, v.n_size - 1)));
    const double ascale = ldexp(1.0, 2 * ilogb(v.radius(lam, v.n_size - 1)));   // 1 / rscale^2
    for (int comp = 0; comp < v.n_comp; ++comp) {
        const int64_t unit = lr * v.n_comp + comp;
        const double *E = v.eff4 + (size_t)unit * v.n_size * 4;
        KSum<T> acc[NB][9];
#pragma unroll
        for (int b = 0; b < NB; ++b)
#pragma unroll
            for (int j = 0; j < 9; ++j) acc[b][j].zero();
        // the inputs of a thread's next size are loaded one iteration ahead,
        // so that their latency overlaps the current size's sums
        const size_t w0 = v.wlam(lam) + ((size_t)rh * v.n_bin * v.n_comp + comp) * v.n_size;
        const size_t wstep = (size_t)v.n_comp * v.n_size;   // between bins
        auto load = [&](int i, double4 &e4, double &rad, T (&wv)[NB]) {
            if (i < v.n_size) {
                e4 = make_double4(E[4 * i], E[4 * i + 1], E[4 * i + 2], E[4 * i + 3]);
                rad = v.radius(lam, i);
#pragma unroll
                for (int b = 0; b < NB; ++b)
                    wv[b] = b < v.n_bin ? (sizeof(T) == 8 ? (T)v.W[w0 + b * wstep + i] : (T)v.Wf[w0 + b * wstep + i]) : (T)0;
            }
        };
        double4 e4n = make_double4(0.0, 0.0, 0.0, 0.0);
        double radn = 0.0;
        T wn[NB];
        load(threadIdx.x, e4n, radn, wn);
        for (int i = threadIdx.x; i < v.n_size; i += blockDim.x) {
            const double4 e4 = e4n;
            const double rad = radn;
            T wv[NB];
#pragma unroll
            for (int b = 0; b < NB; ++b) wv[b] = wn[b];
            load(i + blockDim.x, e4n, radn, wn);
            const T r = (T)(rad * rscale);
            const T A = (T)PI_D * r * r;
            const T qext = (T)e4.x, qsca = (T)e4.y, qb = (T)e4.z, g = (T)e4.w;
            const T qabs = (T)(e4.x - e4.y);
            const T as = A * qsca;
            const T f[9] = {A, qext * A, qsca * A, qabs * A, qb * A, g * as, qsca * A * as, qext * A * as, as};
#pragma unroll
            for (int b = 0; b < NB; ++b) {
                if (b < v.n_bin) {
#pragma unroll
                    for (int j = 0; j < 9; ++j) acc[b][j].add(wv[b] * f[j]);
                }
            }
        }
        // block reduction of the NB x 9 sums: warp shuffles (FP64 for the FP64
        // sums; for the FP32 sums unevaluated FP32 pairs hi + lo combined by
        // two-sum, which keeps FP64 work off the reduction), then one thread
        // per sum over the warps in FP64
#pragma unroll
        for (int b = 0; b < NB; ++b)
#pragma unroll
            for (int j = 0; j < 9; ++j) {
                if (sizeof(T) == 8) {
                    double t = acc[b][j].val();
                    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
                    if ((threadIdx.x & 31) == 0) sRed[threadIdx.x >> 5][b * 9 + j] = t;
                } else {
                    float hi = (float)acc[b][j].s, lo = -(float)acc[b][j].c;
                    for (int o = 16; o > 0; o >>= 1) {
                        const float oh = __shfl_xor_sync(0xffffffffu, hi, o);
                        const float ol = __shfl_xor_sync(0xffffffffu, lo, o);
                        const float sm = hi + oh, bp = sm - hi;
                        lo += ol + ((hi - (sm - bp)) + (oh - bp));
                        hi = sm;
                    }
                    if ((threadIdx.x & 31) == 0) sRed[threadIdx.x >> 5][b * 9 + j] = (double)hi + (double)lo;
                }
            }
        __syncthreads();
        for (int sidx = threadIdx.x; sidx < NB * 9; sidx += blockDim.x) {
            double t = 0.0;
            for (int wq = 0; wq < (int)(blockDim.x >> 5); ++wq) t += sRed[wq][sidx];
            sS[sidx] = t;
        }
        __syncthreads();
        // one thread per bin: bulk values of (bin, comp), weighted by frac
        const int b = threadIdx.x;
        if (b < v.n_bin && b < NB) {
            const double *s = sS + b * 9;
            const double rhop = v.rhop[(size_t)b * v.n_rh + rh];
            const double rhop0 = v.rhop0[b];
            const double *m4 = v.sums + ((((size_t)v.wl(lam) * v.n_rh + rh) * v.n_bin + b) * v.n_comp + comp) * 4;
            const double num = m4[0], s2 = m4[1], s3 = m4[2], s4 = m4[3];
            const double reff0 = v.reff0[((size_t)v.wl(lam) * v.n_bin + b) * v.n_comp + comp];
            const double area = PI_D * s2 / num;
            const double volume = 4.0 / 3.0 * PI_D * s3 / num;
            const double mass = volume * rhop;
            const double reff = s3 / s2;
            const double reffm = s4 / s3;
            const double rmass = 4.0 / 3.0 * PI_D * rhop * reffm * reffm * reffm;
            const double rmass0 = 4.0 / 3.0 * PI_D * rhop0 * reff0 * reff0 * reff0;
            const double i0 = 1.0 / s[0], i8 = 1.0 / s[8];
            const double qext = s[1] * i0, qsca = s[2] * i0, qabs = s[3] * i0;
            const double qbv = s[4] / s[2] * qsca;   // p11back qsca / (4 pi)
            const double g = s[5] * i8, csca = s[6] * i8 * ascale, cext = s[7] * i8 * ascale;
            const double conv = rmass / (rhop * reff * rmass0);
            const double f = v.frac[(size_t)b * v.n_comp + comp];
            const double vals[15] = {qext, qsca, qabs, qbv, g, csca, cext, 0.75 * qsca * conv, 0.75 * qext * conv,
                                     0.75 * qbv * conv / (4.0 * PI_D), mass, volume, area, reff, rmass};
#pragma unroll
            for (int k = 0; k < 15; ++k) sR[b][k] += f * vals[k];
        }
        __syncthreads();
    }
    __syncthreads();
    for (int t = threadIdx.x; t < v.n_bin * 15 && t < NB * 15; t += blockDim.x) {
        const int b = t / 15, k = t % 15;
        const size_t e = (size_t)lr * v.n_bin + b;
        if (k < 10) v.sraw[e * 10 + k] = sR[b][k];
        else v.nlraw[e * 5 + (k - 10)] = sR[b][k];
    }
}

// trapz weights of the angle grid: sum_a f_a tw_a = trapz(f sin(theta), theta)
__global__ void k_tab_trapz(int nang, const double *__restrict__ theta, double *__restrict__ tw)
{
    for (int a = threadIdx.x; a < nang; a += blockDim.x) {
        const double left = a > 0 ? theta[a] - theta[a - 1] : 0.0;
        const double right = a < nang - 1 ? theta[a + 1] - theta[a] : 0.0;
        tw[a] = 0.5 * (left + right) * sin(theta[a]);
    }
}

// Phase normalisation and the per-entry outputs (dointegration.py:950-1001).
// The entry's Mueller sums are first formed from the angular kernels'
// partial sums: over components c, then slots s < used, in that order (a
// fixed order, so that repeated runs give the same bits).  APT > 0: up to
// APT angles per thread (n_ang <= 64 APT), the sums in registers with every
// slot's loads of the thread issued together; APT = 0: any angle count, the
// sums through pacc.
template <int APT>
__global__ void __launch_bounds__(64) k_tab_finalize(TabView v, gbmie_table_out out, int used)
{
    const int blk = blockIdx.x;   // (lam * n_rh + rh) * n_bin + bin
    const int bin = blk % v.n_bin;
    const int64_t lr = blk / v.n_bin;
    const int rh = (int)(lr % v.n_rh), lam = (int)(lr / v.n_rh);
    const int nang = v.n_ang;
    double *P = v.pacc + (size_t)blk * 4 * nang;
    const size_t plane = (size_t)v.n_bin * 4 * nang;
    const double *src = v.part + (size_t)lr * v.n_comp * v.n_slots * plane + (size_t)bin * 4 * nang;
    // trapz(p11 sin(theta), theta) with the precomputed weights
    double tr[1] = {0.0};
    const int nsrc = v.n_comp * v.n_slots;
    double R[APT > 0 ? APT : 1][4];   // APT > 0: the sums of angle threadIdx.x + 64 i
    if (APT > 0) {
#pragma unroll
        for (int i = 0; i < (APT > 0 ? APT : 1); ++i)
#pragma unroll
            for (int k = 0; k < 4; ++k) R[i][k] = 0.0;
#pragma unroll 1
        for (int c = 0; c < nsrc; c += v.n_slots)
#pragma unroll 1
            for (int sl = 0; sl < used; ++sl) {
                const double *__restrict__ q = src + (size_t)(c + sl) * plane + threadIdx.x;
#pragma unroll
                for (int i = 0; i < (APT > 0 ? APT : 1); ++i)
                    if (threadIdx.x + 64 * i < nang)
#pragma unroll
                        for (int k = 0; k < 4; ++k) R[i][k] += __ldg(q + k * nang + 64 * i);
            }
#pragma unroll
        for (int i = 0; i < (APT > 0 ? APT : 1); ++i)
            if (threadIdx.x + 64 * i < nang) tr[0] += R[i][0] * v.tw[threadIdx.x + 64 * i];
    } else {
        for (int a = threadIdx.x; a < nang; a += blockDim.x) {
            for (int k = 0; k < 4; ++k) {
                const double *q = src + k * nang + a;
                double sum = 0.0;
#pragma unroll 1
                for (int c = 0; c < nsrc; c += v.n_slots)
#pragma unroll 8
                    for (int sl = 0; sl < used; ++sl) sum += q[(size_t)(c + sl) * plane];   // loads issued ahead, adds in order
                P[k * nang + a] = sum;   // read back below by this thread only
            }
            tr[0] += P[a] * v.tw[a];
        }
    }
    block_sum<1>(tr);
    const double scale = 2.0 / tr[0];   // p11n / p11, the same at every angle
    const size_t e = ((size_t)bin * v.n_lambda + lam) * v.n_rh + rh;   // output entry
    double *ph = out.phase + e * 6 * nang;
    for (int a = threadIdx.x, i = 0; a < nang; a += blockDim.x, ++i) {
        double p11, p12, p33, p34;
        if (APT > 0) {
            // i < APT here (n_ang <= 64 APT); the index is a compile-time one
            // after unrolling the selection
            p11 = p12 = p33 = p34 = 0.0;
#pragma unroll
            for (int j = 0; j < (APT > 0 ? APT : 1); ++j)
                if (j == i) {
                    p11 = R[j][0];
                    p12 = R[j][1];
                    p33 = R[j][2];
                    p34 = R[j][3];
                }
        } else {
            p11 = P[a];
            p12 = P[nang + a];
            p33 = P[2 * nang + a];
            p34 = P[3 * nang + a];
        }
        const double p11n = p11 * scale;
        const double p12n = p12 * scale, p22n = p11n;
        const double p33n = p33 * scale, p34n = p34 * scale;
        ph[a] = p11n;
        ph[nang + a] = p12n;
        ph[2 * nang + a] = p22n;
        ph[3 * nang + a] = p33n;
        ph[4 * nang + a] = p34n;
        ph[5 * nang + a] = p33n;
        if (a == nang - 1 && out.pback) {
            double *pb = out.pback + e * 6;   // p11 p12 p33 p34 p22 p44
            pb[0] = p11n;
            pb[1] = p12n;
            pb[2] = p33n;
            pb[3] = p34n;
            pb[4] = p22n;
            pb[5] = p33n;
        }
    }
    if (threadIdx.x == 0) {
        const double *s = v.sraw + (size_t)blk * 10;
        const double2 m0 = v.m[(size_t)lr * v.n_comp];
        if (out.scalar) {
            double *o = out.scalar + e * GBMIE_NSCALAR;
            o[GBMIE_S_QEXT] = s[0];
            o[GBMIE_S_QSCA] = s[1];
            o[GBMIE_S_QABS] = s[2];
            o[GBMIE_S_QB] = s[3];
            o[GBMIE_S_G] = s[4];
            o[GBMIE_S_CSCA] = s[5];
            o[GBMIE_S_CEXT] = s[6];
            o[GBMIE_S_SSA] = s[1] / s[0];
            o[GBMIE_S_BSCA] = s[7];
            o[GBMIE_S_BEXT] = s[8];
            o[GBMIE_S_BBCK] = s[9];
            o[GBMIE_S_REFREAL] = m0.x;
            o[GBMIE_S_REFIMAG] = -fabs(m0.y);
            o[GBMIE_S_LIDAR_RATIO] = s[0] / s[3] * 4.0 * PI_D;
        }
        if (out.nl) {
            const double *nl = v.nlraw + (size_t)blk * 5;
            const double *nl0 = v.nlraw + (((size_t)lam * v.n_rh + 0) * v.n_bin + bin) * 5;
            const double mass0 = nl0[1] * v.rhop0[bin];
            double *o = out.nl + e * GBMIE_NNL;
            o[GBMIE_N_MASS] = nl[0];
            o[GBMIE_N_VOLUME] = nl[1] / mass0;
            o[GBMIE_N_AREA] = nl[2] / mass0;
            o[GBMIE_N_REFF] = nl[3];
            o[GBMIE_N_RMASS] = nl[4];
            o[GBMIE_N_RHOP] = v.rhop[(size_t)bin * v.n_rh + rh];
            o[GBMIE_N_GF] = v.gf[rh];
            o[GBMIE_N_RLOW] = v.rlow[bin];
            o[GBMIE_N_RUP] = v.rup[bin];
        }
    }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
static TabView make_view(const gbmie_table_plan *p, char *scr)
{
    const gbmie_table_desc &d = p->d;
    TabView v;
    v.n_lambda = d.n_lambda;
    v.n_rh = d.n_rh;
    v.n_size = d.n_size;
    v.n_bin = d.n_bin;
    v.n_comp = d.n_comp;
    v.n_ang = d.n_ang;
    v.grid_kind = d.grid_kind;
    v.psd_kind = d.psd_kind;
    v.rh0 = d.rh0_index;
    v.lam_shared = (d.grid_kind == GBMIE_GRID_RADIUS && d.psd_kind != GBMIE_PSD_WEIGHTS) ? 1 : 0;
    v.lambda = d.lambda;
    v.grid = d.grid;
    v.dgrid = d.dgrid;
    v.psd_param = d.psd_param;
    v.gf_psd = d.gf_psd;
    v.frac = d.frac;
    v.rhop = d.rhop;
    v.rhop0 = d.rhop0;
    v.gf = d.gf;
    v.rlow = d.rlow;
    v.rup = d.rup;
    v.theta = d.theta;
    v.m = (const double2 *)d.m;
    v.m_core = (const double2 *)d.m_core;
    v.core_ratio = d.core_ratio;
    v.dscr = d.m_core ? (double2 *)(scr + p->o_dscr) : nullptr;
    v.xg = p->xg;
    v.off = p->off;
    v.unit_base = p->unit_base;
    v.pc = (double2 *)(scr + p->o_pc);
    v.an = (double2 *)(scr + p->o_an);
    v.bn = (double2 *)(scr + p->o_bn);
    v.eff4 = (double *)(scr + p->o_eff);
    v.W = (double *)(scr + p->o_w);
    v.sums = (double *)(scr + p->o_sums);
    v.reff0 = (double *)(scr + p->o_reff0);
    v.pacc = (double *)(scr + p->o_pacc);
    v.part = (double *)(scr + p->o_part);
    v.n_slots = p->n_slots;
    v.pq = (const double2 *)(scr + p->o_pq);
    v.sraw = (double *)(scr + p->o_sraw);
    v.nlraw = (double *)(scr + p->o_nlraw);
    v.Wf = p->d.precision == GBMIE_MIXED ? (float *)(scr + p->o_wf) : nullptr;
    v.tw = (double *)(scr + p->o_tw);
    v.rowc = (double4 *)(scr + p->o_rowc);
    v.hidx = (HomogIndex *)(scr + p->o_hidx);
    v.pcd = p->d.precision == GBMIE_MIXED ? (float4 *)(scr + p->o_pcf) : nullptr;
    v.ngrp = p->ngrp;
    v.grel = p->grp;
    v.grow = p->grp ? p->grp + (size_t)p->n_le * (p->ngrp + 1) : nullptr;
    v.gunit = p->grp ? v.grow + p->n_le : nullptr;
    v.hdf = p->d.precision == GBMIE_MIXED ? (float4 *)(scr + p->o_hdf) : nullptr;
    v.rowcd = p->d.precision == GBMIE_MIXED ? (float4 *)(scr + p->o_rowcd) : nullptr;
    return v;
}

// GSF tables of table plans (Gauss nodes, generalized spherical functions,
// interpolation, the digit operand and the row buffers of the tensor-core
// expansion): they depend on the node and moment counts, the angles, the
// entry count and the precision only, so plans with the same key share them
// through the context (plans run one after another on a context, as they
// share its scratch).  Reference-counted; unused entries are evicted.
struct GsfCacheEntry {
    bool used;
    GsfTables t;
    int ng, L, nang, ntab_max, precision;
    double *hkey;   // [2 nang]: cos(theta), theta of the key
    int refs;
};
struct TableCache {
    GsfCacheEntry gsf[2];
};

void table_cache_release(gbmie_ctx *ctx)
{
    TableCache *c = (TableCache *)ctx->table_cache;
    if (!c) return;
    cudaDeviceSynchronize();
    for (GsfCacheEntry &e : c->gsf)
        if (e.used) {
            gsf_release(&e.t, ctx->stream);
            free(e.hkey);
        }
    free(c);
    ctx->table_cache = nullptr;
}

static void table_gsf_release(gbmie_ctx *ctx, int entry)
{
    TableCache *c = (TableCache *)ctx->table_cache;
    if (c && entry >= 0 && c->gsf[entry].refs > 0) --c->gsf[entry].refs;
}

// The GSF tables for a plan: a cached entry with the same key, else freshly
// prepared (into a cache entry when one is free or unused, else plan-owned,
// *entry = -1).  hkey: cos(theta) then theta on the host.
static int table_gsf_get(gbmie_ctx *ctx, int ng, int L, int nang, const double *theta, const double *hkey,
                         int ntab_max, int precision, GsfTables *t, int *entry)
{
    *entry = -1;
    if (!ctx->table_cache) ctx->table_cache = calloc(1, sizeof(TableCache));
    TableCache *c = (TableCache *)ctx->table_cache;
    const int cap = (int)(sizeof(c->gsf) / sizeof(c->gsf[0]));
    for (int i = 0; c && i < cap; ++i) {
        GsfCacheEntry &e = c->gsf[i];
        if (e.used && e.ng == ng && e.L == L && e.nang == nang && e.ntab_max == ntab_max && e.precision == precision &&
            memcmp(e.hkey, hkey, sizeof(double) * 2 * nang) == 0) {
            ++e.refs;
            *t = e.t;
            *entry = i;
            return GBMIE_OK;
        }
    }
    int slot = -1;
    for (int i = 0; c && i < cap && slot < 0; ++i)
        if (!c->gsf[i].used) slot = i;
    for (int i = 0; c && i < cap && slot < 0; ++i)
        if (c->gsf[i].refs == 0) {
            // evict: a run of the plan that last held it may still be in flight
            // on another stream, so the device is idle before the free
            cudaDeviceSynchronize();
            gsf_release(&c->gsf[i].t, ctx->stream);
            free(c->gsf[i].hkey);
            c->gsf[i].used = false;
            slot = i;
        }
    double *hk = slot >= 0 ? (double *)malloc(sizeof(double) * 2 * nang) : nullptr;
    if (slot < 0 || !hk) {   // plan-owned tables outside the cache
        free(hk);
        return gsf_prepare(ctx, ng, L, nang, theta, t, ntab_max, precision);
    }
    GsfCacheEntry &e = c->gsf[slot];
    e.t = GsfTables{};
    const int st = gsf_prepare(ctx, ng, L, nang, theta, &e.t, ntab_max, precision);
    if (st != GBMIE_OK) {
        gsf_release(&e.t, ctx->stream);
        free(hk);
        return st;
    }
    memcpy(hk, hkey, sizeof(double) * 2 * nang);
    e.used = true;
    e.hkey = hk;
    e.ng = ng;
    e.L = L;
    e.nang = nang;
    e.ntab_max = ntab_max;
    e.precision = precision;
    e.refs = 1;
    *t = e.t;
    *entry = slot;
    return GBMIE_OK;
}

// The plan's device arrays are stream-ordered allocations, freed in order on
// the context's stream after its last use there: destroying a plan neither
// waits for the device nor stalls work in flight on other streams.
static void plan_free(gbmie_table_plan *p)
{
    if (!p) return;
    cudaStream_t s = p->ctx->stream;
    if (p->xg) cudaFreeAsync(p->xg, s);
    if (p->off) cudaFreeAsync(p->off, s);
    if (p->unit_base) cudaFreeAsync(p->unit_base, s);
    if (p->unit_order) cudaFreeAsync(p->unit_order, s);
    if (p->tile_cbase) cudaFreeAsync(p->tile_cbase, s);
    if (p->bt) {
        if (p->bt_entry >= 0) ctx_angle_op_release(p->ctx, p->bt_entry);
        else cudaFree(p->bt);
    }
    free(p->hcos);
    if (p->brange) cudaFreeAsync(p->brange, s);
    if (p->unit_cbase) cudaFreeAsync(p->unit_cbase, s);
    if (p->grp) cudaFreeAsync(p->grp, s);
    if (p->ctasks) cudaFreeAsync(p->ctasks, s);
    if (p->gexec) cudaGraphExecDestroy(p->gexec);
    if (p->cap_stream) cudaStreamDestroy(p->cap_stream);
    if (p->has_gsf && p->gsf_entry >= 0) table_gsf_release(p->ctx, p->gsf_entry);
    else gsf_release(&p->gsf, s);
    free(p);
}

extern "C" int gbmie_table_plan_destroy(gbmie_table_plan *plan)
{
    if (plan) {
        cudaSetDevice(plan->ctx->device);
        // a captured graph is destroyed only once no replay is in flight
        if (plan->gexec) cudaStreamSynchronize(plan->ctx->stream);
    }
    plan_free(plan);
    return GBMIE_OK;
}

extern "C" int gbmie_table_plan_create(gbmie_ctx *ctx, const gbmie_table_desc *desc, gbmie_table_plan **out,
                                       int64_t *scratch_bytes)
{
    if (!ctx) return GBMIE_ERR_INVALID;
    if (!desc || !out) return ctx_fail(ctx, GBMIE_ERR_INVALID, "gbmie_table_plan_create: NULL argument");
    *out = nullptr;
    const gbmie_table_desc &d = *desc;
    if (d.n_lambda < 1 || d.n_rh < 1 || d.n_size < 2 || d.n_bin < 1 || d.n_comp < 1 || d.n_ang < 2 ||
        d.n_bin > 8 || d.n_gsf < 0 || (d.n_gsf > 0 && d.n_gsf < 3) || d.rh0_index < 0 || d.rh0_index >= d.n_rh ||
        d.n_gsf_nodes < 0 || (d.n_gsf > 0 && d.n_gsf_nodes > 0 && d.n_gsf_nodes < d.n_gsf))
        return ctx_fail(ctx, GBMIE_ERR_INVALID, "gbmie_table_plan_create: bad sizes (n_size >= 2, n_ang >= 2, "
                                                "1 <= n_bin <= 8, n_gsf = 0 or >= 3, n_gsf_nodes = 0 or "
                                                ">= n_gsf)");
    if (d.grid_kind != GBMIE_GRID_X && d.grid_kind != GBMIE_GRID_RADIUS)
        return ctx_fail(ctx, GBMIE_ERR_INVALID, "gbmie_table_plan_create: bad grid_kind");
    if (d.psd_kind < GBMIE_PSD_LOGNORM || d.psd_kind > GBMIE_PSD_WEIGHTS)
        return ctx_fail(ctx, GBMIE_ERR_INVALID, "gbmie_table_plan_create: bad psd_kind");
    if (d.precision != GBMIE_PLAIN_FP64 && d.precision != GBMIE_MIXED)
        return ctx_fail(ctx, GBMIE_ERR_INVALID, "gbmie_table_plan_create: bad precision");
    if ((d.m_core == nullptr) != (d.core_ratio == nullptr))
        return ctx_fail(ctx, GBMIE_ERR_INVALID, "gbmie_table_plan_create: m_core and core_ratio go together");
    if (!d.lambda || !d.grid || !d.dgrid || !d.m || !d.frac || !d.rhop || !d.rhop0 || !d.gf || !d.rlow || !d.rup ||
        !d.cos_theta || !d.theta || (d.psd_kind != GBMIE_PSD_WEIGHTS && (!d.psd_param || !d.gf_psd)) ||
        (d.psd_kind == GBMIE_PSD_WEIGHTS && !d.weights))
        return ctx_fail(ctx, GBMIE_ERR_INVALID, "gbmie_table_plan_create: missing array");
    cudaSetDevice(ctx->device);
    gbmie_table_plan *p = (gbmie_table_plan *)calloc(1, sizeof(gbmie_table_plan));
    if (!p) return GBMIE_ERR_NOMEM;
    p->ctx = ctx;
    p->d = d;
    p->wait_limit = GBMIE_WAIT_LIMIT_DEFAULT;
    p->n_le = d.grid_kind == GBMIE_GRID_X ? 1 : d.n_lambda;
    p->n_units = (int64_t)d.n_lambda * d.n_rh * d.n_comp;
    p->n_inst = p->n_units * d.n_size;
    p->n_entries = (int64_t)d.n_lambda * d.n_rh * d.n_bin;
    const int64_t nrows = (int64_t)p->n_le * d.n_size;
    int st = ctx_cuda(ctx, cudaMallocAsync((void **)&p->xg, sizeof(double) * nrows, ctx->stream), "plan x grid");
    if (st == GBMIE_OK) st = ctx_cuda(ctx, cudaMallocAsync((void **)&p->off, sizeof(int64_t) * (nrows + 1), ctx->stream), "plan offsets");
    if (st == GBMIE_OK)
        st = ctx_cuda(ctx, cudaMallocAsync((void **)&p->unit_base, sizeof(int64_t) * p->n_units, ctx->stream), "plan unit base");
    if (st == GBMIE_OK) {
        ctx_pre_launch(ctx);
        k_tab_make_x<<<(unsigned)ceil_div64(nrows, 256), 256, 0, ctx->stream>>>(p->n_le, d.n_size, d.grid_kind,
                                                                               d.grid, d.lambda, p->xg,
                                                                               ctx->d_flags);
        st = ctx_check_launch(ctx, "k_tab_make_x");
    }
    int64_t total = 0;
    if (st == GBMIE_OK) st = launch_layout(ctx, nrows, p->xg, 0, p->off, &total);
    int64_t *hoff = nullptr;
    if (st == GBMIE_OK) {
        hoff = (int64_t *)malloc(sizeof(int64_t) * (nrows + 1));
        if (!hoff) st = GBMIE_ERR_NOMEM;
    }
    if (st == GBMIE_OK)
        st = ctx_cuda(ctx, cudaMemcpyAsync(hoff, p->off, sizeof(int64_t) * (nrows + 1), cudaMemcpyDeviceToHost, ctx->stream),
                      "plan offsets copy");
    p->bt_entry = -1;
    p->gsf_entry = -1;
    if (st == GBMIE_OK && (d.precision == GBMIE_MIXED || d.n_gsf > 0)) {
        // the keys of the cached angle operand and GSF tables: cos(theta), theta
        p->hcos = (double *)malloc(sizeof(double) * 2 * d.n_ang);
        if (!p->hcos) st = GBMIE_ERR_NOMEM;
        else
            st = ctx_cuda(ctx, cudaMemcpyAsync(p->hcos, d.cos_theta, sizeof(double) * d.n_ang, cudaMemcpyDeviceToHost, ctx->stream),
                          "plan angles copy");
        if (st == GBMIE_OK)
            st = ctx_cuda(ctx, cudaMemcpyAsync(p->hcos + d.n_ang, d.theta, sizeof(double) * d.n_ang,
                                               cudaMemcpyDeviceToHost, ctx->stream),
                          "plan angles copy");
    }
    if (st == GBMIE_OK) st = ctx_cuda(ctx, cudaStreamSynchronize(ctx->stream), "plan offsets sync");
    if (st == GBMIE_OK) {
        p->pc_total = total;
        int nm = 2;
        for (int64_t j = 0; j < nrows; ++j) {
            const int g = (int)(hoff[j + 1] - hoff[j]);
            if (g > nm) nm = g;
        }
        p->nmax_max = nm;
        int64_t *ub = (int64_t *)malloc(sizeof(int64_t) * p->n_units);
        if (!ub) st = GBMIE_ERR_NOMEM;
        int64_t acc = 0;
        for (int64_t u = 0; ub && u < p->n_units; ++u) {
            const int lam = (int)(u / ((int64_t)d.n_rh * d.n_comp));
            const int le = d.grid_kind == GBMIE_GRID_X ? 0 : lam;
            ub[u] = acc;
            acc += hoff[(int64_t)(le + 1) * d.n_size] - hoff[(int64_t)le * d.n_size];
        }
        p->ab_total = acc;
        // mixed path: units in decreasing order of work (sum of nmax of their size row)
        p->n_pad_total = (d.n_ang + 127) / 128 * 128;
        p->k_pad = (p->nmax_max + 31) / 32 * 32;
        if (ub && d.precision == GBMIE_MIXED && st == GBMIE_OK) {
            int64_t *cost = (int64_t *)malloc(sizeof(int64_t) * p->n_units);
            int *ord = (int *)malloc(sizeof(int) * p->n_units);
            if (!cost || !ord) st = GBMIE_ERR_NOMEM;
            for (int64_t u = 0; st == GBMIE_OK && u < p->n_units; ++u) {
                const int lam = (int)(u / ((int64_t)d.n_rh * d.n_comp));
                const int le = d.grid_kind == GBMIE_GRID_X ? 0 : lam;
                cost[u] = hoff[(int64_t)(le + 1) * d.n_size] - hoff[(int64_t)le * d.n_size];
                ord[u] = (int)u;
            }
            if (st == GBMIE_OK) {
                // insertion-free sort: counting by cost rank is not needed; qsort on (cost desc, id)
                struct K { int64_t c; int u; };
                K *keys = (K *)malloc(sizeof(K) * p->n_units);
                if (!keys) st = GBMIE_ERR_NOMEM;
                for (int64_t u = 0; keys && u < p->n_units; ++u) keys[u] = K{cost[u], (int)u};
                if (keys) {
                    qsort(keys, (size_t)p->n_units, sizeof(K), [](const void *a, const void *b) -> int {
                        const K *x = (const K *)a, *y = (const K *)b;
                        if (x->c != y->c) return x->c > y->c ? -1 : 1;
                        return x->u - y->u;
                    });
                    for (int64_t u = 0; u < p->n_units; ++u) ord[u] = keys[u].u;
                    free(keys);
                }
            }
            // chunks (16 orders up to a tile's largest nmax) of every 64-size tile
            p->ntiles = (d.n_size + 63) / 64;
            const int ntp = p->ntiles + 1;
            int *tcb = st == GBMIE_OK ? (int *)malloc(sizeof(int) * (size_t)p->n_le * ntp) : nullptr;
            int64_t *ucb = st == GBMIE_OK ? (int64_t *)malloc(sizeof(int64_t) * p->n_units) : nullptr;
            if (st == GBMIE_OK && (!tcb || !ucb)) st = GBMIE_ERR_NOMEM;
            for (int le = 0; st == GBMIE_OK && le < p->n_le; ++le) {
                int acc_c = 0;
                for (int t = 0; t < p->ntiles; ++t) {
                    const int t0 = 64 * t, nt = d.n_size - t0 < 64 ? d.n_size - t0 : 64;
                    const int64_t r = (int64_t)le * d.n_size + t0 + nt - 1;
                    tcb[le * ntp + t] = acc_c;
                    acc_c += (int)((hoff[r + 1] - hoff[r] + 15) / 16);
                }
                tcb[le * ntp + p->ntiles] = acc_c;
            }
            int64_t nch = 0;
            for (int64_t u = 0; st == GBMIE_OK && u < p->n_units; ++u) {
                const int lam = (int)(u / ((int64_t)d.n_rh * d.n_comp));
                const int le = d.grid_kind == GBMIE_GRID_X ? 0 : lam;
                ucb[u] = nch;
                nch += tcb[le * ntp + p->ntiles];
            }
            p->n_chunks = nch;
            if (st == GBMIE_OK)
                st = ctx_cuda(ctx, cudaMallocAsync((void **)&p->tile_cbase, sizeof(int) * (size_t)p->n_le * ntp, ctx->stream), "tile chunks");
            if (st == GBMIE_OK)
                st = ctx_cuda(ctx, cudaMallocAsync((void **)&p->unit_cbase, sizeof(int64_t) * p->n_units, ctx->stream), "unit chunks");
            if (st == GBMIE_OK)
                st = ctx_cuda(ctx, cudaMemcpyAsync(p->tile_cbase, tcb, sizeof(int) * (size_t)p->n_le * ntp,
                                              cudaMemcpyHostToDevice, ctx->stream), "tile chunks copy");
            if (st == GBMIE_OK)
                st = ctx_cuda(ctx, cudaMemcpyAsync(p->unit_cbase, ucb, sizeof(int64_t) * p->n_units, cudaMemcpyHostToDevice, ctx->stream),
                              "unit chunks copy");
            free(tcb);
            free(ucb);
            // order-major layout of the mixed recurrences' rows and
            // coefficients in groups of 32 sizes: order k of size 32 g + l at
            // [group base + 32 (k - 1) + l], so that a warp (one group) reads
            // and writes one contiguous 512-byte segment per order.  A group
            // holds 32 x its largest nmax entries.  grp = [n_le][ng + 1]
            // bases within a wavelength's block, [n_le] block bases of the
            // rows, [n_units] block bases of the coefficients.
            p->ngrp = (d.n_size + 31) / 32;
            const size_t ngl = (size_t)p->n_le * (p->ngrp + 1);
            const size_t ngrp_all = ngl + p->n_le + p->n_units;
            int64_t *hg = st == GBMIE_OK ? (int64_t *)malloc(sizeof(int64_t) * ngrp_all) : nullptr;
            if (st == GBMIE_OK && !hg) st = GBMIE_ERR_NOMEM;
            if (st == GBMIE_OK) {
                int64_t rows_acc = 0;
                for (int le = 0; le < p->n_le; ++le) {
                    int64_t acc_g = 0;
                    for (int g = 0; g < p->ngrp; ++g) {
                        hg[(size_t)le * (p->ngrp + 1) + g] = acc_g;
                        int64_t gm = 0;
                        for (int i = 32 * g; i < d.n_size && i < 32 * g + 32; ++i) {
                            const int64_t r = (int64_t)le * d.n_size + i;
                            if (hoff[r + 1] - hoff[r] > gm) gm = hoff[r + 1] - hoff[r];
                        }
                        acc_g += 32 * gm;
                    }
                    hg[(size_t)le * (p->ngrp + 1) + p->ngrp] = acc_g;
                    hg[ngl + le] = rows_acc;
                    rows_acc += acc_g;
                }
                p->pcg_total = rows_acc;
                int64_t cf_acc = 0;
                for (int64_t u = 0; u < p->n_units; ++u) {
                    const int lam = (int)(u / ((int64_t)d.n_rh * d.n_comp));
                    const int le = d.grid_kind == GBMIE_GRID_X ? 0 : lam;
                    hg[ngl + p->n_le + u] = cf_acc;
                    cf_acc += hg[(size_t)le * (p->ngrp + 1) + p->ngrp];
                }
                p->cfg_total = cf_acc;
                st = ctx_cuda(ctx, cudaMallocAsync((void **)&p->grp, sizeof(int64_t) * ngrp_all, ctx->stream), "size groups");
            }
            if (st == GBMIE_OK)
                st = ctx_cuda(ctx, cudaMemcpyAsync(p->grp, hg, sizeof(int64_t) * ngrp_all, cudaMemcpyHostToDevice, ctx->stream),
                              "size groups copy");
            // tasks of the persistent coefficient kernel: (wavelength block,
            // group) by decreasing largest nmax (stable), each with every
            // unit of that block
            if (st == GBMIE_OK) {
                const int nlg = p->n_le * p->ngrp;
                struct G { int64_t gm; int lg; };
                G *gs = (G *)malloc(sizeof(G) * (size_t)nlg);
                const int64_t upl = d.grid_kind == GBMIE_GRID_X ? p->n_units : (int64_t)d.n_rh * d.n_comp;
                int2 *ht = (int2 *)malloc(sizeof(int2) * (size_t)nlg * (size_t)upl);
                if (!gs || !ht) st = GBMIE_ERR_NOMEM;
                for (int k = 0; st == GBMIE_OK && k < nlg; ++k) {
                    const int le = k / p->ngrp, g = k % p->ngrp;
                    const int64_t *rel = hg + (size_t)le * (p->ngrp + 1);
                    gs[k] = G{(rel[g + 1] - rel[g]) / 32, k};
                }
                if (st == GBMIE_OK) {
                    qsort(gs, (size_t)nlg, sizeof(G), [](const void *a, const void *b) -> int {
                        const G *x = (const G *)a, *y = (const G *)b;
                        if (x->gm != y->gm) return x->gm > y->gm ? -1 : 1;
                        return x->lg - y->lg;
                    });
                    int64_t nt = 0;
                    for (int k = 0; k < nlg; ++k) {
                        const int le = gs[k].lg / p->ngrp, g = gs[k].lg % p->ngrp;
                        const int64_t u0 = d.grid_kind == GBMIE_GRID_X ? 0 : (int64_t)le * upl;
                        for (int64_t u = u0; u < u0 + upl; ++u) ht[nt++] = make_int2((int)u, g);
                    }
                    p->n_ctasks = (int)nt;
                    st = ctx_cuda(ctx, cudaMallocAsync((void **)&p->ctasks, sizeof(int2) * (size_t)nt, ctx->stream),
                                  "coefficient tasks");
                    if (st == GBMIE_OK)
                        st = ctx_cuda(ctx, cudaMemcpyAsync(p->ctasks, ht, sizeof(int2) * (size_t)nt, cudaMemcpyHostToDevice,
                                                           ctx->stream),
                                      "coefficient tasks copy");
                }
                free(gs);
                free(ht);
            }
            free(hg);
            if (st == GBMIE_OK) st = ctx_cuda(ctx, cudaMallocAsync((void **)&p->unit_order, sizeof(int) * p->n_units, ctx->stream), "unit order");
            if (st == GBMIE_OK)
                st = ctx_cuda(ctx, cudaMemcpyAsync(p->unit_order, ord, sizeof(int) * p->n_units, cudaMemcpyHostToDevice, ctx->stream),
                              "unit order copy");
            free(cost);
            free(ord);
        }
        if (ub) {
            st = ctx_cuda(ctx, cudaMemcpyAsync(p->unit_base, ub, sizeof(int64_t) * p->n_units, cudaMemcpyHostToDevice, ctx->stream),
                          "plan unit base copy");
            free(ub);
        }
    }
    // nmax buckets of the plain angular kernel: per x grid, the size range
    // whose nmax falls in each bucket (nmax grows with the size index)
    if (st == GBMIE_OK) {
        const int lim[GBMIE_TUNE_BUCKETS - 1] = {16, 64, 256};
        const int nb1 = GBMIE_TUNE_BUCKETS + 1;
        int2 *hb = (int2 *)malloc(sizeof(int2) * nb1 * (size_t)p->n_le);
        if (!hb) st = GBMIE_ERR_NOMEM;
        for (int b = 0; b < nb1; ++b) p->bmaxlen[b] = 0;
        for (int le = 0; hb && le < p->n_le; ++le) {
            int i = 0;
            for (int b = 0; b < GBMIE_TUNE_BUCKETS; ++b) {
                const int i0 = i;
                if (b == GBMIE_TUNE_BUCKETS - 1) i = d.n_size;
                else
                    while (i < d.n_size) {
                        const int64_t r = (int64_t)le * d.n_size + i;
                        if (hoff[r + 1] - hoff[r] > lim[b]) break;
                        ++i;
                    }
                hb[b * p->n_le + le] = make_int2(i0, i);
                if (i - i0 > p->bmaxlen[b]) p->bmaxlen[b] = i - i0;
            }
            hb[GBMIE_TUNE_BUCKETS * p->n_le + le] = make_int2(0, d.n_size);
        }
        p->bmaxlen[GBMIE_TUNE_BUCKETS] = d.n_size;
        if (st == GBMIE_OK)
            st = ctx_cuda(ctx, cudaMallocAsync((void **)&p->brange, sizeof(int2) * nb1 * (size_t)p->n_le, ctx->stream), "bucket ranges");
        if (st == GBMIE_OK)
            st = ctx_cuda(ctx, cudaMemcpyAsync(p->brange, hb, sizeof(int2) * nb1 * (size_t)p->n_le, cudaMemcpyHostToDevice, ctx->stream),
                          "bucket ranges copy");
        free(hb);
        const int thr = d.n_ang >= 256 ? 256 : ((d.n_ang + 31) / 32) * 32;
        for (int b = 0; b < nb1; ++b) {
            p->plain_chunk[b] = 256;
            p->plain_threads[b] = thr;
        }
        p->plain_split = 0;   // one launch over the whole grid until tuned
        p->coef_block = 128;
        p->tc_win = 3;
    }
    free(hoff);
    if (st == GBMIE_OK) {
        size_t o = 0;
        auto carve = [&](size_t bytes) {
            const size_t at = o;
            o = align_up(o + bytes, 256);
            return at;
        };
        const size_t nW = (size_t)d.n_lambda * d.n_rh * d.n_bin * d.n_comp;
        const bool mixed = d.precision == GBMIE_MIXED;
        p->o_pc = carve(sizeof(double2) * (size_t)p->pc_total);
        p->o_an = carve(mixed ? 16 : sizeof(double2) * (size_t)p->ab_total);
        p->o_bn = carve(mixed ? 16 : sizeof(double2) * (size_t)p->ab_total);
        p->o_eff = carve(sizeof(double) * 4 * (size_t)p->n_inst);
        p->o_w = carve(sizeof(double) * nW * d.n_size);
        p->o_sums = carve(sizeof(double) * nW * 4);
        p->o_reff0 = carve(sizeof(double) * (size_t)d.n_lambda * d.n_bin * d.n_comp);
        p->o_pacc = carve(sizeof(double) * (size_t)p->n_entries * 4 * d.n_ang);
        // partial-sum slots per unit: mixed, two size halves per tile range;
        // plain, the chunks of the finest chunking the autotuner tries (64
        // sizes) over the nmax buckets or the whole grid, whichever is more
        if (mixed) {
            int nsm = 0;
            cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, ctx->device);
            if (nsm < 1) nsm = 1;
            // work items of the contraction: (unit, angle block) pairs, each
            // split into tile ranges when there are fewer than four pairs per SM
            const int64_t pairs = p->n_units * (int64_t)(p->n_pad_total / 128);
            int ntr = 1;
            if (pairs < 4 * (int64_t)nsm) {
                const int64_t want = ceil_div64(4 * (int64_t)nsm, pairs);
                ntr = (int)(want < p->ntiles ? want : p->ntiles);
            }
            p->tc_tpr = (p->ntiles + ntr - 1) / ntr;
            p->tc_ntr = (p->ntiles + p->tc_tpr - 1) / p->tc_tpr;
            p->n_slots = 2 * p->tc_ntr;
            p->slots_used = p->n_slots;
        } else {
            int split = 0;
            for (int b = 0; b < GBMIE_TUNE_BUCKETS; ++b) split += (p->bmaxlen[b] + 63) / 64;
            const int whole = (p->bmaxlen[GBMIE_TUNE_BUCKETS] + 63) / 64;
            p->n_slots = split > whole ? split : whole;
            p->slots_used = 0;
        }
        p->o_part = carve(sizeof(double) * (size_t)p->n_units * p->n_slots * d.n_bin * 4 * d.n_ang);
        p->o_pq = carve(mixed ? 16 : sizeof(double2) * (size_t)p->nmax_max * d.n_ang);
        p->o_cf = carve(mixed ? sizeof(float4) * (size_t)(p->ab_total > p->cfg_total ? p->ab_total : p->cfg_total) : 16);
        p->o_eexp = carve(mixed ? sizeof(int) * (size_t)p->n_inst : 16);
        p->o_eunit = carve(mixed ? sizeof(int) * (size_t)p->n_units : 16);
        p->o_asplit = carve(mixed ? (size_t)16384 * (size_t)p->n_chunks : 16);
        p->o_cnext = carve(16);
        p->o_pcf = carve(mixed ? sizeof(float4) * (size_t)p->pcg_total : 16);
        p->o_hdf = carve(mixed ? 4 * sizeof(float4) * (size_t)p->n_units : 16);
        p->o_rowcd = carve(mixed ? 2 * sizeof(float4) * (size_t)p->n_le * d.n_size : 16);
        p->o_dscr = carve(d.m_core ? 5 * sizeof(double2) * (size_t)p->ab_total : 16);
        p->o_wf = carve(mixed ? sizeof(float) * nW * d.n_size : 16);
        p->o_tw = carve(sizeof(double) * d.n_ang);
        p->o_rowc = carve(sizeof(double4) * (size_t)p->n_le * d.n_size);
        p->o_hidx = carve(sizeof(HomogIndex) * (size_t)p->n_units);
        p->o_sraw = carve(sizeof(double) * (size_t)p->n_entries * 10);
        p->o_nlraw = carve(sizeof(double) * (size_t)p->n_entries * 5);
        p->bytes = o;
        void *scr = nullptr;
        st = ctx_scratch(ctx, p->bytes, &scr);
    }
    if (st == GBMIE_OK && d.precision == GBMIE_MIXED) st = build_table_bt(ctx, p);
    if (st == GBMIE_OK) table_tune_lookup(ctx, p);
    if (st == GBMIE_OK && d.n_gsf > 0) {
        st = table_gsf_get(ctx, d.n_gsf_nodes > 0 ? d.n_gsf_nodes : d.n_gsf, d.n_gsf, d.n_ang, d.theta, p->hcos,
                           (int)p->n_entries, d.precision, &p->gsf, &p->gsf_entry);
        p->has_gsf = 1;
    }
    if (st == GBMIE_OK) st = gbmie_ctx_synchronize(ctx);
    if (st != GBMIE_OK) {
        plan_free(p);
        return st;
    }
    if (scratch_bytes) *scratch_bytes = (int64_t)p->bytes;
    *out = p;
    return GBMIE_OK;
}

// integratePSD scalars, normalisation and GSF moments (both precisions).
// The FP32 scalar sums run 64 threads per (wavelength, RH): with ~30 sizes
// per thread the block reduction of the 9 x bins sums is a small part of the
// kernel (0.21 ms on the sulfate-like table against 0.36 ms with 256)
static int launch_table_tail(gbmie_ctx *ctx, gbmie_table_plan *p, TabView &v, const gbmie_table_out *out)
{
    const gbmie_table_desc &d = p->d;
    cudaStream_t st = ctx->stream;
    const unsigned nlr = (unsigned)((int64_t)d.n_lambda * d.n_rh);
    const bool mixed = d.precision == GBMIE_MIXED;
    ctx_pre_launch(ctx);
#define SC_LAUNCH(NBV)                                                                 \
    case NBV:                                                                          \
        if (mixed) k_tab_scalars<NBV, float><<<nlr, 64, 0, st>>>(v);                   \
        else k_tab_scalars<NBV, double><<<nlr, 256, 0, st>>>(v);                       \
        break;
    switch (d.n_bin) {
        SC_LAUNCH(1) SC_LAUNCH(2) SC_LAUNCH(3) SC_LAUNCH(4) SC_LAUNCH(5) SC_LAUNCH(6) SC_LAUNCH(7)
        default:
        SC_LAUNCH(8)
    }
#undef SC_LAUNCH
    GBMIE_TRY(ctx_check_launch(ctx, "k_tab_scalars"));
    ctx_pre_launch(ctx);
    k_tab_trapz<<<1, 256, 0, st>>>(d.n_ang, d.theta, v.tw);
    GBMIE_TRY(ctx_check_launch(ctx, "k_tab_trapz"));
    ctx_pre_launch(ctx);
    {
        const int apt = (d.n_ang + 63) / 64;   // angles per thread of 64-thread blocks
        auto fin = apt <= 1 ? k_tab_finalize<1> : apt == 2 ? k_tab_finalize<2> : apt == 3 ? k_tab_finalize<3>
                 : apt == 4 ? k_tab_finalize<4> : k_tab_finalize<0>;
        fin<<<(unsigned)p->n_entries, 64, 0, st>>>(v, *out, p->slots_used);
    }
    GBMIE_TRY(ctx_check_launch(ctx, "k_tab_finalize"));
    if (p->has_gsf) {
        GsfMap map = {{0, 2, 3, 5, 1, 4}, {0, 4, 2, 5, 1, 3}};
        GBMIE_TRY(launch_gsf_expand(ctx, &p->gsf, (int)p->n_entries, out->phase, (int64_t)6 * d.n_ang, d.n_ang, map,
                                    out->pmom, (int64_t)6 * d.n_gsf, d.n_gsf, nullptr, d.precision));
    }
    return GBMIE_OK;
}

int launch_table_mixed(gbmie_ctx *ctx, gbmie_table_plan *p, TabView &v, char *scr);
int table_tc_win_max();

// The plain angular kernel over one nmax bucket (sizes of every unit whose
// nmax falls in it; bucket GBMIE_TUNE_BUCKETS = the whole grid), `chunk`
// sizes per block, `threads` angles per pass.
static int launch_s12_plain(gbmie_ctx *ctx, gbmie_table_plan *p, TabView &v, int b, int chunk, int threads,
                            int slot0 = 0)
{
    if (p->bmaxlen[b] == 0) return GBMIE_OK;
    const int nchunk = (p->bmaxlen[b] + chunk - 1) / chunk;
    if (slot0 + nchunk > p->n_slots)
        return ctx_fail(ctx, GBMIE_ERR_INVALID, "k_tab_s12_plain: %d partial-sum slots needed, %d held",
                        slot0 + nchunk, p->n_slots);
    const unsigned grid = (unsigned)(p->n_units * nchunk);
    const int2 *br = p->brange + (size_t)b * p->n_le;
    cudaStream_t st = ctx->stream;
    ctx_pre_launch(ctx);
    if (p->d.n_bin <= 1) k_tab_s12_plain<1><<<grid, threads, 0, st>>>(v, chunk, nchunk, br, slot0);
    else if (p->d.n_bin <= 2) k_tab_s12_plain<2><<<grid, threads, 0, st>>>(v, chunk, nchunk, br, slot0);
    else if (p->d.n_bin <= 4) k_tab_s12_plain<4><<<grid, threads, 0, st>>>(v, chunk, nchunk, br, slot0);
    else k_tab_s12_plain<8><<<grid, threads, 0, st>>>(v, chunk, nchunk, br, slot0);
    return ctx_check_launch(ctx, "k_tab_s12_plain");
}

extern "C" int gbmie_table_run(gbmie_ctx *ctx, gbmie_table_plan *p, const gbmie_table_out *out)
{
    if (!ctx || !p || !out || p->ctx != ctx) return ctx_fail(ctx, GBMIE_ERR_INVALID, "gbmie_table_run: bad plan");
    if (!out->phase || (p->has_gsf && !out->pmom))
        return ctx_fail(ctx, GBMIE_ERR_INVALID, "gbmie_table_run: phase (and pmom with n_gsf) required");
    cudaSetDevice(ctx->device);
    void *s = nullptr;
    GBMIE_TRY(ctx_scratch(ctx, p->bytes, &s));
    char *scr = (char *)s;
    TabView v = make_view(p, scr);
    const gbmie_table_desc &d = p->d;
    cudaStream_t st = ctx->stream;
    const int64_t nrows = (int64_t)p->n_le * d.n_size;
    ctx_pre_launch(ctx);
    k_tab_psi_chi<<<(unsigned)ceil_div64(nrows, 128), 128, 0, st>>>(nrows, p->xg, p->off, v.pc, v.rowc, v,
                                                                    d.precision == GBMIE_MIXED && !d.m_core);
    GBMIE_TRY(ctx_check_launch(ctx, "k_tab_psi_chi"));
    ctx_pre_launch(ctx);
    k_tab_index<<<(unsigned)ceil_div64(p->n_units, 128), 128, 0, st>>>(p->n_units, v.m, v.hidx, ctx->d_flags);
    GBMIE_TRY(ctx_check_launch(ctx, "k_tab_index"));
    // the PSD weights on the side stream, alongside the recurrences (they are
    // first read by the angular kernels and the scalar sums: joined there)
    const int64_t nW = (int64_t)(v.lam_shared ? 1 : d.n_lambda) * d.n_rh * d.n_bin * d.n_comp;
    GBMIE_TRY(ctx_cuda(ctx, cudaEventRecord(ctx->ev_fork, st), "fork"));
    GBMIE_TRY(ctx_cuda(ctx, cudaStreamWaitEvent(ctx->side, ctx->ev_fork, 0), "fork"));
    ctx->stream = ctx->side;
    ctx_pre_launch(ctx);
    k_tab_weights<<<(unsigned)nW, 256, 0, ctx->side>>>(v, d.weights);
    const int wst = ctx_check_launch(ctx, "k_tab_weights");
    ctx->stream = st;
    GBMIE_TRY(wst);
    GBMIE_TRY(ctx_cuda(ctx, cudaEventRecord(ctx->ev_join, ctx->side), "join"));
    ctx_pre_launch(ctx);
    if (d.precision == GBMIE_MIXED) {
        GBMIE_TRY(launch_table_mixed(ctx, p, v, scr));
        return launch_table_tail(ctx, p, v, out);
    }
    if (d.m_core) {
        k_tab_coeffs_coated<<<(unsigned)ceil_div64(p->n_inst, 128), 128, 0, st>>>(v, p->n_inst, ctx->d_flags);
        GBMIE_TRY(ctx_check_launch(ctx, "k_tab_coeffs_coated"));
    } else {
        k_tab_coeffs<<<(unsigned)ceil_div64(p->n_inst, 128), 128, 0, st>>>(v, p->n_inst, ctx->d_flags);
        GBMIE_TRY(ctx_check_launch(ctx, "k_tab_coeffs"));
    }
    GBMIE_TRY(ctx_cuda(ctx, cudaStreamWaitEvent(st, ctx->ev_join, 0), "join"));   // the PSD weights
    GBMIE_TRY(launch_pq_table(ctx, d.n_ang, d.cos_theta, p->nmax_max, (double2 *)(scr + p->o_pq)));
    // the buckets' chunks take consecutive partial-sum slots
    int slot = 0;
    if (p->plain_split) {
        for (int b = 0; b < GBMIE_TUNE_BUCKETS; ++b) {
            GBMIE_TRY(launch_s12_plain(ctx, p, v, b, p->plain_chunk[b], p->plain_threads[b], slot));
            if (p->bmaxlen[b] > 0) slot += (p->bmaxlen[b] + p->plain_chunk[b] - 1) / p->plain_chunk[b];
        }
    } else {
        const int b = GBMIE_TUNE_BUCKETS;
        GBMIE_TRY(launch_s12_plain(ctx, p, v, b, p->plain_chunk[b], p->plain_threads[b], 0));
        slot = (p->bmaxlen[b] + p->plain_chunk[b] - 1) / p->plain_chunk[b];
    }
    p->slots_used = slot;
    return launch_table_tail(ctx, p, v, out);
}

// ---------------------------------------------------------------------------
// The whole table as one CUDA graph
// ---------------------------------------------------------------------------
static bool same_out(const gbmie_table_out &a, const gbmie_table_out &b)
{
    return a.phase == b.phase && a.pback == b.pback && a.scalar == b.scalar && a.nl == b.nl && a.pmom == b.pmom;
}

// Capture one gbmie_table_run on the plan's private stream.  Per-kernel event
// timing is off while capturing; the launch count of one run is recorded so
// that replays can report it.
static int capture_table(gbmie_ctx *ctx, gbmie_table_plan *p, const gbmie_table_out *out)
{
    if (p->gexec) {
        cudaGraphExecDestroy(p->gexec);   // an in-flight replay finishes first
        p->gexec = nullptr;
    }
    if (!p->cap_stream)
        GBMIE_TRY(ctx_cuda(ctx, cudaStreamCreateWithFlags(&p->cap_stream, cudaStreamNonBlocking), "capture stream"));
    const cudaStream_t saved = ctx->stream;
    const int saved_timing = ctx->timing;
    const int64_t l0 = ctx->launches;
    ctx->stream = p->cap_stream;
    ctx->timing = 0;
    int st = ctx_cuda(ctx, cudaStreamBeginCapture(p->cap_stream, cudaStreamCaptureModeThreadLocal), "begin capture");
    cudaGraph_t graph = nullptr;
    if (st == GBMIE_OK) {
        st = gbmie_table_run(ctx, p, out);
        const int st2 = ctx_cuda(ctx, cudaStreamEndCapture(p->cap_stream, &graph), "end capture");
        if (st == GBMIE_OK) st = st2;
    }
    ctx->stream = saved;
    ctx->timing = saved_timing;
    p->glaunches = ctx->launches - l0;
    ctx->launches = l0;
    if (st == GBMIE_OK && graph)
        st = ctx_cuda(ctx, cudaGraphInstantiate(&p->gexec, graph, 0), "graph instantiate");
    if (graph) cudaGraphDestroy(graph);
    if (st != GBMIE_OK) {
        if (p->gexec) cudaGraphExecDestroy(p->gexec);
        p->gexec = nullptr;
        cudaGetLastError();   // a failed capture leaves no sticky error behind
        return st;
    }
    p->gout = *out;
    p->gscratch = ctx->scratch;
    return GBMIE_OK;
}

extern "C" int gbmie_table_run_graph(gbmie_ctx *ctx, gbmie_table_plan *p, const gbmie_table_out *out)
{
    if (!ctx || !p || !out || p->ctx != ctx)
        return ctx_fail(ctx, GBMIE_ERR_INVALID, "gbmie_table_run_graph: bad plan");
    if (!out->phase || (p->has_gsf && !out->pmom))
        return ctx_fail(ctx, GBMIE_ERR_INVALID, "gbmie_table_run_graph: phase (and pmom with n_gsf) required");
    cudaSetDevice(ctx->device);
    void *s = nullptr;
    GBMIE_TRY(ctx_scratch(ctx, p->bytes, &s));   // grows (and synchronises) outside the capture only
    if (!p->gexec || !same_out(p->gout, *out) || p->gscratch != ctx->scratch) GBMIE_TRY(capture_table(ctx, p, out));
    ctx_pre_launch(ctx);
    GBMIE_TRY(ctx_cuda(ctx, cudaGraphLaunch(p->gexec, ctx->stream), "graph launch"));
    const int st = ctx_check_launch(ctx, "gbmie_table_graph");
    ctx->launches += p->glaunches - 1;   // the graph's kernels, not the graph launch itself
    return st;
}

// ---------------------------------------------------------------------------
// Autotuning
// ---------------------------------------------------------------------------
static void tune_key(const gbmie_table_plan *p, int64_t *k)
{
    const gbmie_table_desc &d = p->d;
    k[0] = d.precision;
    k[1] = d.n_ang;
    k[2] = d.n_size;
    k[3] = p->n_le;
    k[4] = p->n_units;
    k[5] = d.n_bin;
    k[6] = d.n_comp;
    k[7] = p->nmax_max;
    k[8] = p->pc_total;
    k[9] = d.m_core ? 1 : 0;
}

// parameter vector: split, chunk [5], threads [5], coefficient block, window
static void tune_save(const gbmie_table_plan *p, int32_t *q)
{
    q[0] = p->plain_split;
    for (int b = 0; b <= GBMIE_TUNE_BUCKETS; ++b) {
        q[1 + b] = p->plain_chunk[b];
        q[1 + GBMIE_TUNE_BUCKETS + 1 + b] = p->plain_threads[b];
    }
    q[11] = p->coef_block;
    q[12] = p->tc_win;
}

static void tune_load(gbmie_table_plan *p, const int32_t *q)
{
    p->plain_split = q[0];
    for (int b = 0; b <= GBMIE_TUNE_BUCKETS; ++b) {
        p->plain_chunk[b] = q[1 + b];
        p->plain_threads[b] = q[1 + GBMIE_TUNE_BUCKETS + 1 + b];
    }
    p->coef_block = q[11];
    p->tc_win = q[12];
}

// A plan whose table shape was tuned before in this context takes those
// parameters (called at plan creation).
int table_tune_lookup(gbmie_ctx *ctx, gbmie_table_plan *p)
{
    int64_t k[10];
    tune_key(p, k);
    for (int i = 0; i < ctx->n_tune; ++i)
        if (memcmp(ctx->tune_cache[i].key, k, sizeof(k)) == 0) {
            tune_load(p, ctx->tune_cache[i].params);
            p->tuned = 1;
            return 1;
        }
    return 0;
}

extern "C" int gbmie_table_plan_autotune(gbmie_ctx *ctx, gbmie_table_plan *p, const gbmie_table_out *out)
{
    if (!ctx || !p || !out || p->ctx != ctx) return ctx_fail(ctx, GBMIE_ERR_INVALID, "gbmie_table_plan_autotune: bad plan");
    cudaSetDevice(ctx->device);
    if (p->tuned || table_tune_lookup(ctx, p)) return GBMIE_OK;
    const int save_timing = ctx->timing;
    const int64_t save_launches = ctx->launches;
    ctx->timing = 0;
    int st = gbmie_table_run(ctx, p, out);   // fills coefficients, weights, B tables
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (st == GBMIE_OK) st = ctx_cuda(ctx, cudaEventCreate(&e0), "tune events");
    if (st == GBMIE_OK) st = ctx_cuda(ctx, cudaEventCreate(&e1), "tune events");
    void *s = nullptr;
    if (st == GBMIE_OK) st = ctx_scratch(ctx, p->bytes, &s);
    if (st == GBMIE_OK) {
        char *scr = (char *)s;
        TabView v = make_view(p, scr);
        if (p->d.precision == GBMIE_MIXED) {
            st = tune_table_mixed(ctx, p, v, scr, e0, e1);
        } else {
            // per nmax bucket, and for one launch over the whole grid: sizes per
            // block x angles per pass of the plain kernel; then the bucketed
            // launches against the single one
            const int chunks[4] = {64, 128, 256, 512};
            const int thr_cap = p->d.n_ang >= 256 ? 256 : ((p->d.n_ang + 31) / 32) * 32;
            int thrs[4], nthr = 0;
            for (int t = 64; t <= 256; t *= 2)
                if (t < thr_cap) thrs[nthr++] = t;
            thrs[nthr++] = thr_cap;
            auto timed = [&](auto launch, float &ms_out) -> int {
                float best = 3.4e38f;
                for (int rep = 0; rep < 2; ++rep) {
                    cudaEventRecord(e0, ctx->stream);
                    GBMIE_TRY(launch());
                    cudaEventRecord(e1, ctx->stream);
                    GBMIE_TRY(ctx_cuda(ctx, cudaEventSynchronize(e1), "tune angular sums"));
                    float ms = 0.f;
                    cudaEventElapsedTime(&ms, e0, e1);
                    if (ms < best) best = ms;
                }
                ms_out = best;
                return GBMIE_OK;
            };
            for (int b = 0; st == GBMIE_OK && b <= GBMIE_TUNE_BUCKETS; ++b) {
                if (p->bmaxlen[b] == 0) continue;
                float best = 3.4e38f;
                for (int ci = 0; st == GBMIE_OK && ci < 4; ++ci)
                    for (int ti = 0; st == GBMIE_OK && ti < nthr; ++ti) {
                        float ms = 0.f;
                        st = timed([&] { return launch_s12_plain(ctx, p, v, b, chunks[ci], thrs[ti]); }, ms);
                        if (st == GBMIE_OK && ms < best) {
                            best = ms;
                            p->plain_chunk[b] = chunks[ci];
                            p->plain_threads[b] = thrs[ti];
                        }
                    }
            }
            float t_split = 0.f, t_single = 0.f;
            if (st == GBMIE_OK)
                st = timed([&] {
                    for (int b = 0; b < GBMIE_TUNE_BUCKETS; ++b)
                        GBMIE_TRY(launch_s12_plain(ctx, p, v, b, p->plain_chunk[b], p->plain_threads[b]));
                    return (int)GBMIE_OK;
                }, t_split);
            const int bw = GBMIE_TUNE_BUCKETS;
            if (st == GBMIE_OK)
                st = timed([&] { return launch_s12_plain(ctx, p, v, bw, p->plain_chunk[bw], p->plain_threads[bw]); },
                           t_single);
            p->plain_split = t_split < t_single ? 1 : 0;
        }
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (st == GBMIE_OK) {
        p->tuned = 1;
        int64_t k[10];
        tune_key(p, k);
        const int slot = ctx->n_tune < 16 ? ctx->n_tune++ : 15;
        memcpy(ctx->tune_cache[slot].key, k, sizeof(k));
        tune_save(p, ctx->tune_cache[slot].params);
        if (p->gexec) {   // a captured graph holds the old launch parameters
            cudaGraphExecDestroy(p->gexec);
            p->gexec = nullptr;
        }
        st = gbmie_table_run(ctx, p, out);   // the outputs of the tuned table
    }
    if (st == GBMIE_OK) st = gbmie_ctx_synchronize(ctx);
    ctx->timing = save_timing;
    ctx->launches = save_launches;
    return st;
}

extern "C" int gbmie_table_plan_set_wait_limit(gbmie_table_plan *p, int64_t tries)
{
    if (!p || tries > (int64_t)GBMIE_WAIT_LIMIT_DEFAULT) return GBMIE_ERR_INVALID;
    const uint32_t lim = tries < 0 ? GBMIE_WAIT_LIMIT_DEFAULT : (uint32_t)tries;
    if (lim == p->wait_limit) return GBMIE_OK;
    if (p->gexec) {   // a captured graph holds the old limit; none of its replays may be in flight
        GBMIE_TRY(ctx_cuda(p->ctx, cudaStreamSynchronize(p->ctx->stream), "set_wait_limit"));
        cudaGraphExecDestroy(p->gexec);
        p->gexec = nullptr;
    }
    p->wait_limit = lim;
    return GBMIE_OK;
}

extern "C" int gbmie_table_plan_set_dn_fp64(gbmie_table_plan *p, int32_t enable)
{
    if (!p || (enable != 0 && enable != 1)) return GBMIE_ERR_INVALID;
    if (enable == p->dn_fp64) return GBMIE_OK;
    if (p->gexec) {   // a captured graph holds the other kernel; none of its replays may be in flight
        GBMIE_TRY(ctx_cuda(p->ctx, cudaStreamSynchronize(p->ctx->stream), "set_dn_fp64"));
        cudaGraphExecDestroy(p->gexec);
        p->gexec = nullptr;
    }
    p->dn_fp64 = enable;
    return GBMIE_OK;
}

extern "C" int gbmie_table_plan_tuning(const gbmie_table_plan *p, int32_t *params)
{
    if (!p || !params) return GBMIE_ERR_INVALID;
    params[0] = p->tuned;
    tune_save(p, params + 1);
    params[14] = params[15] = 0;
    return GBMIE_OK;
}

// The inverse of gbmie_table_plan_tuning: launch parameters given by the
// caller (those of an earlier autotuning, say), checked against the choices
// the autotuner itself makes, which the plan's scratch is sized for.
extern "C" int gbmie_table_plan_set_tuning(gbmie_table_plan *p, const int32_t *params)
{
    if (!p || !params) return GBMIE_ERR_INVALID;
    const int32_t *q = params + 1;
    bool ok = q[0] == 0 || q[0] == 1;
    for (int b = 0; b <= GBMIE_TUNE_BUCKETS; ++b) {
        const int c = q[1 + b], t = q[1 + GBMIE_TUNE_BUCKETS + 1 + b];
        ok = ok && (c == 64 || c == 128 || c == 256 || c == 512) && t >= 32 && t <= 256 && t % 32 == 0;
    }
    ok = ok && (q[11] == 64 || q[11] == 128 || q[11] == 256) && q[12] >= 1 && q[12] <= table_tc_win_max();
    if (!ok) return ctx_fail(p->ctx, GBMIE_ERR_INVALID, "gbmie_table_plan_set_tuning: parameters out of range");
    if (p->gexec) {   // a captured graph holds the old launches; none of its replays may be in flight
        GBMIE_TRY(ctx_cuda(p->ctx, cudaStreamSynchronize(p->ctx->stream), "set_tuning"));
        cudaGraphExecDestroy(p->gexec);
        p->gexec = nullptr;
    }
    tune_load(p, q);
    p->tuned = 1;
    return GBMIE_OK;
}

