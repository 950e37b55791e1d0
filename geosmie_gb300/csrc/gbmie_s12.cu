// Angular functions and amplitude functions S1, S2 (FP64), and the
// MultipleMie size sweep.
//
// S1 = sum a_n pi~_n + b_n tau~_n and S2 = sum a_n tau~_n + b_n pi~_n
// (pymiecoated/mie_props.py:133-149) are evaluated as
//   S+ = S1 + S2 = sum (a_n + b_n)(pi~_n + tau~_n),
//   S- = S1 - S2 = sum (a_n - b_n)(pi~_n - tau~_n),
// which halves the multiply-adds; the tables p = pi~ + tau~, q = pi~ - tau~
// are stored order-major [n][angle] so a warp reading one order for 32
// angles is coalesced.
#include "common.cuh"
#include "mie_device.cuh"

// pi_n, tau_n upward recurrences of pymiecoated/mie_props.py:166-192, scaled
// by (2n+1)/(n(n+1)) (mie_props.py:224-229).  One thread per cosine.
// mode 0: pq[(n-1)*nang + a] = (p, q);  mode 1: pi_out/tau_out[a*nmax + n-1].
template <int MODE>
__global__ void k_pitau(int nang, const double *__restrict__ cost, int nmax, double2 *__restrict__ pq,
                        double *__restrict__ pi_out, double *__restrict__ tau_out, int *__restrict__ flags)
{
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= nang) return;
    const double u = cost[a];
    if (!(fabs(u) <= 1.0)) {
        atomicOr(flags, GBMIE_FLAG_INVALID);
        return;
    }
    double pm2 = 0.0, pm1 = 0.0;
    for (int n = 1; n <= nmax; ++n) {
        double p, t;
        if (n == 1) {
            p = 1.0;
            t = u;
        } else if (n == 2) {
            p = 3.0 * u;
            t = 6.0 * u * u - 3.0;
        } else {
            const double dn = (double)(n - 1);   // the reference's 0-based index
            p = (2.0 * dn + 1.0) / dn * pm1 * u - (dn + 1.0) / dn * pm2;
            t = (dn + 1.0) * u * p - (dn + 2.0) * pm1;
        }
        pm2 = pm1;
        pm1 = p;
        const double s = (2.0 * n + 1.0) / ((double)n * (double)(n + 1));
        const double ps = p * s, ts = t * s;
        if (MODE == 0) {
            pq[(int64_t)(n - 1) * nang + a] = make_double2(ps + ts, ps - ts);
        } else {
            pi_out[(int64_t)a * nmax + n - 1] = ps;
            tau_out[(int64_t)a * nmax + n - 1] = ts;
        }
    }
}

int launch_pq_table(gbmie_ctx *ctx, int nang, const double *cost, int nmax, double2 *pq)
{
    ctx_pre_launch(ctx);
    k_pitau<0><<<(nang + 127) / 128, 128, 0, ctx->stream>>>(nang, cost, nmax, pq, nullptr, nullptr, ctx->d_flags);
    return ctx_check_launch(ctx, "k_pitau");
}

extern "C" int gbmie_pitau(gbmie_ctx *ctx, int32_t nang, const double *cos_theta, int32_t nmax, double *pi_out,
                           double *tau_out)
{
    if (!ctx) return GBMIE_ERR_INVALID;
    if (nang < 0 || nmax < 2 || nmax > GBMIE_MAX_NMAX || (nang > 0 && (!cos_theta || !pi_out || !tau_out)))
        return ctx_fail(ctx, GBMIE_ERR_INVALID, "gbmie_pitau: bad arguments");
    if (nang == 0) return GBMIE_OK;
    cudaSetDevice(ctx->device);
    ctx_pre_launch(ctx);
    k_pitau<1><<<(nang + 127) / 128, 128, 0, ctx->stream>>>(nang, cos_theta, nmax, nullptr, pi_out, tau_out,
                                                            ctx->d_flags);
    return ctx_check_launch(ctx, "k_pitau");
}

// One block per instance (grid-stride); coefficients staged in shared memory
// as (a+b, a-b) in chunks of S12_CHUNK orders; threads stride over angles.
#define S12_THREADS 128
#define S12_CHUNK 1024

__global__ void __launch_bounds__(S12_THREADS) k_s12_api(int64_t n, const int64_t *__restrict__ off,
                                                         const double2 *__restrict__ an,
                                                         const double2 *__restrict__ bn, int nang,
                                                         const double2 *__restrict__ pq, double2 *__restrict__ s1,
                                                         double2 *__restrict__ s2)
{
    __shared__ double2 cd[S12_CHUNK][2];
    for (int64_t i = blockIdx.x; i < n; i += gridDim.x) {
        const int64_t o = off[i];
        const int nm = (int)(off[i + 1] - o);
        for (int a0 = 0; a0 < nang; a0 += S12_THREADS) {
            const int a = a0 + threadIdx.x;
            double sp_r = 0.0, sp_i = 0.0, sm_r = 0.0, sm_i = 0.0;
            for (int k0 = 0; k0 < nm; k0 += S12_CHUNK) {
                const int kn = min(S12_CHUNK, nm - k0);
                __syncthreads();
                for (int k = threadIdx.x; k < kn; k += S12_THREADS) {
                    const double2 av = an[o + k0 + k], bv = bn[o + k0 + k];
                    cd[k][0] = make_double2(av.x + bv.x, av.y + bv.y);
                    cd[k][1] = make_double2(av.x - bv.x, av.y - bv.y);
                }
                __syncthreads();
                if (a < nang) {
                    const double2 *col = pq + (int64_t)k0 * nang + a;
#pragma unroll 4
                    for (int k = 0; k < kn; ++k) {
                        const double2 t = col[(int64_t)k * nang];
                        const double2 c = cd[k][0], d = cd[k][1];
                        sp_r = fma(c.x, t.x, sp_r);
                        sp_i = fma(c.y, t.x, sp_i);
                        sm_r = fma(d.x, t.y, sm_r);
                        sm_i = fma(d.y, t.y, sm_i);
                    }
                }
            }
            if (a < nang) {
                s1[i * nang + a] = make_double2(0.5 * (sp_r + sm_r), 0.5 * (sp_i + sm_i));
                s2[i * nang + a] = make_double2(0.5 * (sp_r - sm_r), 0.5 * (sp_i - sm_i));
            }
        }
    }
}

int launch_s12_api(gbmie_ctx *ctx, int64_t n, const int64_t *off, const double2 *an, const double2 *bn, int nang,
                   const double2 *pq, double2 *s1, double2 *s2)
{
    if (n == 0 || nang == 0) return GBMIE_OK;
    const unsigned grid = (unsigned)(n < 152 * 64 ? n : 152 * 64);
    ctx_pre_launch(ctx);
    k_s12_api<<<grid, S12_THREADS, 0, ctx->stream>>>(n, off, an, bn, nang, pq, s1, s2);
    return ctx_check_launch(ctx, "k_s12_api");
}

__global__ void k_max_gap(int64_t n, const int64_t *__restrict__ off, unsigned long long *out)
{
    unsigned long long m = 0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const long long g = off[i + 1] - off[i];
        if (g > 0 && (unsigned long long)g > m) m = (unsigned long long)g;
    }
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long t = __shfl_xor_sync(0xffffffffu, m, o);
        m = t > m ? t : m;
    }
    if ((threadIdx.x & 31) == 0) atomicMax(out, m);
}

extern "C" int gbmie_s12(gbmie_ctx *ctx, int64_t n, const int64_t *offsets, const gbmie_complex *an,
                         const gbmie_complex *bn, int32_t nang, const double *cos_theta, gbmie_complex *s1,
                         gbmie_complex *s2)
{
    if (!ctx) return GBMIE_ERR_INVALID;
    if (n < 0 || nang < 0 || (n > 0 && nang > 0 && (!offsets || !an || !bn || !cos_theta || !s1 || !s2)))
        return ctx_fail(ctx, GBMIE_ERR_INVALID, "gbmie_s12: bad arguments");
    if (n == 0 || nang == 0) return GBMIE_OK;
    cudaSetDevice(ctx->device);
    // largest nmax -> table size (synchronous)
    unsigned long long *dmax = nullptr;
    GBMIE_TRY(ctx_cuda(ctx, cudaMallocAsync((void **)&dmax, sizeof(unsigned long long), ctx->stream), "s12"));
    cudaMemsetAsync(dmax, 0, sizeof(unsigned long long), ctx->stream);
    ctx_pre_launch(ctx);
    k_max_gap<<<152, 256, 0, ctx->stream>>>(n, offsets, dmax);
    int st = ctx_check_launch(ctx, "k_max_gap");
    if (st == GBMIE_OK)
        st = ctx_cuda(ctx, cudaMemcpyAsync(ctx->h_pinned, dmax, 8, cudaMemcpyDeviceToHost, ctx->stream), "s12");
    cudaFreeAsync(dmax, ctx->stream);
    GBMIE_TRY(st);
    GBMIE_TRY(ctx_cuda(ctx, cudaStreamSynchronize(ctx->stream), "s12"));
    const int64_t nmx = ctx->h_pinned[0];
    if (nmx < 1 || nmx > GBMIE_MAX_NMAX) return ctx_fail(ctx, GBMIE_ERR_INVALID, "gbmie_s12: bad offsets");
    const int nt = (int)(nmx < 2 ? 2 : nmx);
    void *p = nullptr;
    GBMIE_TRY(ctx_scratch(ctx, (size_t)nt * nang * sizeof(double2), &p));
    GBMIE_TRY(launch_pq_table(ctx, nang, cos_theta, nt, (double2 *)p));
    return launch_s12_api(ctx, n, offsets, (const double2 *)an, (const double2 *)bn, nang, (const double2 *)p,
                          (double2 *)s1, (double2 *)s2);
}

// S1, S2 from caller-supplied pi~/tau~ rows (mie_props.py:115-149): one warp
// per (instance, angle), lanes over orders, FP64 sums reduced across the warp.
// An instance with more orders than a row holds is flagged and skipped.
__global__ void k_s12_pt(int64_t n, const int64_t *__restrict__ off, const double2 *__restrict__ an,
                         const double2 *__restrict__ bn, int nang, int ld, const double *__restrict__ pin,
                         const double *__restrict__ tin, double2 *__restrict__ s1, double2 *__restrict__ s2,
                         int *__restrict__ flags)
{
    const int lane = threadIdx.x & 31;
    const int64_t nwarp = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t w = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); w < n * nang; w += nwarp) {
        const int64_t i = w / nang;
        const int a = (int)(w - i * nang);
        const int64_t o = off[i];
        const int64_t nm = off[i + 1] - o;
        if (nm < 0 || nm > ld) {
            if (lane == 0) atomicOr(flags, GBMIE_FLAG_NMAX);
            continue;   // uniform across the warp
        }
        const double *pr = pin + (int64_t)a * ld, *tr = tin + (int64_t)a * ld;
        double r1 = 0.0, i1 = 0.0, r2 = 0.0, i2 = 0.0;
        for (int64_t k = lane; k < nm; k += 32) {
            const double2 av = an[o + k], bv = bn[o + k];
            const double p = pr[k], t = tr[k];
            r1 = fma(av.x, p, fma(bv.x, t, r1));
            i1 = fma(av.y, p, fma(bv.y, t, i1));
            r2 = fma(av.x, t, fma(bv.x, p, r2));
            i2 = fma(av.y, t, fma(bv.y, p, i2));
        }
        for (int m = 16; m > 0; m >>= 1) {
            r1 += __shfl_xor_sync(0xffffffffu, r1, m);
            i1 += __shfl_xor_sync(0xffffffffu, i1, m);
            r2 += __shfl_xor_sync(0xffffffffu, r2, m);
            i2 += __shfl_xor_sync(0xffffffffu, i2, m);
        }
        if (lane == 0) {
            s1[i * nang + a] = make_double2(r1, i1);
            s2[i * nang + a] = make_double2(r2, i2);
        }
    }
}

extern "C" int gbmie_s12_pt(gbmie_ctx *ctx, int64_t n, const int64_t *offsets, const gbmie_complex *an,
                            const gbmie_complex *bn, int32_t nang, int32_t ld, const double *pi_rows,
                            const double *tau_rows, gbmie_complex *s1, gbmie_complex *s2)
{
    if (!ctx) return GBMIE_ERR_INVALID;
    if (n < 0 || nang < 0 || ld < 1 ||
        (n > 0 && nang > 0 && (!offsets || !an || !bn || !pi_rows || !tau_rows || !s1 || !s2)))
        return ctx_fail(ctx, GBMIE_ERR_INVALID, "gbmie_s12_pt: bad arguments");
    if (n == 0 || nang == 0) return GBMIE_OK;
    cudaSetDevice(ctx->device);
    const int64_t warps = n * nang;
    const int64_t blocks = ceil_div64(warps, 8);
    ctx_pre_launch(ctx);
    k_s12_pt<<<(unsigned)(blocks < 152 * 32 ? blocks : 152 * 32), 256, 0, ctx->stream>>>(
        n, offsets, (const double2 *)an, (const double2 *)bn, nang, ld, pi_rows, tau_rows, (double2 *)s1,
        (double2 *)s2, ctx->d_flags);
    return ctx_check_launch(ctx, "k_s12_pt");
}

int launch_coeffs_uniform(gbmie_ctx *ctx, int64_t n, const double *x, double2 eps, const int64_t *off,
                          double2 *an, double2 *bn, double *eff);

extern "C" int gbmie_size_range(gbmie_ctx *ctx, int64_t n, const double *x, double mr, double mi, int32_t nang,
                                const double *cos_theta, gbmie_complex *s1, gbmie_complex *s2, double *eff)
{
    if (!ctx) return GBMIE_ERR_INVALID;
    if (n < 0 || nang < 0 || (n > 0 && (!x || (nang > 0 && (!cos_theta || !s1 || !s2)))) || !isfinite(mr) ||
        !isfinite(mi))
        return ctx_fail(ctx, GBMIE_ERR_INVALID, "gbmie_size_range: bad arguments");
    if (n == 0) return GBMIE_OK;
    cudaSetDevice(ctx->device);
    // layout into the head of the scratch (offsets, n+1 int64), totals on the host
    int64_t *off = nullptr;
    GBMIE_TRY(ctx_cuda(ctx, cudaMallocAsync((void **)&off, (size_t)(n + 1) * sizeof(int64_t), ctx->stream),
                       "size_range offsets"));
    int64_t total = 0, nmx = 0;
    int st = launch_layout(ctx, n, x, 0, off, &total);
    // maximum nmax (for the angular table)
    if (st == GBMIE_OK) {
        unsigned long long *dm = nullptr;
        st = ctx_cuda(ctx, cudaMallocAsync((void **)&dm, 8, ctx->stream), "size_range max");
        if (st == GBMIE_OK) {
            cudaMemsetAsync(dm, 0, 8, ctx->stream);
            ctx_pre_launch(ctx);
            k_max_gap<<<152, 256, 0, ctx->stream>>>(n, off, dm);
            st = ctx_check_launch(ctx, "k_max_gap");
            if (st == GBMIE_OK)
                st = ctx_cuda(ctx, cudaMemcpyAsync(ctx->h_pinned + 1, dm, 8, cudaMemcpyDeviceToHost, ctx->stream),
                              "size_range max");
            cudaFreeAsync(dm, ctx->stream);
            if (st == GBMIE_OK) st = ctx_cuda(ctx, cudaStreamSynchronize(ctx->stream), "size_range max");
            nmx = ctx->h_pinned[1];
        }
    }
    if (st != GBMIE_OK) {
        cudaFreeAsync(off, ctx->stream);
        return st;
    }
    const int nt = (int)(nmx < 2 ? 2 : nmx);
    const size_t b_ab = align_up((size_t)total * sizeof(double2), 256);
    const size_t b_pq = (size_t)nt * (nang > 0 ? nang : 1) * sizeof(double2);
    void *p = nullptr;
    st = ctx_scratch(ctx, 2 * b_ab + b_pq, &p);
    if (st == GBMIE_OK) {
        double2 *an = (double2 *)p, *bn = (double2 *)((char *)p + b_ab), *pq = (double2 *)((char *)p + 2 * b_ab);
        const double2 eps = make_double2(mr * mr - mi * mi, 2.0 * mr * mi);
        st = launch_coeffs_uniform(ctx, n, x, eps, off, an, bn, eff);
        if (st == GBMIE_OK && nang > 0) st = launch_pq_table(ctx, nang, cos_theta, nt, pq);
        if (st == GBMIE_OK && nang > 0)
            st = launch_s12_api(ctx, n, off, an, bn, nang, pq, (double2 *)s1, (double2 *)s2);
    }
    cudaFreeAsync(off, ctx->stream);
    return st;
}
