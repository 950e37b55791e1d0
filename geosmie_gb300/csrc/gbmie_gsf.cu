// Generalized-spherical-function (GSF) expansion of scattering matrices
// (gsf/spher_expan.f restated for the GPU, FP64).
//
//  k_gsf_nodes   Gauss-Legendre nodes/weights (GAUSS, spher_expan.f:520-579):
//                Newton iteration on P_n with the reference's recurrence,
//                step and stopping rule; one thread per node, started from
//                cos(pi (i - 1/4) / (n + 1/2)) instead of the reference's
//                extrapolated guesses (same roots), weights 2 (1-x^2) /
//                (n P_{n-1})^2 as the reference's PA^2 (1-x^2) times 2.
//  k_gsf_gener   P1..P4 at every node for l = 0..L-1 (GENER, :363-407, with
//                its loop bound LMAX = L1MAX-1, which fills index L1MAX).
//  k_gsf_interp  interval index and fraction of acos(node) in the table's
//                angle grid, with linear extrapolation (LINTERPOL IEX = 1,
//                :593-623).
//  k_gsf_expand  alpha1..alpha4, beta1, beta2 (SPHER_EXPAN :269-358) and the
//                normalisation by 1/alpha1(0) (main program :95-106).
#include "common.cuh"
#include "gsf.cuh"

__global__ void k_gsf_nodes(int n, double *__restrict__ z, double *__restrict__ w)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;   // 0-based node, ascending order
    if (i >= n) return;
    // descending root index k (k = 1 is the largest root)
    const int k = n - i;
    double x = cos(3.14159265358979323846 * ((double)k - 0.25) / ((double)n + 0.5));
    const double A = 1.0, B = 2.0, f = (double)n;
    double pa = 0.0, pb = 0.0, pc = 0.0;
    double check = 1e-16;
    for (int it = 1; it <= 200; ++it) {
        if (it > 100) check *= 10.0;
        pb = 1.0;
        pc = x;
        double dj = A;
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
    if ((n & 1) && i == n / 2) x = 0.0;   // the reference sets the middle node to 0 exactly
    z[i] = x;
    w[i] = B * (pa * pa * (A - x * x));
}

// P[t][g][l], t = 0..3 (P1..P4), node g, order l = 0..L-1.
__global__ void k_gsf_gener(int ng, int L, const double *__restrict__ z, double *__restrict__ P)
{
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= ng) return;
    const double u = z[g];
    const size_t plane = (size_t)ng * L;
    double *P1 = P + (size_t)g * L, *P2 = P1 + plane, *P3 = P2 + plane, *P4 = P3 + plane;
    const double d6 = 0.25 * sqrt(6.0);
    const double dup = 1.0 + u, dum = 1.0 - u, du = u * u;
    // 0-based l: values at l = 0, 1, 2
    double a1m = 1.0, a1 = u, a2m = 0.0, a2 = 0.0, a3m = 0.0, a3 = 0.0, a4m = 0.0, a4 = 0.0;
    if (L > 0) { P1[0] = 1.0; P2[0] = 0.0; P3[0] = 0.0; P4[0] = 0.0; }
    if (L > 1) { P1[1] = u; P2[1] = 0.0; P3[1] = 0.0; P4[1] = 0.0; }
    if (L > 2) {
        P1[2] = 0.5 * (3.0 * du - 1.0);
        P2[2] = 0.25 * dup * dup;
        P3[2] = 0.25 * dum * dum;
        P4[2] = d6 * (du - 1.0);
    }
    a1m = u;
    a1 = 0.5 * (3.0 * du - 1.0);
    a2m = 0.0;
    a2 = 0.25 * dup * dup;
    a3m = 0.0;
    a3 = 0.25 * dum * dum;
    a4m = 0.0;
    a4 = d6 * (du - 1.0);
    // reference loop L1 = 3..LMAX (1-based) computes index L1+1, i.e. 0-based
    // l = L1 from l-1 = L1-1 (value a*) and l-2 (a*m); coefficients use the
    // reference's L = L1-1.
    for (int L1 = 3; L1 <= L - 1; ++L1) {
        const int l = L1 - 1;   // the reference's L
        const double c1 = 1.0 / (double)(l + 1);
        const double c2 = (double)(2 * l + 1);
        const double c3 = 1.0 / sqrt((double)((l + 1) * (l + 1) - 4));
        const double c4 = sqrt((double)(l * l - 4));
        const double c5 = 1.0 / ((double)l * (double)((l + 1) * (l + 1) - 4));
        const double c6 = (double)(2 * l + 1) * (double)(l * (l + 1));
        const double c7 = (double)((2 * l + 1) * 4);
        const double c8 = (double)(l + 1) * (double)(l * l - 4);
        const double cu1 = c2 * u, cu2 = c6 * u;
        const double dl = (double)(L1 - 1);
        const double n1 = c1 * (cu1 * a1 - dl * a1m);
        const double n2 = c5 * ((cu2 - c7) * a2 - c8 * a2m);
        const double n3 = c5 * ((cu2 + c7) * a3 - c8 * a3m);
        const double n4 = c3 * (cu1 * a4 - c4 * a4m);
        P1[L1] = n1; P2[L1] = n2; P3[L1] = n3; P4[L1] = n4;
        a1m = a1; a1 = n1;
        a2m = a2; a2 = n2;
        a3m = a3; a3 = n3;
        a4m = a4; a4 = n4;
    }
}

__global__ void k_gsf_interp(int ng, int nang, const double *__restrict__ z, const double *__restrict__ theta,
                             int *__restrict__ base, double *__restrict__ frac)
{
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= ng) return;
    const double x = acos(z[g]);
    int b;
    if (x < theta[0]) {
        b = 0;
    } else if (x > theta[nang - 1]) {
        b = nang - 2;
    } else {   // first I (1-based, from 2) with XX(I) > X
        int lo = 1, hi = nang - 1;   // 0-based candidates for I-1 .. search smallest j >= 1 with theta[j] > x
        while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (theta[mid] > x) hi = mid;
            else lo = mid + 1;
        }
        b = lo - 1;
    }
    base[g] = b;
    frac[g] = (x - theta[b]) / (theta[b + 1] - theta[b]);
}

// One block per table entry; threads over the orders l.  F element rows are
// read through fmap (Mishchenko order F11 F22 F33 F44 F12 F34 -> row index
// in the entry's block of erows rows of nang values); output row r of the
// 6 coefficients (alpha1 alpha2 alpha3 alpha4 beta1 beta2) goes to omap[r].
#define GSF_NODE_CHUNK 256
__global__ void k_gsf_expand(int ntab, int nang, int ng, int L, const double *__restrict__ F, int64_t entry_stride,
                             int64_t row_stride, GsfMap map, const double *__restrict__ w,
                             const double *__restrict__ P, const int *__restrict__ base,
                             const double *__restrict__ frac, double *__restrict__ coef, int64_t out_stride,
                             int64_t out_row_stride, double *__restrict__ cnorm)
{
    __shared__ double Fs[GSF_NODE_CHUNK][6];
    __shared__ double s_norm;
    const size_t plane = (size_t)ng * L;
    for (int e = blockIdx.x; e < ntab; e += gridDim.x) {
        const double *Fe = F + (size_t)e * entry_stride;
        for (int l0 = 0; l0 < L; l0 += blockDim.x) {
            const int l = l0 + threadIdx.x;
            double al1 = 0, al2 = 0, al3 = 0, al4 = 0, be1 = 0, be2 = 0;
            for (int g0 = 0; g0 < ng; g0 += GSF_NODE_CHUNK) {
                const int gn = min(GSF_NODE_CHUNK, ng - g0);
                __syncthreads();
                for (int t = threadIdx.x; t < gn * 6; t += blockDim.x) {
                    const int g = g0 + t / 6, el = t % 6;
                    const double *row = Fe + (size_t)map.f[el] * row_stride;
                    const int b = base[g];
                    const double y0 = row[b], y1 = row[b + 1];
                    Fs[t / 6][el] = (y0 + (y1 - y0) * frac[g]) * w[g];
                }
                __syncthreads();
                if (l < L) {
                    for (int gg = 0; gg < gn; ++gg) {
                        const size_t pi = (size_t)(g0 + gg) * L + l;
                        const double p1 = P[pi], p2 = P[pi + plane], p3 = P[pi + 2 * plane], p4 = P[pi + 3 * plane];
                        const double f11 = Fs[gg][0], f22 = Fs[gg][1], f33 = Fs[gg][2], f44 = Fs[gg][3];
                        const double f12 = Fs[gg][4], f34 = Fs[gg][5];
                        al1 = fma(f11, p1, al1);
                        al4 = fma(f44, p1, al4);
                        al2 = fma(f22 + f33, p2, al2);
                        al3 = fma(f22 - f33, p3, al3);
                        be1 = fma(f12, p4, be1);
                        be2 = fma(f34, p4, be2);
                    }
                }
            }
            const double cl = (double)l + 0.5;
            const double a2 = al2 * cl * 0.5, a3 = al3 * cl * 0.5;
            double v[6] = {al1 * cl, a2 + a3, a2 - a3, al4 * cl, be1 * cl, be2 * cl};
            if (l0 == 0) {
                __syncthreads();
                if (threadIdx.x == 0) s_norm = 1.0 / v[0];
                __syncthreads();
            }
            if (l < L) {
                const double cn = s_norm;
                double *out = coef + (size_t)e * out_stride + l;
                for (int r = 0; r < 6; ++r) out[(size_t)map.o[r] * out_row_stride] = v[r] * cn;
                if (l == 0 && cnorm) cnorm[e] = cn;
            }
        }
    }
}

int gsf_prepare(gbmie_ctx *ctx, int ng, int L, int nang, const double *theta, GsfTables *t, int ntab_max,
                int precision)
{
    t->ng = ng;
    t->L = L;
    t->nang = nang;
    const size_t bytes = sizeof(double) * (2 * (size_t)ng + 4 * (size_t)ng * L + ng) + sizeof(int) * ng;
    GBMIE_TRY(ctx_cuda(ctx, cudaMallocAsync(&t->mem, bytes, ctx->stream), "gsf tables"));
    char *p = (char *)t->mem;
    t->z = (double *)p; p += sizeof(double) * ng;
    t->w = (double *)p; p += sizeof(double) * ng;
    t->P = (double *)p; p += sizeof(double) * 4 * (size_t)ng * L;
    t->frac = (double *)p; p += sizeof(double) * ng;
    t->base = (int *)p;
    const int tb = 128, nb = (ng + tb - 1) / tb;
    ctx_pre_launch(ctx);
    k_gsf_nodes<<<nb, tb, 0, ctx->stream>>>(ng, t->z, t->w);
    GBMIE_TRY(ctx_check_launch(ctx, "k_gsf_nodes"));
    ctx_pre_launch(ctx);
    k_gsf_gener<<<nb, tb, 0, ctx->stream>>>(ng, t->L, t->z, t->P);
    GBMIE_TRY(ctx_check_launch(ctx, "k_gsf_gener"));
    ctx_pre_launch(ctx);
    k_gsf_interp<<<nb, tb, 0, ctx->stream>>>(ng, nang, t->z, theta, t->base, t->frac);
    GBMIE_TRY(ctx_check_launch(ctx, "k_gsf_interp"));
    if (precision == GBMIE_MIXED) GBMIE_TRY(gsf_tc_prepare(ctx, t, ntab_max));
    return GBMIE_OK;
}

void gsf_release(GsfTables *t, cudaStream_t s)
{
    if (t->mem) cudaFreeAsync(t->mem, s);
    t->mem = nullptr;
    if (t->tc.mem) cudaFreeAsync(t->tc.mem, s);
    t->tc.mem = nullptr;
}

int launch_gsf_expand(gbmie_ctx *ctx, const GsfTables *t, int ntab, const double *F, int64_t entry_stride,
                      int64_t row_stride, GsfMap map, double *coef, int64_t out_stride, int64_t out_row_stride,
                      double *cnorm, int precision)
{
    if (ntab <= 0) return GBMIE_OK;
    int threads = ((t->L + 31) / 32) * 32;
    if (threads > 256) threads = 256;
    const int grid = ntab < 152 * 16 ? ntab : 152 * 16;
    if (precision == GBMIE_MIXED)
        return launch_gsf_expand_tc(ctx, t, ntab, F, entry_stride, row_stride, map, coef, out_stride, out_row_stride,
                                    cnorm);
    ctx_pre_launch(ctx);
    k_gsf_expand<<<grid, threads, 0, ctx->stream>>>(ntab, t->nang, t->ng, t->L, F, entry_stride, row_stride, map,
                                                    t->w, t->P, t->base, t->frac, coef, out_stride, out_row_stride,
                                                    cnorm);
    return ctx_check_launch(ctx, "k_gsf_expand");
}

__global__ void k_deg2rad(int n, const double *__restrict__ deg, double *__restrict__ rad, int *flags)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double d2r = 3.14159265358979323846 / 180.0;
    rad[i] = deg[i] * d2r;
    if (i > 0 && !(deg[i] > deg[i - 1])) atomicOr(flags, GBMIE_FLAG_INVALID);
}

extern "C" int gbmie_gsf(gbmie_ctx *ctx, int32_t ntab, int32_t nang, const double *ang_deg, const double *F,
                         int32_t nnodes, double *coef, double *cnorm, int32_t precision)
{
    if (!ctx) return GBMIE_ERR_INVALID;
    if (ntab < 0 || nang < 2 || nnodes < 3 || (ntab > 0 && (!ang_deg || !F || !coef)))
        return ctx_fail(ctx, GBMIE_ERR_INVALID, "gbmie_gsf: bad arguments (nang >= 2, nnodes >= 3)");
    if (precision != GBMIE_PLAIN_FP64 && precision != GBMIE_MIXED)
        return ctx_fail(ctx, GBMIE_ERR_INVALID, "gbmie_gsf: bad precision");
    if (ntab == 0) return GBMIE_OK;
    cudaSetDevice(ctx->device);
    void *p = nullptr;
    GBMIE_TRY(ctx_scratch(ctx, sizeof(double) * nang, &p));
    double *theta = (double *)p;
    ctx_pre_launch(ctx);
    k_deg2rad<<<(nang + 127) / 128, 128, 0, ctx->stream>>>(nang, ang_deg, theta, ctx->d_flags);
    GBMIE_TRY(ctx_check_launch(ctx, "k_deg2rad"));
    GsfTables t{};
    GBMIE_TRY(gsf_prepare(ctx, nnodes, nnodes, nang, theta, &t, ntab, precision));
    GsfMap map;
    for (int i = 0; i < 6; ++i) map.f[i] = i, map.o[i] = i;
    int st = launch_gsf_expand(ctx, &t, ntab, F, (int64_t)6 * nang, nang, map, coef, (int64_t)6 * nnodes, nnodes,
                               cnorm, precision);
    cudaStreamSynchronize(ctx->stream);
    gsf_release(&t, ctx->stream);
    return st;
}
