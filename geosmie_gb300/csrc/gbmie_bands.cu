// Band averages of table quantities (geosmie/bandaverage.py doAverage
// :18-50, looped by fun :163-179): for every variable, bin, band and RH the
// mean of the variable linearly interpolated in wavenumber at 100 points
// spaced evenly between the band's edges and clipped to the table's
// wavenumber range.  The arithmetic follows the reference's numpy/scipy
// operations step by step, so the results agree to the last bit where the
// host compiles numpy without contracting multiply-adds:
//   numpy.linspace   x_i = i * step + beg (step = (end - beg) / 99), x_99 = end
//   numpy.clip       min(max(x, w_min), w_max)
//   scipy interp1d   sorts the table by wavenumber (stable) and, for 1-D
//                    float64 data, calls numpy.interp: j = the last node with
//                    w_j <= x; y = f_j at the last node or an exact node,
//                    else slope (x - w_j) + f_j with
//                    slope = (f_j+1 - f_j) / (w_j+1 - w_j)
//   numpy.sum        pairwise summation: 8 running sums over the first 96
//                    values, combined ((r0+r1)+(r2+r3))+((r4+r5)+(r6+r7)),
//                    then the last 4 added in order; divided by 100.
// Every product and sum is rounded on its own (__dmul_rn / __dadd_rn).
#include "common.cuh"

#define BAND_NSUB 100

// Stable ascending order of the table's wavenumbers (scipy interp1d sorts
// with a stable mergesort): rank of element i among all, ties by index.
__global__ void k_band_rank(int n, const double *__restrict__ wn, double *__restrict__ sorted,
                            int *__restrict__ perm)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double w = wn[i];
    int r = 0;
    for (int j = 0; j < n; ++j) {
        const double u = wn[j];
        r += (u < w || (u == w && j < i)) ? 1 : 0;
    }
    sorted[r] = w;
    perm[r] = i;
}

// numpy.interp at x on the sorted nodes (x already clipped into their range)
__device__ __forceinline__ double band_interp(double x, int n, const double *__restrict__ ws,
                                              const double *__restrict__ f, int64_t fstride,
                                              const int *__restrict__ perm)
{
    // j = (number of nodes <= x) - 1
    int lo = 0, hi = n;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (ws[mid] <= x) lo = mid + 1;
        else hi = mid;
    }
    const int j = lo - 1;
    if (j < 0) return f[(int64_t)perm[0] * fstride];   // not reached after the clip
    const double fj = f[(int64_t)perm[j] * fstride];
    if (j == n - 1 || ws[j] == x) return fj;
    const double fj1 = f[(int64_t)perm[j + 1] * fstride];
    const double slope = __ddiv_rn(__dsub_rn(fj1, fj), __dsub_rn(ws[j + 1], ws[j]));
    double y = __dadd_rn(__dmul_rn(slope, __dsub_rn(x, ws[j])), fj);
    if (isnan(y)) {
        y = __dadd_rn(__dmul_rn(slope, __dsub_rn(x, ws[j + 1])), fj1);
        if (isnan(y) && fj == fj1) y = fj;
    }
    return y;
}

// One thread per (variable, bin, band, RH).  vin [nvar][nbin][nlam][nrh],
// out [nvar][nbin][nband][nrh].
__global__ void k_band_average(int nvar, int nbin, int nlam, int nrh, int nband, const double *__restrict__ ws,
                               const int *__restrict__ perm, const double *__restrict__ vin,
                               const double *__restrict__ ea, const double *__restrict__ eb,
                               double *__restrict__ out)
{
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t total = (int64_t)nvar * nbin * nband * nrh;
    if (t >= total) return;
    const int r = (int)(t % nrh);
    const int k = (int)((t / nrh) % nband);
    const int64_t vb = t / ((int64_t)nrh * nband);   // variable * nbin + bin
    const double *f = vin + vb * nlam * nrh + r;
    const double a = ea[k], b = eb[k];
    const double beg = a < b ? a : b, end = a < b ? b : a;
    const double wmin = ws[0], wmax = ws[nlam - 1];
    const double step = __ddiv_rn(__dsub_rn(end, beg), (double)(BAND_NSUB - 1));
    double acc[8];
    double res = 0.0;
    for (int i = 0; i < BAND_NSUB; ++i) {
        double x = i == BAND_NSUB - 1 ? end : __dadd_rn(__dmul_rn((double)i, step), beg);
        x = fmin(fmax(x, wmin), wmax);
        const double y = band_interp(x, nlam, ws, f, nrh, perm);
        if (i < 8) {
            acc[i] = y;
        } else if (i < BAND_NSUB - BAND_NSUB % 8) {
            acc[i & 7] = __dadd_rn(acc[i & 7], y);
        } else {
            if (i == BAND_NSUB - BAND_NSUB % 8)
                res = __dadd_rn(__dadd_rn(__dadd_rn(acc[0], acc[1]), __dadd_rn(acc[2], acc[3])),
                                __dadd_rn(__dadd_rn(acc[4], acc[5]), __dadd_rn(acc[6], acc[7])));
            res = __dadd_rn(res, y);
        }
    }
    out[(vb * nband + k) * nrh + r] = __ddiv_rn(res, (double)BAND_NSUB);
}

extern "C" int gbmie_band_average(gbmie_ctx *ctx, int32_t nvar, int32_t nbin, int32_t nlam, int32_t nrh,
                                  const double *wavenum, const double *vin, int32_t nband, const double *edge_a,
                                  const double *edge_b, double *out)
{
    if (!ctx) return GBMIE_ERR_INVALID;
    if (nvar < 0 || nbin < 0 || nlam < 1 || nrh < 0 || nband < 0)
        return ctx_fail(ctx, GBMIE_ERR_INVALID, "gbmie_band_average: bad sizes (nlam >= 1)");
    const int64_t total = (int64_t)nvar * nbin * nband * nrh;
    if (total == 0) return GBMIE_OK;
    if (!wavenum || !vin || !edge_a || !edge_b || !out)
        return ctx_fail(ctx, GBMIE_ERR_INVALID, "gbmie_band_average: null pointer");
    cudaSetDevice(ctx->device);
    void *p = nullptr;
    GBMIE_TRY(ctx_scratch(ctx, align_up(sizeof(double) * nlam, 256) + sizeof(int) * nlam, &p));
    double *ws = (double *)p;
    int *perm = (int *)((char *)p + align_up(sizeof(double) * nlam, 256));
    ctx_pre_launch(ctx);
    k_band_rank<<<(nlam + 127) / 128, 128, 0, ctx->stream>>>(nlam, wavenum, ws, perm);
    GBMIE_TRY(ctx_check_launch(ctx, "k_band_rank"));
    ctx_pre_launch(ctx);
    k_band_average<<<(unsigned)ceil_div64(total, 128), 128, 0, ctx->stream>>>(nvar, nbin, nlam, nrh, nband, ws, perm,
                                                                             vin, edge_a, edge_b, out);
    return ctx_check_launch(ctx, "k_band_average");
}
