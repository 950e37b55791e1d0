// gbmie_coeffs: Mie coefficients and efficiencies of independent instances.
//
// One thread per instance (FP64 recurrences are inherently sequential in n;
// on GB300 FP64 issue is the scarce resource, so the work-optimal thread-
// per-instance form is used and warps are kept uniform by the caller's
// ordering of instances).  Homogeneous instances run in place: the
// Riccati-Bessel rows are built in the a_n output and overwritten by a_n as
// the downward pass consumes them, so they need no scratch.  Coated
// instances park D_n(u), D_n(v), D_n(w), psi_n(v), psi_n(w) in context
// scratch (5 complex per order).
#include "common.cuh"
#include "mie_device.cuh"

struct EmitAB {
    double2 *an, *bn;
    __device__ __forceinline__ void operator()(int k, cplx a, cplx b) const {
        an[k - 1] = d2(a);
        bn[k - 1] = d2(b);
    }
};

__device__ __forceinline__ bool same(cplx a, cplx b) { return a.re == b.re && a.im == b.im; }
__device__ __forceinline__ bool finite_c(cplx a) { return isfinite(a.re) && isfinite(a.im); }

// Dispatch of pymiecoated/mie_coeffs.py:53-71 for instance i.
__device__ __forceinline__ void coeffs_one(int64_t i, const double *__restrict__ x, const double *__restrict__ y,
                                           const double2 *__restrict__ eps, const double2 *__restrict__ mu,
                                           const double2 *__restrict__ eps2, const int64_t *__restrict__ off,
                                           double2 *an, double2 *bn, double *__restrict__ eff,
                                           double2 *__restrict__ dscr, int *__restrict__ flags)
{
    const double xi = x[i];
    const bool coated = (y != nullptr);
    const double yi = coated ? y[i] : xi;
    const cplx e1 = cx(eps[i]);
    const cplx mv = mu ? cx(mu[i]) : cx(1.0, 0.0);
    const cplx e2 = coated ? cx(eps2[i]) : e1;
    const int64_t o = off[i];
    const int nmax = (int)(off[i + 1] - o);
    bool bad = !(xi >= 0.0) || !isfinite(xi) || !(yi >= xi) || !isfinite(yi) || !finite_c(e1) || !finite_c(mv) ||
               !finite_c(e2) || (coated && !(mv.re == 1.0 && mv.im == 0.0));
    if (!bad && nmax != mie_nmax(yi)) bad = true;   // layout does not match the sizes
    double *e = eff ? eff + 6 * i : nullptr;
    if (bad) {
        atomicOr(flags, GBMIE_FLAG_INVALID);
        if (e)
            for (int j = 0; j < 6; ++j) e[j] = nan("");
        return;
    }
    double2 *a = an + o, *b = bn + o;
    EmitAB emit{a, b};
    EffSums es;
    es.init();
    if (yi == 0.0) {   // x = y = 0: the reference's intended zero result (mie_coated.py:186-189)
        for (int k = 0; k < nmax; ++k) a[k] = b[k] = make_double2(0.0, 0.0);
        if (e)
            for (int j = 0; j < 6; ++j) e[j] = 0.0;
        return;
    }
    psi_chi_row(yi, nmax, a);
    if (!coated || xi == yi || same(e1, e2)) {
        homog_instance(yi, e1, mv, a, nmax, emit, es);
    } else if (xi == 0.0) {
        homog_instance(yi, e2, mv, a, nmax, emit, es);
    } else {
        coated_instance(xi, yi, e1, e2, a, nmax, dscr + 5 * o, emit, es);
    }
    if (e) es.finish(yi, e);
}

__global__ void __launch_bounds__(128) k_coeffs_api(int64_t n, const double *__restrict__ x,
                                                    const double *__restrict__ y,
                                                    const double2 *__restrict__ eps,
                                                    const double2 *__restrict__ mu,
                                                    const double2 *__restrict__ eps2,
                                                    const int64_t *__restrict__ off, double2 *an, double2 *bn,
                                                    double *__restrict__ eff, double2 *__restrict__ dscr,
                                                    int *__restrict__ flags)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) coeffs_one(i, x, y, eps, mu, eps2, off, an, bn, eff, dscr, flags);
}

// Same with a uniform permittivity (MultipleMie: eps = (mr + i mi)^2, mu = 1).
__global__ void __launch_bounds__(128) k_coeffs_uniform(int64_t n, const double *__restrict__ x, double2 eps,
                                                        const int64_t *__restrict__ off, double2 *an, double2 *bn,
                                                        double *__restrict__ eff, int *__restrict__ flags)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double xi = x[i];
    const int64_t o = off[i];
    const int nmax = (int)(off[i + 1] - o);
    double *e = eff ? eff + 6 * i : nullptr;
    if (!(xi >= 0.0) || !isfinite(xi) || nmax != mie_nmax(xi)) {
        atomicOr(flags, GBMIE_FLAG_INVALID);
        if (e)
            for (int j = 0; j < 6; ++j) e[j] = nan("");
        return;
    }
    double2 *a = an + o, *b = bn + o;
    if (xi == 0.0) {
        for (int k = 0; k < nmax; ++k) a[k] = b[k] = make_double2(0.0, 0.0);
        if (e)
            for (int j = 0; j < 6; ++j) e[j] = 0.0;
        return;
    }
    EmitAB emit{a, b};
    EffSums es;
    psi_chi_row(xi, nmax, a);
    homog_instance(xi, cx(eps), cx(1.0, 0.0), a, nmax, emit, es);
    if (e) es.finish(xi, e);
}

int launch_coeffs_uniform(gbmie_ctx *ctx, int64_t n, const double *x, double2 eps, const int64_t *off,
                          double2 *an, double2 *bn, double *eff)
{
    if (n == 0) return GBMIE_OK;
    ctx_pre_launch(ctx);
    k_coeffs_uniform<<<(unsigned)ceil_div64(n, 128), 128, 0, ctx->stream>>>(n, x, eps, off, an, bn, eff,
                                                                             ctx->d_flags);
    return ctx_check_launch(ctx, "k_coeffs_uniform");
}

extern "C" int gbmie_coeffs(gbmie_ctx *ctx, int64_t n, const double *x, const double *y, const gbmie_complex *eps,
                            const gbmie_complex *mu, const gbmie_complex *eps2, const int64_t *offsets,
                            gbmie_complex *an, gbmie_complex *bn, double *eff)
{
    if (!ctx) return GBMIE_ERR_INVALID;
    if (n < 0 || (n > 0 && (!x || !eps || !offsets || !an || !bn)) || ((y == nullptr) != (eps2 == nullptr)))
        return ctx_fail(ctx, GBMIE_ERR_INVALID, "gbmie_coeffs: x, eps, offsets, an, bn are required; "
                                                "y and eps2 go together");
    if (n == 0) return GBMIE_OK;
    cudaSetDevice(ctx->device);
    double2 *dscr = nullptr;
    if (y) {   // coated instances need 5 complex per order of scratch
        GBMIE_TRY(ctx_cuda(ctx, cudaMemcpyAsync(ctx->h_pinned, offsets + n, sizeof(int64_t),
                                                cudaMemcpyDeviceToHost, ctx->stream), "offsets total"));
        GBMIE_TRY(ctx_cuda(ctx, cudaStreamSynchronize(ctx->stream), "offsets total"));
        const int64_t total = ctx->h_pinned[0];
        if (total < 0) return ctx_fail(ctx, GBMIE_ERR_INVALID, "gbmie_coeffs: bad offsets");
        void *p = nullptr;
        GBMIE_TRY(ctx_scratch(ctx, (size_t)(5 * total + 1) * sizeof(double2), &p));
        dscr = (double2 *)p;
    }
    ctx_pre_launch(ctx);
    k_coeffs_api<<<(unsigned)ceil_div64(n, 128), 128, 0, ctx->stream>>>(
        n, x, y, (const double2 *)eps, (const double2 *)mu, (const double2 *)eps2, offsets, (double2 *)an,
        (double2 *)bn, eff, dscr, ctx->d_flags);
    return ctx_check_launch(ctx, "k_coeffs_api");
}
