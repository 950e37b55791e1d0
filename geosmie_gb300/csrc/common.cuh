// Shared definitions of the gbmie CUDA library (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>
#include <stdarg.h>

#include "../../include/gbmie.h"

// ---------------------------------------------------------------------------
// complex double arithmetic (storage type double2 / gbmie_complex)
// ---------------------------------------------------------------------------
struct cplx {
    double re, im;
};

__host__ __device__ __forceinline__ cplx cx(double r, double i) { return cplx{r, i}; }
__host__ __device__ __forceinline__ cplx cx(double2 v) { return cplx{v.x, v.y}; }
__host__ __device__ __forceinline__ double2 d2(cplx a) { return make_double2(a.re, a.im); }
__host__ __device__ __forceinline__ cplx operator+(cplx a, cplx b) { return cx(a.re + b.re, a.im + b.im); }
__host__ __device__ __forceinline__ cplx operator-(cplx a, cplx b) { return cx(a.re - b.re, a.im - b.im); }
__host__ __device__ __forceinline__ cplx operator-(cplx a) { return cx(-a.re, -a.im); }
__host__ __device__ __forceinline__ cplx operator*(cplx a, cplx b) {
    return cx(a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re);
}
__host__ __device__ __forceinline__ cplx operator*(cplx a, double s) { return cx(a.re * s, a.im * s); }
__host__ __device__ __forceinline__ cplx operator*(double s, cplx a) { return cx(a.re * s, a.im * s); }
__host__ __device__ __forceinline__ cplx operator+(cplx a, double s) { return cx(a.re + s, a.im); }
__host__ __device__ __forceinline__ cplx operator-(cplx a, double s) { return cx(a.re - s, a.im); }
__host__ __device__ __forceinline__ cplx conjg(cplx a) { return cx(a.re, -a.im); }
__host__ __device__ __forceinline__ double abs2(cplx a) { return a.re * a.re + a.im * a.im; }
__host__ __device__ __forceinline__ double cabs(cplx a) { return hypot(a.re, a.im); }
// 1/a = conj(a)/|a|^2.  Magnitudes on this path stay far inside the double
// range (|a|^2 < 1e300), so the unscaled form is used.
__host__ __device__ __forceinline__ cplx cinv(cplx a) {
    double s = 1.0 / abs2(a);
    return cx(a.re * s, -a.im * s);
}
__host__ __device__ __forceinline__ cplx operator/(cplx a, cplx b) {
    double s = 1.0 / abs2(b);
    return cx((a.re * b.re + a.im * b.im) * s, (a.im * b.re - a.re * b.im) * s);
}
__host__ __device__ __forceinline__ cplx operator/(double a, cplx b) {
    double s = a / abs2(b);
    return cx(b.re * s, -b.im * s);
}
// principal square root
__host__ __device__ __forceinline__ cplx csqrt(cplx a) {
    double r = hypot(a.re, a.im);
    if (r == 0.0) return cx(0.0, 0.0);
    double t = sqrt(0.5 * (r + fabs(a.re)));
    if (a.re >= 0.0) return cx(t, a.im / (2.0 * t));
    return cx(fabs(a.im) / (2.0 * t), copysign(t, a.im));
}
__device__ __forceinline__ cplx csin(cplx a) {
    double s, c;
    sincos(a.re, &s, &c);
    return cx(s * cosh(a.im), c * sinh(a.im));
}
__device__ __forceinline__ cplx ccos(cplx a) {
    double s, c;
    sincos(a.re, &s, &c);
    return cx(c * cosh(a.im), -s * sinh(a.im));
}

// Number of partial waves, round(2 + x + 4 x^(1/3)) (pymiecoated
// mie_coeffs.py:99).  rint() rounds half to even like Python's round().
__host__ __device__ __forceinline__ int mie_nmax(double x) {
    return (int)rint(2.0 + x + 4.0 * pow(x, 1.0 / 3.0));
}
// Start of the downward Riccati-Bessel ratio recurrence for psi_n(x), x real.
// nmax + 16 + 4 x^(1/3) reaches full double accuracy for x up to 1e4
// (checked against mpmath at 40 digits).
__host__ __device__ __forceinline__ int psi_start(double x, int nmax) {
    return nmax + 16 + (int)ceil(4.0 * pow(x, 1.0 / 3.0));
}

// device-side error flags (bit set with atomicOr, read at synchronise time)
#define GBMIE_FLAG_INVALID 1
#define GBMIE_FLAG_NMAX 2
#define GBMIE_FLAG_TIMEOUT 4

// ---------------------------------------------------------------------------
// context
// ---------------------------------------------------------------------------
#define GBMIE_TIMER_CAP 8192
struct gbmie_timer_rec {
    const char *name;
    cudaEvent_t start, stop;
};

struct gbmie_ctx {
    int device;
    cudaStream_t stream;
    // a side stream for independent work inside a table run (forked from and
    // joined back into `stream` by the two events)
    cudaStream_t side;
    cudaEvent_t ev_fork, ev_join;
    int timing;               // per-kernel event timing enabled
    int timer_open;           // a start event is recorded and awaits its kernel
    int ntimer;
    gbmie_timer_rec *timers;  // GBMIE_TIMER_CAP records (events created lazily)
    void *scratch;            // grown on demand
    size_t scratch_bytes;
    int *d_flags;             // device error flags
    int *h_flags;             // pinned mirror
    int64_t *h_pinned;        // pinned scratch for small host results
    int64_t launches;
    char err[512];
    // autotuned launch parameters of table plans, keyed by the table's shape
    struct TuneEntry {
        int64_t key[10];
        int32_t params[13];
    } tune_cache[16];
    int n_tune;
    // angle-function operands of mixed table plans (they depend only on the
    // angles and the largest nmax): shared by plans with the same key,
    // reference-counted, freed when evicted unused or with the context
    struct AngleOp {
        void *bt;
        int n_ang, n_pad, k_pad, nmax;
        double *hcos;   // host copy of the key's cos(theta)
        int refs;
    } angle_ops[4];
    void *table_cache;   // GSF tables of table plans (gbmie_table.cu), or NULL
};

// Frees the context's cached table-plan tables (gbmie_table.cu).
void table_cache_release(gbmie_ctx *ctx);

// Angle-function operand for (cos theta on the host, sizes): a cached one
// or a fresh cache entry the caller fills; *entry is its index (release it
// with ctx_angle_op_release).  *fresh = 1 when the caller must build it.
int ctx_angle_op_get(gbmie_ctx *ctx, const double *hcos, int n_ang, int n_pad, int k_pad, int nmax, size_t bytes,
                     void **bt, int *entry, int *fresh);
void ctx_angle_op_release(gbmie_ctx *ctx, int entry);

int ctx_fail(gbmie_ctx *ctx, int status, const char *fmt, ...);
int ctx_cuda(gbmie_ctx *ctx, cudaError_t e, const char *what);
// Grow the context scratch to at least `bytes` (synchronises the stream when
// it must reallocate).  Returns GBMIE_OK or an error status.
int ctx_scratch(gbmie_ctx *ctx, size_t bytes, void **ptr);
int ctx_check_launch(gbmie_ctx *ctx, const char *what);
// Call right before a kernel launch: records the start event when timing is
// enabled (ctx_check_launch records the matching stop event).
void ctx_pre_launch(gbmie_ctx *ctx);

#define GBMIE_TRY(expr)                         \
    do {                                        \
        int _st = (expr);                       \
        if (_st != GBMIE_OK) return _st;        \
    } while (0)

static inline int64_t ceil_div64(int64_t a, int64_t b) { return (a + b - 1) / b; }
static inline size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

// ---------------------------------------------------------------------------
// launch helpers shared between translation units
// ---------------------------------------------------------------------------
// CSR layout: offsets[i+1] - offsets[i] = nmax(size[i]) + add_per_row; the
// total is returned on the host (synchronous) when total_host != NULL.
int launch_layout(gbmie_ctx *ctx, int64_t n, const double *size, int64_t add_per_row, int64_t *offsets,
                  int64_t *total_host);
// (p, q) = (pi~ + tau~, pi~ - tau~) at orders 1..nmax, [n-1][angle].
int launch_pq_table(gbmie_ctx *ctx, int nang, const double *cost, int nmax, double2 *pq);
