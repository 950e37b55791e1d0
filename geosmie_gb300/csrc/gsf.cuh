// GSF expansion tables and launch helpers (definitions in gbmie_gsf.cu).
#pragma once
#include "common.cuh"
#include <cuda_fp16.h>

// Buffers of the tensor-core expansion (gbmie_gsf_tc.cu): split A operand
// per table (chunks of 128 rows x 16 nodes), FP64 moment sums and row
// exponents, sized for ntab_max entries.
struct GsfTcBuf {
    uint8_t *a;
    size_t a_off[4];
    long long *c;     // [4][rows_cap][lpad] exact integer sums of the digit products
    int *rexp;        // [4][rows_cap]
    int64_t rows_cap;
    int lpad;
};

struct GsfTables {
    int ng, L, nang;
    void *mem;        // one cudaMalloc block holding everything below
    double *z, *w;    // nodes (ascending) and weights [ng]
    double *P;        // [4][ng][L] generalized spherical functions P1..P4, l < L
    double *frac;     // [ng] interpolation fraction
    int *base;        // [ng] interpolation interval start
    struct {          // mixed precision: the tensor-core expansion
        void *mem;
        __half *bt;   // P1..P4 split into FP16 hi/lo, [4][ntn][nkc] chunks of 64 moments x 16 nodes
        int ntn, nkc, lpad, ntab_max;
        GsfTcBuf buf;
    } tc;
};

// f[k]: row of the k-th input element (F11 F22 F33 F44 F12 F34) within an
// entry; o[r]: output row of coefficient r (alpha1 alpha2 alpha3 alpha4
// beta1 beta2).
struct GsfMap {
    int f[6];
    int o[6];
};

// ng Gauss nodes, the first L <= ng coefficients; with precision
// GBMIE_MIXED also the tensor-core tables and buffers for ntab_max entries
int gsf_prepare(gbmie_ctx *ctx, int ng, int L, int nang, const double *theta_rad, GsfTables *t, int ntab_max,
                int precision);
int gsf_tc_prepare(gbmie_ctx *ctx, GsfTables *t, int ntab_max);
int launch_gsf_expand_tc(gbmie_ctx *ctx, const GsfTables *t, int ntab, const double *F, int64_t entry_stride,
                         int64_t row_stride, GsfMap map, double *coef, int64_t out_stride, int64_t out_row_stride,
                         double *cnorm);
// stream-ordered free of the tables on s (after their last use there)
void gsf_release(GsfTables *t, cudaStream_t s);
// precision: GBMIE_PLAIN_FP64 (FP64 sums) or GBMIE_MIXED (split-FP16
// tensor-core GEMMs, gbmie_gsf_tc.cu)
int launch_gsf_expand(gbmie_ctx *ctx, const GsfTables *t, int ntab, const double *F, int64_t entry_stride,
                      int64_t row_stride, GsfMap map, double *coef, int64_t out_stride, int64_t out_row_stride,
                      double *cnorm, int precision);
