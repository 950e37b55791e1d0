// GSF expansion tables and launch helpers (definitions in gbmie_gsf.cu).
#pragma once
#include "common.cuh"

struct GsfTables {
    int ng, L, nang;
    void *mem;        // one cudaMalloc block holding everything below
    double *z, *w;    // nodes (ascending) and weights [ng]
    double *P;        // [4][ng][L] generalized spherical functions P1..P4, l < L
    float *Ph, *Pl;   // P split into FP32 hi + lo (P = Ph + Pl to ~2^-48)
    double *frac;     // [ng] interpolation fraction
    int *base;        // [ng] interpolation interval start
};

// f[k]: row of the k-th input element (F11 F22 F33 F44 F12 F34) within an
// entry; o[r]: output row of coefficient r (alpha1 alpha2 alpha3 alpha4
// beta1 beta2).
struct GsfMap {
    int f[6];
    int o[6];
};

// ng Gauss nodes, the first L <= ng coefficients
int gsf_prepare(gbmie_ctx *ctx, int ng, int L, int nang, const double *theta_rad, GsfTables *t);
void gsf_release(GsfTables *t);
// precision: GBMIE_PLAIN_FP64 (FP64 sums) or GBMIE_MIXED (split-FP32
// products, Kahan-compensated FP32 sums)
int launch_gsf_expand(gbmie_ctx *ctx, const GsfTables *t, int ntab, const double *F, int64_t entry_stride,
                      int64_t row_stride, GsfMap map, double *coef, int64_t out_stride, int64_t out_row_stride,
                      double *cnorm, int precision);
