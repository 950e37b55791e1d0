// Internal structures of the table pipeline shared by gbmie_table.cu (plain
// FP64 kernels, plan/run) and gbmie_table_tc.cu (tensor-core kernels).
#pragma once
#include "common.cuh"
#include "gsf.cuh"
#include "mie_device.cuh"
#include <cuda_fp16.h>

// nmax buckets of the plain angular kernel: nmax <= 16, <= 64, <= 256, more
#define GBMIE_TUNE_BUCKETS 4

#define TWO_PI 6.28318530717958647692
#define PI_D 3.14159265358979323846

struct gbmie_table_plan {
    gbmie_ctx *ctx;
    gbmie_table_desc d;
    int n_le;
    int64_t n_units, n_inst, n_entries;
    double *xg;          // [n_le][n_size]
    int64_t *off;        // [n_le * n_size + 1]
    int64_t *unit_base;  // [n_units]
    int64_t pc_total, ab_total;
    int nmax_max;
    size_t o_pc, o_an, o_bn, o_eff, o_w, o_sums, o_reff0, o_pacc, o_pq, o_sraw, o_nlraw, bytes;
    // Partial Mueller sums of the angular kernels, one plane [bin][4][ang]
    // per (unit, slot): a slot is a block's share of a unit's sizes (plain:
    // a size chunk of an nmax bucket; mixed: a tile range and a size half),
    // written with plain stores and summed in a fixed order into pacc, so
    // that a table's bits do not depend on the order in which blocks finish
    size_t o_part;
    int n_slots;     // slots per unit the buffer holds
    int slots_used;  // slots per unit the last launch layout wrote
    int tc_ntr, tc_tpr;   // mixed: tile ranges per (unit, angle block), tiles per range
    // mixed precision (tensor-core) path
    size_t o_cf, o_eexp, o_eunit, o_wf, o_tw, o_rowc, o_hidx, o_pcf, o_dscr, o_hdf, o_rowcd;
    __half *bt;          // angle-function operand of the contraction (built once per key, see ctx angle_ops)
    int bt_entry;        // its context cache entry, or -1 when plan-owned
    double *hcos;        // host copy of cos(theta) (plan creation only)
    int n_pad_total;     // angles padded to whole 128-angle blocks (mixed path)
    int k_pad;           // orders padded to 32
    int *unit_order;     // [n_units] units by decreasing work (plan-owned)
    // split A operand of the tensor-core contraction: per unit, per 64-size
    // tile, per 16-order chunk one 16 KB block in the shared-memory layout
    int ntiles;          // 64-size tiles per unit
    int *tile_cbase;     // [n_le][ntiles + 1] chunk offset of a tile within its unit (plan-owned)
    int64_t *unit_cbase; // [n_units] first chunk of a unit (plan-owned)
    int64_t n_chunks;    // chunks of the whole table
    size_t o_asplit;
    // order-major size groups of the mixed recurrences (TabView grel, grow,
    // gunit: one plan-owned block)
    int ngrp;
    int64_t *grp;
    int64_t pcg_total, cfg_total;
    // tasks of the persistent mixed coefficient kernel: (unit, group) pairs
    // by decreasing largest nmax of the group (plan-owned), and the scratch
    // offset of its task counter
    int2 *ctasks;
    int n_ctasks;
    size_t o_cnext;
    GsfTables gsf;
    int has_gsf;
    int gsf_entry;       // its context cache entry, or -1 when plan-owned
    // CUDA graph of one gbmie_table_run (gbmie_table_run_graph): captured on
    // a private stream, replayed on the context stream
    cudaStream_t cap_stream;
    cudaGraphExec_t gexec;
    gbmie_table_out gout;   // output pointers the graph was captured with
    void *gscratch;         // context scratch block the graph was captured with
    int64_t glaunches;      // kernel launches in one replay
    // launch parameters, defaults until gbmie_table_plan_autotune (or a
    // context cache hit) sets them
    // [GBMIE_TUNE_BUCKETS + 1][n_le] size range [begin, end) of each nmax
    // bucket, then the whole grid (plan-owned)
    int2 *brange;
    int bmaxlen[GBMIE_TUNE_BUCKETS + 1];   // longest range of a bucket over the x grids
    int plain_chunk[GBMIE_TUNE_BUCKETS + 1], plain_threads[GBMIE_TUNE_BUCKETS + 1];
    int plain_split;        // 1: one launch per nmax bucket, 0: one launch over the whole grid
    int coef_block;         // block size of k_tab_coeffs_mixed
    int tc_win;             // accumulation window of k_tab_s12_tc (16-order chunks)
    int tuned;
    // tries of every pipeline wait of k_tab_s12_tc before it gives up and
    // flags a timeout (default GBMIE_WAIT_LIMIT_DEFAULT;
    // gbmie_table_plan_set_wait_limit)
    uint32_t wait_limit;
    // mixed path: D_n recurrence in FP64 from the reference's start
    // (gbmie_table_plan_set_dn_fp64; a measurement variant)
    int dn_fp64;
};
#define GBMIE_WAIT_LIMIT_DEFAULT (1u << 26)

// ---------------------------------------------------------------------------
// block reduction of K doubles (all threads receive the totals)
// ---------------------------------------------------------------------------
template <int K>
__device__ __forceinline__ void block_sum(double (&v)[K])
{
    __shared__ double red[32][K];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
#pragma unroll
    for (int k = 0; k < K; ++k)
        for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_xor_sync(0xffffffffu, v[k], o);
    __syncthreads();
    if (lane == 0)
#pragma unroll
        for (int k = 0; k < K; ++k) red[wid][k] = v[k];
    __syncthreads();
    if (wid == 0) {
#pragma unroll
        for (int k = 0; k < K; ++k) {
            double t = lane < nw ? red[lane][k] : 0.0;
            for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
            if (lane == 0) red[0][k] = t;
        }
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < K; ++k) v[k] = red[0][k];
    __syncthreads();
}

struct TabView {
    int n_lambda, n_rh, n_size, n_bin, n_comp, n_ang, grid_kind, psd_kind, rh0;
    const double *lambda, *grid, *dgrid, *psd_param, *gf_psd, *frac, *rhop, *rhop0, *gf, *rlow, *rup;
    const double *theta;
    const double2 *m;
    const double2 *m_core;   // coated: core index per unit, or NULL
    const double *core_ratio;
    double2 *dscr;           // coated: 5 complex per order of every instance
    const double *xg;
    const int64_t *off, *unit_base;
    double2 *pc, *an, *bn;
    double *eff4, *W, *sums, *reff0, *pacc, *sraw, *nlraw;
    double *part;   // [n_units][n_slots][bin][4][ang] partial Mueller sums
    int n_slots;
    float *Wf;   // FP32 copy of W (mixed path), or NULL
    double *tw;  // trapz weights of the angle grid [n_ang]
    double4 *rowc;      // per size row: sin x, cos x, 1/x
    HomogIndex *hidx;   // per unit: medium constants of the recurrences
    const double2 *pq;
    // pc as FP32 pairs (psi hi, lo, chi hi, lo; mixed path) in order-major
    // groups of 32 sizes: order k of size i = 32 g + l of wavelength block le
    // at pcd[grow[le] + grel[le][g] + 32 (k - 1) + l]; the mixed
    // coefficients (cf) of unit u in the same layout from gunit[u]
    float4 *pcd;
    int ngrp;                   // groups per wavelength block, (n_size + 31) / 32
    const int64_t *grel;        // [n_le][ngrp + 1] group bases within a block
    const int64_t *grow;        // [n_le] block bases of pcd
    const int64_t *gunit;       // [n_units] block bases of cf
    float4 *hdf;        // per unit, FP32 pairs: m, 1/m, x/z, (|z|/x) (mixed path)
    float4 *rowcd;      // per size row, FP32 pairs: (sin x, cos x), (1/x, x) (mixed path)
    // PSD weights, their radius moments and reff0 do not depend on the
    // wavelength when the grid is a radius grid and the PSD is analytic
    // (x = 2 pi r / lambda: the lognormal argument ln(x / x_mode) and the
    // r^-4 law are wavelength-free and the 1/x factor cancels in the
    // normalisation); they are then stored once (lam_shared = 1).
    int lam_shared;
    __device__ __forceinline__ int le(int lam) const { return grid_kind == GBMIE_GRID_X ? 0 : lam; }
    __device__ __forceinline__ int wl(int lam) const { return lam_shared ? 0 : lam; }
    // offset of wavelength lam's block of W ([rh][bin][comp][size])
    __device__ __forceinline__ size_t wlam(int lam) const {
        return (size_t)wl(lam) * n_rh * n_bin * n_comp * n_size;
    }
    __device__ __forceinline__ double radius(int lam, int i) const {
        return grid_kind == GBMIE_GRID_RADIUS ? grid[i] : xg[i] * lambda[lam] / TWO_PI;
    }
};

// Coated units (pymiecoated Mie(m=core, m2=shell, x=core, y=outer)): the
// reference's dispatch (mie_coeffs.py:62-71) and the FP64 coated recurrences
// (:183-251), one thread per instance; the grid is the outer size.  DFD:
// the D_n recurrences in double-float (coated_instance; the mixed path).
template <class Emit, bool DFD = false>
__device__ __forceinline__ void coated_table_instance(const TabView &v, int64_t unit, int64_t c, int64_t o, int nmax,
                                                      double x, Emit &emit, EffSums &es, int *flags)
{
    const int rh = (int)((unit / v.n_comp) % v.n_rh);
    const cplx ms = cx(v.m[unit]), mc = cx(v.m_core[unit]);
    const double ratio = v.core_ratio[rh];
    if (!(ratio >= 0.0 && ratio <= 1.0) || !isfinite(mc.re) || !isfinite(mc.im)) atomicOr(flags, GBMIE_FLAG_INVALID);
    const cplx e1 = mc * mc, e2 = ms * ms;
    const double xc = ratio * x;
    if (xc == x || (e1.re == e2.re && e1.im == e2.im)) homog_instance(x, e1, cx(1.0, 0.0), v.pc + o, nmax, emit, es);
    else if (xc == 0.0) homog_instance(x, e2, cx(1.0, 0.0), v.pc + o, nmax, emit, es);
    else coated_instance<Emit, DFD>(xc, x, e1, e2, v.pc + o, nmax, v.dscr + 5 * c, emit, es);
}

// Mixed path (gbmie_table_tc.cu): the contraction's B operand tables, built
// once per plan.
int build_table_bt(gbmie_ctx *ctx, gbmie_table_plan *p);
int tune_table_mixed(gbmie_ctx *ctx, gbmie_table_plan *p, TabView &v, char *scr, cudaEvent_t e0, cudaEvent_t e1);
// gbmie_table.cu: launch parameters tuned before for this table shape, if any
int table_tune_lookup(gbmie_ctx *ctx, gbmie_table_plan *p);
