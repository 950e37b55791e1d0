// Tensor-core GSF expansion (mixed precision): the moment sums of
// gsf/spher_expan.f:269-358 (SPHER_EXPAN)
//   alpha_l(row) = sum_g F'_g(row) P_t(l, g),   F' = F(acos z_g) w_g
// for every table entry and element combination row as GEMMs on tcgen05:
//   A_t [rows x nodes]  node values of the rows that use table t
//                        (t = 0: F11, F44 with P1; 1: F22 + F33 with P2;
//                         2: F22 - F33 with P3; 3: F12, F34 with P4),
//   B_t [moments x nodes] the generalised spherical functions P1..P4.
//
// Numerics: fixed-point digits, exact tensor-core sums.  Every A row is
// scaled by its own power of two (|F' s| < 2^7) and P by 2^7, and both are
// written as GT_ND signed base-2^8 digits, v = sum_k d_k 2^(-8k), |d_k| <= 128
// (rounded digits; FP16 holds them exactly).  Digit products are integers
// below 2^14; the digit-pair classes c = i + j each get their own TMEM
// accumulator, and a class sum over a window of GT_WIN chunks of 16 nodes
// stays below 2^24 (at most GT_ND products per node): the FP32 tensor-core
// accumulation is exact, whatever its alignment and truncation.  The class
// sums are combined as integers (int64) and summed over the windows, so the
// only error is the digit truncation, ~2^-31 of the row's largest value and
// of |P| <= 1.  (A hi/lo FP16 split, 22 bits, gave 1.8e-6 of alpha1(0) at
// l ~ 40 for Henyey-Greenstein g = 0.85: the (l + 1/2) factor amplifies the
// rounding of the raw sums.)
//
// k_gsf_tc_tables  B_t digit tables (plan time)
// k_gsf_tc_rows    A_t: interpolation to the nodes (LINTERPOL, :593-623),
//                  weights, combinations, per-row scale, digits
// k_gsf_tc_gemm    the GEMMs, one CTA per (table, 128-row tile, 64-moment
//                  tile): warps 0-3 read the window sums back from TMEM,
//                  warp 4 (one thread) issues the bulk copies and the MMAs
// k_gsf_tc_finish  (l + 1/2) factors, alpha2/alpha3 recombination (:335-345),
//                  normalisation by 1/alpha1(0) (main program :95-106)
#include "common.cuh"
#include "gsf.cuh"
#include "tc.cuh"

#define GT_ND 4                            // digits per operand
#define GT_KC 16                           // nodes per K chunk
#define GT_NT 64                           // moments per N tile
#define GT_MT 128                          // rows per M tile
#define GT_WIN 16                          // chunks per exact accumulation window
#define GT_A_MAT (GT_KC * GT_MT * 2)       // one digit plane of an A chunk: 4 KB
#define GT_B_MAT (GT_KC * GT_NT * 2)       // one digit plane of a B chunk: 2 KB
#define GT_A_CHUNK (GT_ND * GT_A_MAT)
#define GT_B_CHUNK (GT_ND * GT_B_MAT)
#define GT_STAGE (GT_A_CHUNK + GT_B_CHUNK) // 24 KB
#define GT_NS 4                            // load stages
#define GT_SMEM (116 * 1024)               // > half an SM: one CTA per SM owns all 512 TMEM columns
#define GT_THREADS 160
#define GT_TMEM_COLS (2 * GT_ND * GT_NT)   // two windows in flight
#define GT_SHIFT (8 * (GT_ND - 1))         // int64 sum = sum_c class_c 2^(8 (ND - 1 - c))

static_assert(GT_NS * GT_STAGE <= GT_SMEM, "stages exceed the shared-memory request");
static_assert(GT_TMEM_COLS <= 512, "TMEM columns");
static_assert(GT_ND * GT_WIN * GT_KC * 128 * 128 <= (1 << 24), "window class sums must stay exact in FP32");

__constant__ int c_gt_rows_per_entry[4] = {2, 1, 1, 2};

// byte offset of (row r, node k) inside one K-major no-swizzle matrix of R
// rows and 16 nodes: core matrices of 8 rows x 8 nodes, K groups R/8 apart
__device__ __forceinline__ uint32_t gt_off(int r, int k, int R)
{
    return ((k >> 3) * (R >> 3) + (r >> 3)) * 128 + (r & 7) * 16 + (k & 7) * 2;
}

// the six combination rows (F11, F44, F22 + F33, F22 - F33, F12, F34) of
// entry Fe at node g, interpolated and weighted
__device__ __forceinline__ void gt_node_values(const double *Fe, int64_t row_stride, const GsfMap &map, int g,
                                               const int *base, const double *frac, const double *w, double *f)
{
    const int b = base[g];
    const double fr = frac[g], wg = w[g];
    double v[6];
#pragma unroll
    for (int el = 0; el < 6; ++el) {
        const double *row = Fe + (size_t)map.f[el] * row_stride;
        const double y0 = row[b], y1 = row[b + 1];
        v[el] = (y0 + (y1 - y0) * fr) * wg;
    }
    f[0] = v[0];
    f[1] = v[3];
    f[2] = v[1] + v[2];
    f[3] = v[1] - v[2];
    f[4] = v[4];
    f[5] = v[5];
}

// GT_ND balanced base-2^8 digits of n = rint(v 2^(8 (GT_ND - 1))), |v| < 2^7:
// v ~ sum_k d_k 2^(-8k), d_k in [-128, 128]
__device__ __forceinline__ void gt_digits_int(long long n, __half *d)
{
#pragma unroll
    for (int k = GT_ND - 1; k > 0; --k) {
        const int r = (int)(((n + 128) & 255) - 128);
        d[k] = __int2half_rn(r);
        n = (n - r) >> 8;
    }
    d[0] = __int2half_rn((int)n);
}

__global__ void k_gsf_tc_tables(int ng, int L, int ntn, int nkc, const double *__restrict__ P, __half *__restrict__ bt)
{
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t per_t = (int64_t)ntn * GT_NT * nkc * GT_KC;
    if (idx >= 4 * per_t) return;
    const int t = (int)(idx / per_t);
    const int64_t rem = idx % per_t;
    const int l = (int)(rem / ((int64_t)nkc * GT_KC)), g = (int)(rem % ((int64_t)nkc * GT_KC));
    const double v = (l < L && g < ng) ? P[((size_t)t * ng + g) * L + l] : 0.0;   // |P| <= 1
    __half d[GT_ND];
    gt_digits_int(__double2ll_rn(ldexp(v, 7 + GT_SHIFT)), d);
    uint8_t *chunk = (uint8_t *)bt + ((size_t)(t * ntn + l / GT_NT) * nkc + g / GT_KC) * GT_B_CHUNK;
    const uint32_t o = gt_off(l % GT_NT, g % GT_KC, GT_NT);
#pragma unroll
    for (int k = 0; k < GT_ND; ++k) *(__half *)(chunk + k * GT_B_MAT + o) = d[k];
}

// One block per entry: per-row exponents (first pass over the nodes), then
// the digit rows of all six combinations (second pass).
__global__ void __launch_bounds__(128) k_gsf_tc_rows(int ntab, int ng, int nkc, const double *__restrict__ F,
                                                     int64_t entry_stride, int64_t row_stride, GsfMap map,
                                                     const double *__restrict__ w, const int *__restrict__ base,
                                                     const double *__restrict__ frac, GsfTcBuf buf)
{
    __shared__ int s_exp[6];
    const int e = blockIdx.x;
    if (e >= ntab) return;
    const double *Fe = F + (size_t)e * entry_stride;
    if (threadIdx.x < 6) s_exp[threadIdx.x] = -1100;
    __syncthreads();
    int em[6];
#pragma unroll
    for (int c = 0; c < 6; ++c) em[c] = -1100;
    // with at most one node per thread its values are kept for the digit
    // pass below (the same thread takes the same node there)
    const bool keep = ng <= (int)blockDim.x;
    double fk[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    for (int g = threadIdx.x; g < ng; g += blockDim.x) {
        double f[6];
        gt_node_values(Fe, row_stride, map, g, base, frac, w, f);
#pragma unroll
        for (int c = 0; c < 6; ++c) {
            if (f[c] != 0.0) em[c] = max(em[c], ilogb(f[c]));
            fk[c] = f[c];
        }
    }
#pragma unroll
    for (int c = 0; c < 6; ++c) {
        for (int o = 16; o > 0; o >>= 1) em[c] = max(em[c], __shfl_xor_sync(0xffffffffu, em[c], o));
        if ((threadIdx.x & 31) == 0) atomicMax(&s_exp[c], em[c]);
    }
    __syncthreads();
    const int tab_of[6] = {0, 0, 1, 2, 3, 3}, sub_of[6] = {0, 1, 0, 0, 0, 1};
    double sc[6];
    uint8_t *arow[6];
    int r[6];
#pragma unroll
    for (int c = 0; c < 6; ++c) {
        const int t = tab_of[c];
        const int64_t row = (int64_t)e * c_gt_rows_per_entry[t] + sub_of[c];
        const int ex = s_exp[c];
        if (threadIdx.x == 0) buf.rexp[(size_t)t * buf.rows_cap + row] = ex;
        // |value 2^(6 - ex)| < 2^7, times 2^(8 (GT_ND - 1)) for the integer digits
        sc[c] = ex > -1100 ? ldexp(1.0, 6 - ex + GT_SHIFT) : 0.0;
        arow[c] = buf.a + buf.a_off[t] + (size_t)(row / GT_MT) * nkc * GT_A_CHUNK;
        r[c] = (int)(row % GT_MT);
    }
    for (int g = threadIdx.x; g < nkc * GT_KC; g += blockDim.x) {
        double f[6] = {0, 0, 0, 0, 0, 0};
        if (g < ng) {
            if (keep) {
#pragma unroll
                for (int c = 0; c < 6; ++c) f[c] = fk[c];
            } else {
                gt_node_values(Fe, row_stride, map, g, base, frac, w, f);
            }
        }
        const size_t cofs = (size_t)(g / GT_KC) * GT_A_CHUNK;
#pragma unroll
        for (int c = 0; c < 6; ++c) {
            __half d[GT_ND];
            gt_digits_int(__double2ll_rn(f[c] * sc[c]), d);
            uint8_t *chunk = arow[c] + cofs;
            const uint32_t o = gt_off(r[c], g % GT_KC, GT_MT);
#pragma unroll
            for (int k = 0; k < GT_ND; ++k) *(__half *)(chunk + k * GT_A_MAT + o) = d[k];
        }
    }
}

// rows of A_t beyond the entries' rows stay zero (set once per buffer)
__global__ void k_gsf_tc_zero(size_t n, uint4 *__restrict__ p)
{
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) p[i] = make_uint4(0u, 0u, 0u, 0u);
}

// Barriers: full[s] (bulk copies of stage s landed), empty[s] (MMAs reading
// stage s done), accf[b] (window in TMEM buffer b complete), acce[b] (buffer
// b read back by the four epilogue warps).  Chunk kc uses stage kc % GT_NS
// (phase kc / GT_NS); window w uses buffer w & 1 (phase w >> 1).  Every wait
// is bounded and also ends when another role raised s_abort.  nsplit > 1:
// the K chunks of an output tile are split over nsplit blocks (tables with
// fewer tiles than SMs), each adding its exact int64 sums into the zeroed
// output with integer atomics, so the result does not depend on the split.
__global__ void __launch_bounds__(GT_THREADS, 1) k_gsf_tc_gemm(int ntab, int L, int ntn, int nkc, int nsplit,
                                                               const __half *__restrict__ bt, GsfTcBuf buf,
                                                               int *flags)
{
    extern __shared__ __align__(1024) uint8_t smem[];
    __shared__ uint64_t full[GT_NS], empty[GT_NS], accf[2], acce[2], drain;
    __shared__ uint32_t s_tmem;
    __shared__ int s_abort_i;
    volatile int *s_abort = &s_abort_i;
    // block -> (table, M tile, N tile, K split)
    const int split = blockIdx.x % nsplit;
    int blk = blockIdx.x / nsplit, t = 0, nmt = 0;
    for (t = 0; t < 4; ++t) {
        nmt = (ntab * c_gt_rows_per_entry[t] + GT_MT - 1) / GT_MT;
        if (blk < nmt * ntn) break;
        blk -= nmt * ntn;
    }
    if (t == 4) return;
    const int mt = blk / ntn, nt = blk % ntn;
    const int rows = ntab * c_gt_rows_per_entry[t];
    // this block's chunks: [k_lo, k_lo + nk) of the tile's nkc
    const int cps = (nkc + nsplit - 1) / nsplit;
    const int k_lo = min(nkc, split * cps), nk = min(nkc, k_lo + cps) - k_lo;
    const uint8_t *ga = buf.a + buf.a_off[t] + ((size_t)mt * nkc + k_lo) * GT_A_CHUNK;
    const uint8_t *gb = (const uint8_t *)bt + ((size_t)(t * ntn + nt) * nkc + k_lo) * GT_B_CHUNK;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int nwin = (nk + GT_WIN - 1) / GT_WIN;
    if (warp == 0) tmem_alloc(&s_tmem, GT_TMEM_COLS);
    if (tid == 0) {
        for (int i = 0; i < GT_NS; ++i) {
            mbar_init(full + i, 1);
            mbar_init(empty + i, 1);
        }
        for (int i = 0; i < 2; ++i) {
            mbar_init(accf + i, 1);
            mbar_init(acce + i, 4);
        }
        mbar_init(&drain, 1);
        fence_mbar_init();
        s_abort_i = 0;
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = s_tmem;
    if (warp == 4) {
        // ---------------- producer + MMA issuer (one thread) ----------------
        if (lane == 0) {
            const uint32_t idesc = idesc_f16_f32(GT_MT, GT_NT);
            int last_ld = -1;
            auto load = [&](int kc) {
                uint8_t *st = smem + (kc % GT_NS) * GT_STAGE;
                mbar_arrive_expect_tx(full + kc % GT_NS, GT_STAGE);
                bulk_g2s(st, ga + (size_t)kc * GT_A_CHUNK, GT_A_CHUNK, full + kc % GT_NS);
                bulk_g2s(st + GT_A_CHUNK, gb + (size_t)kc * GT_B_CHUNK, GT_B_CHUNK, full + kc % GT_NS);
                last_ld = kc;
            };
            for (int kc = 0; kc < nk && kc < GT_NS; ++kc) load(kc);
            bool ok = true;
            for (int w = 0; w < nwin && ok; ++w) {
                const int b = w & 1;
                if (w >= 2 && !mbar_wait_or_abort(acce + b, ((w - 2) >> 1) & 1u, s_abort)) {
                    ok = false;
                    break;
                }
                tc_fence_after();
                const int k0 = w * GT_WIN, k1 = min(nk, k0 + GT_WIN);
                for (int kc = k0; kc < k1; ++kc) {
                    if (!mbar_wait_or_abort(full + kc % GT_NS, (kc / GT_NS) & 1u, s_abort)) {
                        ok = false;
                        break;
                    }
                    tc_fence_after();
                    const uint32_t sa = smem_u32(smem + (kc % GT_NS) * GT_STAGE), sb = sa + GT_A_CHUNK;
#pragma unroll
                    for (int c = 0; c < GT_ND; ++c) {
                        const uint32_t d = tmem + b * (GT_ND * GT_NT) + c * GT_NT;
#pragma unroll
                        for (int i = 0; i <= c; ++i) {
                            const uint64_t ad = smem_desc(sa + i * GT_A_MAT, (GT_MT / 8) * 128, 128);
                            const uint64_t bd = smem_desc(sb + (c - i) * GT_B_MAT, (GT_NT / 8) * 128, 128);
                            mma_f16(d, ad, bd, idesc, (kc > k0 || i > 0) ? 1u : 0u);
                        }
                    }
                    mma_commit(empty + kc % GT_NS);
                    // refill the stage of the previous chunk (its MMAs were issued one step ago)
                    const int kp = kc - 1;
                    if (kp >= 0 && kp + GT_NS < nk) {
                        if (!mbar_wait_or_abort(empty + kp % GT_NS, (kp / GT_NS) & 1u, s_abort)) {
                            ok = false;
                            break;
                        }
                        load(kp + GT_NS);
                    }
                }
                if (ok) mma_commit(accf + b);
            }
            if (!ok) {
                *s_abort = 1;
                atomicOr(flags, GBMIE_FLAG_TIMEOUT);
                // copies and MMAs still in flight finish before the block ends
                for (int kk = last_ld - GT_NS + 1; kk <= last_ld; ++kk)
                    if (kk >= 0) mbar_wait(full + kk % GT_NS, (kk / GT_NS) & 1u, 1u << 20);
                mma_commit(&drain);
                mbar_wait(&drain, 0, 1u << 20);
            }
        }
        __syncwarp();
    } else {
        // ---------------- epilogue: window class sums -> int64 ----------------
        long long sum[GT_NT];
#pragma unroll
        for (int j = 0; j < GT_NT; ++j) sum[j] = 0;
        for (int w = 0; w < nwin; ++w) {
            const int b = w & 1;
            if (!mbar_wait_or_abort(accf + b, (w >> 1) & 1u, s_abort, 64)) {
                *s_abort = 1;
                atomicOr(flags, GBMIE_FLAG_TIMEOUT);
                break;
            }
            tc_fence_after();
#pragma unroll 1
            for (int c = 0; c < GT_ND; ++c)
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    float v[32];
                    tmem_ld32(tmem + ((uint32_t)(32 * warp) << 16) + b * (GT_ND * GT_NT) + c * GT_NT + 32 * h, v);
#pragma unroll
                    for (int j = 0; j < 32; ++j)   // exact integers below 2^24
                        sum[32 * h + j] += (long long)__float2int_rn(v[j]) * (1ll << (8 * (GT_ND - 1 - c)));
                }
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(acce + b);
        }
        __syncwarp();
        const int row = mt * GT_MT + 32 * warp + lane;
        if (!*s_abort && row < rows) {
            long long *c = buf.c + ((size_t)t * buf.rows_cap + row) * buf.lpad + nt * GT_NT;
            if (nsplit == 1) {
#pragma unroll
                for (int j = 0; j < GT_NT; ++j)
                    if (nt * GT_NT + j < L) c[j] = sum[j];
            } else {   // exact: two's complement sums in any order
#pragma unroll
                for (int j = 0; j < GT_NT; ++j)
                    if (nt * GT_NT + j < L && nk > 0)
                        atomicAdd((unsigned long long *)(c + j), (unsigned long long)sum[j]);
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 0) tmem_dealloc(tmem, GT_TMEM_COLS);
}

// One block per entry, threads over l: the SPHER_EXPAN tail and the
// normalisation of the main program.
__global__ void k_gsf_tc_finish(int ntab, int L, GsfTcBuf buf, GsfMap map, double *__restrict__ coef,
                                int64_t out_stride, int64_t out_row_stride, double *__restrict__ cnorm)
{
    __shared__ double s_norm;
    const int e = blockIdx.x;
    if (e >= ntab) return;
    const int tab_of[6] = {0, 0, 1, 2, 3, 3}, sub_of[6] = {0, 1, 0, 0, 0, 1};
    for (int l0 = 0; l0 < L; l0 += blockDim.x) {
        const int l = l0 + threadIdx.x;
        double al[6] = {0, 0, 0, 0, 0, 0};
        if (l < L)
#pragma unroll
            for (int c = 0; c < 6; ++c) {
                const int t = tab_of[c];
                const int64_t row = (int64_t)e * c_gt_rows_per_entry[t] + sub_of[c];
                const int ex = buf.rexp[(size_t)t * buf.rows_cap + row];
                if (ex > -1100)
                    al[c] = ldexp((double)buf.c[((size_t)t * buf.rows_cap + row) * buf.lpad + l], ex - 13 - GT_SHIFT);
            }
        const double cl = (double)l + 0.5;
        const double a2 = al[2] * cl * 0.5, a3 = al[3] * cl * 0.5;
        const double v[6] = {al[0] * cl, a2 + a3, a2 - a3, al[1] * cl, al[4] * cl, al[5] * cl};
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

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
int gsf_tc_prepare(gbmie_ctx *ctx, GsfTables *t, int ntab_max)
{
    t->tc.ntn = (t->L + GT_NT - 1) / GT_NT;
    t->tc.nkc = (t->ng + GT_KC - 1) / GT_KC;
    t->tc.lpad = t->tc.ntn * GT_NT;
    t->tc.ntab_max = ntab_max;
    const int ntn = t->tc.ntn, nkc = t->tc.nkc;
    GsfTcBuf &b = t->tc.buf;
    b.rows_cap = 2 * (int64_t)ntab_max;
    b.lpad = t->tc.lpad;
    size_t a_bytes = 0;
    for (int k = 0; k < 4; ++k) {
        const int rpe = k == 0 || k == 3 ? 2 : 1;
        const int64_t nmt = ((int64_t)ntab_max * rpe + GT_MT - 1) / GT_MT;
        b.a_off[k] = a_bytes;
        a_bytes += (size_t)nmt * nkc * GT_A_CHUNK;
    }
    const size_t bt_bytes = (size_t)4 * ntn * nkc * GT_B_CHUNK;
    const size_t c_bytes = sizeof(long long) * 4 * (size_t)b.rows_cap * b.lpad;
    const size_t e_bytes = sizeof(int) * 4 * (size_t)b.rows_cap;
    const size_t total = align_up(bt_bytes, 256) + align_up(a_bytes, 256) + align_up(c_bytes, 256) + e_bytes;
    GBMIE_TRY(ctx_cuda(ctx, cudaMallocAsync(&t->tc.mem, total, ctx->stream), "gsf tensor-core buffers"));
    char *p = (char *)t->tc.mem;
    t->tc.bt = (__half *)p;
    p += align_up(bt_bytes, 256);
    b.a = (uint8_t *)p;
    p += align_up(a_bytes, 256);
    b.c = (long long *)p;
    p += align_up(c_bytes, 256);
    b.rexp = (int *)p;
    if (nkc > (1 << 16)) return ctx_fail(ctx, GBMIE_ERR_INVALID, "gsf: more than 2^20 Gauss nodes");
    const int64_t nb = 4 * (int64_t)ntn * GT_NT * nkc * GT_KC;
    ctx_pre_launch(ctx);
    k_gsf_tc_tables<<<(unsigned)ceil_div64(nb, 256), 256, 0, ctx->stream>>>(t->ng, t->L, ntn, nkc, t->P, t->tc.bt);
    GBMIE_TRY(ctx_check_launch(ctx, "k_gsf_tc_tables"));
    const size_t n16 = a_bytes / 16;
    ctx_pre_launch(ctx);
    k_gsf_tc_zero<<<(unsigned)ceil_div64((int64_t)n16, 256), 256, 0, ctx->stream>>>(n16, (uint4 *)b.a);
    return ctx_check_launch(ctx, "k_gsf_tc_zero");
}

int launch_gsf_expand_tc(gbmie_ctx *ctx, const GsfTables *t, int ntab, const double *F, int64_t entry_stride,
                         int64_t row_stride, GsfMap map, double *coef, int64_t out_stride, int64_t out_row_stride,
                         double *cnorm)
{
    if (ntab > t->tc.ntab_max) return ctx_fail(ctx, GBMIE_ERR_INVALID, "gsf: more entries than planned");
    const int ntn = t->tc.ntn, nkc = t->tc.nkc;
    cudaStream_t st = ctx->stream;
    ctx_pre_launch(ctx);
    k_gsf_tc_rows<<<ntab, t->ng <= 64 ? 64 : 128, 0, st>>>(ntab, t->ng, nkc, F, entry_stride, row_stride, map, t->w, t->base, t->frac,
                                         t->tc.buf);
    GBMIE_TRY(ctx_check_launch(ctx, "k_gsf_tc_rows"));
    int nblk = 0;
    for (int k = 0; k < 4; ++k) {
        const int rpe = k == 0 || k == 3 ? 2 : 1;
        nblk += (int)(((int64_t)ntab * rpe + GT_MT - 1) / GT_MT) * ntn;
    }
    const size_t smem = GT_SMEM;
    cudaError_t e = cudaFuncSetAttribute(k_gsf_tc_gemm, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    GBMIE_TRY(ctx_cuda(ctx, e, "k_gsf_tc_gemm smem attribute"));
    // K split: tables with fewer output tiles than SMs (one block per SM)
    int nsm = 0;
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, ctx->device);
    int nsplit = nblk > 0 && nblk < nsm ? nsm / nblk : 1;
    nsplit = max(1, min(nsplit, nkc / 4));   // at least 4 chunks per split
    if (nsplit > 1) {
        const size_t c_bytes = sizeof(long long) * 4 * (size_t)t->tc.buf.rows_cap * t->tc.buf.lpad;
        GBMIE_TRY(ctx_cuda(ctx, cudaMemsetAsync(t->tc.buf.c, 0, c_bytes, st), "gsf split sums"));
    }
    ctx_pre_launch(ctx);
    k_gsf_tc_gemm<<<nblk * nsplit, GT_THREADS, smem, st>>>(ntab, t->L, ntn, nkc, nsplit, t->tc.bt, t->tc.buf,
                                                          ctx->d_flags);
    GBMIE_TRY(ctx_check_launch(ctx, "k_gsf_tc_gemm"));
    const int thr = t->L >= 256 ? 256 : ((t->L + 31) / 32) * 32;
    ctx_pre_launch(ctx);
    k_gsf_tc_finish<<<ntab, thr, 0, st>>>(ntab, t->L, t->tc.buf, map, coef, out_stride, out_row_stride, cnorm);
    return ctx_check_launch(ctx, "k_gsf_tc_finish");
}
