// Mixed-precision table path: tensor-core (tcgen05) angular contraction with
// the Mueller elements and the size-distribution integration fused into the
// epilogue.
//
// The recurrences stay FP64 (k_tab_coeffs_mixed: D_n, psi/chi rows, a_n,
// b_n and the efficiency sums).  The coefficients leave it as FP32
//   c_n = a_n + b_n,  d_n = a_n - b_n   (float4 per order)
// with a per-instance exponent e_i = floor(log2 max |c|, |d|).  The two
// contractions
//   S+ = S1 + S2 = sum_n c_n (pi~_n + tau~_n),   S- = S1 - S2 = sum_n d_n (pi~_n - tau~_n)
// are GEMMs [instances x orders] x [orders x angles]: rows are (instance,
// Re/Im) pairs, 64 instances = M 128 per tile; columns are angles in blocks of
// up to 192 (N).  Each operand is split into FP16 hi + lo halves (values
// scaled by 2^(13 - e_i) so the row maximum sits just below 2^14), and
//   C P ~ C_hi P_hi + C_hi P_lo + C_lo P_hi
// is accumulated in FP32 in tensor memory: three tcgen05.mma per product and
// K step of 16 orders, six per step for S+ and S-.  The epilogue reads S+/S-
// rows from TMEM (tcgen05.ld), pairs Re/Im lanes, forms s11, s12, s33, s34
// and reduces them over the tile's 64 sizes with the PSD weights of every
// bin (the weights absorb 2^(2(e_i - E)) with E the unit's largest
// exponent), accumulating per unit in FP64.  Per-size phase matrices never
// reach global memory.
#include "common.cuh"
#include "mie_device.cuh"
#include "table_internal.cuh"
#include "tc.cuh"

#define TC_INST 64        // sizes per tile (M = 128 rows: Re, Im)
#define TC_KC 32          // orders per K chunk (two MMA K steps)
#define TC_NBLK 192       // angles per column block (N)
#define TC_THREADS 256
#define TC_ROUNDS (TC_NBLK / 64)
#define SHIFT_BITS 13

// ---------------------------------------------------------------------------
// FP64 coefficients -> FP32 (c, d) + exponent
// ---------------------------------------------------------------------------
// Emits FP32 (c, d) and accumulates the efficiency sums from them: with
// c = a + b and d = a - b,
//   Re a + Re b = Re c,   |a|^2 + |b|^2 = (|c|^2 + |d|^2) / 2,
//   Re(a_n a*_{n+1} + b_n b*_{n+1}) = (Re(c_n c*_{n+1}) + Re(d_n d*_{n+1})) / 2,
// while Re(a_n b*_n) is formed from the FP64 a_n, b_n ((|c|^2 - |d|^2) / 4
// would cancel for small particles, where |a_1| >> |b_1|).
// qext, qsca and the asymmetry sum are accumulated in FP32 with Kahan
// compensation (the accumulated rounding then stays at the FP32 unit
// roundoff whatever nmax is, and the terms do not cancel in the PSD-weighted
// bulk values); the
// back-scattering sum sum (2n+1)(-1)^n (a_n - b_n) cancels strongly for
// large particles and stays FP64 from the FP64 d_n.
__device__ __forceinline__ void kahan(float &sum, float &comp, float v)
{
    const float y = v - comp;
    const float t = sum + y;
    comp = (t - sum) - y;
    sum = t;
}

struct EmitMixed {
    float4 *cf;
    float amax;
    float ext, sca, asy;
    float ext_c, sca_c, asy_c;   // Kahan compensations
    double qbr, qbi;
    float4 prev;         // (c, d) of order n+1 (zero above nmax)
    float inv_n1;        // 1/(n+1)
    __device__ __forceinline__ void operator()(int k, cplx a, cplx b) {
        const double dr = a.re - b.re, di = a.im - b.im;
        const float4 q = make_float4((float)(a.re + b.re), (float)(a.im + b.im), (float)dr, (float)di);
        cf[k - 1] = q;
        amax = fmaxf(amax, fmaxf(fmaxf(fabsf(q.x), fabsf(q.y)), fmaxf(fabsf(q.z), fabsf(q.w))));
        const float fk = (float)k;
        const float cn = 2.f * fk + 1.f;
        const float inv_n = 1.f / fk;
        const float c2 = q.x * q.x + q.y * q.y, d2v = q.z * q.z + q.w * q.w;
        kahan(ext, ext_c, cn * q.x);
        kahan(sca, sca_c, cn * 0.5f * (c2 + d2v));
        // Re(a b*) from FP64 a, b: (|c|^2 - |d|^2) / 4 cancels when |a| >> |b|
        const float rab = (float)fma(a.re, b.re, a.im * b.im);
        kahan(asy, asy_c, ((fk + 1.f) - inv_n1) * 0.5f * (q.x * prev.x + q.y * prev.y + q.z * prev.z + q.w * prev.w) +
                              (inv_n + inv_n1) * rab);
        const double sg = (double)((k & 1) ? -(2 * k + 1) : (2 * k + 1));   // (2k+1)(-1)^k
        qbr = fma(sg, dr, qbr);
        qbi = fma(sg, di, qbi);
        prev = q;
        inv_n1 = inv_n;
    }
};

// The homogeneous recurrences without the FP64 efficiency sums (they are
// accumulated by EmitMixed): same D_n, psi/chi and a_n/b_n arithmetic as
// homog_instance.
struct NoSums {
    static constexpr bool needs_inv_n = false;
    __device__ __forceinline__ void init() {}
    __device__ __forceinline__ void add_rcp(int, cplx, cplx, double, double) {}
};

__global__ void __launch_bounds__(128) k_tab_coeffs_mixed(TabView v, int64_t n_inst, float4 *__restrict__ cf,
                                                          int *__restrict__ eexp, int *__restrict__ eunit,
                                                          int *flags)
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
    const HomogIndex h = v.hidx[unit];
    EmitMixed emit;
    emit.cf = cf + c;
    emit.amax = 0.f;
    emit.ext = emit.sca = emit.asy = 0.f;
    emit.ext_c = emit.sca_c = emit.asy_c = 0.f;
    emit.qbr = emit.qbi = 0.0;
    emit.prev = make_float4(0.f, 0.f, 0.f, 0.f);
    emit.inv_n1 = 1.f / (float)(nmax + 1);
    NoSums ns;
    homog_core(x, rc.z, rc.x, rc.y, h, v.pc + o, nmax, emit, ns);
    const double iy2 = rc.z * rc.z;   // 1 / x^2
    const double qext = 2.0 * (double)emit.ext * iy2;
    const double qsca = 2.0 * (double)emit.sca * iy2;
    double *o4 = v.eff4 + t * 4;
    o4[0] = qext;
    o4[1] = qsca;
    o4[2] = (emit.qbr * emit.qbr + emit.qbi * emit.qbi) * iy2;
    o4[3] = 2.0 * (double)emit.asy / (double)emit.sca;   // 4/x^2 asy / qsca
    const int ex = emit.amax > 0.f ? ilogbf(emit.amax) : -1000;
    eexp[t] = ex;
    atomicMax(eunit + unit, ex);
}

__global__ void k_fill_int(int n, int *p, int val)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) p[i] = val;
}

// ---------------------------------------------------------------------------
// B operands: (p, q) = (pi~ + tau~, pi~ - tau~) split into FP16 hi/lo, in the
// no-swizzle K-major canonical layout [k/8][angle/8][8 angles][8 orders].
// Matrices 0..3: P_hi, P_lo, Q_hi, Q_lo, each n_pad x k_pad halves.
// ---------------------------------------------------------------------------
__global__ void k_tab_bt_f16(int nang, int n_pad, int k_pad, int nmax, const double *__restrict__ cost,
                             __half *__restrict__ bt)
{
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= n_pad) return;
    const size_t mat = (size_t)n_pad * k_pad;
    const double u = a < nang ? cost[a] : 0.0;
    double pm2 = 0.0, pm1 = 0.0;
    for (int n = 1; n <= k_pad; ++n) {
        float p = 0.f, q = 0.f;
        if (a < nang && n <= nmax) {
            double pv, tv;
            if (n == 1) {
                pv = 1.0;
                tv = u;
            } else if (n == 2) {
                pv = 3.0 * u;
                tv = 6.0 * u * u - 3.0;
            } else {
                const double dn = (double)(n - 1);
                pv = (2.0 * dn + 1.0) / dn * pm1 * u - (dn + 1.0) / dn * pm2;
                tv = (dn + 1.0) * u * pv - (dn + 2.0) * pm1;
            }
            pm2 = pm1;
            pm1 = pv;
            const double s = (2.0 * n + 1.0) / ((double)n * (double)(n + 1));
            p = (float)(pv * s + tv * s);
            q = (float)(pv * s - tv * s);
        }
        const int k = n - 1;
        const size_t off = ((size_t)(k >> 3) * (n_pad >> 3) + (a >> 3)) * 64 + (a & 7) * 8 + (k & 7);
        __half h, l;
        split_f16(p, h, l);
        bt[off] = h;
        bt[mat + off] = l;
        split_f16(q, h, l);
        bt[2 * mat + off] = h;
        bt[3 * mat + off] = l;
    }
}

// ---------------------------------------------------------------------------
// The tensor-core contraction with the fused epilogue.
// ---------------------------------------------------------------------------
struct TcArgs {
    TabView v;
    const float4 *cf;
    const int *eexp;
    const int *eunit;
    const __half *bt;
    int n_pad, k_pad;
    const int *unit_order;
    int *counter;
    int *flags;
};

// shared-memory carve (bytes)
#define TC_A_BYTES (TC_KC * 128 * 2)                   // one A matrix chunk: 8 KB
#define TC_B_BYTES (TC_KC * TC_NBLK * 2)               // one B matrix chunk: 12 KB
#define TC_STAGE_PITCH 66                              // 64 columns + 2: conflict-free pair writes
#define TC_STAGE_FLOATS (4 * TC_INST * TC_STAGE_PITCH) // Mueller staging [k][size][col]: 66 KB
#define TC_SMEM_BYTES (4 * TC_A_BYTES + 8 * TC_B_BYTES + TC_STAGE_FLOATS * 4 + 8 * TC_INST * 4 + 256)

// One K chunk (TC_KC orders from k0) of angle block blk of the four B
// matrices into shared memory, [m][kg][ng][8][16 B]; plain 16-byte loads.
__device__ __forceinline__ void copy_b_chunk(const TcArgs &g, uint8_t *dstbase, int k0, int blk, int tid)
{
    const int nkg = TC_KC / 8, nng = TC_NBLK / 8, ngt = g.n_pad / 8;
    const size_t mat = (size_t)g.n_pad * g.k_pad;
    for (int idx = tid; idx < 4 * nkg * nng * 8; idx += TC_THREADS) {
        const int rr = idx & 7;
        const int ng = (idx >> 3) % nng;
        const int kg = ((idx >> 3) / nng) % nkg;
        const int m = (idx >> 3) / (nng * nkg);
        const size_t src = m * mat + (((size_t)(k0 / 8 + kg) * ngt + blk * nng + ng) * 64 + rr * 8);
        const uint32_t dst = m * TC_B_BYTES + (kg * nng + ng) * 128 + rr * 16;
        *(uint4 *)(dstbase + dst) = *(const uint4 *)(g.bt + src);
    }
}

template <int NB>
__global__ void __launch_bounds__(TC_THREADS, 1) k_tab_s12_tc(TcArgs g)
{
    extern __shared__ __align__(1024) uint8_t smem[];
    uint8_t *sA = smem;                                     // 4 x TC_A_BYTES
    uint8_t *sB0 = sA + 4 * TC_A_BYTES;                     // chunk 0 of the angle block, resident
    uint8_t *sB1 = sB0 + 4 * TC_B_BYTES;                    // later chunks
    float *stage = (float *)(sB1 + 4 * TC_B_BYTES);         // [4][64][65]
    float *sw = stage + TC_STAGE_FLOATS;                    // [64 sizes][8 bins]
    uint64_t *bar = (uint64_t *)(sw + 8 * TC_INST);
    uint32_t *s_tmem = (uint32_t *)(bar + 1);
    int *s_unit = (int *)(s_tmem + 1);
    int *s_abort = s_unit + 1;

    const TabView &v = g.v;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    int s_blk_loaded = -1;   // angle block whose chunk 0 sits in sB0 (same value in every thread)
    if (warp == 0) tmem_alloc(s_tmem, 512);
    if (tid == 0) {
        mbar_init(bar, 1);
        fence_mbar_init();
        *s_abort = 0;
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *s_tmem;
    const uint32_t idesc = idesc_f16_f32(128, TC_NBLK);
    uint32_t phase = 0;
    const int64_t n_units = (int64_t)v.n_lambda * v.n_rh * v.n_comp;
    const int nblocks = g.n_pad / TC_NBLK;

    for (;;) {
        if (tid == 0) *s_unit = atomicAdd(g.counter, 1);
        __syncthreads();
        const int uidx = *s_unit;
        __syncthreads();
        if (uidx >= n_units) break;
        const int64_t unit = g.unit_order[uidx];
        const int comp = (int)(unit % v.n_comp);
        const int64_t lr = unit / v.n_comp;
        const int lam = (int)(lr / v.n_rh);
        const int le = v.le(lam);
        const int64_t *off = v.off + (int64_t)le * v.n_size;
        const int64_t cbase = v.unit_base[unit] - off[0];
        const float4 *cf = g.cf + cbase;
        const int *ex = g.eexp + unit * v.n_size;
        const int E = g.eunit[unit];
        const int rhi = (int)(lr % v.n_rh);
        const float *Wb = v.Wf + v.wlam(lam) + ((size_t)rhi * v.n_bin * v.n_comp + comp) * v.n_size;

        for (int blk = 0; blk < nblocks; ++blk) {
            // per-unit sums of this thread's two columns per round as
            // unevaluated FP32 pairs (hi + lo, two-sum)
            float uh[TC_ROUNDS][2][NB], ul[TC_ROUNDS][2][NB];
#pragma unroll
            for (int r = 0; r < TC_ROUNDS; ++r)
#pragma unroll
                for (int c = 0; c < 2; ++c)
#pragma unroll
                    for (int b = 0; b < NB; ++b) uh[r][c][b] = ul[r][c][b] = 0.f;
            if (blk != s_blk_loaded) {   // uniform: chunk 0 of this angle block into sB0
                copy_b_chunk(g, sB0, 0, blk, tid);
                s_blk_loaded = blk;
            }

            for (int t0 = 0; t0 < v.n_size; t0 += TC_INST) {
                const int ntile = min(TC_INST, v.n_size - t0);
                const int kt = (int)(off[t0 + ntile] - off[t0 + ntile - 1]);   // largest nmax of the tile
                const int ktile = (kt + TC_KC - 1) / TC_KC * TC_KC;
                // scaled weights of the tile
                for (int idx = tid; idx < 8 * TC_INST; idx += TC_THREADS) {
                    const int b = idx & 7, i = idx >> 3;
                    float w = 0.f;
                    if (i < ntile && b < v.n_bin && b < NB)
                        w = ldexpf(Wb[(size_t)b * v.n_comp * v.n_size + t0 + i], max(-300, 2 * (ex[t0 + i] - E)));
                    sw[idx] = w;
                }
                // A-row data of this thread: size i = tid / 4, orders 8 (tid % 4) .. + 8 of each chunk
                const int ia = tid >> 2, seg = tid & 3;
                const bool has = ia < ntile;
                const int64_t pa = has ? off[t0 + ia] : 0;
                const int nma = has ? (int)(off[t0 + ia + 1] - pa) : 0;
                const float sc = has ? ldexpf(1.0f, max(-126, min(126, SHIFT_BITS - ex[t0 + ia]))) : 0.f;

                for (int k0 = 0; k0 < ktile; k0 += TC_KC) {
                    // ---- A: FP32 (c, d) -> scaled FP16 hi/lo, rows 2i (Re), 2i+1 (Im)
                    {
                        __half ch[4][8], cl[4][8];   // [c.re, c.im, d.re, d.im][order]
#pragma unroll
                        for (int j = 0; j < 8; ++j) {
                            const int k = k0 + 8 * seg + j;
                            float4 q = make_float4(0.f, 0.f, 0.f, 0.f);
                            if (k < nma) q = cf[pa + k];
                            split_f16(q.x * sc, ch[0][j], cl[0][j]);
                            split_f16(q.y * sc, ch[1][j], cl[1][j]);
                            split_f16(q.z * sc, ch[2][j], cl[2][j]);
                            split_f16(q.w * sc, ch[3][j], cl[3][j]);
                        }
                        // core matrix (kg = seg, mg = row / 8): offset (kg * 16 + mg) * 128 + (row % 8) * 16
                        const int r0 = 2 * ia, r1 = 2 * ia + 1;
                        const uint32_t o0 = (seg * 16 + (r0 >> 3)) * 128 + (r0 & 7) * 16;
                        const uint32_t o1 = (seg * 16 + (r1 >> 3)) * 128 + (r1 & 7) * 16;
                        // matrices: 0 C_hi, 1 C_lo, 2 D_hi, 3 D_lo
                        *(uint4 *)(sA + 0 * TC_A_BYTES + o0) = *(uint4 *)ch[0];
                        *(uint4 *)(sA + 0 * TC_A_BYTES + o1) = *(uint4 *)ch[1];
                        *(uint4 *)(sA + 1 * TC_A_BYTES + o0) = *(uint4 *)cl[0];
                        *(uint4 *)(sA + 1 * TC_A_BYTES + o1) = *(uint4 *)cl[1];
                        *(uint4 *)(sA + 2 * TC_A_BYTES + o0) = *(uint4 *)ch[2];
                        *(uint4 *)(sA + 2 * TC_A_BYTES + o1) = *(uint4 *)ch[3];
                        *(uint4 *)(sA + 3 * TC_A_BYTES + o0) = *(uint4 *)cl[2];
                        *(uint4 *)(sA + 3 * TC_A_BYTES + o1) = *(uint4 *)cl[3];
                    }
                    // ---- B: chunk 0 is resident; later chunks go to sB1
                    if (k0 > 0) copy_b_chunk(g, sB1, k0, blk, tid);
                    uint8_t *sB = k0 > 0 ? sB1 : sB0;
                    fence_proxy_async_smem();
                    __syncthreads();
                    if (tid == 0) {
                        tc_fence_after();
                        const uint32_t aA = smem_u32(sA), aB = smem_u32(sB);
#pragma unroll
                        for (int ks = 0; ks < TC_KC / 16; ++ks) {
                            const uint32_t acc = (k0 > 0 || ks > 0) ? 1u : 0u;
                            // A: LBO (K step of 8) = 16 core matrices, SBO (8 rows) = 128 B
                            const uint32_t ao = ks * 2 * 16 * 128;
                            const uint32_t bo = ks * 2 * (TC_NBLK / 8) * 128;
                            const uint64_t a_chi = smem_desc(aA + 0 * TC_A_BYTES + ao, 16 * 128, 128);
                            const uint64_t a_clo = smem_desc(aA + 1 * TC_A_BYTES + ao, 16 * 128, 128);
                            const uint64_t a_dhi = smem_desc(aA + 2 * TC_A_BYTES + ao, 16 * 128, 128);
                            const uint64_t a_dlo = smem_desc(aA + 3 * TC_A_BYTES + ao, 16 * 128, 128);
                            const uint64_t b_phi = smem_desc(aB + 0 * TC_B_BYTES + bo, (TC_NBLK / 8) * 128, 128);
                            const uint64_t b_plo = smem_desc(aB + 1 * TC_B_BYTES + bo, (TC_NBLK / 8) * 128, 128);
                            const uint64_t b_qhi = smem_desc(aB + 2 * TC_B_BYTES + bo, (TC_NBLK / 8) * 128, 128);
                            const uint64_t b_qlo = smem_desc(aB + 3 * TC_B_BYTES + bo, (TC_NBLK / 8) * 128, 128);
                            mma_f16(tmem, a_chi, b_phi, idesc, acc);
                            mma_f16(tmem, a_chi, b_plo, idesc, 1u);
                            mma_f16(tmem, a_clo, b_phi, idesc, 1u);
                            mma_f16(tmem + 256, a_dhi, b_qhi, idesc, acc);
                            mma_f16(tmem + 256, a_dhi, b_qlo, idesc, 1u);
                            mma_f16(tmem + 256, a_dlo, b_qhi, idesc, 1u);
                        }
                        mma_commit(bar);
                    }
                    // the MMAs read shared memory until the commit arrives; a wait
                    // that runs out aborts the whole block (uniformly, after a barrier)
                    if (!mbar_wait(bar, phase)) {
                        *s_abort = 1;
                        atomicOr(g.flags, GBMIE_FLAG_TIMEOUT);
                    }
                    phase ^= 1u;
                    tc_fence_after();
                    __syncthreads();
                    if (*s_abort) goto done;
                }
                // ---- epilogue: S+/S- -> Mueller -> weighted sums over the tile's sizes.
                // Mueller phase: warp (q = TMEM lane quarter, half = warp / 4)
                // holds rows 32 q .. + 31 (sizes 16 q .. + 15, Re/Im lane
                // pairs) for 32 columns.  Lanes exchange one value per column
                // pair so that the even lane forms column 2p and the odd lane
                // column 2p + 1 (no idle lanes).
                // Reduction phase: warp w sums element kk = w / 2, columns
                // 32 (w % 2) + 2 cp + {0, 1} (cp = lane % 16) over sizes
                // 32 h .. + 31 (h = lane / 16) for every bin; the two size
                // halves meet by a shuffle.
                const int q = warp & 3;
                const int il = 16 * q + (lane >> 1);
                const bool odd = lane & 1;
                const int kk = warp >> 1, cg = warp & 1, hh = lane >> 4, cp = lane & 15;
#pragma unroll
                for (int r = 0; r < TC_ROUNDS; ++r) {   // unrolled: uh/ul stay in registers
                    const int chunk = 2 * r + (warp >> 2);
                    float sp[32], sm[32];
                    tmem_ld32(tmem + ((uint32_t)(32 * q) << 16) + 32 * chunk, sp);
                    tmem_ld32(tmem + ((uint32_t)(32 * q) << 16) + 256 + 32 * chunk, sm);
                    float *strow = stage + il * TC_STAGE_PITCH + 32 * (warp >> 2) + (odd ? 1 : 0);
#pragma unroll
                    for (int pj = 0; pj < 16; ++pj) {
                        const int j0 = 2 * pj, j1 = 2 * pj + 1;
                        const float rp = __shfl_xor_sync(0xffffffffu, odd ? sp[j0] : sp[j1], 1);
                        const float rm = __shfl_xor_sync(0xffffffffu, odd ? sm[j0] : sm[j1], 1);
                        const float pr = odd ? rp : sp[j0], pi = odd ? sp[j1] : rp;
                        const float mr = odd ? rm : sm[j0], mi = odd ? sm[j1] : rm;
                        const float A2 = pr * pr + pi * pi, B2 = mr * mr + mi * mi;
                        float *st = strow + j0;
                        st[0 * TC_INST * TC_STAGE_PITCH] = 0.25f * (A2 + B2);
                        st[1 * TC_INST * TC_STAGE_PITCH] = -0.5f * (pr * mr + pi * mi);
                        st[2 * TC_INST * TC_STAGE_PITCH] = 0.25f * (A2 - B2);
                        st[3 * TC_INST * TC_STAGE_PITCH] = -0.5f * (mr * pi - mi * pr);
                    }
                    __syncthreads();
                    {
                        float acc[2][NB];
#pragma unroll
                        for (int c = 0; c < 2; ++c)
#pragma unroll
                            for (int b = 0; b < NB; ++b) acc[c][b] = 0.f;
                        const float *src = stage + (kk * TC_INST + 32 * hh) * TC_STAGE_PITCH + 32 * cg + 2 * cp;
                        const float *wsrc = sw + 32 * hh * 8;
#pragma unroll 4
                        for (int i = 0; i < 32; ++i) {
                            const float2 sv = *(const float2 *)(src + i * TC_STAGE_PITCH);
                            const float4 w0 = *(const float4 *)(wsrc + 8 * i);
                            float wv[8] = {w0.x, w0.y, w0.z, w0.w, 0.f, 0.f, 0.f, 0.f};
                            if (NB > 4) {
                                const float4 w1 = *(const float4 *)(wsrc + 8 * i + 4);
                                wv[4] = w1.x;
                                wv[5] = w1.y;
                                wv[6] = w1.z;
                                wv[7] = w1.w;
                            }
#pragma unroll
                            for (int b = 0; b < NB; ++b) {
                                acc[0][b] = fmaf(wv[b], sv.x, acc[0][b]);
                                acc[1][b] = fmaf(wv[b], sv.y, acc[1][b]);
                            }
                        }
#pragma unroll
                        for (int c = 0; c < 2; ++c)
#pragma unroll
                            for (int b = 0; b < NB; ++b) {
                                const float a = acc[c][b] + __shfl_xor_sync(0xffffffffu, acc[c][b], 16);
                                // two-sum: (uh + ul) += a exactly-rounded
                                const float sum = uh[r][c][b] + a;
                                const float bp = sum - uh[r][c][b];
                                ul[r][c][b] += (uh[r][c][b] - (sum - bp)) + (a - bp);
                                uh[r][c][b] = sum;
                            }
                    }
                    __syncthreads();
                }
                tc_fence_before();
            }
            // unit results of this angle block: lanes of the first size half
            // hold the combined sums of (element kk, two columns) per round
            if ((lane >> 4) == 0) {
                const int kk = warp >> 1;
                const double f2 = ldexp(1.0, 2 * (E - SHIFT_BITS));
#pragma unroll
                for (int r = 0; r < TC_ROUNDS; ++r) {
#pragma unroll
                    for (int c = 0; c < 2; ++c) {
                        const int col = blk * TC_NBLK + 64 * r + 32 * (warp & 1) + 2 * (lane & 15) + c;
                        if (col < v.n_ang) {
#pragma unroll
                            for (int b = 0; b < NB; ++b) {
                                if (b < v.n_bin) {
                                    const double f = v.frac[(size_t)b * v.n_comp + comp];
                                    atomicAdd(v.pacc + (((size_t)lr * v.n_bin + b) * 4 + kk) * v.n_ang + col,
                                              f * ((double)uh[r][c][b] + (double)ul[r][c][b]) * f2);
                                }
                            }
                        }
                    }
                }
            }
        }
    }
done:
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 0) tmem_dealloc(tmem, 512);
}

// ---------------------------------------------------------------------------
// host launchers (called from gbmie_table_run)
// ---------------------------------------------------------------------------
int launch_table_mixed(gbmie_ctx *ctx, gbmie_table_plan *p, TabView &v, char *scr)
{
    const gbmie_table_desc &d = p->d;
    cudaStream_t st = ctx->stream;
    float4 *cf = (float4 *)(scr + p->o_cf);
    int *eexp = (int *)(scr + p->o_eexp);
    int *eunit = (int *)(scr + p->o_eunit);
    __half *bt = (__half *)(scr + p->o_bt);
    int *counter = (int *)(scr + p->o_counter);
    ctx_pre_launch(ctx);
    k_fill_int<<<(unsigned)ceil_div64(p->n_units, 256), 256, 0, st>>>((int)p->n_units, eunit, -100000);
    GBMIE_TRY(ctx_check_launch(ctx, "k_fill_int"));
    ctx_pre_launch(ctx);
    k_tab_coeffs_mixed<<<(unsigned)ceil_div64(p->n_inst, 128), 128, 0, st>>>(v, p->n_inst, cf, eexp, eunit,
                                                                            ctx->d_flags);
    GBMIE_TRY(ctx_check_launch(ctx, "k_tab_coeffs_mixed"));
    ctx_pre_launch(ctx);
    k_tab_bt_f16<<<(p->n_pad_total + 127) / 128, 128, 0, st>>>(d.n_ang, p->n_pad_total, p->k_pad, p->nmax_max,
                                                                d.cos_theta, bt);
    GBMIE_TRY(ctx_check_launch(ctx, "k_tab_bt_f16"));
    GBMIE_TRY(ctx_cuda(ctx, cudaMemsetAsync(counter, 0, sizeof(int), st), "counter clear"));
    TcArgs a;
    a.v = v;
    a.cf = cf;
    a.eexp = eexp;
    a.eunit = eunit;
    a.bt = bt;
    a.n_pad = p->n_pad_total;
    a.k_pad = p->k_pad;
    a.unit_order = p->unit_order;
    a.counter = counter;
    a.flags = ctx->d_flags;
    int nsm = 0;
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, ctx->device);
    const int grid = (int)(p->n_units < nsm ? p->n_units : nsm);
    const size_t smem = TC_SMEM_BYTES;
    cudaError_t e = cudaSuccess;
    ctx_pre_launch(ctx);
#define TC_LAUNCH(NBV)                                                                                   \
    case NBV:                                                                                            \
        e = cudaFuncSetAttribute(k_tab_s12_tc<NBV>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem); \
        k_tab_s12_tc<NBV><<<grid, TC_THREADS, smem, st>>>(a);                                            \
        break;
    switch (d.n_bin) {
        TC_LAUNCH(1) TC_LAUNCH(2) TC_LAUNCH(3) TC_LAUNCH(4) TC_LAUNCH(5) TC_LAUNCH(6) TC_LAUNCH(7)
        default:
        TC_LAUNCH(8)
    }
#undef TC_LAUNCH
    GBMIE_TRY(ctx_cuda(ctx, e, "k_tab_s12_tc smem attribute"));
    return ctx_check_launch(ctx, "k_tab_s12_tc");
}

size_t table_mixed_smem_bytes() { return TC_SMEM_BYTES; }
