// gbmie_s12_noalloc: S1/S2 from Mie coefficients without any device
// allocation, for callers that cannot call cudaMalloc -- code that runs
// inside another framework's memory pool or allocator-owned region (which
// forbids foreign cudaMalloc/cudaFree), and embedded callers that must not
// grow the device footprint after start-up.  They pass their own inputs and
// outputs; the only other device memory used is the fixed array below.  The
// call returns after its stream has finished (it reads the status word back
// into host memory).
//
// The angular table (pi~_n + tau~_n, pi~_n - tau~_n) lives in the
// file-scope array g_noalloc_pq of GBMIE_NOALLOC_PQ_BYTES (4 MiB), which
// every GPU that loads the library keeps until the process exits.  The
// status word g_noalloc_status lives next to it.  Host code must not pass
// the symbols themselves to a kernel (on the host they are stand-ins, not
// device addresses): their device addresses are looked up once per device
// with cudaGetSymbolAddress, on the first call made with that device
// current, and cached.  That first call should therefore happen before any
// stream capture.
//
// Every call shares the array and leaves its contents behind; the table is
// rewritten in full before each use and the status word is cleared at the
// start of each call.  Two calls that overlap on the GPU (different streams,
// or different host threads on one device) race on the array and must be
// serialised by the caller.
#include "common.cuh"

#include <mutex>

#define GBMIE_NOALLOC_PQ_BYTES (4u << 20)
#define GBMIE_NOALLOC_PQ_ELEMS (GBMIE_NOALLOC_PQ_BYTES / sizeof(double2))
#define GBMIE_NOALLOC_MAX_DEVICES 64

static __device__ __align__(256) double2 g_noalloc_pq[GBMIE_NOALLOC_PQ_ELEMS];
static __device__ __align__(256) int g_noalloc_status;

// (p, q) at orders 1..nmax and nang cosines, [n-1][angle]; the upward
// recurrences of pymiecoated/mie_props.py:166-192 scaled by (2n+1)/(n(n+1)).
__global__ void k_noalloc_pq(int nang, const double *__restrict__ cost, int nmax, double2 *__restrict__ pq,
                             int *__restrict__ status)
{
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= nang) return;
    const double u = cost[a];
    if (!(fabs(u) <= 1.0)) {
        atomicOr(status, GBMIE_FLAG_INVALID);
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
            const double dn = (double)(n - 1);
            p = (2.0 * dn + 1.0) / dn * pm1 * u - (dn + 1.0) / dn * pm2;
            t = (dn + 1.0) * u * p - (dn + 2.0) * pm1;
        }
        pm2 = pm1;
        pm1 = p;
        const double s = (2.0 * n + 1.0) / ((double)n * (double)(n + 1));
        pq[(int64_t)(n - 1) * nang + a] = make_double2(p * s + t * s, p * s - t * s);
    }
}

// One block per instance (grid-stride), coefficients staged in shared memory
// as (a+b, a-b); an instance with more orders than the table holds is
// skipped and flagged instead of reading past the table.
#define NOALLOC_THREADS 128
#define NOALLOC_CHUNK 1024
__global__ void __launch_bounds__(NOALLOC_THREADS) k_noalloc_s12(int64_t n, const int64_t *__restrict__ off,
                                                                 const double2 *__restrict__ an,
                                                                 const double2 *__restrict__ bn, int nmax_table,
                                                                 int nang, const double2 *__restrict__ pq,
                                                                 double2 *__restrict__ s1, double2 *__restrict__ s2,
                                                                 int *__restrict__ status)
{
    __shared__ double2 cd[NOALLOC_CHUNK][2];
    for (int64_t i = blockIdx.x; i < n; i += gridDim.x) {
        const int64_t o = off[i];
        const int64_t nm64 = off[i + 1] - o;
        if (nm64 < 0 || nm64 > nmax_table) {
            if (threadIdx.x == 0) atomicOr(status, GBMIE_FLAG_NMAX);
            continue;   // uniform across the block
        }
        const int nm = (int)nm64;
        for (int a0 = 0; a0 < nang; a0 += NOALLOC_THREADS) {
            const int a = a0 + threadIdx.x;
            double sp_r = 0.0, sp_i = 0.0, sm_r = 0.0, sm_i = 0.0;
            for (int k0 = 0; k0 < nm; k0 += NOALLOC_CHUNK) {
                const int kn = min(NOALLOC_CHUNK, nm - k0);
                __syncthreads();
                for (int k = threadIdx.x; k < kn; k += NOALLOC_THREADS) {
                    const double2 av = an[o + k0 + k], bv = bn[o + k0 + k];
                    cd[k][0] = make_double2(av.x + bv.x, av.y + bv.y);
                    cd[k][1] = make_double2(av.x - bv.x, av.y - bv.y);
                }
                __syncthreads();
                if (a < nang) {
                    const double2 *col = pq + (int64_t)k0 * nang + a;
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

// Device addresses of the two arrays, looked up once per device.
struct NoallocSymbols {
    double2 *pq;
    int *status;
    bool ready;
};
static NoallocSymbols g_symbols[GBMIE_NOALLOC_MAX_DEVICES];
static std::mutex g_symbols_mutex;

static int noalloc_symbols(int device, NoallocSymbols *out)
{
    std::lock_guard<std::mutex> lock(g_symbols_mutex);
    NoallocSymbols &s = g_symbols[device];
    if (!s.ready) {
        void *p = nullptr, *f = nullptr;
        if (cudaGetSymbolAddress(&p, g_noalloc_pq) != cudaSuccess) return GBMIE_ERR_CUDA;
        if (cudaGetSymbolAddress(&f, g_noalloc_status) != cudaSuccess) return GBMIE_ERR_CUDA;
        s.pq = (double2 *)p;
        s.status = (int *)f;
        s.ready = true;
    }
    *out = s;
    return GBMIE_OK;
}

extern "C" int gbmie_s12_noalloc(void *stream, int64_t n, const int64_t *offsets, const gbmie_complex *an,
                                 const gbmie_complex *bn, int32_t nmax_max, int32_t nang, const double *cos_theta,
                                 gbmie_complex *s1, gbmie_complex *s2)
{
    if (n < 0 || nang < 0 || nmax_max < 1 || nmax_max > GBMIE_MAX_NMAX) return GBMIE_ERR_INVALID;
    if (n == 0 || nang == 0) return GBMIE_OK;
    if (!offsets || !an || !bn || !cos_theta || !s1 || !s2) return GBMIE_ERR_INVALID;
    const int nt = nmax_max < 2 ? 2 : nmax_max;
    if ((uint64_t)nt * (uint64_t)nang > (uint64_t)GBMIE_NOALLOC_PQ_ELEMS) return GBMIE_ERR_CAPACITY;
    int device = 0;
    if (cudaGetDevice(&device) != cudaSuccess || device < 0 || device >= GBMIE_NOALLOC_MAX_DEVICES)
        return GBMIE_ERR_CUDA;
    NoallocSymbols sym;
    GBMIE_TRY(noalloc_symbols(device, &sym));
    cudaStream_t st = (cudaStream_t)stream;
    if (cudaMemsetAsync(sym.status, 0, sizeof(int), st) != cudaSuccess) return GBMIE_ERR_CUDA;
    k_noalloc_pq<<<(nang + 127) / 128, 128, 0, st>>>(nang, cos_theta, nt, sym.pq, sym.status);
    if (cudaGetLastError() != cudaSuccess) return GBMIE_ERR_CUDA;
    const unsigned grid = (unsigned)(n < 152 * 64 ? n : 152 * 64);
    k_noalloc_s12<<<grid, NOALLOC_THREADS, 0, st>>>(n, offsets, (const double2 *)an, (const double2 *)bn, nt, nang,
                                                    sym.pq, (double2 *)s1, (double2 *)s2, sym.status);
    if (cudaGetLastError() != cudaSuccess) return GBMIE_ERR_CUDA;
    int status = 0;
    if (cudaMemcpyAsync(&status, sym.status, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess)
        return GBMIE_ERR_CUDA;
    if (cudaStreamSynchronize(st) != cudaSuccess) return GBMIE_ERR_CUDA;
    if (status & GBMIE_FLAG_NMAX) return GBMIE_ERR_NMAX;
    if (status) return GBMIE_ERR_INVALID;
    return GBMIE_OK;
}
