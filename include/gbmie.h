/*
 * gbmie.h -- C ABI of the GB300 (sm_103a) Mie hot path of GEOSmie.
 *
 * The reference (GEOS-ESM/GEOSmie) is a Python package; its hot path is the
 * pymiecoated Mie kernel (pymiecoated/mie_coeffs.py, mie_props.py,
 * mie_coated.py), the size/humidity integration of the runoptics table
 * builder (geosmie/dointegration.py) and the GSF expansion program
 * (gsf/spher_expan.f, reached through os.system in gsf/convertncdf.py:188).
 * It has no FFI of its own, so each entry point below states the reference
 * function whose work it replaces; the Python layer in geosmie_gb300/ binds
 * these with ctypes behind the reference's own Python signatures.
 *
 * Conventions
 *  - Every call returns an int status (GBMIE_OK == 0).  The message of the
 *    last failure on a context is available from gbmie_last_error().
 *  - Array arguments are DEVICE pointers owned by the caller unless a
 *    comment says "host".  Complex numbers are two doubles (re, im), the
 *    memory layout of numpy complex128 and CUDA double2.
 *  - Calls are asynchronous on the context's stream (gbmie_ctx_set_stream)
 *    except where a host result is returned (gbmie_layout, gbmie_table_plan).
 *  - A context is used by one host thread at a time.
 *  - Refractive indices follow pymiecoated: Im(m) > 0 is absorbing,
 *    eps = m^2, mu = 1 unless given.
 */
#ifndef GBMIE_H
#define GBMIE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define GBMIE_OK 0
#define GBMIE_ERR_INVALID 1     /* bad argument: x < 0, y < x, NaN/Inf, |u| > 1,
                                   coated with mu != 1, bad sizes or pointers */
#define GBMIE_ERR_NMAX 2        /* an instance needs more partial waves than
                                   GBMIE_MAX_NMAX */
#define GBMIE_ERR_CUDA 3        /* a CUDA runtime call failed */
#define GBMIE_ERR_TIMEOUT 4     /* a device-side wait hit its iteration limit */
#define GBMIE_ERR_NOMEM 5       /* device allocation failed */
#define GBMIE_ERR_UNSUPPORTED 6 /* option not implemented */
#define GBMIE_ERR_CAPACITY 7    /* request larger than gbmie_s12_noalloc's fixed
                                   device array */

#define GBMIE_MAX_NMAX 100000   /* x up to about 9.9e4 */

/* precision of the contractions (S1/S2 angular sums, size integration, GSF) */
#define GBMIE_PLAIN_FP64 0      /* everything in FP64 */
#define GBMIE_MIXED 1           /* FP64 recurrences, tensor-core split-FP16
                                   contractions with FP32 accumulation */

typedef struct gbmie_ctx gbmie_ctx;
typedef struct { double re, im; } gbmie_complex;

/* ---- context ----------------------------------------------------------- */
int gbmie_ctx_create(int device, gbmie_ctx **ctx);
int gbmie_ctx_destroy(gbmie_ctx *ctx);
/* stream: a cudaStream_t (NULL = legacy default stream). */
int gbmie_ctx_set_stream(gbmie_ctx *ctx, void *stream);
int gbmie_ctx_synchronize(gbmie_ctx *ctx);
const char *gbmie_status_string(int status);
const char *gbmie_last_error(const gbmie_ctx *ctx);
/* Kernel launches issued by this context so far (host counter). */
int64_t gbmie_launch_count(const gbmie_ctx *ctx);
/* Per-kernel device timing: when enabled, every kernel the context launches
 * is bracketed by CUDA events on its stream.  gbmie_ctx_kernel_times
 * synchronises and reports, for up to `cap` distinct kernels, the name (a
 * static string owned by the library), the launch count and the summed
 * device time in ms; *n receives the number of kernels.  Enabling clears
 * earlier records.  No counterpart in the reference (measurement only). */
int gbmie_ctx_set_timing(gbmie_ctx *ctx, int enable);
int gbmie_ctx_kernel_times(gbmie_ctx *ctx, int32_t cap, const char **names, int64_t *launches,
                           double *total_ms, int32_t *n);

/* Number of partial waves round(2 + x + 4 x^(1/3)) for one size parameter,
 * computed by the same device function the kernels use (host result).
 * Replaces the nmax expression of pymiecoated/mie_coeffs.py:99,148,203. */
int gbmie_nmax(gbmie_ctx *ctx, double x, int32_t *nmax /* host */);

/* CSR layout of ragged per-instance coefficient arrays: offsets[0] = 0,
 * offsets[i+1] = offsets[i] + nmax(size[i]).  size = x (homogeneous) or
 * y (coated).  *total (host) receives offsets[n].  Synchronous. */
int gbmie_layout(gbmie_ctx *ctx, int64_t n, const double *size,
                 int64_t *offsets, int64_t *total /* host */);

/* Mie coefficients a_n, b_n (n = 1..nmax) and the six efficiencies
 * (qext, qsca, qabs, qb, asy, qratio) of n instances.
 * Replaces pymiecoated/mie_coeffs.py:36-73 (mie_coeffs dispatch),
 * :83-180 (homogeneous), :183-251 (coated) and mie_props.py:28-70.
 *   x[n]                 core (or only) size parameter
 *   y[n] or NULL         shell size parameter (coated if y != x and
 *                        eps2 != eps, as the reference dispatches)
 *   eps[n]               permittivity (core)
 *   mu[n] or NULL        permeability (homogeneous only; NULL = 1)
 *   eps2[n] or NULL      shell permittivity (required with y)
 *   offsets[n+1]         from gbmie_layout on max(x, y); may be NULL when
 *                        an and bn are NULL
 *   an, bn or NULL       [offsets[n]] complex
 *   eff or NULL          [n][6]
 * Uses scratch device memory owned by the context. */
int gbmie_coeffs(gbmie_ctx *ctx, int64_t n, const double *x, const double *y,
                 const gbmie_complex *eps, const gbmie_complex *mu,
                 const gbmie_complex *eps2, const int64_t *offsets,
                 gbmie_complex *an, gbmie_complex *bn, double *eff);

/* Scaled angular functions pi~_n(u) and tau~_n(u) (times (2n+1)/(n(n+1))),
 * n = 1..nmax, at nang cosines: pi_out, tau_out [nang][nmax].
 * Replaces pymiecoated/mie_props.py:166-231 and mie_coated.py:160-179. */
int gbmie_pitau(gbmie_ctx *ctx, int32_t nang, const double *cos_theta,
                int32_t nmax, double *pi_out, double *tau_out);

/* Amplitude functions S1, S2 [n][nang] of n instances from their
 * coefficients (CSR by offsets).  Replaces mie_props.py:108-149 and
 * mie_coated.py:31-39 (runS12Loop).  |cos_theta| <= 1 is required. */
int gbmie_s12(gbmie_ctx *ctx, int64_t n, const int64_t *offsets,
              const gbmie_complex *an, const gbmie_complex *bn, int32_t nang,
              const double *cos_theta, gbmie_complex *s1, gbmie_complex *s2);

/* Amplitude functions S1, S2 [n][nang] of n instances from their
 * coefficients (CSR by offsets) and caller-supplied scaled angular functions
 * pi~_n, tau~_n (times (2n+1)/(n(n+1))) given as rows pi[nang][ld],
 * tau[nang][ld], order n at column n-1; every instance's nmax must be <= ld
 * (else GBMIE_ERR_NMAX).  S1 = sum a_n pi~_n + b_n tau~_n, S2 = sum a_n
 * tau~_n + b_n pi~_n over the instance's own orders.  Replaces
 * pymiecoated/mie_props.py:115-149 (mie_S12_pt, Mie.S12_pt) and
 * mie_coated.py:51-59 (MultipleMie.calculateS12WithParams over its
 * precomputed parr/tarr rows).  Allocates nothing. */
int gbmie_s12_pt(gbmie_ctx *ctx, int64_t n, const int64_t *offsets, const gbmie_complex *an,
                 const gbmie_complex *bn, int32_t nang, int32_t ld, const double *pi_rows,
                 const double *tau_rows, gbmie_complex *s1, gbmie_complex *s2);

/* gbmie_s12 for callers that cannot allocate device memory: code running
 * inside another framework's memory pool or allocator-owned region (which
 * forbids foreign cudaMalloc/cudaFree), and embedded callers that must not
 * grow the device footprint after start-up.  No counterpart in the
 * reference.  Allocates nothing: no context, no scratch;
 * the angular table lives in a fixed 4 MiB device array inside the library
 * (held by every GPU that loads it until exit), so nmax_max * nang must not
 * exceed 262144 (e.g. nmax 700 with 371 angles), else GBMIE_ERR_CAPACITY.
 * nmax_max (host) bounds every instance's offsets[i+1] - offsets[i]; an
 * instance above it returns GBMIE_ERR_NMAX (that instance is skipped).
 * Runs on `stream` (a cudaStream_t, NULL = legacy default) with the current
 * device and returns after the stream finishes.  The first call on a device
 * looks up the array's device address (cudaGetSymbolAddress); make it before
 * any stream capture.  Calls share the array: calls that overlap on the GPU
 * race and must be serialised by the caller. */
int gbmie_s12_noalloc(void *stream, int64_t n, const int64_t *offsets, const gbmie_complex *an,
                      const gbmie_complex *bn, int32_t nmax_max, int32_t nang, const double *cos_theta,
                      gbmie_complex *s1, gbmie_complex *s2);

/* One MultipleMie(xArr, None, costarr).calculateS12SizeRange(mr, mi) call:
 * eps = (mr + i mi)^2, mu = 1; S1, S2 [n][nang] and eff [n][6] for every x.
 * Replaces pymiecoated/mie_coated.py:61-89.  Uses context scratch. */
int gbmie_size_range(gbmie_ctx *ctx, int64_t n, const double *x, double mr,
                     double mi, int32_t nang, const double *cos_theta,
                     gbmie_complex *s1, gbmie_complex *s2, double *eff);

/* ---- table generation (runoptics / dointegration.fun) ------------------ */
#define GBMIE_GRID_X 0          /* grid = size parameters, shared by all
                                   wavelengths (dointegration.py:791) */
#define GBMIE_GRID_RADIUS 1     /* grid = radii (m); x = 2 pi r / lambda */

#define GBMIE_PSD_LOGNORM 0     /* particleparams.py:113-127 x dgrid,
                                   dointegration.py:546-583 */
#define GBMIE_PSD_POWER4 1      /* r^-4 in [rmin, rmax] x dgrid,
                                   dointegration.py:626-662 */
#define GBMIE_PSD_WEIGHTS 2     /* caller-supplied normalised weights */

/* scalar outputs per (bin, lambda, rh) */
enum {
    GBMIE_S_QEXT = 0, GBMIE_S_QSCA, GBMIE_S_QABS, GBMIE_S_QB, GBMIE_S_G,
    GBMIE_S_CSCA, GBMIE_S_CEXT, GBMIE_S_SSA, GBMIE_S_BSCA, GBMIE_S_BEXT,
    GBMIE_S_BBCK, GBMIE_S_REFREAL, GBMIE_S_REFIMAG, GBMIE_S_LIDAR_RATIO,
    GBMIE_NSCALAR
};
/* wavelength-independent outputs per (bin, lambda, rh); the reference file
 * keeps the values of the last wavelength */
enum {
    GBMIE_N_MASS = 0, GBMIE_N_VOLUME, GBMIE_N_AREA, GBMIE_N_REFF,
    GBMIE_N_RMASS, GBMIE_N_RHOP, GBMIE_N_GF, GBMIE_N_RLOW, GBMIE_N_RUP,
    GBMIE_NNL
};

typedef struct {
    int32_t n_lambda, n_rh, n_size, n_bin, n_comp, n_ang;
    int32_t grid_kind;          /* GBMIE_GRID_* */
    int32_t psd_kind;           /* GBMIE_PSD_* */
    int32_t precision;          /* GBMIE_PLAIN_FP64 or GBMIE_MIXED */
    int32_t n_gsf;              /* moments of the GSF expansion; the
                                   reference keeps 129 (its Gauss node
                                   count); 0 = no expansion */
    const double *lambda;       /* [n_lambda] m */
    const double *grid;         /* [n_size] ascending, see grid_kind */
    const double *dgrid;        /* [n_size] PSD widths (drarr), same unit */
    const gbmie_complex *m;     /* [n_lambda][n_rh][n_comp], Im > 0 absorbing */
    const double *psd_param;    /* [n_bin][n_comp][4]: lognormal r0, rmin0,
                                   rmax0, sigma; power4 rmin, rmax, -, - (m) */
    const double *gf_psd;       /* [n_rh] growth applied to r0 and rmax0
                                   (particleparams.py:85-91) */
    int32_t rh0_index;          /* rh index whose growth defines the dry
                                   effective radius reff0 (dointegration.py:841) */
    int32_t n_gsf_nodes;        /* Gauss nodes of the GSF expansion, >= n_gsf;
                                   0 = n_gsf nodes (the reference's
                                   L1MAX = NG, spher_expan.f:156).  The first
                                   n_gsf coefficients of an expansion do not
                                   depend on how many are kept. */
    const double *frac;         /* [n_bin][n_comp] */
    const double *weights;      /* GBMIE_PSD_WEIGHTS: [n_lambda][n_rh][n_bin]
                                   [n_comp][n_size]; weights of rh0_index give
                                   reff0 */
    const double *rhop;         /* [n_bin][n_rh] wet density */
    const double *rhop0;        /* [n_bin] dry density */
    const double *gf;           /* [n_rh] growth factor recorded in the table */
    const double *rlow;         /* [n_bin] */
    const double *rup;          /* [n_bin] */
    const double *cos_theta;    /* [n_ang] */
    const double *theta;        /* [n_ang] radians, ascending */
    /* Coated spheres (pymiecoated Mie(m=core, m2=shell, x, y),
     * mie_coeffs.py:183-251), or NULL for homogeneous spheres: the grid is
     * the outer size, m the shell index and m_core the core index per
     * (lambda, rh, comp); the core size parameter is core_ratio[rh] times the
     * outer one (0 <= core_ratio <= 1; 0 gives the shell alone, 1 or equal
     * indices the homogeneous core sphere, mie_coeffs.py:62-71). */
    const gbmie_complex *m_core;  /* [n_lambda][n_rh][n_comp] or NULL */
    const double *core_ratio;     /* [n_rh], with m_core */
} gbmie_table_desc;

typedef struct {
    double *phase;   /* [n_bin][n_lambda][n_rh][6][n_ang]: p11 p12 p22 p33 p34 p44 */
    double *pback;   /* [n_bin][n_lambda][n_rh][6]: p11 p12 p33 p34 p22 p44 at the
                        last angle (dointegration.py:990-991) */
    double *scalar;  /* [n_bin][n_lambda][n_rh][GBMIE_NSCALAR] */
    double *nl;      /* [n_bin][n_lambda][n_rh][GBMIE_NNL] */
    double *pmom;    /* [n_bin][n_lambda][n_rh][6][n_gsf] alpha1..alpha4, beta1,
                        beta2 normalised to alpha1(0) = 1, or NULL */
} gbmie_table_out;

typedef struct gbmie_table_plan gbmie_table_plan;

/* Plan a table: validates the descriptor, computes the per-wavelength
 * coefficient layout on the device and sizes the scratch memory.  Its
 * device work runs on the context's stream at the time of the call and it
 * returns once that stream has done it (other streams are not waited for:
 * a plan can be created on a side stream while tables run on another).
 * The plan's arrays are stream-ordered allocations; the angle-function
 * operand of mixed plans is shared, through the context, by plans with the
 * same angles and largest nmax.  The descriptor's pointers must stay valid
 * until the plan is destroyed.  *scratch_bytes (host) receives the scratch
 * size. */
int gbmie_table_plan_create(gbmie_ctx *ctx, const gbmie_table_desc *desc,
                            gbmie_table_plan **plan, int64_t *scratch_bytes);
/* Destroy a plan: its arrays are freed in order on the context's stream at
 * the time of the call (bind the stream of the plan's last run); no wait
 * for the device unless the plan holds a captured graph. */
int gbmie_table_plan_destroy(gbmie_table_plan *plan);
/* Run a planned table: replaces the (bin x lambda x RH) loop of
 * geosmie/dointegration.py:786-1031 (rawMie, calculateScatVals,
 * calculatePSD, integratePSD, the phase normalisation) and, when n_gsf > 0,
 * the pygeos pass of gsf/convertncdf.py:319-401 + gsf/spher_expan.f.
 * Asynchronous; uses context scratch sized by the plan. */
int gbmie_table_run(gbmie_ctx *ctx, gbmie_table_plan *plan, const gbmie_table_out *out);
/* The same table as one CUDA graph: the first call (and any call whose
 * output pointers differ from the captured ones, or after the context's
 * scratch block was reallocated by a larger plan) captures gbmie_table_run
 * on a private stream and instantiates it; every call then launches the
 * graph on the context stream.  Results equal gbmie_table_run's bit for
 * bit (the angular kernels' partial sums are added in a fixed order, so a
 * table's bits do not depend on block timing).  With timing
 * enabled the whole graph is timed as one record, "gbmie_table_graph".  No
 * counterpart in the reference (its table loop is Python,
 * geosmie/dointegration.py:786-1031). */
int gbmie_table_run_graph(gbmie_ctx *ctx, gbmie_table_plan *plan, const gbmie_table_out *out);
/* Autotuning (synchronous): times launch parameters on the plan's own data
 * and keeps the fastest; the plain FP64 path tunes sizes per block and
 * angles per pass of its angular kernel for each nmax bucket (nmax <= 16,
 * <= 64, <= 256, more) and for one launch over the whole grid, then keeps
 * the faster of the two layouts; the mixed path the block size of its coefficient
 * kernel and the accumulation window of its tensor-core contraction.  The
 * choice is cached in the context by table shape: later plans of the same
 * shape take it at creation.  Ends with a run of the tuned table into out.
 * No counterpart in the reference (its loops run in Python). */
int gbmie_table_plan_autotune(gbmie_ctx *ctx, gbmie_table_plan *plan, const gbmie_table_out *out);
/* Tries of every pipeline wait (mbarrier waits between the roles of the
 * tensor-core contraction of mixed plans) before the kernel gives up: it
 * then raises GBMIE_FLAG_TIMEOUT, lets its in-flight copies and MMAs finish,
 * frees its tensor memory and returns, and the next gbmie_ctx_synchronize
 * reports GBMIE_ERR_TIMEOUT.  tries < 0 restores the default (2^26); 0 makes
 * every wait give up at once, so that callers can test their handling of a
 * device timeout without a hang (the context stays usable).  Drops a
 * captured graph of the plan (synchronising the context stream first).  No
 * counterpart in the reference (its loops run in Python). */
int gbmie_table_plan_set_wait_limit(gbmie_table_plan *plan, int64_t tries);
/* Mixed plans of homogeneous spheres: enable = 1 runs the downward D_n
 * recurrence of the coefficient kernel in FP64 from the reference's start
 * (zero at round(max(nmax, |m x|) + 16), pymiecoated/mie_coeffs.py:101,
 * 119-121) instead of double-float pairs with a warm-up shortened to an
 * e^-23 damping; 0 restores the default.  A measurement variant (the cost of
 * keeping D_n in FP64 on this GPU); drops a captured graph of the plan. */
int gbmie_table_plan_set_dn_fp64(gbmie_table_plan *plan, int32_t enable);
/* params[16]: [0] 1 when tuned (or taken from the cache); [1] 1 = the plain
 * angular kernel runs one launch per nmax bucket, 0 = one launch over the
 * whole grid; [2..6] sizes per block and [7..11] angles per pass of the four
 * buckets and of the whole-grid launch; [12] coefficient block size of the
 * mixed path; [13] its accumulation window. */
int gbmie_table_plan_tuning(const gbmie_table_plan *plan, int32_t *params);
/* Sets the launch parameters in the layout of gbmie_table_plan_tuning
 * (params[0] is ignored): chunks of 64, 128, 256 or 512 sizes, 32 to 256
 * angles per pass (multiples of 32), coefficient block 64, 128 or 256,
 * accumulation window 1 to 4; else GBMIE_ERR_INVALID.  A table's bits
 * depend on its launch layout only (repeated runs, graph replays and other
 * plans with the same parameters give identical outputs), so parameters
 * saved from one process reproduce its tables in another.  Drops a captured
 * graph of the plan.  No counterpart in the reference. */
int gbmie_table_plan_set_tuning(gbmie_table_plan *plan, const int32_t *params);

/* ---- GSF expansion ------------------------------------------------------ */
/* Expansion coefficients of ntab scattering matrices given on one angle grid:
 * ang_deg [nang] ascending degrees; F [ntab][6][nang] in the order F11 F22
 * F33 F44 F12 F34; coef [ntab][6][nnodes] alpha1 alpha2 alpha3 alpha4 beta1
 * beta2 (l = 0..nnodes-1) normalised so alpha1(0) = 1; cnorm [ntab] or NULL
 * receives 1/alpha1(0).  Replaces gsf/spher_expan.f:93-107,120-180,269-407,
 * 520-623 (one program run per matrix in the reference).  precision
 * GBMIE_PLAIN_FP64: FP64 sums; GBMIE_MIXED: tensor-core GEMMs on
 * fixed-point digits (exact integer sums; coefficients within ~1e-7 of
 * alpha1(0)). */
int gbmie_gsf(gbmie_ctx *ctx, int32_t ntab, int32_t nang, const double *ang_deg,
              const double *F, int32_t nnodes, double *coef, double *cnorm,
              int32_t precision);

/* ---- band averages ------------------------------------------------------- */
/* Band averages of table quantities: for every variable, bin, band and RH
 * the mean of the variable linearly interpolated in wavenumber at 100 points
 * spaced evenly between the band's two edges (either order), clipped to the
 * table's wavenumber range.  Replaces geosmie/bandaverage.py doAverage
 * (:18-50) as looped by fun (:163-179); the arithmetic follows its numpy
 * linspace / clip / interp / pairwise-sum steps.  wavenum [nlam]: the
 * table's wavenumbers in cm^-1 (any order, 1/(100 lambda[m])); vin
 * [nvar][nbin][nlam][nrh]; edge_a, edge_b [nband] band edges in cm^-1;
 * out [nvar][nbin][nband][nrh].  Device pointers; nlam >= 1. */
int gbmie_band_average(gbmie_ctx *ctx, int32_t nvar, int32_t nbin, int32_t nlam, int32_t nrh,
                       const double *wavenum, const double *vin, int32_t nband,
                       const double *edge_a, const double *edge_b, double *out);

/* ---- measurement helper ------------------------------------------------- */
/* Sustained FP64 FMA throughput of this device (GFLOP/s, host), measured by
 * a dependent-chain-free DFMA loop over the whole GPU. */
int gbmie_measure_fp64_peak(gbmie_ctx *ctx, double *gflops);

#ifdef __cplusplus
}
#endif
#endif /* GBMIE_H */
