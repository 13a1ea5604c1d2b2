/*
 * oneka_gb300.h -- C ABI of liboneka_gb300.so, the GB300 (sm_103a) engine for
 * OnekaPy's per-realization hot path:
 *
 *   realization draw -> weighted least-squares fit of A..F -> multivariate-
 *   normal draw -> Dormand-Prince backtrace of npaths particles -> chronicle
 *   of every trace into the ProbabilityField grid.
 *
 * The OnekaPy reference (Python/NumPy, single thread) has no FFI; its
 * operator surface is the Python functions cited beside each entry point.
 * These entry points are what a binding of that surface calls (ctypes,
 * cffi, or a C/C++ host).
 *
 * Conventions
 *   - Every array pointer is a DEVICE pointer owned by the caller unless the
 *     comment says "host".  Struct arguments themselves live in host memory.
 *   - Calls are ordered on `stream` (a cudaStream_t; NULL = legacy default
 *     stream) and return ONEKA_OK (0) or a negative ONEKA_ERR_* code.  They
 *     never abort the process.  oneka_last_error() describes the last failure
 *     of the calling thread.
 *   - Per-particle and per-realization outcomes are status codes, not errors:
 *     a dry cell ends a trace with the vertices so far (the reference's
 *     AquiferError path), and an attempt cap ends a trace that would never
 *     finish (the reference loops forever on a NaN velocity).
 *   - Arrays are row-major and C-contiguous.
 */
#ifndef ONEKA_GB300_H
#define ONEKA_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ONEKA_ABI_VERSION 1

#if defined(__GNUC__)
#define ONEKA_API __attribute__((visibility("default")))
#else
#define ONEKA_API
#endif

/* return codes */
#define ONEKA_OK 0
#define ONEKA_ERR_INVALID (-1)   /* bad argument (null pointer, size, option) */
#define ONEKA_ERR_CUDA (-2)      /* a CUDA launch or runtime call failed */
#define ONEKA_ERR_SCRATCH (-3)   /* scratch buffer too small for one realization slot */

/* per-realization status (oneka_realize; skipped by oneka_track) */
#define ONEKA_REAL_OK 0
#define ONEKA_REAL_RANGE 1       /* an observed head is at or below the base (model.py:558-559 RangeError) */
#define ONEKA_REAL_NOT_SPD 2     /* normal equations not positive definite (model.py:604 LinAlgError) */
#define ONEKA_REAL_NOT_FINITE 3  /* the fitted or drawn coefficients are not finite, e.g. an observation on a
                                    well (log 0 in construct_fit, model.py:565); the reference would then
                                    backtrace with NaN velocities and never end.  Not tracked. */

/* per-particle status (oneka_track) */
#define ONEKA_TRACE_OK 0         /* reached |duration| */
#define ONEKA_TRACE_DRY 1        /* potential <= 0 or head <= 0 (model.py:343, :380 AquiferError) */
#define ONEKA_TRACE_STEP_LIMIT 2 /* attempt cap reached */

/* distribution kinds (generate_random_variate, stochastic.py:297-304; LOGNORMAL is an extension) */
#define ONEKA_DIST_CONST 0       /* p0 */
#define ONEKA_DIST_UNIFORM 1     /* U(p0, p1) */
#define ONEKA_DIST_TRIANGULAR 2  /* (min p0, mode p1, max p2) */
#define ONEKA_DIST_LOGNORMAL 3   /* exp(N(mu = p0, sigma = p1)) */

/* oneka_realize modes */
#define ONEKA_MODE_STOCHASTIC 0  /* draw q, K, n, H; fit; draw A..F (stochastic.py:220-241) */
#define ONEKA_MODE_MEAN 1        /* distribution means; fit; A..F = fitted mean (deterministic.py:175-199) */
#define ONEKA_MODE_GIVEN 2       /* q and aquifer are inputs; fit; draw A..F */
#define ONEKA_MODE_GIVEN_EV 3    /* q and aquifer are inputs; fit; A..F = fitted mean */

/* oneka_track precision */
#define ONEKA_FP64 0             /* parity build: the reference's FP64 arithmetic, bit-exact counts */
#define ONEKA_FP32 1             /* fast build: FP32 tracking, FP64 where digits are lost */

typedef struct OnekaDist {
    int32_t kind;
    int32_t pad;
    double p0, p1, p2;
} OnekaDist;

/* One site: wells, observations and the regional-flow origin. */
typedef struct OnekaSite {
    int32_t nwells;          /* wells in the reference's list order */
    int32_t nobs;
    int32_t target;          /* index of the target well (centre of the release ring) */
    int32_t pad;
    double base;             /* aquifer base elevation [m] */
    double xo, yo;           /* regional-flow origin; the stochastic driver uses the target well.
                                The FP32 tracker measures coordinates from it. */
    const double* wells;     /* [nwells][3]: xw, yw, rw */
    const double* obs;       /* [nobs][4]: x, y, z_ev, z_std (may be NULL when nobs == 0) */
} OnekaSite;

/* Per-realization parameters, structure of arrays ([nreal] leading). */
typedef struct OnekaRealizations {
    double* coef;            /* [nreal][6] A..F used for tracking */
    double* coef_ev;         /* [nreal][6] fitted expected value, or NULL */
    double* coef_cov;        /* [nreal][36] fitted covariance, or NULL */
    double* q;               /* [nreal][nwells] well discharges [m^3/d] */
    double* aquifer;         /* [nreal][3] conductivity, porosity, thickness */
    int32_t* status;         /* [nreal] ONEKA_REAL_* */
} OnekaRealizations;

/* Node grid: node (i, j) at (xmin + j*dx, ymin + i*dy), i < nrows, j < ncols. */
typedef struct OnekaGrid {
    double xmin, ymin, dx, dy;
    int32_t nrows, ncols;
} OnekaGrid;

/*
 * The grid a particle's trace is rasterized against when the caller replays
 * the reference's auto-expanding ProbabilityField: its origin at that time
 * and its offset (columns, rows) inside the final grid.
 */
typedef struct OnekaFrame {
    double xmin, ymin;
    int32_t coff, roff;
    int32_t ncols, nrows;
} OnekaFrame;

typedef struct OnekaTrackOpts {
    double duration;         /* [d]; negative tracks forward (capturezone.py:143) */
    double tol;              /* local error tolerance [m] */
    double maxstep;          /* maximum space step [m] */
    double umbra;            /* vector-to-raster range [m] */
    int32_t confined;        /* 1: compute_velocity_confined; 0: compute_velocity */
    int32_t precision;       /* ONEKA_FP64 or ONEKA_FP32 */
    int32_t max_attempts;    /* step attempts per particle before STEP_LIMIT; <= 0: 1,000,000 */
    int32_t block;           /* threads per block: 32, 64, 128 or 256; 0: 256 (FP32), 128 (FP64) */
    int32_t window_kb;       /* shared-memory chronicle window per block in KiB (0: 32; < 0: none) */
    int32_t occupancy;       /* FP32 build: resident blocks per SM to compile for (4, 6, 8 at 128
                                threads; 2, 3, 4 at 256); 0: the lowest */
    int32_t head64;          /* FP32 build, general path: 1 re-inverts a head within 1 % of the
                                aquifer top in FP64 from the compensated potential (off: FP32);
                                runs the 256 x 3 launch shape; not for batched launches */
} OnekaTrackOpts;

/* Optional per-particle outputs ([nreal][npaths] leading); any pointer may be NULL. */
typedef struct OnekaTrackOut {
    double* endpoint;        /* [..][2] last vertex */
    double* bbox;            /* [..][4] xmin, xmax, ymin, ymax over the vertices */
    int32_t* naccept;        /* accepted steps */
    int32_t* nattempt;       /* attempted steps */
    int32_t* status;         /* ONEKA_TRACE_* */
    double* vertices;        /* [..][max_vertices][2] first vertices of each trace */
    int32_t* nvertices;      /* vertices in the full trace (may exceed max_vertices) */
    int32_t max_vertices;
    int32_t pad;
    int64_t* counters;       /* [8] summed over all particles: step attempts, accepted steps,
                                chronicle node tests, chronicle word ORs, DRY traces, STEP_LIMIT
                                traces, traces reaching the grid's outer nodes (clipped by a fixed
                                window; the reference would expand its grid), 0; or NULL */
} OnekaTrackOut;

/* ---------------------------------------------------------------------- */

/* ABI version of the loaded library (ONEKA_ABI_VERSION). */
ONEKA_API int oneka_abi_version(void);

/* Description of the last failure on the calling thread ("" if none). */
ONEKA_API const char* oneka_last_error(void);

/*
 * log(r^2) from every observation to every well, [nobs][nwells], FP64.
 * The fit reuses it for every realization of the site; the well term of the
 * observation potential is then (q * logr2) * 1/(4 pi) in the reference's
 * order (model.py:258-264).
 */
ONEKA_API int oneka_site_logr2(const OnekaSite* site, double* logr2, void* stream);

/*
 * Realization draw + WLS fit + MVN draw for realizations
 * [first, first + nreal) of the Philox stream `seed` (one warp each).
 *   stochastic.py:220-241 (draws, fit, MVN); model.py:497-606 (FOSM rows,
 *   lstsq + inv, here FP64 normal equations with a Jacobi-scaled Cholesky
 *   factor; the MVN draw uses the same factor).
 *   qdist: [nwells] distributions of the discharges; adist: host [3] for
 *   conductivity, porosity, thickness.  logr2 from oneka_site_logr2, or NULL.
 *   For ONEKA_MODE_GIVEN*, out->q and out->aquifer are read, not written.
 */
ONEKA_API int oneka_realize(const OnekaSite* site, const OnekaDist* qdist, const OnekaDist* adist,
                  const double* logr2, uint64_t seed, uint64_t first, int32_t nreal,
                  int32_t mode, OnekaRealizations* out, void* stream);

/*
 * Model.construct_fit (model.py:497-567) for one model on the device: the
 * weighted rows WA [nobs][6] and right-hand side Wb [nobs] of the regional-
 * flow least-squares problem, with the wells' discharges q [nwells] and the
 * aquifer's conductivity and thickness, about the origin (site->xo, site->yo).
 * FP64 in the reference's operation order.  *status (device int32) is set to
 * ONEKA_REAL_OK, or ONEKA_REAL_RANGE where an observed head is at or below
 * the base (the reference's RangeError; that row is NaN).
 */
ONEKA_API int oneka_fit_rows(const OnekaSite* site, const double* q, double conductivity, double thickness,
                             double* WA, double* Wb, int32_t* status, void* stream);

/*
 * Model.compute_fit (model.py:571-606) for nfit independent problems:
 * coef_ev [nfit][6], the least-squares solution of WA c = Wb (WA [nfit][nobs][6],
 * Wb [nfit][nobs]), and coef_cov [nfit][36] = inv(WA^T WA), FP64 normal
 * equations with a Jacobi-scaled Cholesky factor (one warp per problem).
 * status [nfit] (may be NULL): ONEKA_REAL_OK, ONEKA_REAL_NOT_SPD (the
 * reference's LinAlgError), or ONEKA_REAL_NOT_FINITE for a non-finite row.
 */
ONEKA_API int oneka_fit_solve(const double* WA, const double* Wb, int32_t nobs, int32_t nfit, double* coef_ev,
                              double* coef_cov, int32_t* status, void* stream);

/* Bytes of scratch oneka_track needs for `slots` realizations in flight. */
ONEKA_API size_t oneka_track_scratch_bytes(const OnekaGrid* grid, int32_t slots);

/*
 * Backtrack npaths particles for each realization and chronicle the traces.
 *   capturezone.py:51-253 (release ring given as `release` [npaths][2];
 *   Dormand-Prince 5(4) with the reference's step control), model.py:207-427
 *   (velocity), probabilityfield.py:264-372 (rasterize within umbra,
 *   per-realization OR, register with weight 1).
 *   counts [nrows][ncols] int32 is incremented once per realization for each
 *   node any of its traces marks; `registered` (int64, may be NULL) is
 *   incremented once per realization tracked (status ONEKA_REAL_OK).
 *   frames: [nreal][npaths] or NULL (every trace against `grid`).
 *   scratch (16-byte aligned) holds realization slots of
 *   oneka_track_scratch_bytes(grid, 1) bytes each (a bitmask of
 *   ceil(ncols/32) words per row plus a small header).  It must be all
 *   zero on entry (zero it once after allocating it):
 *     counts != NULL: working slots, at least one; more slots let more
 *       realizations run per launch.  Every slot used is zero again on
 *       return, so the same scratch serves the next call as it is.
 *     counts == NULL, scratch != NULL ("mark only"): realization k ORs its
 *       traces into slot k (nreal slots needed); nothing is cleared or
 *       registered, so the caller can register with a weight
 *       (oneka_register_weighted).
 *     both NULL: tracking only, for the per-particle outputs.
 */
ONEKA_API int oneka_track(const OnekaSite* site, const OnekaRealizations* real, int32_t nreal,
                const double* release, int32_t npaths, const OnekaTrackOpts* opts,
                const OnekaGrid* grid, const OnekaFrame* frames, int32_t* counts,
                int64_t* registered, const OnekaTrackOut* out, void* scratch,
                size_t scratch_bytes, void* stream);

/* One site of a batched launch (oneka_track_batched); pointers to structs are host pointers. */
typedef struct OnekaTrackJob {
    const OnekaSite* site;
    const OnekaRealizations* real;
    int32_t nreal, npaths;
    const double* release;           /* device [npaths][2] */
    const OnekaTrackOpts* opts;      /* precision must be ONEKA_FP32; block/occupancy of job 0 apply to all */
    const OnekaGrid* grid;
    int32_t* counts;                 /* device [nrows][ncols] int32 */
    int64_t* registered;             /* device, may be NULL */
    const OnekaTrackOut* out;        /* may be NULL */
} OnekaTrackJob;

/* Scratch bytes oneka_track_batched needs to run every realization of the jobs in one wave. */
ONEKA_API size_t oneka_track_batched_scratch_bytes(const OnekaTrackJob* jobs, int32_t njobs);

/*
 * Many sites in one launch (FP32 build): every realization of every job --
 * sites with uneven well counts, npaths, durations, grids, confined or not --
 * is a block row of one persistent tracking kernel whose lanes refill from
 * their realization's particles, followed by one register kernel.  Rows are
 * packed into waves that fit `scratch` (zero on entry, zero on return, like
 * oneka_track).  Up to 80 jobs form one launch; more jobs run as further
 * launches.  Each job's semantics are those of oneka_track with the same
 * arguments.  No host synchronization; capturable in a CUDA graph.
 */
ONEKA_API int oneka_track_batched(const OnekaTrackJob* jobs, int32_t njobs, void* scratch,
                                  size_t scratch_bytes, void* stream);

/* Size of the fixed scratch array inside the library that oneka_track_noalloc uses. */
#define ONEKA_NOALLOC_SCRATCH_BYTES (32u << 20)

/*
 * oneka_track for callers that cannot allocate device memory.  No counterpart
 * in the reference: it exists for hosts that cannot call cudaMalloc -- a
 * plugin whose device memory the host's own allocator has already divided
 * up, or a binding that can only pass buffers the host owns.  It takes the
 * same arguments as oneka_track minus the scratch, which comes from a
 * file-scope array of ONEKA_NOALLOC_SCRATCH_BYTES (32 MiB) inside the library,
 * held by every GPU that loads the library until the process exits.
 *   - Inputs and outputs are still the caller's device buffers.
 *   - A grid whose realization slot (oneka_track_scratch_bytes(grid, 1))
 *     exceeds 32 MiB is rejected with ONEKA_ERR_SCRATCH; smaller grids run
 *     32 MiB / slot realizations per launch.
 *   - The call allocates nothing: no cudaMalloc/cudaFree, no allocating
 *     library routine.
 *   - Every call on a device shares the array and clears the part it uses
 *     first; calls that overlap on the GPU (other streams or threads) race on
 *     it, so order them on one stream.
 *   - The array is reserved on a device when the library's device code is
 *     first loaded there, i.e. at the first call on that device, not when the
 *     library is loaded.  A host whose own allocator takes the GPU after its
 *     set-up should make one call during that set-up.
 *   - The first call on each device (with that device current) looks up the
 *     array's device address and caches it; make that first call before any
 *     stream capture.  A cudaDeviceReset invalidates the cached address: it
 *     is not supported while the library is in use.
 */
ONEKA_API int oneka_track_noalloc(const OnekaSite* site, const OnekaRealizations* real, int32_t nreal,
                                  const double* release, int32_t npaths, const OnekaTrackOpts* opts,
                                  const OnekaGrid* grid, const OnekaFrame* frames, int32_t* counts,
                                  int64_t* registered, const OnekaTrackOut* out, void* stream);

/*
 * Model evaluation at npts points (model.py:207-427): potential, discharge
 * [npts][2], head, velocity [npts][2] (general when confined == 0, else the
 * confined shortcut) and status (ONEKA_TRACE_DRY where the reference raises
 * AquiferError).  Any output may be NULL.  coef is host [6].
 */
ONEKA_API int oneka_evaluate(const OnekaSite* site, const double* q, double conductivity, double porosity,
                   double thickness, const double* coef, const double* points, int64_t npts,
                   int32_t confined, double* potential, double* discharge, double* head,
                   double* velocity, int32_t* status, void* stream);

/*
 * ProbabilityField.rasterize (probabilityfield.py:313-339) without expand:
 * OR the nodes within umbra of the polyline xy [n][2] into `mask`, a
 * realization bitmask of oneka_track_scratch_bytes(grid, 1) bytes
 * (row-major, ceil(ncols/32) words per row).  frame may be NULL.
 */
ONEKA_API int oneka_rasterize(const OnekaGrid* grid, const OnekaFrame* frame, const double* xy, int64_t n,
                    double umbra, uint32_t* mask, void* stream);

/*
 * ProbabilityField.register (probabilityfield.py:357-359) for one bitmask:
 * pgrid[marked] += weight, then the mask is cleared.
 */
ONEKA_API int oneka_register_weighted(const OnekaGrid* grid, uint32_t* mask, double weight, double* pgrid,
                            void* stream);

/*
 * Smoothed capture probability (oneka/visualize.py:232-233,
 * scipy.ndimage.gaussian_filter(Z, smooth, mode='constant', cval=0)): two
 * separable FP64 passes (columns, then rows) with zero padding.  weights:
 * device [2*radius+1], normalized; tmp: a caller buffer like out.
 */
ONEKA_API int oneka_gaussian_filter(const double* in, double* out, double* tmp, int32_t nrows,
                                    int32_t ncols, const double* weights, int32_t radius, void* stream);

/*
 * Histogram of integer visit counts (values clamped to [0, nbins - 1]),
 * added into hist (uint64 [nbins]).  The impact curve of
 * oneka/visualize.py:382-385 (probabilities sorted in decreasing order
 * against cumulative area) and the decile table of oneka/oneka.py:278-288
 * follow from its cumulative sums, since every probability is count / R.
 */
ONEKA_API int oneka_count_histogram(const int32_t* counts, int64_t n, int32_t nbins, uint64_t* hist,
                                    void* stream);

/* ---------------------------------------------------------------------- */
/* Learned surrogate (no counterpart in the reference): an MLP from a
 * realization's parameters (A..F, discharges, K, porosity) to per-cell
 * capture logits, trained on the tracker's own per-realization masks.
 * BF16 operands, FP32 accumulation, FP32 master weights.  All arrays are
 * device memory; bf16 arrays are raw 16-bit words. */

/*
 * C[M][N] = A . B (+ bias[N]) (then GELU) on the tensor cores, FP32
 * accumulate.  A is [M][lda] when a_kmajor, else [K][lda] (A^T stored
 * row-major); B is [N][ldb] when b_kmajor, else [K][ldb].  C is FP32 when
 * c_f32, else BF16.  Z (optional, BF16, ldc) receives the pre-activation.
 * K % 32 == 0; lda, ldb, ldc % 8 == 0; matrices and bias 16-byte aligned.  splitk > 1 adds
 * partial products into a zeroed FP32 C (no GELU, no Z).
 *
 * K-major A and B with K % 64 == 0 run on the tcgen05 kernel (TMA-staged
 * operands, accumulator in tensor memory; FP32 C, also split-K, or BF16 C
 * with GELU and Z); everything else on an mma.sync kernel.  An output with
 * an even number of 128-row tiles runs on clusters of two CTAs that share
 * each B slice by TMA multicast.  flags bit 0 forces the mma.sync kernel;
 * bit 1 keeps the tcgen05 kernel to one CTA per tile.
 */
ONEKA_API int oneka_gemm_bf16(const void* A, int32_t lda, int32_t a_kmajor, const void* B, int32_t ldb,
                              int32_t b_kmajor, void* C, int32_t ldc, int32_t c_f32, const float* bias,
                              int32_t gelu, void* Z, int32_t M, int32_t N, int32_t K, int32_t splitk,
                              int32_t flags, void* stream);

/* dst[c][r] = src[r][c] for a BF16 matrix src [rows][lds] into dst [cols][ldd]: the backward
 * GEMMs' operands turned K-major for the tcgen05 kernel. */
ONEKA_API int oneka_transpose_bf16(const void* src, int32_t rows, int32_t cols, int64_t lds, void* dst, int64_t ldd,
                                   void* stream);

/* 1 when oneka_gemm_bf16 with these arguments runs on the tcgen05 kernel, else 0 (host only). */
ONEKA_API int oneka_gemm_bf16_path(int32_t a_kmajor, int32_t b_kmajor, int32_t K, int32_t splitk, int32_t c_f32,
                                   int32_t gelu, int32_t has_z, int32_t sigsum, int32_t flags);

/*
 * The tcgen05 kernel's device status: *code = 0, or 1 when a wait inside it
 * timed out (the kernel then skipped its stores); reading clears it.
 * Synchronizes the device.
 */
ONEKA_API int oneka_gemm_tc_status(int32_t* code);

/*
 * out[n] += sum over m of sigmoid((A B^T)[m][n] + bias[n]) for k-major A [M][lda]
 * and B [N][ldb] (BF16): the surrogate's last layer fused with the sum of its
 * capture probabilities over realizations; the logits are never stored.
 */
ONEKA_API int oneka_gemm_bf16_sigmoid_colsum(const void* A, int32_t lda, const void* B, int32_t ldb,
                                             const float* bias, float* out, int32_t M, int32_t N, int32_t K,
                                             int32_t flags, void* stream);

/*
 * Binary cross-entropy of logits [B][ncells] (FP32) against chronicle masks
 * (sample b's bits at masks + b * slot_words, wpr words per grid row):
 * loss += scale * sum(bce); dlogits (BF16, optional) = scale * (sigmoid - y).
 */
ONEKA_API int oneka_bce_bitmask(const float* logits, const uint32_t* masks, int64_t slot_words, int32_t wpr,
                                int32_t ncols, int32_t B, int32_t ncells, float scale, void* dlogits,
                                float* loss, void* stream);

/* dz = dh * GELU'(z): dh FP32, z and dz BF16, n elements. */
ONEKA_API int oneka_gelu_backward(const float* dh, const void* z, void* dz, int64_t n, void* stream);

/* out[c] = sum over rows of x[r][c], x BF16 [rows][cols]. */
ONEKA_API int oneka_colsum_bf16(const void* x, int32_t rows, int32_t cols, float* out, void* stream);

/* AdamW step `step` (>= 1) on FP32 w, m, v with gradient g; writes the BF16 copy w_bf16 if given. */
ONEKA_API int oneka_adamw(float* w, float* m, float* v, const float* g, void* w_bf16, int64_t n, float lr,
                          float beta1, float beta2, float eps, float weight_decay, int32_t step, void* stream);

/* oneka_adamw with the step's learning rate and bias corrections read from device memory,
 * hyper = [lr, 1 - beta1^t, 1 - beta2^t], so that a training step captured in a CUDA graph
 * follows a schedule written into hyper between replays. */
ONEKA_API int oneka_adamw_scheduled(float* w, float* m, float* v, const float* g, void* w_bf16, int64_t n,
                                    const float* hyper, float beta1, float beta2, float eps, float weight_decay,
                                    void* stream);

/*
 * oneka_bce_bitmask that also writes the gradient transposed, dlogits_t
 * [ncells][ldt] (BF16), for the weight-gradient GEMM's K-major operand.
 * ncols and B multiples of 64, ldt a multiple of 8 and >= B.
 */
ONEKA_API int oneka_bce_bitmask_t(const float* logits, const uint32_t* masks, int64_t slot_words, int32_t wpr,
                                  int32_t ncols, int32_t B, int32_t ncells, float scale, void* dlogits,
                                  void* dlogits_t, int64_t ldt, float* loss, void* stream);

/*
 * oneka_adamw_scheduled for a weight matrix w [rows][cols] that also writes
 * the BF16 copy transposed, w_bf16_t [cols][ldt], for the backward pass's
 * K-major operand.  rows and cols multiples of 64, ldt a multiple of 8 and
 * >= rows.
 */
ONEKA_API int oneka_adamw_scheduled_t(float* w, float* m, float* v, const float* g, void* w_bf16, void* w_bf16_t,
                                      int64_t ldt, int32_t rows, int32_t cols, const float* hyper, float beta1,
                                      float beta2, float eps, float weight_decay, void* stream);

/* Standardized BF16 features [n][ld] of realizations: A..F, discharges, K, porosity (nf = 8 + nwells). */
ONEKA_API int oneka_features(const double* coef, const double* q, const double* aquifer, int32_t nwells,
                             int32_t n, const float* mean, const float* inv_std, int32_t nf, int32_t ld,
                             void* x, void* stream);

/* out[c] += sum over rows of sigmoid(logits[r][c]) (logits FP32 [rows][cols]). */
ONEKA_API int oneka_sigmoid_colsum(const float* logits, int32_t rows, int32_t cols, float* out, void* stream);

/*
 * Measurement helper (no reference counterpart): sustained FMA throughput of
 * this GPU in FLOP/s for FP32 (fp64 == 0) or FP64 (fp64 != 0), from a
 * register-resident FMA loop over every SM.  Synchronizes `stream`.
 */
ONEKA_API int oneka_fma_peak(int32_t fp64, double* flops_per_s, void* stream);

/* ProbabilityField.distancesquared (probabilityfield.py:380-427) for n queries [n][6]. */
ONEKA_API int oneka_distancesquared(const double* abc, double* d2, int64_t n, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* ONEKA_GB300_H */
