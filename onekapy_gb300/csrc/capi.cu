// capi.cu -- extern "C" entry points of liboneka_gb300.so (include/oneka_gb300.h).
#include <math.h>
#include <stdarg.h>

#include <algorithm>
#include <memory>
#include <vector>
#include <stdio.h>
#include <string.h>

#include "oneka_internal.cuh"

namespace oneka {

cudaError_t launch_realize(const OnekaSite& site, const OnekaDist* qdist, const OnekaDist* adist,
                           const double* logr2, unsigned long long seed, unsigned long long first,
                           int nreal, int mode, const OnekaRealizations& out, cudaStream_t s);
cudaError_t launch_logr2(const OnekaSite& site, double* logr2, cudaStream_t s);
cudaError_t launch_fit_rows(const OnekaSite& site, const double* q, double K, double H, double* WA, double* Wb,
                            int32_t* status, cudaStream_t s);
cudaError_t launch_fit_solve(const double* WA, const double* Wb, int nobs, int nfit, double* coef_ev,
                             double* coef_cov, int32_t* status, cudaStream_t s);
cudaError_t launch_register_weighted(uint32_t* mask, const OnekaGrid& g, double weight, double* pgrid,
                                     cudaStream_t s);
cudaError_t launch_rasterize(const OnekaGrid& g, const OnekaFrame& f, const double* xy, long long n,
                             double umbra, uint32_t* mask, cudaStream_t s);
cudaError_t launch_distancesquared(const double* abc, double* d2, long long n, cudaStream_t s);
cudaError_t probe_fma(int fp64, double* flops_per_s, cudaStream_t s);
cudaError_t launch_gaussian(const double* in, double* out, double* tmp, int nrows, int ncols, const double* w,
                            int radius, cudaStream_t s);
cudaError_t launch_histogram(const int32_t* counts, long long n, int nbins, unsigned long long* hist,
                             cudaStream_t s);
cudaError_t launch_gemm_bf16(const void* A, int lda, int a_kmajor, const void* B, int ldb, int b_kmajor, void* C,
                             int ldc, int c_f32, const float* bias, int gelu, void* Z, int M, int N, int K,
                             int splitk, float* sigsum, int flags, cudaStream_t s);
int gemm_path(int a_kmajor, int b_kmajor, int K, int splitk, int c_f32, int gelu, void* Z, float* sigsum, int flags);
cudaError_t gemm_tc_take_error(int* code);
cudaError_t launch_bce_bitmask(const float* logits, const uint32_t* masks, long long slot_words, int wpr, int ncols,
                               int B, int ncells, float scale, void* dlogits, float* loss, cudaStream_t s);
cudaError_t launch_gelu_backward(const float* dh, const void* z, void* dz, long long n, cudaStream_t s);
cudaError_t launch_colsum(const void* x, int rows, int cols, float* out, cudaStream_t s);
cudaError_t launch_adamw(float* w, float* m, float* v, const float* g, void* wb, long long n, float lr, float b1,
                         float b2, float eps, float wd, int step, cudaStream_t s);
cudaError_t launch_features(const double* coef, const double* q, const double* aquifer, int nwells, int n,
                            const float* mean, const float* inv_std, int nf, int ld, void* x, cudaStream_t s);
cudaError_t launch_sigmoid_colsum(const float* logits, int rows, int cols, float* out, cudaStream_t s);
cudaError_t launch_transpose_bf16(const void* src, int rows, int cols, long long lds, void* dst, long long ldd,
                                  cudaStream_t s);
cudaError_t launch_adamw_scheduled(float* w, float* m, float* v, const float* g, void* wb, long long n,
                                   const float* hyper, float b1, float b2, float eps, float wd, cudaStream_t s);
cudaError_t launch_bce_bitmask_t(const float* logits, const uint32_t* masks, long long slot_words, int wpr,
                                 int ncols, int B, int ncells, float scale, void* dlogits, void* dlogits_t,
                                 long long ldt, float* loss, cudaStream_t s);
cudaError_t launch_adamw_t(float* w, float* m, float* v, const float* g, void* wb, void* wbt, long long ldt, int rows,
                           int cols, const float* hyper, float b1, float b2, float eps, float wd, cudaStream_t s);

cudaError_t launch_evaluate(const OnekaSite& site, const double* q, double K, double n, double H,
                            const double* coef, const double* pts, long long npts, int confined,
                            double* potential, double* discharge, double* head, double* velocity,
                            int32_t* status, cudaStream_t s);

static thread_local char g_err[512];

void set_error(const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
}

}  // namespace oneka

using namespace oneka;

#define ONEKA_CHECK_ARG(cond, msg)          \
    do {                                    \
        if (!(cond)) {                      \
            set_error("invalid argument: %s", msg); \
            return ONEKA_ERR_INVALID;       \
        }                                   \
    } while (0)

#define ONEKA_CHECK_CUDA(expr)                                                  \
    do {                                                                        \
        cudaError_t e_ = (expr);                                                \
        if (e_ != cudaSuccess) {                                                \
            set_error("%s: %s", #expr, cudaGetErrorString(e_));                \
            return ONEKA_ERR_CUDA;                                              \
        }                                                                       \
    } while (0)

static bool grid_ok(const OnekaGrid* g) {
    return g && g->nrows > 0 && g->ncols > 0 && g->dx > 0 && g->dy > 0;
}

// The shared-memory chronicle window: the whole grid when it fits the
// budget, else a window about square in nodes centred on the regional origin
// (the target well), where traces start and overlap most.
static void set_window(TrackLaunch& L, const OnekaGrid& g, int window_kb) {
    L.win_r0 = L.win_w0 = L.win_rows = L.win_words = 0;
    if (window_kb < 0) return;
    const long long budget = (long long)(window_kb == 0 ? 32 : window_kb) * 256;   // words
    const int wpr = words_per_row(g.ncols);
    if ((long long)g.nrows * wpr <= budget) {
        L.win_rows = g.nrows;
        L.win_words = wpr;
        return;
    }
    int ww = 1;
    while ((long long)(ww + 1) * (ww + 1) * 32 <= budget) ++ww;
    if (ww > wpr) ww = wpr;
    long long wr = budget / ww;
    if (wr > g.nrows) wr = g.nrows;
    const int row_t = (int)floor((L.yt - g.ymin) / g.dy + 0.5);
    const int col_t = (int)floor((L.xt - g.xmin) / g.dx + 0.5);
    int r0 = row_t - (int)(wr / 2), w0 = (col_t >> 5) - ww / 2;
    if (r0 > g.nrows - (int)wr) r0 = g.nrows - (int)wr;
    if (r0 < 0) r0 = 0;
    if (w0 > wpr - ww) w0 = wpr - ww;
    if (w0 < 0) w0 = 0;
    L.win_r0 = r0;
    L.win_w0 = w0;
    L.win_rows = (int)wr;
    L.win_words = ww;
}

// Argument checks shared by oneka_track and oneka_track_batched.
static int check_track_args(const OnekaSite* site, const OnekaRealizations* real, int32_t nreal,
                            const double* release, int32_t npaths, const OnekaTrackOpts* opts,
                            const OnekaGrid* grid, const OnekaTrackOut* out) {
    ONEKA_CHECK_ARG(site && real && opts && grid, "site/real/opts/grid");
    ONEKA_CHECK_ARG(grid_ok(grid), "grid (nrows, ncols, dx, dy must be > 0)");
    ONEKA_CHECK_ARG(nreal >= 0 && npaths >= 0, "nreal/npaths");
    ONEKA_CHECK_ARG(npaths == 0 || release, "release");
    ONEKA_CHECK_ARG(site->nwells >= 1 && site->nwells <= 2048 && site->wells, "wells (1..2048)");
    ONEKA_CHECK_ARG(site->target >= 0 && site->target < site->nwells, "target index");
    ONEKA_CHECK_ARG(real->coef && real->q && real->aquifer, "realization arrays");
    ONEKA_CHECK_ARG(opts->precision == ONEKA_FP64 || opts->precision == ONEKA_FP32, "precision");
    ONEKA_CHECK_ARG(opts->tol > 0 && opts->maxstep > 0 && opts->umbra >= 0, "tol/maxstep/umbra");
    ONEKA_CHECK_ARG(opts->block == 0 || opts->block == 32 || opts->block == 64 || opts->block == 128 ||
                    opts->block == 256, "block must be 32, 64, 128 or 256");
    ONEKA_CHECK_ARG(!out || out->max_vertices >= 0, "max_vertices");
    ONEKA_CHECK_ARG(!out || !out->vertices || out->max_vertices > 0, "vertices without max_vertices");
    return ONEKA_OK;
}

static void fill_launch(TrackLaunch& L, const OnekaSite* site, const OnekaRealizations* real,
                        const double* release, int32_t npaths, const OnekaTrackOpts* opts,
                        const OnekaGrid* grid, const OnekaFrame* frames, int64_t* registered,
                        const OnekaTrackOut* out) {
    memset(&L, 0, sizeof(L));
    L.nwells = site->nwells;
    L.npaths = npaths;
    L.wells = site->wells;
    L.xo = site->xo;
    L.yo = site->yo;
    // The regional origin anchors the FP32 build's relative coordinates (the
    // stochastic driver puts it on the target well).
    L.xt = site->xo;
    L.yt = site->yo;
    L.coef = real->coef;
    L.q = real->q;
    L.aquifer = real->aquifer;
    L.rstatus = real->status;
    L.release = release;
    L.opts = *opts;
    L.grid = *grid;
    L.frames = frames;
    L.wpr = words_per_row(grid->ncols);
    L.slot_words = slot_words(*grid);
    L.mask_words = mask_words(*grid);
    L.registered = (unsigned long long*)registered;
    if (out) L.out = *out;
    L.max_attempts = opts->max_attempts > 0 ? opts->max_attempts : kDefaultMaxAttempts;
    set_window(L, *grid, opts->window_kb);
}

extern "C" {

int oneka_abi_version(void) { return ONEKA_ABI_VERSION; }

const char* oneka_last_error(void) { return g_err; }

int oneka_site_logr2(const OnekaSite* site, double* logr2, void* stream) {
    g_err[0] = 0;
    ONEKA_CHECK_ARG(site && logr2, "site/logr2");
    ONEKA_CHECK_ARG(site->nwells >= 0 && site->nobs >= 0, "sizes");
    ONEKA_CHECK_ARG(site->nobs == 0 || (site->obs && site->wells), "site arrays");
    ONEKA_CHECK_CUDA(launch_logr2(*site, logr2, (cudaStream_t)stream));
    return ONEKA_OK;
}

int oneka_realize(const OnekaSite* site, const OnekaDist* qdist, const OnekaDist* adist,
                  const double* logr2, uint64_t seed, uint64_t first, int32_t nreal, int32_t mode,
                  OnekaRealizations* out, void* stream) {
    g_err[0] = 0;
    ONEKA_CHECK_ARG(site && out && adist, "site/out/adist");
    ONEKA_CHECK_ARG(nreal >= 0, "nreal");
    ONEKA_CHECK_ARG(mode >= ONEKA_MODE_STOCHASTIC && mode <= ONEKA_MODE_GIVEN_EV, "mode");
    ONEKA_CHECK_ARG(site->nwells >= 1 && site->nwells <= 4096, "nwells must be in [1, 4096]");
    ONEKA_CHECK_ARG(site->nobs >= 0 && (site->nobs == 0 || site->obs), "observations");
    ONEKA_CHECK_ARG(site->wells, "wells");
    ONEKA_CHECK_ARG(out->coef && out->q && out->aquifer, "out->coef/q/aquifer");
    ONEKA_CHECK_ARG(mode == ONEKA_MODE_GIVEN || mode == ONEKA_MODE_GIVEN_EV || qdist, "qdist");
    for (int a = 0; a < 3; ++a)
        ONEKA_CHECK_ARG(adist[a].kind >= ONEKA_DIST_CONST && adist[a].kind <= ONEKA_DIST_LOGNORMAL,
                        "adist kind");
    ONEKA_CHECK_CUDA(launch_realize(*site, qdist, adist, logr2, seed, first, nreal, mode, *out,
                                    (cudaStream_t)stream));
    return ONEKA_OK;
}

int oneka_fit_rows(const OnekaSite* site, const double* q, double conductivity, double thickness, double* WA,
                   double* Wb, int32_t* status, void* stream) {
    g_err[0] = 0;
    ONEKA_CHECK_ARG(site && status, "site/status");
    ONEKA_CHECK_ARG(site->nwells >= 0 && (site->nwells == 0 || (site->wells && q)), "wells/q");
    ONEKA_CHECK_ARG(site->nobs >= 0 && (site->nobs == 0 || (site->obs && WA && Wb)), "observations/WA/Wb");
    ONEKA_CHECK_CUDA(cudaMemsetAsync(status, 0, sizeof(int32_t), (cudaStream_t)stream));
    ONEKA_CHECK_CUDA(launch_fit_rows(*site, q, conductivity, thickness, WA, Wb, status, (cudaStream_t)stream));
    return ONEKA_OK;
}

int oneka_fit_solve(const double* WA, const double* Wb, int32_t nobs, int32_t nfit, double* coef_ev,
                    double* coef_cov, int32_t* status, void* stream) {
    g_err[0] = 0;
    ONEKA_CHECK_ARG(nobs >= 0 && nfit >= 0, "nobs/nfit");
    ONEKA_CHECK_ARG(nfit == 0 || (coef_ev && coef_cov), "coef_ev/coef_cov");
    ONEKA_CHECK_ARG(nfit == 0 || nobs == 0 || (WA && Wb), "WA/Wb");
    ONEKA_CHECK_CUDA(launch_fit_solve(WA, Wb, nobs, nfit, coef_ev, coef_cov, status, (cudaStream_t)stream));
    return ONEKA_OK;
}

size_t oneka_track_scratch_bytes(const OnekaGrid* grid, int32_t slots) {
    if (!grid_ok(grid) || slots < 0) return 0;
    return (size_t)slot_words(*grid) * 4u * (size_t)slots;
}

int oneka_track(const OnekaSite* site, const OnekaRealizations* real, int32_t nreal,
                const double* release, int32_t npaths, const OnekaTrackOpts* opts,
                const OnekaGrid* grid, const OnekaFrame* frames, int32_t* counts,
                int64_t* registered, const OnekaTrackOut* out, void* scratch,
                size_t scratch_bytes, void* stream) {
    g_err[0] = 0;
    const int rc = check_track_args(site, real, nreal, release, npaths, opts, grid, out);
    if (rc != ONEKA_OK) return rc;
    if (nreal == 0) return ONEKA_OK;

    cudaStream_t s = (cudaStream_t)stream;
    TrackLaunch L;
    fill_launch(L, site, real, release, npaths, opts, grid, frames, registered, out);

    int wave = nreal < 65535 ? nreal : 65535;
    if (!counts && scratch) {
        // mark-only: realization k ORs its traces into slot k of scratch; no
        // clearing and no register (the caller registers, e.g. with weights)
        const size_t need = (size_t)L.slot_words * 4u * (size_t)nreal;
        if (scratch_bytes < need) {
            set_error("mark-only scratch of %zu bytes is smaller than %d slots (%zu bytes)",
                      scratch_bytes, nreal, need);
            return ONEKA_ERR_SCRATCH;
        }
        ONEKA_CHECK_ARG(((uintptr_t)scratch & 15u) == 0, "scratch must be 16-byte aligned");
        L.slots = (uint32_t*)scratch;
        for (int r0 = 0; r0 < nreal; r0 += wave) {
            L.r0 = r0;
            L.nr = (nreal - r0) < wave ? (nreal - r0) : wave;
            TrackLaunch Lw = L;
            Lw.slots = L.slots + (long long)r0 * L.slot_words;
            ONEKA_CHECK_CUDA(opts->precision == ONEKA_FP64 ? launch_track64(Lw, s) : launch_track32(Lw, s));
        }
        return ONEKA_OK;
    }
    if (counts) {
        const size_t slot_bytes = (size_t)L.slot_words * 4u;
        ONEKA_CHECK_ARG(scratch != nullptr, "scratch is required when counts is given");
        if (scratch_bytes < slot_bytes) {
            set_error("scratch of %zu bytes is smaller than one realization slot (%zu bytes)",
                      scratch_bytes, slot_bytes);
            return ONEKA_ERR_SCRATCH;
        }
        ONEKA_CHECK_ARG(((uintptr_t)scratch & 15u) == 0, "scratch must be 16-byte aligned");
        const size_t fit = scratch_bytes / slot_bytes;
        if ((size_t)wave > fit) wave = (int)fit;
        L.slots = (uint32_t*)scratch;
    }
    for (int r0 = 0; r0 < nreal; r0 += wave) {
        L.r0 = r0;
        L.nr = (nreal - r0) < wave ? (nreal - r0) : wave;
        ONEKA_CHECK_CUDA(opts->precision == ONEKA_FP64 ? launch_track64(L, s) : launch_track32(L, s));
        if (counts) ONEKA_CHECK_CUDA(launch_register_counts(L.slots, L.nr, *grid, counts, s));
    }
    return ONEKA_OK;
}

static size_t align256(size_t v) { return (v + 255) & ~(size_t)255; }

size_t oneka_track_batched_scratch_bytes(const OnekaTrackJob* jobs, int32_t njobs) {
    if (!jobs || njobs < 0) return 0;
    size_t total = 0;
    for (int j = 0; j < njobs; ++j) {
        if (!jobs[j].grid || !grid_ok(jobs[j].grid) || jobs[j].nreal < 0) return 0;
        total += align256((size_t)slot_words(*jobs[j].grid) * 4u * (size_t)jobs[j].nreal);
    }
    return total;
}

int oneka_track_batched(const OnekaTrackJob* jobs, int32_t njobs, void* scratch, size_t scratch_bytes,
                        void* stream) {
    g_err[0] = 0;
    ONEKA_CHECK_ARG(jobs && njobs >= 0, "jobs");
    ONEKA_CHECK_ARG(scratch && ((uintptr_t)scratch & 255u) == 0, "scratch must be 256-byte aligned");
    for (int j = 0; j < njobs; ++j) {
        const OnekaTrackJob& J = jobs[j];
        const int rc = check_track_args(J.site, J.real, J.nreal, J.release, J.npaths, J.opts, J.grid, J.out);
        if (rc != ONEKA_OK) return rc;
        ONEKA_CHECK_ARG(J.opts->precision == ONEKA_FP32, "batched launches run the FP32 build");
        ONEKA_CHECK_ARG(!J.opts->head64, "batched launches do not take head64");
        ONEKA_CHECK_ARG(J.counts, "counts");
    }
    cudaStream_t s = (cudaStream_t)stream;
    std::unique_ptr<JobTable> T(new JobTable());
    int n = 0, rows = 0;
    size_t off = 0;
    auto flush = [&]() -> int {
        if (n == 0) return ONEKA_OK;
        T->first[n] = rows;
        T->njobs = n;
        ONEKA_CHECK_CUDA(launch_track32_batch(*T, rows, s));
        ONEKA_CHECK_CUDA(launch_register_batch(*T, rows, s));
        n = rows = 0;
        off = 0;
        return ONEKA_OK;
    };
    // costliest jobs first: their blocks are dispatched first, and the cheap
    // ones fill the tail (realizations x paths x well terms x duration)
    std::vector<int> order(njobs);
    for (int j = 0; j < njobs; ++j) order[j] = j;
    auto cost = [&](int j) {
        const OnekaTrackJob& J = jobs[j];
        return (double)J.nreal * (double)J.npaths * (double)(J.site->nwells + 8) * fabs(J.opts->duration);
    };
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return cost(a) > cost(b); });
    constexpr int kMaxRows = 1 << 30;
    for (int jj = 0; jj < njobs; ++jj) {
        const OnekaTrackJob& J = jobs[order[jj]];
        TrackLaunch base;
        fill_launch(base, J.site, J.real, J.release, J.npaths, J.opts, J.grid, nullptr, J.registered, J.out);
        base.counts = J.counts;
        // every job shares job 0's launch shape
        base.opts.block = jobs[0].opts->block;
        base.opts.occupancy = jobs[0].opts->occupancy;
        const size_t slot = (size_t)base.slot_words * 4u;
        int r = 0;
        while (r < J.nreal) {
            const size_t room = off < scratch_bytes ? (scratch_bytes - off) / slot : 0;
            if (room == 0 || n == kMaxJobs || rows == kMaxRows) {
                if (n == 0) {
                    set_error("scratch of %zu bytes is smaller than one realization slot (%zu bytes)",
                              scratch_bytes, slot);
                    return ONEKA_ERR_SCRATCH;
                }
                const int rc = flush();
                if (rc != ONEKA_OK) return rc;
                continue;
            }
            int take = J.nreal - r;
            if ((size_t)take > room) take = (int)room;
            if (take > kMaxRows - rows) take = kMaxRows - rows;
            TrackLaunch& L = T->job[n];
            L = base;
            L.r0 = r;
            L.nr = take;
            L.slots = (uint32_t*)((char*)scratch + off);
            T->first[n] = rows;
            ++n;
            rows += take;
            off = align256(off + (size_t)take * slot);
            r += take;
        }
    }
    return flush();
}

int oneka_evaluate(const OnekaSite* site, const double* q, double conductivity, double porosity,
                   double thickness, const double* coef, const double* points, int64_t npts,
                   int32_t confined, double* potential, double* discharge, double* head,
                   double* velocity, int32_t* status, void* stream) {
    g_err[0] = 0;
    ONEKA_CHECK_ARG(site && coef && (npts == 0 || points), "site/coef/points");
    ONEKA_CHECK_ARG(site->nwells >= 0 && (site->nwells == 0 || (site->wells && q)), "wells/q");
    ONEKA_CHECK_ARG(npts >= 0, "npts");
    ONEKA_CHECK_CUDA(launch_evaluate(*site, q, conductivity, porosity, thickness, coef, points, npts,
                                     confined, potential, discharge, head, velocity, status,
                                     (cudaStream_t)stream));
    return ONEKA_OK;
}

int oneka_rasterize(const OnekaGrid* grid, const OnekaFrame* frame, const double* xy, int64_t n,
                    double umbra, uint32_t* mask, void* stream) {
    g_err[0] = 0;
    ONEKA_CHECK_ARG(grid_ok(grid) && mask && n >= 0 && (n == 0 || xy), "grid/mask/xy");
    ONEKA_CHECK_ARG(umbra >= 0, "umbra");
    OnekaFrame f;
    if (frame) {
        f = *frame;
    } else {
        f.xmin = grid->xmin;
        f.ymin = grid->ymin;
        f.coff = f.roff = 0;
        f.ncols = grid->ncols;
        f.nrows = grid->nrows;
    }
    ONEKA_CHECK_CUDA(launch_rasterize(*grid, f, xy, n, umbra, mask, (cudaStream_t)stream));
    return ONEKA_OK;
}

int oneka_register_weighted(const OnekaGrid* grid, uint32_t* mask, double weight, double* pgrid,
                            void* stream) {
    g_err[0] = 0;
    ONEKA_CHECK_ARG(grid_ok(grid) && mask && pgrid, "grid/mask/pgrid");
    ONEKA_CHECK_CUDA(launch_register_weighted(mask, *grid, weight, pgrid, (cudaStream_t)stream));
    return ONEKA_OK;
}

int oneka_gaussian_filter(const double* in, double* out, double* tmp, int32_t nrows, int32_t ncols,
                          const double* weights, int32_t radius, void* stream) {
    g_err[0] = 0;
    ONEKA_CHECK_ARG(in && out && tmp && weights && nrows > 0 && ncols > 0, "in/out/tmp/weights/shape");
    ONEKA_CHECK_ARG(radius >= 0 && radius <= 4096, "radius");
    ONEKA_CHECK_ARG(in != tmp && out != tmp, "tmp must not alias in or out");
    ONEKA_CHECK_CUDA(launch_gaussian(in, out, tmp, nrows, ncols, weights, radius, (cudaStream_t)stream));
    return ONEKA_OK;
}

int oneka_count_histogram(const int32_t* counts, int64_t n, int32_t nbins, uint64_t* hist, void* stream) {
    g_err[0] = 0;
    ONEKA_CHECK_ARG(counts && hist && n >= 0 && nbins > 0 && nbins <= 12000, "counts/hist/n/nbins");
    ONEKA_CHECK_CUDA(launch_histogram(counts, n, nbins, (unsigned long long*)hist, (cudaStream_t)stream));
    return ONEKA_OK;
}

static bool al16(const void* p) { return ((uintptr_t)p & 15u) == 0; }

int oneka_gemm_bf16(const void* A, int32_t lda, int32_t a_kmajor, const void* B, int32_t ldb, int32_t b_kmajor,
                    void* C, int32_t ldc, int32_t c_f32, const float* bias, int32_t gelu, void* Z, int32_t M,
                    int32_t N, int32_t K, int32_t splitk, int32_t flags, void* stream) {
    g_err[0] = 0;
    ONEKA_CHECK_ARG(A && B && C && M > 0 && N > 0 && K > 0, "A/B/C/M/N/K");
    ONEKA_CHECK_ARG(K % 32 == 0, "K must be a multiple of 32");
    ONEKA_CHECK_ARG(lda % 8 == 0 && ldb % 8 == 0 && ldc % 8 == 0, "leading dimensions must be multiples of 8");
    ONEKA_CHECK_ARG(al16(A) && al16(B) && al16(C) && (!Z || al16(Z)) && (!bias || al16(bias)),
                    "16-byte aligned matrices and bias");
    ONEKA_CHECK_ARG(lda >= (a_kmajor ? K : M) && ldb >= (b_kmajor ? K : N) && ldc >= N, "leading dimensions");
    ONEKA_CHECK_ARG(splitk <= 1 || (c_f32 && !gelu && !Z), "split-K needs an FP32 output without GELU");
    ONEKA_CHECK_CUDA(launch_gemm_bf16(A, lda, a_kmajor, B, ldb, b_kmajor, C, ldc, c_f32, bias, gelu, Z, M, N, K,
                                      splitk, nullptr, flags, (cudaStream_t)stream));
    return ONEKA_OK;
}

int oneka_transpose_bf16(const void* src, int32_t rows, int32_t cols, int64_t lds, void* dst, int64_t ldd,
                         void* stream) {
    g_err[0] = 0;
    ONEKA_CHECK_ARG(src && dst && rows >= 0 && cols >= 0, "src/dst/rows/cols");
    ONEKA_CHECK_ARG(lds >= cols && ldd >= rows, "leading dimensions");
    ONEKA_CHECK_CUDA(launch_transpose_bf16(src, rows, cols, lds, dst, ldd, (cudaStream_t)stream));
    return ONEKA_OK;
}

int oneka_gemm_bf16_path(int32_t a_kmajor, int32_t b_kmajor, int32_t K, int32_t splitk, int32_t c_f32, int32_t gelu,
                         int32_t has_z, int32_t sigsum, int32_t flags) {
    return gemm_path(a_kmajor, b_kmajor, K, splitk, c_f32, gelu, has_z ? (void*)1 : nullptr,
                     sigsum ? (float*)1 : nullptr, flags);
}

int oneka_gemm_tc_status(int32_t* code) {
    g_err[0] = 0;
    ONEKA_CHECK_ARG(code, "code");
    int c = 0;
    ONEKA_CHECK_CUDA(gemm_tc_take_error(&c));
    *code = c;
    return ONEKA_OK;
}

int oneka_gemm_bf16_sigmoid_colsum(const void* A, int32_t lda, const void* B, int32_t ldb, const float* bias,
                                   float* out, int32_t M, int32_t N, int32_t K, int32_t flags, void* stream) {
    g_err[0] = 0;
    ONEKA_CHECK_ARG(A && B && out && M > 0 && N > 0 && K > 0, "A/B/out/M/N/K");
    ONEKA_CHECK_ARG(K % 32 == 0, "K must be a multiple of 32");
    ONEKA_CHECK_ARG(lda % 8 == 0 && ldb % 8 == 0 && lda >= K && ldb >= K, "leading dimensions");
    ONEKA_CHECK_ARG(al16(A) && al16(B) && (!bias || al16(bias)), "16-byte aligned matrices and bias");
    ONEKA_CHECK_CUDA(launch_gemm_bf16(A, lda, 1, B, ldb, 1, nullptr, N, 1, bias, 0, nullptr, M, N, K, 1, out,
                                      flags, (cudaStream_t)stream));
    return ONEKA_OK;
}

int oneka_bce_bitmask(const float* logits, const uint32_t* masks, int64_t slot_words, int32_t wpr, int32_t ncols,
                      int32_t B, int32_t ncells, float scale, void* dlogits, float* loss, void* stream) {
    g_err[0] = 0;
    ONEKA_CHECK_ARG(logits && masks && B > 0 && ncells > 0 && ncols > 0 && wpr * 32 >= ncols, "bce arguments");
    ONEKA_CHECK_CUDA(launch_bce_bitmask(logits, masks, slot_words, wpr, ncols, B, ncells, scale, dlogits, loss,
                                        (cudaStream_t)stream));
    return ONEKA_OK;
}

int oneka_gelu_backward(const float* dh, const void* z, void* dz, int64_t n, void* stream) {
    g_err[0] = 0;
    ONEKA_CHECK_ARG(dh && z && dz && n >= 0, "gelu_backward arguments");
    ONEKA_CHECK_CUDA(launch_gelu_backward(dh, z, dz, n, (cudaStream_t)stream));
    return ONEKA_OK;
}

int oneka_colsum_bf16(const void* x, int32_t rows, int32_t cols, float* out, void* stream) {
    g_err[0] = 0;
    ONEKA_CHECK_ARG(x && out && rows > 0 && cols > 0, "colsum arguments");
    ONEKA_CHECK_CUDA(launch_colsum(x, rows, cols, out, (cudaStream_t)stream));
    return ONEKA_OK;
}

int oneka_adamw(float* w, float* m, float* v, const float* g, void* w_bf16, int64_t n, float lr, float beta1,
                float beta2, float eps, float weight_decay, int32_t step, void* stream) {
    g_err[0] = 0;
    ONEKA_CHECK_ARG(w && m && v && g && n >= 0 && step >= 1, "adamw arguments");
    ONEKA_CHECK_CUDA(launch_adamw(w, m, v, g, w_bf16, n, lr, beta1, beta2, eps, weight_decay, step,
                                  (cudaStream_t)stream));
    return ONEKA_OK;
}

int oneka_adamw_scheduled(float* w, float* m, float* v, const float* g, void* w_bf16, int64_t n, const float* hyper,
                          float beta1, float beta2, float eps, float weight_decay, void* stream) {
    g_err[0] = 0;
    ONEKA_CHECK_ARG(w && m && v && g && hyper && n >= 0, "adamw arguments");
    ONEKA_CHECK_CUDA(launch_adamw_scheduled(w, m, v, g, w_bf16, n, hyper, beta1, beta2, eps, weight_decay,
                                            (cudaStream_t)stream));
    return ONEKA_OK;
}

int oneka_bce_bitmask_t(const float* logits, const uint32_t* masks, int64_t slot_words, int32_t wpr, int32_t ncols,
                        int32_t B, int32_t ncells, float scale, void* dlogits, void* dlogits_t, int64_t ldt,
                        float* loss, void* stream) {
    g_err[0] = 0;
    ONEKA_CHECK_ARG(logits && masks && dlogits && dlogits_t && B > 0 && ncells > 0 && ncols > 0, "bce arguments");
    ONEKA_CHECK_ARG(ncols % 64 == 0 && ncells % ncols == 0 && B % 64 == 0 && B <= 65535 * 64 && ldt % 8 == 0 &&
                    ldt >= B, "ncols and B must be multiples of 64, ldt of 8 and >= B");
    ONEKA_CHECK_ARG(al16(logits) && al16(dlogits) && al16(dlogits_t), "16-byte alignment");
    ONEKA_CHECK_CUDA(launch_bce_bitmask_t(logits, masks, slot_words, wpr, ncols, B, ncells, scale, dlogits, dlogits_t,
                                          ldt, loss, (cudaStream_t)stream));
    return ONEKA_OK;
}

int oneka_adamw_scheduled_t(float* w, float* m, float* v, const float* g, void* w_bf16, void* w_bf16_t, int64_t ldt,
                            int32_t rows, int32_t cols, const float* hyper, float beta1, float beta2, float eps,
                            float weight_decay, void* stream) {
    g_err[0] = 0;
    ONEKA_CHECK_ARG(w && m && v && g && w_bf16 && w_bf16_t && hyper && rows > 0 && cols > 0, "adamw arguments");
    ONEKA_CHECK_ARG(rows % 64 == 0 && cols % 64 == 0 && rows <= 65535 * 64 && ldt % 8 == 0 && ldt >= rows,
                    "rows and cols must be multiples of 64, ldt of 8 and >= rows");
    ONEKA_CHECK_ARG(al16(w) && al16(m) && al16(v) && al16(g) && al16(w_bf16) && al16(w_bf16_t), "16-byte alignment");
    ONEKA_CHECK_CUDA(launch_adamw_t(w, m, v, g, w_bf16, w_bf16_t, ldt, rows, cols, hyper, beta1, beta2, eps,
                                    weight_decay, (cudaStream_t)stream));
    return ONEKA_OK;
}

int oneka_features(const double* coef, const double* q, const double* aquifer, int32_t nwells, int32_t n,
                   const float* mean, const float* inv_std, int32_t nf, int32_t ld, void* x, void* stream) {
    g_err[0] = 0;
    ONEKA_CHECK_ARG(coef && q && aquifer && mean && inv_std && x && n >= 0, "features arguments");
    ONEKA_CHECK_ARG(nf == 6 + nwells + 2 && ld >= nf, "nf = 6 + nwells + 2 and ld >= nf");
    ONEKA_CHECK_CUDA(launch_features(coef, q, aquifer, nwells, n, mean, inv_std, nf, ld, x, (cudaStream_t)stream));
    return ONEKA_OK;
}

int oneka_sigmoid_colsum(const float* logits, int32_t rows, int32_t cols, float* out, void* stream) {
    g_err[0] = 0;
    ONEKA_CHECK_ARG(logits && out && rows > 0 && cols > 0, "sigmoid_colsum arguments");
    ONEKA_CHECK_CUDA(launch_sigmoid_colsum(logits, rows, cols, out, (cudaStream_t)stream));
    return ONEKA_OK;
}

int oneka_fma_peak(int32_t fp64, double* flops_per_s, void* stream) {
    g_err[0] = 0;
    ONEKA_CHECK_ARG(flops_per_s, "flops_per_s");
    ONEKA_CHECK_CUDA(probe_fma(fp64, flops_per_s, (cudaStream_t)stream));
    return ONEKA_OK;
}

int oneka_distancesquared(const double* abc, double* d2, int64_t n, void* stream) {
    g_err[0] = 0;
    ONEKA_CHECK_ARG(n >= 0 && (n == 0 || (abc && d2)), "abc/d2");
    ONEKA_CHECK_CUDA(launch_distancesquared(abc, d2, n, (cudaStream_t)stream));
    return ONEKA_OK;
}

}  // extern "C"
