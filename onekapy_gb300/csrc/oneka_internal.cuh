// oneka_internal.cuh -- shared declarations of liboneka_gb300 (not part of the ABI).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/oneka_gb300.h"

namespace oneka {

constexpr int kTraceSkipped = 3;              // per-particle status of an untracked realization
constexpr int kDefaultMaxAttempts = 1000000;

// Everything one tracking launch needs, passed by value as the kernel parameter.
struct TrackLaunch {
    const double* wells;        // [nwells][3]
    int nwells;
    int npaths;
    double xo, yo;              // regional origin
    double xt, yt;              // target well (FP32 build: coordinates relative to it)
    const double* coef;         // [nreal][6]
    const double* q;            // [nreal][nwells]
    const double* aquifer;      // [nreal][3]
    const int32_t* rstatus;     // [nreal] or null
    int r0;                     // first realization of this wave
    int nr;                     // realizations in this wave
    const double* release;      // [npaths][2]
    OnekaTrackOpts opts;
    OnekaGrid grid;
    const OnekaFrame* frames;   // [nreal][npaths] or null
    uint32_t* slots;            // wave-local realization k uses slots + k * slot_words; null: no chronicle
    int wpr;                    // words per grid row
    long long slot_words;
    long long mask_words;
    unsigned long long* registered;
    OnekaTrackOut out;
    int max_attempts;
    // shared-memory window of each realization slot: rows [win_r0, win_r0 + win_rows),
    // words [win_w0, win_w0 + win_words) of every row; win_rows == 0: no window
    int win_r0, win_w0, win_rows, win_words;
    int32_t* counts;            // register target of this launch (batched launches)
};

// The jobs of one batched launch (oneka_track_batched), passed whole as a
// __grid_constant__ kernel parameter: first[j] is job j's first block row.
constexpr int kMaxJobs = 80;
struct JobTable {
    TrackLaunch job[kMaxJobs];
    int first[kMaxJobs + 1];
    int njobs;
};
static_assert(sizeof(JobTable) < 32000, "JobTable must fit the 32 KB kernel-parameter limit");

// Where a chronicle mark goes: the block's shared-memory window of the slot
// when the word lies inside it, else the slot in global memory.
struct Chron {
    uint32_t* slot;
    uint32_t* win;
    int wpr, r0, w0, nr, nw;
    __device__ __forceinline__ void orw(int gi, int w, uint32_t bits) const {
        const int ri = gi - r0, wi = w - w0;
        if (win && (unsigned)ri < (unsigned)nr && (unsigned)wi < (unsigned)nw)
            atomicOr(win + ri * nw + wi, bits);
        else
            atomicOr(slot + (long long)gi * wpr + w, bits);
    }
};

__device__ __forceinline__ Chron make_chron(const TrackLaunch& L, uint32_t* slot, uint32_t* win) {
    Chron c;
    c.slot = slot;
    c.win = (slot && L.win_rows > 0) ? win : nullptr;
    c.wpr = L.wpr;
    c.r0 = L.win_r0;
    c.w0 = L.win_w0;
    c.nr = L.win_rows;
    c.nw = L.win_words;
    return c;
}

// Zero the block's window (before the first mark) ...
__device__ __forceinline__ void window_clear(const Chron& c) {
    if (!c.win) return;
    for (int i = threadIdx.x; i < c.nr * c.nw; i += blockDim.x) c.win[i] = 0u;
}

// ... and OR its nonzero words into the global slot (after the last mark).
__device__ __forceinline__ void window_flush(const Chron& c) {
    if (!c.win) return;
    for (int i = threadIdx.x; i < c.nr * c.nw; i += blockDim.x) {
        const uint32_t v = c.win[i];
        if (v) atomicOr(c.slot + (long long)(c.r0 + i / c.nw) * c.wpr + (c.w0 + i % c.nw), v);
    }
}

// A realization slot: the bitmask (nrows rows of words_per_row words), padded
// to a multiple of 4 words, then a 4-word header { h0, h1, 0, 0 } recording
// the rows touched: h0 = max(nrows - row), h1 = max(row + 1) over marked
// rows, so an all-zero slot is an empty one.
inline int words_per_row(int ncols) { return (ncols + 31) / 32; }
inline long long mask_words(const OnekaGrid& g) {
    long long w = (long long)g.nrows * words_per_row(g.ncols);
    return (w + 3) / 4 * 4;
}
inline long long slot_words(const OnekaGrid& g) { return mask_words(g) + 4; }

cudaError_t launch_track64(const TrackLaunch& L, cudaStream_t s);
cudaError_t launch_track32(const TrackLaunch& L, cudaStream_t s);
cudaError_t launch_track32_batch(const JobTable& T, int rows, cudaStream_t s);
cudaError_t launch_register_batch(const JobTable& T, int rows, cudaStream_t s);
cudaError_t launch_register_counts(uint32_t* slots, int nslots, const OnekaGrid& g, int32_t* counts,
                                   cudaStream_t s);

void set_error(const char* fmt, ...);

// Dormand-Prince 5(4) tableau (capturezone.py:202-209); every entry is the
// double nearest the rational, as Python's true division gives.
struct DP {
    static constexpr double a2 = 1.0 / 5.0;
    static constexpr double a31 = 3.0 / 40.0, a32 = 9.0 / 40.0;
    static constexpr double a41 = 44.0 / 45.0, a42 = -56.0 / 15.0, a43 = 32.0 / 9.0;
    static constexpr double a51 = 19372.0 / 6561.0, a52 = -25360.0 / 2187.0,
                            a53 = 64448.0 / 6561.0, a54 = -212.0 / 729.0;
    static constexpr double a61 = 9017.0 / 3168.0, a62 = -355.0 / 33.0, a63 = 46732.0 / 5247.0,
                            a64 = 49.0 / 176.0, a65 = -5103.0 / 18656.0;
    static constexpr double a71 = 35.0 / 384.0, a73 = 500.0 / 1113.0, a74 = 125.0 / 192.0,
                            a75 = -2187.0 / 6784.0, a76 = 11.0 / 84.0;
    static constexpr double e1 = 71.0 / 57600.0, e2 = -1.0 / 40.0, e3 = -71.0 / 16695.0,
                            e4 = 71.0 / 1920.0, e5 = -17253.0 / 339200.0, e6 = 22.0 / 525.0;
    static constexpr double eps = 2.220446049250313e-16;   // np.finfo(float).eps
};

// Python's min(a, b): the first argument unless the second is strictly smaller.
__device__ __forceinline__ double py_min(double a, double b) { return (b < a) ? b : a; }
__device__ __forceinline__ double py_max(double a, double b) { return (b > a) ? b : a; }

// The frame a particle's trace is rasterized against.
__device__ __forceinline__ OnekaFrame frame_of(const TrackLaunch& L, int r, int p) {
    if (L.frames) return L.frames[(long long)r * L.npaths + p];
    OnekaFrame f;
    f.xmin = L.grid.xmin;
    f.ymin = L.grid.ymin;
    f.coff = 0;
    f.roff = 0;
    f.ncols = L.grid.ncols;
    f.nrows = L.grid.nrows;
    return f;
}

// Clamp floor() results (as doubles) to a half-open index range [0, n).
__device__ __forceinline__ bool clip_range(double lo, double hi, int n, int& ilo, int& ihi) {
    if (!(lo < (double)n) || !(hi > 0.0)) return false;
    ilo = lo < 0.0 ? 0 : (int)lo;
    ihi = hi > (double)n ? n : (int)hi;
    return ilo < ihi;
}

// ProbabilityField.distancesquared(...) < umbra**2 with the reference's FP64
// operations (probabilityfield.py:407-427).  A reciprocal replaces the two
// divisions unless the result lies within 1e-12 (relative) of the threshold,
// where the exact quotients decide; the outcome equals the reference's.
__device__ __forceinline__ bool in_umbra64(double bax, double bay, double cax, double cay,
                                           double length2, double inv, bool fast_ok, double u2) {
    const double perpdot = bax * cay - bay * cax;
    const double dot = bax * cax + bay * cay;
    if (fast_ok) {
        const double a2 = perpdot * perpdot * inv;
        const double b2 = dot * dot * inv;
        double d2;
        if (dot < 0) d2 = a2 + b2;
        else if (b2 > length2) d2 = a2 + b2 - 2 * dot + length2;
        else d2 = a2;
        const double margin = 1e-12 * (a2 + b2 + 2 * fabs(dot) + length2 + u2);
        if (d2 < u2 - margin) return true;
        if (d2 > u2 + margin) return false;
    }
    const double alpha2 = perpdot * perpdot / length2;
    const double beta2 = dot * dot / length2;
    double d2;
    if (dot < 0) d2 = alpha2 + beta2;
    else if (beta2 > length2) d2 = alpha2 + beta2 - 2 * dot + length2;
    else d2 = alpha2;
    return d2 < u2;
}

// ProbabilityField.insert (probabilityfield.py:296-310) into a realization
// bitmask: every node of the frame within umbra of segment a-b is OR-ed in,
// one atomicOr per touched 32-node word of a row.
// The reference's node test from the node's indices (the exact path of
// insert64's FP32 pre-test).  Kept out of line so that the compiler cannot
// evaluate it speculatively for every node: it runs for about 1 node in 5,000.
static __device__ __noinline__ bool in_umbra64_node(double fxmin, int j, double dx, double ax, double bax, double bay,
                                             double cay, double length2, double inv, bool fast_ok, double u2) {
    const double cx = fxmin + (double)j * dx;
    const double cax = cx - ax;
    return in_umbra64(bax, bay, cax, cay, length2, inv, fast_ok, u2);
}

__device__ __forceinline__ void insert64(const Chron& ch, int gnrows, int gncols,
                                         const OnekaFrame& f, double dx, double dy, double umbra,
                                         double ax, double ay, double bx, double by,
                                         long long& ntest, long long& natom, int& rlo, int& rhi) {
    const double u2 = umbra * umbra;
    int left, right, bottom, top;
    if (!clip_range(floor((py_min(ax, bx) - umbra - f.xmin) / dx),
                    floor((py_max(ax, bx) + umbra - f.xmin) / dx) + 1, f.ncols, left, right))
        return;
    if (!clip_range(floor((py_min(ay, by) - umbra - f.ymin) / dy),
                    floor((py_max(ay, by) + umbra - f.ymin) / dy) + 1, f.nrows, bottom, top))
        return;
    ntest += (long long)(right - left) * (top - bottom);
    const double bax = bx - ax;
    const double bay = by - ay;
    const double length2 = bax * bax + bay * bay;
    const double inv = 1.0 / length2;
    const bool fast_ok = (length2 > 1e-250) && (inv < 1e250);
    // FP32 pre-test.  The distance^2 of each node is first evaluated in FP32
    // (cancellation-free form); a node whose FP32 value lies farther than
    // `mf` from umbra^2 is decided by it, the others by the reference's FP64
    // formula.  S bounds every coordinate magnitude of the node box
    // (|cax| <= |bax| + umbra + dx, |cay| <= |bay| + umbra + dy), so each FP32
    // operation errs by at most 2^-24 S^2 in the squared terms; the margin
    // (256 + 4 k) 2^-24 S^2 covers them, the conversions, the k-node row
    // offset and the reference's own FP64 rounding many times over.  The
    // decisions, hence the counts, are the FP64 formula's.
    const bool f32_ok = (length2 > 1e-20) && (length2 < 1e20) && (right - left) < (1 << 20);
    float bxf = 0.0f, byf = 0.0f, l2f = 0.0f, u2f = 0.0f, dxf = 0.0f, mf = 0.0f;
    if (f32_ok) {
        bxf = (float)bax;
        byf = (float)bay;
        l2f = bxf * bxf + byf * byf;
        u2f = (float)u2;
        dxf = (float)dx;
        const double S = 2.0 * (fabs(bax) + fabs(bay)) + 2.0 * umbra + dx + dy;
        mf = (float)((256.0 + 4.0 * (right - left)) * 5.9604644775390625e-08 * S * S);
    }
    for (int i = bottom; i < top; ++i) {
        const int gi = i + f.roff;
        if (gi < 0 || gi >= gnrows) continue;
        const double cy = f.ymin + (double)i * dy;
        const double cay = cy - ay;
        float cayf = 0.0f, cax0f = 0.0f;
        if (f32_ok) {
            cayf = (float)cay;
            cax0f = (float)((f.xmin + (double)left * dx) - ax);
        }
        uint32_t acc = 0;
        int curw = -1;
        for (int j = left; j < right; ++j) {
            const int gj = j + f.coff;
            if (gj < 0 || gj >= gncols) continue;
            int decided = 0;                    // 1: inside, -1: outside, 0: FP64
            if (f32_ok) {
                // j - left as a float without the (FP64-pipe) I2F: exact below 2^22
                const float kf = __int_as_float(0x4B400000 + (j - left)) - 12582912.0f;
                const float caxf = fmaf(kf, dxf, cax0f);
                const float dot = bxf * caxf + byf * cayf;
                float d2;
                if (dot < 0.0f) {
                    d2 = caxf * caxf + cayf * cayf;
                } else if (dot > l2f) {
                    const float ex = caxf - bxf, ey = cayf - byf;
                    d2 = ex * ex + ey * ey;
                } else {
                    const float p = bxf * cayf - byf * caxf;
                    d2 = p * p / l2f;
                }
                if (d2 < u2f - mf) decided = 1;
                else if (d2 > u2f + mf) decided = -1;
            }
            bool inside;
            if (__builtin_expect(decided != 0, 1))
                inside = decided > 0;
            else
                inside = in_umbra64_node(f.xmin, j, dx, ax, bax, bay, cay, length2, inv, fast_ok, u2);
            if (inside) {
                const int w = gj >> 5;
                if (w != curw) {
                    if (acc) { ch.orw(gi, curw, acc); ++natom; }
                    curw = w;
                    acc = 0;
                }
                acc |= 1u << (gj & 31);
            }
        }
        if (curw >= 0) {
            if (acc) { ch.orw(gi, curw, acc); ++natom; }
            rlo = gi < rlo ? gi : rlo;
            rhi = gi > rhi ? gi : rhi;
        }
    }
}

// Record the rows a particle marked in its slot's header (see slot_words).
__device__ __forceinline__ void note_rows(uint32_t* slot, long long mwords, int nrows, int rlo, int rhi) {
    if (!slot || rhi < rlo) return;
    atomicMax(slot + mwords, (uint32_t)(nrows - rlo));
    atomicMax(slot + mwords + 1, (uint32_t)(rhi + 1));
}

// Per-particle counters, added into OnekaTrackOut.counters when the trace
// ends: [0] step attempts, [1] accepted steps, [2] chronicle node tests,
// [3] chronicle word ORs, [4] DRY traces, [5] STEP_LIMIT traces, [6] traces
// that left the grid (their bounding box reaches the grid's outer nodes,
// where the reference's ProbabilityField.expand would grow the grid,
// oneka/probabilityfield.py:228-244; a fixed window clips them), [7] 0.
__device__ __forceinline__ void add_counters(long long* c, long long att, long long acc, long long ntest,
                                             long long natom, int status, const OnekaGrid& g, double bx0,
                                             double bx1, double by0, double by1) {
    if (!c) return;
    unsigned long long* u = (unsigned long long*)c;
    atomicAdd(u + 0, (unsigned long long)att);
    atomicAdd(u + 1, (unsigned long long)acc);
    atomicAdd(u + 2, (unsigned long long)ntest);
    atomicAdd(u + 3, (unsigned long long)natom);
    if (status == ONEKA_TRACE_DRY) atomicAdd(u + 4, 1ull);
    if (status == ONEKA_TRACE_STEP_LIMIT) atomicAdd(u + 5, 1ull);
    const double xmax = g.xmin + (g.ncols - 1) * g.dx, ymax = g.ymin + (g.nrows - 1) * g.dy;
    if (bx0 <= g.xmin || bx1 >= xmax || by0 <= g.ymin || by1 >= ymax) atomicAdd(u + 6, 1ull);
}

}  // namespace oneka
