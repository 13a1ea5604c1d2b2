// chronicle.cu -- ProbabilityField kernels and pointwise model evaluation (FP64).
//
// Built with --fmad=false (reference FP64 arithmetic).  References (paths
// within OnekaPy):
//   oneka/probabilityfield.py:313-339   rasterize / insert      -> rasterize_kernel
//   oneka/probabilityfield.py:342-372   register / reset        -> register_*_kernel
//   oneka/probabilityfield.py:380-427   distancesquared         -> distancesquared_kernel
//   oneka/model.py:207-427              potential .. velocity   -> evaluate_kernel
#include <math.h>

#include "oneka_internal.cuh"

namespace oneka {
namespace {

// One block per realization slot: scan the rows its particles touched (the
// slot header), add 1 to counts for every marked node, and clear the words
// and the header as they are read (register() then rgrid[:] = False).
__device__ __forceinline__ void register_slot(uint32_t* __restrict__ slot, long long mask_words, int nrows,
                                              int ncols, int wpr, int32_t* __restrict__ counts) {
    const uint32_t h0 = slot[mask_words], h1 = slot[mask_words + 1];
    if (h1 == 0) return;
    // the header is written only by the tracker; clamping keeps a corrupted
    // header from leading the scan outside the slot
    const int rlo = h0 > (uint32_t)nrows ? 0 : nrows - (int)h0;
    const int rhi = h1 > (uint32_t)nrows ? nrows - 1 : (int)h1 - 1;
    const long long w0 = (long long)rlo * wpr, w1 = (long long)(rhi + 1) * wpr;
    for (long long w = w0 + threadIdx.x; w < w1; w += blockDim.x) {
        uint32_t v = slot[w];
        if (!v) continue;
        slot[w] = 0u;
        const int row = (int)(w / wpr);
        const int col0 = (int)(w % wpr) * 32;
        // bits past the last column are never set by the trackers; dropping
        // them keeps a stray one from counting into the next row
        if (ncols - col0 < 32) v &= (1u << (ncols - col0)) - 1u;
        int32_t* crow = counts + (long long)row * ncols + col0;
        while (v) {
            const int b = __ffs(v) - 1;
            v &= v - 1;
            atomicAdd(crow + b, 1);
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        slot[mask_words] = 0u;
        slot[mask_words + 1] = 0u;
    }
}

__global__ void __launch_bounds__(256) register_counts_kernel(uint32_t* __restrict__ slots,
                                                              long long slot_words, long long mask_words,
                                                              int nrows, int ncols, int wpr,
                                                              int32_t* __restrict__ counts) {
    register_slot(slots + (long long)blockIdx.x * slot_words, mask_words, nrows, ncols, wpr, counts);
}

// Register nslots slots column by column: the thread of (word w, slot range
// blockIdx.y) sums bit b of word w over the slots of its range in bit-sliced
// counters (plane i holds bit i of every one of the 32 column counts; 16
// planes count to 65,535), clears the words it read, and adds each nonzero
// column count with one reduction.  A block first lists the slots of its
// range whose headers (the rows they marked) meet its rows, so untouched
// rows are neither read nor tested; its threads then load those slots' words
// eight at a time.  The reductions fall from one per visited node
// (register_slot) to one per column and slot range.
constexpr int kColumnsSlotsPerRange = 1024;
// Launches of this many slots or more register column by column (measured on
// the 10,000-realization site: 48.5 against 50.3 ms for track + register at
// 10,000 slots, equal at 2,048, 0.05-0.2 ms slower at 200-1,000 slots).
constexpr int kColumnsMinSlots = 4096;

__global__ void __launch_bounds__(256) register_columns_kernel(uint32_t* __restrict__ slots, long long slot_words,
                                                               long long mask_words, int nslots, int nrows,
                                                               int ncols, int wpr, int32_t* __restrict__ counts) {
    __shared__ int list[kColumnsSlotsPerRange];
    __shared__ int nlist;
    const long long nw = (long long)nrows * wpr;
    const long long wb = (long long)blockIdx.x * blockDim.x;
    const long long w = wb + threadIdx.x;
    const bool valid = w < nw;
    const int row = valid ? (int)(w / wpr) : 0;
    const int rfirst = (int)(wb / wpr);
    const int rlast = (int)((min(nw, wb + blockDim.x) - 1) / wpr);
    const int r0 = blockIdx.y * kColumnsSlotsPerRange;
    const int r1 = min(nslots, r0 + kColumnsSlotsPerRange);
    if (threadIdx.x == 0) nlist = 0;
    __syncthreads();
    for (int r = r0 + (int)threadIdx.x; r < r1; r += blockDim.x) {
        const uint32_t* sl = slots + (long long)r * slot_words;
        const uint32_t h0 = sl[mask_words], h1 = sl[mask_words + 1];
        // rows [nrows - h0, h1 - 1] (a zero header: an empty slot)
        const int rlo = h0 > (uint32_t)nrows ? 0 : nrows - (int)h0;
        const int rhi = h1 > (uint32_t)nrows ? nrows - 1 : (int)h1 - 1;
        if (h1 != 0u && rlo <= rlast && rhi >= rfirst) list[atomicAdd(&nlist, 1)] = r;
    }
    __syncthreads();
    const int n = nlist;
    if (!valid) return;      // no block-wide synchronization below
    uint32_t plane[16];
#pragma unroll
    for (int i = 0; i < 16; ++i) plane[i] = 0u;
    uint32_t seen = 0u;
    for (int m = 0; m < n; m += 8) {
        uint32_t x[8];
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            x[k] = 0u;
            if (m + k < n) {
                const uint32_t* sl = slots + (long long)list[m + k] * slot_words;
                const uint32_t h0 = sl[mask_words], h1 = sl[mask_words + 1];
                const int rlo = h0 > (uint32_t)nrows ? 0 : nrows - (int)h0;
                if (row >= rlo && row < (int)h1) x[k] = 1u;
            }
        }
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            if (x[k]) {
                uint32_t* p = slots + (long long)list[m + k] * slot_words + w;
                x[k] = *p;
                if (x[k]) *p = 0u;
            }
        }
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            uint32_t carry = x[k];
            seen |= carry;
#pragma unroll
            for (int i = 0; i < 16; ++i) {
                if (!carry) break;
                const uint32_t t = plane[i] & carry;
                plane[i] ^= carry;
                carry = t;
            }
        }
    }
    if (!seen) return;
    const int col0 = (int)(w % wpr) * 32;
    const int nb = min(32, ncols - col0);      // bits past the last column are never counted
    int32_t* crow = counts + (long long)row * ncols + col0;
    for (int b = 0; b < nb; ++b) {
        if (!((seen >> b) & 1u)) continue;
        int c = 0;
#pragma unroll
        for (int i = 0; i < 16; ++i) c |= (int)((plane[i] >> b) & 1u) << i;
        atomicAdd(crow + b, c);
    }
}

// Clear the headers of nslots slots (after register_columns_kernel has read them).
__global__ void clear_headers_kernel(uint32_t* __restrict__ slots, long long slot_words, long long mask_words,
                                     int nslots) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nslots) return;
    slots[(long long)r * slot_words + mask_words] = 0u;
    slots[(long long)r * slot_words + mask_words + 1] = 0u;
}

// Register every slot of a batched launch: block row -> (job, realization).
__global__ void __launch_bounds__(256) register_batch_kernel(const __grid_constant__ JobTable T) {
    const int row = blockIdx.x;
    int lo = 0, hi = T.njobs - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (T.first[mid] <= row) lo = mid; else hi = mid - 1;
    }
    const TrackLaunch& J = T.job[lo];
    if (!J.slots || !J.counts) return;
    register_slot(J.slots + (long long)(row - T.first[lo]) * J.slot_words, J.mask_words, J.grid.nrows,
                  J.grid.ncols, J.wpr, J.counts);
}

__global__ void register_weighted_kernel(uint32_t* __restrict__ mask, long long mwords, int nrows, int ncols,
                                         int wpr, double weight, double* __restrict__ pgrid) {
    const long long word = (long long)blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (word >= (long long)nrows * wpr) return;
    const uint32_t w = mask[word];
    const int row = (int)(word / wpr);
    const int col = (int)(word % wpr) * 32 + lane;
    if (((w >> lane) & 1u) && col < ncols) {
        double* cell = pgrid + (long long)row * ncols + col;
        *cell = *cell + weight;
    }
    __syncwarp();
    if (lane == 0) mask[word] = 0u;
    if (word == 0 && lane < 4) mask[mwords + lane] = 0u;
}

__global__ void rasterize_kernel(OnekaGrid g, OnekaFrame f, const double* __restrict__ xy, long long n,
                                 double umbra, uint32_t* mask, int wpr) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i + 1 >= n) return;
    long long ntest = 0, natom = 0;
    int rlo = 0x7fffffff, rhi = -1;
    Chron ch;
    ch.slot = mask;
    ch.win = nullptr;
    ch.wpr = wpr;
    ch.r0 = ch.w0 = ch.nr = ch.nw = 0;
    insert64(ch, g.nrows, g.ncols, f, g.dx, g.dy, umbra, xy[2 * i], xy[2 * i + 1], xy[2 * i + 2],
             xy[2 * i + 3], ntest, natom, rlo, rhi);
}

__global__ void distancesquared_kernel(const double* __restrict__ abc, double* __restrict__ d2, long long n) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double* a = abc + 6 * i;
    const double bax = a[2] - a[0];
    const double bay = a[3] - a[1];
    const double cax = a[4] - a[0];
    const double cay = a[5] - a[1];
    const double perpdot = bax * cay - bay * cax;
    const double dot = bax * cax + bay * cay;
    const double length2 = bax * bax + bay * bay;
    const double alpha2 = perpdot * perpdot / length2;
    const double beta2 = dot * dot / length2;
    double r;
    if (dot < 0) r = alpha2 + beta2;
    else if (beta2 > length2) r = alpha2 + beta2 - 2 * dot + length2;
    else r = alpha2;
    d2[i] = r;
}

struct EvalModel {
    const double* wells;   // [nw][3]
    const double* q;       // [nw]
    int nw;
    double xo, yo, c[6], K, n, H;
};

__global__ void evaluate_kernel(EvalModel m, const double* __restrict__ pts, long long npts, int confined,
                                double* potential, double* discharge, double* head, double* velocity,
                                int32_t* status) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= npts) return;
    const double x = pts[2 * i], y = pts[2 * i + 1];
    // compute_discharge (model.py:299-315)
    double dx = x - m.xo, dy = y - m.yo;
    double Qx = -(2.0 * m.c[0] * dx + m.c[2] * dy + m.c[3]);
    double Qy = -(2.0 * m.c[1] * dy + m.c[2] * dx + m.c[4]);
    // compute_potential (model.py:225-237)
    double pot = (m.c[0] * (dx * dx) + m.c[1] * (dy * dy) + m.c[2] * dx * dy + m.c[3] * dx + m.c[4] * dy + m.c[5]);
    double pw = 0.0;
    for (int w = 0; w < m.nw; ++w) {
        const double ddx = x - m.wells[3 * w], ddy = y - m.wells[3 * w + 1];
        const double r2 = ddx * ddx + ddy * ddy;
        Qx += -m.q[w] * ddx / r2 * 0.15915494309189535;
        Qy += -m.q[w] * ddy / r2 * 0.15915494309189535;
        pw += m.q[w] * log(r2) * 0.07957747154594767;
    }
    pot += pw;
    // compute_head (model.py:341-350)
    int st = ONEKA_TRACE_OK;
    double h = NAN;
    if (pot <= 0) {
        st = ONEKA_TRACE_DRY;
    } else {
        const double kh2 = 0.5 * m.K * (m.H * m.H);
        h = (pot < kh2) ? sqrt(2.0 * pot / m.K) : (pot + kh2) / (m.K * m.H);
    }
    // compute_velocity / compute_velocity_confined (model.py:377-389, 423-427)
    double vx = NAN, vy = NAN;
    if (confined) {
        vx = Qx / (m.H * m.n);
        vy = Qy / (m.H * m.n);
    } else if (st == ONEKA_TRACE_OK) {
        if (h <= 0) {
            st = ONEKA_TRACE_DRY;
        } else if (h > m.H) {
            vx = Qx / (m.H * m.n);
            vy = Qy / (m.H * m.n);
        } else {
            vx = Qx / (h * m.n);
            vy = Qy / (h * m.n);
        }
    }
    if (potential) potential[i] = pot;
    if (discharge) { discharge[2 * i] = Qx; discharge[2 * i + 1] = Qy; }
    if (head) head[i] = h;
    if (velocity) { velocity[2 * i] = vx; velocity[2 * i + 1] = vy; }
    if (status) status[i] = confined ? ONEKA_TRACE_OK : st;
}

// One pass of a separable Gaussian filter with zero padding outside the grid
// (scipy.ndimage.gaussian_filter(..., mode='constant', cval=0), used by
// oneka/visualize.py:232-233): along rows (axis 1) when along_cols == 0, else
// along columns (axis 0).  w: the 2*radius+1 normalized weights.
__global__ void gauss_pass_kernel(const double* __restrict__ in, double* __restrict__ out, int nrows, int ncols,
                                  const double* __restrict__ w, int radius, int along_cols) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long long)nrows * ncols) return;
    const int row = (int)(i / ncols), col = (int)(i % ncols);
    double acc = 0.0;
    for (int k = -radius; k <= radius; ++k) {
        const int rr = along_cols ? row + k : row;
        const int cc = along_cols ? col : col + k;
        if (rr < 0 || rr >= nrows || cc < 0 || cc >= ncols) continue;
        acc += w[k + radius] * in[(long long)rr * ncols + cc];
    }
    out[i] = acc;
}

// Histogram of int32 counts in [0, nbins); values outside are clamped into
// the last bin (shared-memory privatized).
__global__ void count_histogram_kernel(const int32_t* __restrict__ counts, long long n, int nbins,
                                       unsigned long long* __restrict__ hist) {
    extern __shared__ unsigned int sh[];
    for (int b = threadIdx.x; b < nbins; b += blockDim.x) sh[b] = 0u;
    __syncthreads();
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        int v = counts[i];
        v = v < 0 ? 0 : (v >= nbins ? nbins - 1 : v);
        atomicAdd(&sh[v], 1u);
    }
    __syncthreads();
    for (int b = threadIdx.x; b < nbins; b += blockDim.x)
        if (sh[b]) atomicAdd(&hist[b], (unsigned long long)sh[b]);
}

unsigned blocks_for(long long n, int per_block) { return (unsigned)((n + per_block - 1) / per_block); }

}  // namespace

cudaError_t launch_register_counts(uint32_t* slots, int nslots, const OnekaGrid& g, int32_t* counts,
                                   cudaStream_t s) {
    if (nslots <= 0) return cudaSuccess;
    const long long nw = (long long)g.nrows * words_per_row(g.ncols);
    const long long wblocks = (nw + 255) / 256;
    const int ranges = (nslots + kColumnsSlotsPerRange - 1) / kColumnsSlotsPerRange;
    if (nslots >= kColumnsMinSlots && wblocks <= 0x7fffffffLL && ranges <= 65535) {
        // many slots: column by column (one reduction per column and slot range)
        register_columns_kernel<<<dim3((unsigned)wblocks, (unsigned)ranges), 256, 0, s>>>(
            slots, slot_words(g), mask_words(g), nslots, g.nrows, g.ncols, words_per_row(g.ncols), counts);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
        clear_headers_kernel<<<(unsigned)((nslots + 255) / 256), 256, 0, s>>>(slots, slot_words(g), mask_words(g),
                                                                             nslots);
        return cudaGetLastError();
    }
    register_counts_kernel<<<(unsigned)nslots, 256, 0, s>>>(slots, slot_words(g), mask_words(g), g.nrows,
                                                            g.ncols, words_per_row(g.ncols), counts);
    return cudaGetLastError();
}

cudaError_t launch_gaussian(const double* in, double* out, double* tmp, int nrows, int ncols, const double* w,
                            int radius, cudaStream_t s) {
    const long long n = (long long)nrows * ncols;
    if (n <= 0) return cudaSuccess;
    // axis 0 first, then axis 1, as scipy.ndimage.gaussian_filter applies its 1-D passes
    gauss_pass_kernel<<<blocks_for(n, 256), 256, 0, s>>>(in, tmp, nrows, ncols, w, radius, 1);
    gauss_pass_kernel<<<blocks_for(n, 256), 256, 0, s>>>(tmp, out, nrows, ncols, w, radius, 0);
    return cudaGetLastError();
}

cudaError_t launch_histogram(const int32_t* counts, long long n, int nbins, unsigned long long* hist,
                             cudaStream_t s) {
    if (n <= 0 || nbins <= 0) return cudaSuccess;
    long long blocks = blocks_for(n, 256);
    if (blocks > 1216) blocks = 1216;
    count_histogram_kernel<<<(unsigned)blocks, 256, sizeof(unsigned) * (size_t)nbins, s>>>(counts, n, nbins,
                                                                                        hist);
    return cudaGetLastError();
}

// (Registering the jobs of 4,096 slots or more column by column, one launch
// each, measured the same on the 64 uneven sites: 9.94 s either way.)
cudaError_t launch_register_batch(const JobTable& T, int rows, cudaStream_t s) {
    if (rows <= 0) return cudaSuccess;
    register_batch_kernel<<<(unsigned)rows, 256, 0, s>>>(T);
    return cudaGetLastError();
}

cudaError_t launch_register_weighted(uint32_t* mask, const OnekaGrid& g, double weight, double* pgrid,
                                     cudaStream_t s) {
    const int wpr = words_per_row(g.ncols);
    const long long words = (long long)g.nrows * wpr;
    register_weighted_kernel<<<blocks_for(words, 8), 256, 0, s>>>(mask, mask_words(g), g.nrows, g.ncols, wpr,
                                                                  weight, pgrid);
    return cudaGetLastError();
}

cudaError_t launch_rasterize(const OnekaGrid& g, const OnekaFrame& f, const double* xy, long long n,
                             double umbra, uint32_t* mask, cudaStream_t s) {
    if (n < 2) return cudaSuccess;
    rasterize_kernel<<<blocks_for(n - 1, 128), 128, 0, s>>>(g, f, xy, n, umbra, mask, words_per_row(g.ncols));
    return cudaGetLastError();
}

cudaError_t launch_distancesquared(const double* abc, double* d2, long long n, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    distancesquared_kernel<<<blocks_for(n, 256), 256, 0, s>>>(abc, d2, n);
    return cudaGetLastError();
}

cudaError_t launch_evaluate(const OnekaSite& site, const double* q, double K, double n, double H,
                            const double* coef, const double* pts, long long npts, int confined,
                            double* potential, double* discharge, double* head, double* velocity,
                            int32_t* status, cudaStream_t s) {
    if (npts <= 0) return cudaSuccess;
    EvalModel m;
    m.wells = site.wells;
    m.q = q;
    m.nw = site.nwells;
    m.xo = site.xo;
    m.yo = site.yo;
    for (int i = 0; i < 6; ++i) m.c[i] = coef[i];
    m.K = K;
    m.n = n;
    m.H = H;
    evaluate_kernel<<<blocks_for(npts, 128), 128, 0, s>>>(m, pts, npts, confined, potential, discharge,
                                                          head, velocity, status);
    return cudaGetLastError();
}

}  // namespace oneka
