// track64.cu -- FP64 parity tracker: one thread per particle.
//
// Built with --fmad=false: every multiply and add rounds on its own, as in
// Python float / NumPy scalar arithmetic, so a trace reproduces the
// reference's vertices and the chronicle its visit counts.  References
// (paths within OnekaPy):
//   oneka/capturezone.py:198-253   Dormand-Prince 5(4), step control, partial traces
//   oneka/model.py:269-315         compute_discharge
//   oneka/model.py:318-389         compute_head / compute_velocity (general)
//   oneka/model.py:392-427         compute_velocity_confined
//   oneka/stochastic.py:253-260    feval = -velocity
//   oneka/probabilityfield.py:264-339  rasterize / insert (per accepted segment)
#include <math.h>

#include "crpow.cuh"
#include "oneka_internal.cuh"

namespace oneka {
namespace {

struct Model64 {
    const double* wx;
    const double* wy;
    const double* wq;
    int nw;
    double xo, yo;
    double c0, c1, c2, c3, c4, c5;
    double K, n, H;
};

// feval: -V at (x, y); false where the reference raises AquiferError.
template <bool CONFINED>
__device__ __forceinline__ bool feval64(const Model64& m, double x, double y, double& kx, double& ky) {
    const double dxo = x - m.xo;
    const double dyo = y - m.yo;
    double Qx = -(2.0 * m.c0 * dxo + m.c2 * dyo + m.c3);
    double Qy = -(2.0 * m.c1 * dyo + m.c2 * dxo + m.c4);
    double pw = 0.0;
    for (int i = 0; i < m.nw; ++i) {
        const double dx = x - m.wx[i];
        const double dy = y - m.wy[i];
        const double r2 = dx * dx + dy * dy;
        Qx += -m.wq[i] * dx / r2 * 0.15915494309189535;
        Qy += -m.wq[i] * dy / r2 * 0.15915494309189535;
        if (!CONFINED) pw += m.wq[i] * log(r2) * 0.07957747154594767;
    }
    double hn;
    if (CONFINED) {
        hn = m.H * m.n;
    } else {
        double pot = m.c0 * (dxo * dxo) + m.c1 * (dyo * dyo) + m.c2 * dxo * dyo + m.c3 * dxo +
                     m.c4 * dyo + m.c5;
        pot += pw;
        if (pot <= 0.0) return false;
        const double kh2 = 0.5 * m.K * (m.H * m.H);
        double head;
        if (pot < kh2)
            head = sqrt(2.0 * pot / m.K);
        else
            head = (pot + kh2) / (m.K * m.H);
        if (head <= 0.0) return false;
        hn = (head > m.H) ? m.H * m.n : head * m.n;
    }
    kx = -(Qx / hn);
    ky = -(Qy / hn);
    return true;
}

struct VertexSink {
    double* v;       // this particle's [max_vertices][2] or null
    int maxv;
    int n;
    double bx0, bx1, by0, by1;
    __device__ void push(double x, double y) {
        if (v && n < maxv) {
            v[2 * n] = x;
            v[2 * n + 1] = y;
        }
        if (n == 0) {
            bx0 = bx1 = x;
            by0 = by1 = y;
        } else {
            bx0 = fmin(bx0, x);
            bx1 = fmax(bx1, x);
            by0 = fmin(by0, y);
            by1 = fmax(by1, y);
        }
        ++n;
    }
};

template <bool CONFINED>
__device__ __forceinline__ void trace64(const TrackLaunch& L, int r, int p, long long idx, bool live,
                                        const double* wx, const double* wy, const double* wq, const Chron& ch);

template <bool CONFINED>
__global__ void __launch_bounds__(128) track64_kernel(const TrackLaunch L) {
    extern __shared__ double sm64[];
    const int k = blockIdx.y;
    const int r = L.r0 + k;
    double* wx = sm64;
    double* wy = sm64 + L.nwells;
    double* wq = sm64 + 2 * L.nwells;
    uint32_t* slot = L.slots ? L.slots + (long long)k * L.slot_words : nullptr;
    const Chron ch = make_chron(L, slot, reinterpret_cast<uint32_t*>(sm64 + 3 * L.nwells));
    for (int i = threadIdx.x; i < L.nwells; i += blockDim.x) {
        wx[i] = L.wells[3 * i];
        wy[i] = L.wells[3 * i + 1];
        wq[i] = L.q[(long long)r * L.nwells + i];
    }
    window_clear(ch);
    __syncthreads();
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    const long long idx = (long long)r * L.npaths + p;
    const bool skip = L.rstatus && L.rstatus[r] != ONEKA_REAL_OK;
    if (!skip && blockIdx.x == 0 && threadIdx.x == 0 && L.registered) atomicAdd(L.registered, 1ull);
    if (p < L.npaths && skip && L.out.status) L.out.status[idx] = kTraceSkipped;
    // Every lane enters: the step loop is warp-uniform (see trace64).
    trace64<CONFINED>(L, r, p, idx, p < L.npaths && !skip, wx, wy, wq, ch);
    __syncthreads();
    window_flush(ch);
}

// One particle per lane.  `live` is false for the lanes past npaths and for a
// realization that is not tracked; such a lane reads and writes nothing but
// still takes part in the warp's loop.
//
// The step loop is warp-uniform: it runs until every lane of the warp is done
// (a __any_sync vote at the top), and lanes that are done sit out the body.
// Only the chronicle insertion of an accepted step diverges, and the vote
// brings the lanes back together before the next attempt, so the six stage
// evaluations (k2..k7) issue once per warp rather than once per group of
// lanes that happened to split apart in a variable-length insertion.  Each
// lane's arithmetic is unchanged.
template <bool CONFINED>
__device__ __forceinline__ void trace64(const TrackLaunch& L, int r, int p, long long idx, bool live,
                                        const double* wx, const double* wy, const double* wq, const Chron& ch) {

    Model64 m;
    m.wx = wx;
    m.wy = wy;
    m.wq = wq;
    m.nw = L.nwells;
    m.xo = L.xo;
    m.yo = L.yo;
    const double* c = L.coef + 6LL * r;
    m.c0 = c[0]; m.c1 = c[1]; m.c2 = c[2]; m.c3 = c[3]; m.c4 = c[4]; m.c5 = c[5];
    m.K = L.aquifer[3LL * r];
    m.n = L.aquifer[3LL * r + 1];
    m.H = L.aquifer[3LL * r + 2];

    OnekaFrame f = {};
    if (live) f = frame_of(L, r, p);
    uint32_t* slot = ch.slot;

    const double dur = L.opts.duration;
    const double tol = L.opts.tol;
    const double maxstep = L.opts.maxstep;
    double t = 0.0;
    double dt = 0.1 * (dur > 0.0 ? 1.0 : (dur < 0.0 ? -1.0 : 0.0));
    double x = 0.0, y = 0.0;
    if (live) {
        x = L.release[2 * p];
        y = L.release[2 * p + 1];
    }

    VertexSink vs;
    vs.v = (live && L.out.vertices) ? L.out.vertices + idx * 2LL * L.out.max_vertices : nullptr;
    vs.maxv = L.out.max_vertices;
    vs.n = 0;
    vs.push(x, y);

    int status = ONEKA_TRACE_OK;
    int acc = 0, att = 0;
    long long ntest = 0, natom = 0;
    int rlo = 0x7fffffff, rhi = -1;
    double k1x = 0.0, k1y = 0.0, k2x, k2y, k3x, k3y, k4x, k4y, k5x, k5y, k6x, k6y, k7x = 0.0, k7y = 0.0;
    bool done = !live;
    if (live && !feval64<CONFINED>(m, x, y, k1x, k1y)) {
        status = ONEKA_TRACE_DRY;
        done = true;
    }
    while (__any_sync(0xffffffffu, !done)) {
        bool accept = false;
        double xn = x, yn = y;
        if (!done) do {
            if (!(fabs(t) < fabs(dur))) {
                done = true;
                break;
            }
            if (att >= L.max_attempts) {
                status = ONEKA_TRACE_STEP_LIMIT;
                done = true;
                break;
            }
            ++att;
            if (fabs(t + dt) > fabs(dur)) dt = dur - t;
            double px, py;
            px = x + dt * (DP::a2 * k1x);
            py = y + dt * (DP::a2 * k1y);
            if (!feval64<CONFINED>(m, px, py, k2x, k2y)) { status = ONEKA_TRACE_DRY; done = true; break; }
            px = x + dt * (DP::a31 * k1x + DP::a32 * k2x);
            py = y + dt * (DP::a31 * k1y + DP::a32 * k2y);
            if (!feval64<CONFINED>(m, px, py, k3x, k3y)) { status = ONEKA_TRACE_DRY; done = true; break; }
            px = x + dt * (DP::a41 * k1x + DP::a42 * k2x + DP::a43 * k3x);
            py = y + dt * (DP::a41 * k1y + DP::a42 * k2y + DP::a43 * k3y);
            if (!feval64<CONFINED>(m, px, py, k4x, k4y)) { status = ONEKA_TRACE_DRY; done = true; break; }
            px = x + dt * (DP::a51 * k1x + DP::a52 * k2x + DP::a53 * k3x + DP::a54 * k4x);
            py = y + dt * (DP::a51 * k1y + DP::a52 * k2y + DP::a53 * k3y + DP::a54 * k4y);
            if (!feval64<CONFINED>(m, px, py, k5x, k5y)) { status = ONEKA_TRACE_DRY; done = true; break; }
            px = x + dt * (DP::a61 * k1x + DP::a62 * k2x + DP::a63 * k3x + DP::a64 * k4x + DP::a65 * k5x);
            py = y + dt * (DP::a61 * k1y + DP::a62 * k2y + DP::a63 * k3y + DP::a64 * k4y + DP::a65 * k5y);
            if (!feval64<CONFINED>(m, px, py, k6x, k6y)) { status = ONEKA_TRACE_DRY; done = true; break; }
            xn = x + dt * (DP::a71 * k1x + DP::a73 * k3x + DP::a74 * k4x + DP::a75 * k5x + DP::a76 * k6x);
            yn = y + dt * (DP::a71 * k1y + DP::a73 * k3y + DP::a74 * k4y + DP::a75 * k5y + DP::a76 * k6y);
            if (!feval64<CONFINED>(m, xn, yn, k7x, k7y)) { status = ONEKA_TRACE_DRY; done = true; break; }
            const double ex = dt * (DP::e1 * k1x + DP::e2 * k7x + DP::e3 * k3x + DP::e4 * k4x +
                                    DP::e5 * k5x + DP::e6 * k6x);
            const double ey = dt * (DP::e1 * k1y + DP::e2 * k7y + DP::e3 * k3y + DP::e4 * k4y +
                                    DP::e5 * k5y + DP::e6 * k6y);
            const double aex = fabs(ex), aey = fabs(ey);
            const double est = (isnan(aex) || isnan(aey)) ? (double)NAN : (aey > aex ? aey : aex);
            const double d0 = xn - x, d1 = yn - y;
            const double ds = sqrt(fma(d1, d1, d0 * d0));   // numpy.linalg.norm (OpenBLAS ddot)
            accept = (est < tol) && (ds < maxstep);
            if (accept) t = t + dt;
            // dt = 0.9 * min((tol/(est+EPS))**(1/5), maxstep/(ds+EPS), 10) * dt  (:247)
            const double fstep = maxstep / (ds + DP::eps);
            const double xq = tol / (est + DP::eps);
            double lower = fstep;
            if (10.0 < lower) lower = 10.0;
            double fac;
            if (pow(xq, 0.2) > lower * (1.0 + 1e-13)) {
                fac = lower;                        // the power cannot be the minimum
            } else {
                fac = cr_pow_fifth(xq);             // it may be: evaluate it exactly
                if (fstep < fac) fac = fstep;
                if (10.0 < fac) fac = 10.0;
            }
            dt = 0.9 * fac * dt;
        } while (0);
        if (accept) {
            if (slot)
                insert64(ch, L.grid.nrows, L.grid.ncols, f, L.grid.dx, L.grid.dy, L.opts.umbra, x, y, xn, yn,
                         ntest, natom, rlo, rhi);
            k1x = k7x;
            k1y = k7y;
            x = xn;
            y = yn;
            vs.push(x, y);
            ++acc;
        }
    }
    if (!live) return;
    if (L.out.endpoint) {
        L.out.endpoint[2 * idx] = x;
        L.out.endpoint[2 * idx + 1] = y;
    }
    if (L.out.bbox) {
        L.out.bbox[4 * idx] = vs.bx0;
        L.out.bbox[4 * idx + 1] = vs.bx1;
        L.out.bbox[4 * idx + 2] = vs.by0;
        L.out.bbox[4 * idx + 3] = vs.by1;
    }
    if (L.out.naccept) L.out.naccept[idx] = acc;
    if (L.out.nattempt) L.out.nattempt[idx] = att;
    if (L.out.status) L.out.status[idx] = status;
    if (L.out.nvertices) L.out.nvertices[idx] = vs.n;
    note_rows(slot, L.mask_words, L.grid.nrows, rlo, rhi);
    add_counters((long long*)L.out.counters, att, acc, ntest, natom, status, L.grid, vs.bx0, vs.bx1, vs.by0,
                 vs.by1);
}

}  // namespace

cudaError_t launch_track64(const TrackLaunch& L, cudaStream_t s) {
    const int block = 128;
    dim3 grid((unsigned)((L.npaths + block - 1) / block), (unsigned)L.nr);
    if (grid.x == 0) grid.x = 1;
    const size_t smem = sizeof(double) * 3 * (size_t)L.nwells + 4 * (size_t)L.win_rows * L.win_words;
    if (L.opts.confined) {
        cudaFuncSetAttribute(track64_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        track64_kernel<true><<<grid, block, smem, s>>>(L);
    } else {
        cudaFuncSetAttribute(track64_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        track64_kernel<false><<<grid, block, smem, s>>>(L);
    }
    return cudaGetLastError();
}

}  // namespace oneka
