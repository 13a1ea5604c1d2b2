// track32.cu -- FP32 fast tracker: one thread per particle.
//
// Same algorithm as the FP64 parity build (oneka/capturezone.py:198-253 step
// control, oneka/model.py:269-427 velocity, oneka/probabilityfield.py:264-339
// chronicle) with the bulk arithmetic in FP32:
//   * coordinates are relative to the target well; the particle position is
//     a float pair (hi + lo) updated with an error-free two-sum, so the
//     position keeps ~48 bits over hundreds of steps;
//   * well terms are summed with Kahan compensation (discharge and potential);
//   * where the potential lies within 1% of K*H^2/2 (the confined/unconfined
//     switch) the head is inverted in FP64 from the compensated potential;
//   * elapsed time is kept in FP64.
#include <math.h>

#include "oneka_internal.cuh"

namespace oneka {
namespace {

struct Model32 {
    const float4* w;     // per well: x, y (relative to the target), -q/(2 pi), q/(4 pi)
    int nw;
    float ox, oy;        // regional origin relative to the target
    float c0, c1, c2, c3, c4, c5;
    float K, n, H;
    float inv_hn;        // 1 / (H n)
    double kh2;          // 0.5 K H^2 in FP64
};

struct Kahan {
    float s, c;
    __device__ __forceinline__ void add(float v) {
        const float y = v - c;
        const float t = s + y;
        c = (t - s) - y;
        s = t;
    }
};

template <bool CONFINED>
__device__ __forceinline__ bool feval32(const Model32& m, float x, float y, float& kx, float& ky) {
    const float dxo = x - m.ox;
    const float dyo = y - m.oy;
    Kahan qx{-(2.0f * m.c0 * dxo + m.c2 * dyo + m.c3), 0.0f};
    Kahan qy{-(2.0f * m.c1 * dyo + m.c2 * dxo + m.c4), 0.0f};
    Kahan pot{0.0f, 0.0f};
    if (!CONFINED)
        pot.s = m.c0 * dxo * dxo + m.c1 * dyo * dyo + m.c2 * dxo * dyo + m.c3 * dxo + m.c4 * dyo + m.c5;
#pragma unroll 4
    for (int i = 0; i < m.nw; ++i) {
        const float4 w = m.w[i];
        const float dx = x - w.x;
        const float dy = y - w.y;
        const float r2 = dx * dx + dy * dy;
        const float s = __fdividef(w.z, r2);
        qx.add(s * dx);
        qy.add(s * dy);
        if (!CONFINED) pot.add(w.w * __logf(r2));
    }
    if (CONFINED) {
        kx = -(qx.s * m.inv_hn);
        ky = -(qy.s * m.inv_hn);
        return true;
    }
    const float phi = pot.s - pot.c;
    if (phi <= 0.0f) return false;
    float head;
    const float kh2 = (float)m.kh2;
    if (fabsf(phi - kh2) < 0.01f * kh2) {
        // Near the top of the aquifer: invert in FP64 from the compensated sum.
        const double pd = (double)pot.s - (double)pot.c;
        if (pd <= 0.0) return false;
        double hd;
        if (pd < m.kh2)
            hd = sqrt(2.0 * pd / (double)m.K);
        else
            hd = (pd + m.kh2) / ((double)m.K * (double)m.H);
        head = (float)hd;
    } else if (phi < kh2) {
        head = sqrtf(2.0f * phi / m.K);
    } else {
        head = (phi + kh2) / (m.K * m.H);
    }
    if (head <= 0.0f) return false;
    const float inv = (head > m.H) ? m.inv_hn : 1.0f / (head * m.n);
    kx = -(qx.s * inv);
    ky = -(qy.s * inv);
    return true;
}

// Error-free a + b = s + e (Knuth's two-sum).
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
    s = a + b;
    const float bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}

// OR the nodes gj in [glo, ghi] of grid row gi into the chronicle.
__device__ __forceinline__ void or_span(const Chron& ch, int gi, int glo, int ghi, long long& natom) {
    int w = glo >> 5;
    const int wl = ghi >> 5;
    uint32_t m = 0xffffffffu << (glo & 31);
    for (; w <= wl; ++w) {
        if (w == wl) m &= 0xffffffffu >> (31 - (ghi & 31));
        ch.orw(gi, w, m);
        ++natom;
        m = 0xffffffffu;
    }
}

// Chronicle one segment in FP32: for every grid row the nodes within umbra
// of the segment form one interval, the row's intersection with the capsule
// (the two end disks and the band between them); the interval's nodes are
// set as whole bit ranges.  Nodes strictly closer than umbra are marked, as
// in ProbabilityField.insert (probabilityfield.py:296-310); FP32 rounding can
// move a node lying within ~1e-6 m of the boundary across it.
__device__ __forceinline__ void insert32(const Chron& ch, int gnrows, int gncols, const OnekaFrame& f,
                                         float fx0, float fy0, float dx, float dy, float umbra,
                                         float ax, float ay, float bx, float by, long long& ntest,
                                         long long& natom, int& rlo, int& rhi) {
    const float bax = bx - ax;
    const float bay = by - ay;
    const float length2 = bax * bax + bay * bay;
    if (!(length2 > 0.0f)) return;           // the reference's 0/0 marks nothing
    int left, right, bottom, top;
    if (!clip_range(floorf((fminf(ax, bx) - umbra - fx0) / dx),
                    floorf((fmaxf(ax, bx) + umbra - fx0) / dx) + 1.0f, f.ncols, left, right))
        return;
    if (!clip_range(floorf((fminf(ay, by) - umbra - fy0) / dy),
                    floorf((fmaxf(ay, by) + umbra - fy0) / dy) + 1.0f, f.nrows, bottom, top))
        return;
    ntest += (long long)(right - left) * (top - bottom);
    const float u2 = umbra * umbra;
    const float uL = umbra * sqrtf(length2);
    const float inv_bay = (bay != 0.0f) ? 1.0f / bay : 0.0f;
    const float inv_bax = (bax != 0.0f) ? 1.0f / bax : 0.0f;
    const float inv_dx = 1.0f / dx;
    for (int i = bottom; i < top; ++i) {
        const int gi = i + f.roff;
        if (gi < 0 || gi >= gnrows) continue;
        const float cy = fy0 + (float)i * dy;
        const float cay = cy - ay, cby = cy - by;
        float lo = INFINITY, hi = -INFINITY;
        const float ha = u2 - cay * cay;
        if (ha > 0.0f) { const float h = sqrtf(ha); lo = ax - h; hi = ax + h; }
        const float hb = u2 - cby * cby;
        if (hb > 0.0f) { const float h = sqrtf(hb); lo = fminf(lo, bx - h); hi = fmaxf(hi, bx + h); }
        // band: s = x - ax with |bay s - bax cay| < u L and 0 <= bax s + bay cay <= L^2
        float slo = -INFINITY, shi = INFINITY;
        const float bc = bax * cay;
        if (bay != 0.0f) {
            const float c1 = (bc - uL) * inv_bay, c2 = (bc + uL) * inv_bay;
            slo = fminf(c1, c2);
            shi = fmaxf(c1, c2);
        } else if (!(fabsf(bc) < uL)) {
            slo = INFINITY;
        }
        const float yc = bay * cay;
        if (bax != 0.0f) {
            const float d1 = -yc * inv_bax, d2 = (length2 - yc) * inv_bax;
            slo = fmaxf(slo, fminf(d1, d2));
            shi = fminf(shi, fmaxf(d1, d2));
        } else if (!(yc >= 0.0f && yc <= length2)) {
            slo = INFINITY;
        }
        if (slo < shi) { lo = fminf(lo, ax + slo); hi = fmaxf(hi, ax + shi); }
        if (!(lo < hi)) continue;
        int jlo = (int)fmaxf(ceilf((lo - fx0) * inv_dx), (float)left);
        int jhi = (int)fminf(floorf((hi - fx0) * inv_dx), (float)(right - 1));
        // strictly inside: drop an end node that sits on the boundary
        if (jlo <= jhi && fx0 + (float)jlo * dx <= lo) ++jlo;
        if (jlo <= jhi && fx0 + (float)jhi * dx >= hi) --jhi;
        int glo = jlo + f.coff, ghi = jhi + f.coff;
        glo = glo < 0 ? 0 : glo;
        ghi = ghi >= gncols ? gncols - 1 : ghi;
        if (glo > ghi) continue;
        or_span(ch, gi, glo, ghi, natom);
        rlo = gi < rlo ? gi : rlo;
        rhi = gi > rhi ? gi : rhi;
    }
}

template <bool CONFINED>
__device__ __forceinline__ void trace32(const TrackLaunch& L, int r, int p, long long idx, const float4* sm32,
                                        const Chron& ch);

template <bool CONFINED>
__global__ void __launch_bounds__(256) track32_kernel(const TrackLaunch L) {
    extern __shared__ float4 sm32[];
    const int k = blockIdx.y;
    const int r = L.r0 + k;
    uint32_t* slot = L.slots ? L.slots + (long long)k * L.slot_words : nullptr;
    const Chron ch = make_chron(L, slot, reinterpret_cast<uint32_t*>(sm32 + L.nwells));
    for (int i = threadIdx.x; i < L.nwells; i += blockDim.x) {
        const double q = L.q[(long long)r * L.nwells + i];
        sm32[i] = make_float4((float)(L.wells[3 * i] - L.xt), (float)(L.wells[3 * i + 1] - L.yt),
                              (float)(-q * 0.15915494309189535), (float)(q * 0.07957747154594767));
    }
    window_clear(ch);
    __syncthreads();
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    const long long idx = (long long)r * L.npaths + p;
    const bool skip = L.rstatus && L.rstatus[r] != ONEKA_REAL_OK;
    if (!skip && blockIdx.x == 0 && threadIdx.x == 0 && L.registered) atomicAdd(L.registered, 1ull);
    if (p < L.npaths) {
        if (skip) {
            if (L.out.status) L.out.status[idx] = kTraceSkipped;
        } else {
            trace32<CONFINED>(L, r, p, idx, sm32, ch);
        }
    }
    __syncthreads();
    window_flush(ch);
}

template <bool CONFINED>
__device__ __forceinline__ void trace32(const TrackLaunch& L, int r, int p, long long idx, const float4* sm32,
                                        const Chron& ch) {

    Model32 m;
    m.w = sm32;
    m.nw = L.nwells;
    m.ox = (float)(L.xo - L.xt);
    m.oy = (float)(L.yo - L.yt);
    const double* c = L.coef + 6LL * r;
    m.c0 = (float)c[0]; m.c1 = (float)c[1]; m.c2 = (float)c[2];
    m.c3 = (float)c[3]; m.c4 = (float)c[4]; m.c5 = (float)c[5];
    const double Kd = L.aquifer[3LL * r], nd = L.aquifer[3LL * r + 1], Hd = L.aquifer[3LL * r + 2];
    m.K = (float)Kd;
    m.n = (float)nd;
    m.H = (float)Hd;
    m.inv_hn = (float)(1.0 / (Hd * nd));
    m.kh2 = 0.5 * Kd * (Hd * Hd);

    const OnekaFrame f = frame_of(L, r, p);
    const float fx0 = (float)(f.xmin - L.xt);
    const float fy0 = (float)(f.ymin - L.yt);
    uint32_t* slot = ch.slot;
    const float gdx = (float)L.grid.dx, gdy = (float)L.grid.dy, umbra = (float)L.opts.umbra;

    const double dur = L.opts.duration;
    const float tol = (float)L.opts.tol;
    const float maxstep = (float)L.opts.maxstep;
    const float eps = (float)DP::eps;
    double t = 0.0;
    float dt = 0.1f * (dur > 0.0 ? 1.0f : (dur < 0.0 ? -1.0f : 0.0f));
    float xh = (float)(L.release[2 * p] - L.xt), yh = (float)(L.release[2 * p + 1] - L.yt);
    float xl = (float)((L.release[2 * p] - L.xt) - (double)xh);
    float yl = (float)((L.release[2 * p + 1] - L.yt) - (double)yh);

    double* vout = L.out.vertices ? L.out.vertices + idx * 2LL * L.out.max_vertices : nullptr;
    int nv = 0;
    float bx0 = xh + xl, bx1 = bx0, by0 = yh + yl, by1 = by0;
    auto push = [&](float ph, float pl, float qh, float ql) {
        if (vout && nv < L.out.max_vertices) {
            vout[2 * nv] = L.xt + ((double)ph + (double)pl);
            vout[2 * nv + 1] = L.yt + ((double)qh + (double)ql);
        }
        ++nv;
    };
    push(xh, xl, yh, yl);

    int status = ONEKA_TRACE_OK;
    int acc = 0, att = 0;
    long long ntest = 0, natom = 0;
    int rlo = 0x7fffffff, rhi = -1;
    float k1x, k1y, k2x, k2y, k3x, k3y, k4x, k4y, k5x, k5y, k6x, k6y, k7x, k7y;
    constexpr float a2 = (float)DP::a2, a31 = (float)DP::a31, a32 = (float)DP::a32;
    constexpr float a41 = (float)DP::a41, a42 = (float)DP::a42, a43 = (float)DP::a43;
    constexpr float a51 = (float)DP::a51, a52 = (float)DP::a52, a53 = (float)DP::a53, a54 = (float)DP::a54;
    constexpr float a61 = (float)DP::a61, a62 = (float)DP::a62, a63 = (float)DP::a63, a64 = (float)DP::a64,
                    a65 = (float)DP::a65;
    constexpr float a71 = (float)DP::a71, a73 = (float)DP::a73, a74 = (float)DP::a74, a75 = (float)DP::a75,
                    a76 = (float)DP::a76;
    constexpr float e1 = (float)DP::e1, e2 = (float)DP::e2, e3 = (float)DP::e3, e4 = (float)DP::e4,
                    e5 = (float)DP::e5, e6 = (float)DP::e6;
    if (!feval32<CONFINED>(m, xh + xl, yh + yl, k1x, k1y)) {
        status = ONEKA_TRACE_DRY;
    } else {
        while (fabs(t) < fabs(dur)) {
            if (att >= L.max_attempts) {
                status = ONEKA_TRACE_STEP_LIMIT;
                break;
            }
            ++att;
            bool last = false;
            if (fabs(t + (double)dt) > fabs(dur)) {
                dt = (float)(dur - t);
                last = true;
            }
            if (!feval32<CONFINED>(m, xh + (xl + dt * (a2 * k1x)), yh + (yl + dt * (a2 * k1y)), k2x, k2y)) {
                status = ONEKA_TRACE_DRY; break;
            }
            if (!feval32<CONFINED>(m, xh + (xl + dt * (a31 * k1x + a32 * k2x)),
                                   yh + (yl + dt * (a31 * k1y + a32 * k2y)), k3x, k3y)) {
                status = ONEKA_TRACE_DRY; break;
            }
            if (!feval32<CONFINED>(m, xh + (xl + dt * (a41 * k1x + a42 * k2x + a43 * k3x)),
                                   yh + (yl + dt * (a41 * k1y + a42 * k2y + a43 * k3y)), k4x, k4y)) {
                status = ONEKA_TRACE_DRY; break;
            }
            if (!feval32<CONFINED>(m, xh + (xl + dt * (a51 * k1x + a52 * k2x + a53 * k3x + a54 * k4x)),
                                   yh + (yl + dt * (a51 * k1y + a52 * k2y + a53 * k3y + a54 * k4y)), k5x, k5y)) {
                status = ONEKA_TRACE_DRY; break;
            }
            if (!feval32<CONFINED>(m, xh + (xl + dt * (a61 * k1x + a62 * k2x + a63 * k3x + a64 * k4x + a65 * k5x)),
                                   yh + (yl + dt * (a61 * k1y + a62 * k2y + a63 * k3y + a64 * k4y + a65 * k5y)),
                                   k6x, k6y)) {
                status = ONEKA_TRACE_DRY; break;
            }
            const float sx = dt * (a71 * k1x + a73 * k3x + a74 * k4x + a75 * k5x + a76 * k6x);
            const float sy = dt * (a71 * k1y + a73 * k3y + a74 * k4y + a75 * k5y + a76 * k6y);
            if (!feval32<CONFINED>(m, xh + (xl + sx), yh + (yl + sy), k7x, k7y)) {
                status = ONEKA_TRACE_DRY; break;
            }
            const float ex = dt * (e1 * k1x + e2 * k7x + e3 * k3x + e4 * k4x + e5 * k5x + e6 * k6x);
            const float ey = dt * (e1 * k1y + e2 * k7y + e3 * k3y + e4 * k4y + e5 * k5y + e6 * k6y);
            const float est = fmaxf(fabsf(ex), fabsf(ey));
            const float ds = sqrtf(sx * sx + sy * sy);
            if ((est < tol) && (ds < maxstep)) {
                t = last ? dur : t + (double)dt;
                const float ax = xh + xl, ay = yh + yl;
                float s, e;
                two_sum(xh, sx, s, e);
                xl += e;
                two_sum(s, xl, xh, e);
                xl = e;
                two_sum(yh, sy, s, e);
                yl += e;
                two_sum(s, yl, yh, e);
                yl = e;
                const float bxn = xh + xl, byn = yh + yl;
                if (slot)
                    insert32(ch, L.grid.nrows, L.grid.ncols, f, fx0, fy0, gdx, gdy, umbra,
                             ax, ay, bxn, byn, ntest, natom, rlo, rhi);
                bx0 = fminf(bx0, bxn); bx1 = fmaxf(bx1, bxn);
                by0 = fminf(by0, byn); by1 = fmaxf(by1, byn);
                k1x = k7x;
                k1y = k7y;
                push(xh, xl, yh, yl);
                ++acc;
            }
            float fac = __powf(tol / (est + eps), 0.2f);
            const float fstep = maxstep / (ds + eps);
            if (fstep < fac) fac = fstep;
            if (10.0f < fac) fac = 10.0f;
            dt = 0.9f * fac * dt;
        }
    }
    if (L.out.endpoint) {
        L.out.endpoint[2 * idx] = L.xt + ((double)xh + (double)xl);
        L.out.endpoint[2 * idx + 1] = L.yt + ((double)yh + (double)yl);
    }
    if (L.out.bbox) {
        L.out.bbox[4 * idx] = L.xt + (double)bx0;
        L.out.bbox[4 * idx + 1] = L.xt + (double)bx1;
        L.out.bbox[4 * idx + 2] = L.yt + (double)by0;
        L.out.bbox[4 * idx + 3] = L.yt + (double)by1;
    }
    if (L.out.naccept) L.out.naccept[idx] = acc;
    if (L.out.nattempt) L.out.nattempt[idx] = att;
    if (L.out.status) L.out.status[idx] = status;
    if (L.out.nvertices) L.out.nvertices[idx] = nv;
    note_rows(slot, L.mask_words, L.grid.nrows, rlo, rhi);
    add_counters((long long*)L.out.counters, att, acc, ntest, natom);
}

}  // namespace

cudaError_t launch_track32(const TrackLaunch& L, cudaStream_t s) {
    const int block = L.opts.block > 0 ? L.opts.block : 128;
    dim3 grid((unsigned)((L.npaths + block - 1) / block), (unsigned)L.nr);
    if (grid.x == 0) grid.x = 1;
    const size_t smem = sizeof(float4) * (size_t)L.nwells + 4 * (size_t)L.win_rows * L.win_words;
    if (L.opts.confined) {
        cudaFuncSetAttribute(track32_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        track32_kernel<true><<<grid, block, smem, s>>>(L);
    } else {
        cudaFuncSetAttribute(track32_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        track32_kernel<false><<<grid, block, smem, s>>>(L);
    }
    return cudaGetLastError();
}

}  // namespace oneka
