// track32.cu -- FP32 fast tracker: persistent lanes over a realization's particles.
//
// Same algorithm as the FP64 parity build (oneka/capturezone.py:198-253 step
// control, oneka/model.py:269-427 velocity, oneka/probabilityfield.py:264-339
// chronicle) with the bulk arithmetic in FP32:
//   * coordinates are relative to the target well, where every trace starts;
//     the particle position is a float pair (hi + lo) updated with an
//     error-free two-sum, so the position keeps ~48 bits over hundreds of
//     steps;
//   * every well's position is a float pair too, and its distance to the
//     particle is differenced pair by pair, (x_hi - xw_hi) + (x_lo - xw_lo):
//     the high difference is exact near the well (Sterbenz), so r^2 about
//     each well keeps the particle's full position, not one rounded to a
//     float (the recentred r^2);
//   * x and y travel together as packed FP32 pairs (Blackwell's FADD2 /
//     FMUL2 / FFMA2), one instruction for both coordinates;
//   * the discharge's well terms are summed with Kahan compensation, one
//     compensated addition per group of four wells (the potential's per
//     well in the FP64 head-inversion mode);
//   * the head is inverted from the compensated potential in FP32 (the
//     inversion is well conditioned; see feval32);
//   * the time left is a float pair counting down to zero, so no FP64
//     instruction runs in the step loop (GB300's FP64 pipe is ~1/64 of FP32,
//     and float<->int conversions use FP32 magic-constant arithmetic).
//
// Work layout: one block per realization (or per chunk of its particles when
// the realizations alone cannot fill the GPU).  Each lane takes the next
// particle from a shared counter as soon as its trace ends, so a block's
// lanes stay busy until its last particles, and no lane waits for the
// slowest trace of a fixed group.  The Dormand-Prince stages are folded into
// register running sums of the tableau rows (the six velocity evaluations of
// an attempt are unrolled, so every row index is a compile-time constant);
// the cold per-particle state (bounding box, counters, frame, vertex count)
// sits in shared-memory columns, one per lane.
#include <math.h>

#include <type_traits>

#include "oneka_internal.cuh"

namespace oneka {
namespace {

// Packed FP32 pairs: (x, y) in one 64-bit register pair, one instruction for
// both (FADD2 / FMUL2 / FFMA2 on sm_100 and later); every operation rounds
// each lane once, as its scalar form does.
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
// b - a with one rounding (a * -1 is exact).
__device__ __forceinline__ float2 rsub2(float2 a, float2 b) { return __ffma2_rn(a, make_float2(-1.0f, -1.0f), b); }
__device__ __forceinline__ float2 splat(float v) { return make_float2(v, v); }

struct Model32 {
    const float4* wp;    // per well: -x_hi, -y_hi, -x_lo, -y_lo (relative to the target)
    const float2* wq;    // per well: -q/(2 pi), q ln(2)/(4 pi)
    int nw;
    float ox, oy;        // regional origin relative to the target
    float c0, c1, c2, c3, c4, c5;
    float K, n, H;
    float inv_hn;        // 1 / (H n)
    float kh2f;          // 0.5 K H^2
    float inv_k;         // 1 / K
    float inv_kh;        // 1 / (K H)
    const double* d64;   // {K, n, H} in FP64 (read only by the near-top inversion of kGeneralHead64)
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

// Kahan summation of (x, y) pairs; the compensation is kept negated, so the
// total is s + cn and every step is one packed instruction.  Terms are added
// in groups: a group's products are chained by FMA onto the compensation
// (one rounding per term, as a per-term Kahan step has) and the group enters
// the running sum with one compensated addition, so the rounding of the
// large running sum is still recovered while the compensation costs three
// instructions per group instead of per term.
struct Kahan2 {
    float2 s, cn;
    __device__ __forceinline__ void add(float2 y) {   // += y, where y already carries cn
        const float2 t = add2(s, y);
        cn = rsub2(rsub2(s, t), y);     // y - (t - s)
        s = t;
    }
};

// Velocity modes of the FP32 build: the general (mixed) path, the confined
// path, and the general path with the optional FP64 near-top head inversion.
enum Mode32 { kGeneral = 0, kConfined = 1, kGeneralHead64 = 2 };

// -V at the point ph + pl (hi and lo parts of x and y), in k.  Returns false
// at a dry point (potential or head <= 0, the reference's AquiferError).
template <int MODE>
__device__ __forceinline__ bool feval32(const Model32& m, float2 ph, float2 pl, float2& k) {
    constexpr bool CONFINED = MODE == kConfined;
    const float2 p = add2(ph, pl);                 // the point rounded to floats, for the regional terms
    const float dxo = p.x - m.ox;
    const float dyo = p.y - m.oy;
    Kahan2 q{make_float2(-(2.0f * m.c0 * dxo + m.c2 * dyo + m.c3), -(2.0f * m.c1 * dyo + m.c2 * dxo + m.c4)),
             make_float2(0.0f, 0.0f)};
    Kahan pot{0.0f, 0.0f};
    if (!CONFINED)
        pot.s = m.c0 * dxo * dxo + m.c1 * dyo * dyo + m.c2 * dxo * dyo + m.c3 * dxo + m.c4 * dyo + m.c5;
    // well i's discharge term onto y, its potential term into pot; wq = its
    // constants (-q/(2 pi), q ln(2)/(4 pi))
    auto well = [&](int i, float2 wq, float2 y) {
        const float4 w = m.wp[i];
        // recentred difference: (x_hi - xw_hi) + (x_lo - xw_lo), both coordinates at once
        const float2 d = add2(add2(ph, make_float2(w.x, w.y)), add2(pl, make_float2(w.z, w.w)));
        const float r2 = d.x * d.x + d.y * d.y;
        // q/(4 pi) ln r^2 (ln 2 folded into wq.y).  The discharge sums carry
        // the trace's accuracy and are compensated; the potential only
        // selects the head branch and scales the velocity, and compensating
        // it changed no measured drift, so it is compensated only where the
        // FP64 head inversion reads the unrounded pair.
        if (!CONFINED) {
            if (MODE == kGeneralHead64)
                pot.add(wq.y * __log2f(r2));
            else
                pot.s += wq.y * __log2f(r2);
        }
        return fma2(splat(__fdividef(wq.x, r2)), d, y);
    };
    // the constants of wells 2j and 2j + 1 in one 16-byte load (the array
    // is padded to whole float4s)
    const float4* wq4 = reinterpret_cast<const float4*>(m.wq);
    constexpr int G = 4;       // wells per compensated group
    int i = 0;
#pragma unroll 1
    for (; i + G <= m.nw; i += G) {
        const float4 qa = wq4[i >> 1], qb = wq4[(i >> 1) + 1];
        float2 y = q.cn;
        y = well(i, make_float2(qa.x, qa.y), y);
        y = well(i + 1, make_float2(qa.z, qa.w), y);
        y = well(i + 2, make_float2(qb.x, qb.y), y);
        y = well(i + 3, make_float2(qb.z, qb.w), y);
        q.add(y);
    }
    if (i < m.nw) {            // the last, partial group
        float2 y = q.cn;
#pragma unroll 1
        for (; i + 1 < m.nw; i += 2) {
            const float4 qa = wq4[i >> 1];
            y = well(i, make_float2(qa.x, qa.y), y);
            y = well(i + 1, make_float2(qa.z, qa.w), y);
        }
        if (i < m.nw) y = well(i, m.wq[i], y);
        q.add(y);
    }
    const float2 qt = add2(q.s, q.cn);
    if (CONFINED) {
        k = mul2(qt, splat(-m.inv_hn));
        return true;
    }
    // Head from the potential (model.py:341-350).  The inversion itself is
    // well conditioned (sqrt halves relative errors; the confined branch is
    // linear), so FP32 keeps the digits the potential delivers.  An FP64
    // inversion near the aquifer top would add nothing to an FP32 result and,
    // on GB300, costs the whole warp ~1000 FP64-pipe cycles whenever one lane
    // takes it.  Computed without branches.
    const float phi = pot.s - pot.c;
    const float kh2 = m.kh2f;
    const float hu = sqrtf(fmaxf(2.0f * phi * m.inv_k, 0.0f));
    const float hc = (phi + kh2) * m.inv_kh;
    float head = (phi < kh2) ? hu : hc;
    float inv = (head > m.H) ? m.inv_hn : __fdividef(1.0f, head * m.n);
    if (MODE == kGeneralHead64 && fabsf(head - m.H) < 0.01f * m.H) {
        // optional: the inversion in FP64 from the unrounded compensated pair
        // (model.py:341-350 operation order)
        const double K = m.d64[0], n = m.d64[1], H = m.d64[2];
        const double ph64 = (double)pot.s - (double)pot.c;
        const double h = (ph64 < 0.5 * K * H * H) ? sqrt(2.0 * ph64 / K) : (ph64 + 0.5 * K * H * H) / (K * H);
        head = (float)h;
        inv = (h > H) ? m.inv_hn : (float)(1.0 / (h * n));
    }
    k = mul2(qt, splat(-inv));
    return (phi > 0.0f) && (head > 0.0f);
}

// Error-free a + b = s + e (Knuth's two-sum), scalar and for (x, y) pairs.
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
    s = a + b;
    const float bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}

__device__ __forceinline__ void two_sum2(float2 a, float2 b, float2& s, float2& e) {
    s = add2(a, b);
    const float2 bb = rsub2(a, s);                           // s - a
    e = add2(rsub2(rsub2(bb, s), a), rsub2(bb, b));          // (a - (s - bb)) + (b - bb)
}

// Conversions without the FP64 pipe.  On GB300, I2F/F2I and float rounding
// instructions issue on the (narrow) FP64 pipe; these use an FADD with
// 1.5 * 2^23, whose low mantissa bits then hold the integer, and integer
// arithmetic.  Exact for |values| < 2^22 (arguments are clamped to that).
constexpr float kMagic = 12582912.0f;   // 1.5 * 2^23
constexpr int kMagicBits = 0x4B400000;

__device__ __forceinline__ float i2f_small(int i) { return __fsub_rn(__int_as_float(kMagicBits + i), kMagic); }

__device__ __forceinline__ int floor_small(float x) {
    x = fminf(fmaxf(x, -4.0e6f), 4.0e6f);
    const float b = __fadd_rn(x, kMagic);               // round to nearest integer (+M)
    const float r = __fsub_rn(b, kMagic);
    return (__float_as_int(b) - kMagicBits) - (r > x ? 1 : 0);
}

// clip_range for integer bounds [lo, hi) of a range of n nodes.
__device__ __forceinline__ bool clip_int(int lo, int hi, int n, int& ilo, int& ihi) {
    ilo = lo < 0 ? 0 : lo;
    ihi = hi > n ? n : hi;
    return ilo < ihi;
}

// OR the nodes gj in [glo, ghi] of one grid row into the chronicle.
// or_win: the caller has established that the whole span lies in the
// shared-memory window, whose word (row, 0) is at ch.win + base.  or_span:
// otherwise; the row's window test is made once and each word's once.
// Masks: bits lo.. of a word are 0 - (1 << lo), bits ..hi are (2 << hi) - 1
// (2 << 31 wraps to 0), bits lo..hi of one word (2 << hi) - (1 << lo).
__device__ __forceinline__ void or_win(const Chron& ch, int base, int glo, int ghi, unsigned& natom) {
    int w = glo >> 5;
    const int wl = ghi >> 5;
    natom += wl - w + 1;
    const uint32_t lo_bit = 1u << (glo & 31);
    const uint32_t hi_end = 2u << (ghi & 31);
    if (w == wl) {                       // most spans lie in one word
        atomicOr(ch.win + (base + w), hi_end - lo_bit);
        return;
    }
    atomicOr(ch.win + (base + w), 0u - lo_bit);
    for (++w; w < wl; ++w) atomicOr(ch.win + (base + w), 0xffffffffu);
    atomicOr(ch.win + (base + wl), hi_end - 1u);
}

__device__ __forceinline__ void or_span(const Chron& ch, int gi, int glo, int ghi, unsigned& natom) {
    const int ri = gi - ch.r0;
    const bool row_in = ch.win && (unsigned)ri < (unsigned)ch.nr;
    int w = glo >> 5;
    const int wl = ghi >> 5;
    natom += wl - w + 1;
    uint32_t m = 0u - (1u << (glo & 31));
    for (; w <= wl; ++w) {
        if (w == wl) m &= (2u << (ghi & 31)) - 1u;
        const int wi = w - ch.w0;
        if (row_in && (unsigned)wi < (unsigned)ch.nw)
            atomicOr(ch.win + ri * ch.nw + wi, m);
        else
            atomicOr(ch.slot + (long long)gi * ch.wpr + w, m);
        m = 0xffffffffu;
    }
}

// Grid constants of the FP32 chronicle, converted once per block.
struct Raster32 {
    float dx, dy, inv_dx, inv_dy;
    float U, U2;         // umbra and umbra^2 in units of dx
    float ryy;           // row spacing in units of dx (dy / dx)
    float umbra;
};

// Chronicle one segment in FP32: for every grid row the nodes within umbra
// of the segment form one open interval (LO, HI), the row's intersection
// with the capsule (the band and the end disk at b; see below for the disk
// at a); its nodes floor(LO) + 1 .. ceil(HI) - 1 are set as whole bit
// ranges.  Nodes strictly
// closer than umbra are marked, as in ProbabilityField.insert
// (probabilityfield.py:296-310); FP32 rounding can move a node lying within
// a few ulps of its frame coordinate (about 1e-4 of a cell on a 1,601-node
// frame) of the boundary across it.
//
// A trace's capsules overlap at their joints: segment i starts where the
// last segment of nonzero length before it ended, whose capsule holds the
// disk about that point, so a segment does not mark the disk about its
// start a.  The one disk no segment marks, about the release point, is
// marked by disk32 once per trace (after the block's traces end), for every
// trace with a segment that reached the row loop; a trace whose segments
// were all clipped away has no node of that disk in its frame.  The union of
// the marks is the reference's (in exact arithmetic).
//
// Geometry is in units of dx with x measured from the frame's first column,
// so LO and HI are node indices; every per-row quantity is one multiply-add
// of the row's offset from the segment's start (the band's limits are
// linear in it, with their order fixed per segment).
__device__ __forceinline__ void insert32(const Chron& ch, int gnrows, int gncols, int coff, int roff,
                                         int fncols, int fnrows, float fx0, float fy0, const Raster32& g,
                                         float ax, float ay, float bx, float by, unsigned& ntest,
                                         unsigned& natom, int& rlo, int& rhi) {
    // the grid constants live in shared memory next to the window that the
    // row loop ORs into; registers copies keep them from being reloaded
    // after every atomic
    const float umbra = g.umbra, inv_dx = g.inv_dx, inv_dy = g.inv_dy;
    const float U = g.U, U2 = g.U2, ryy = g.ryy;
    const float bax = bx - ax;
    const float bay = by - ay;
    if (!(bax * bax + bay * bay > 0.0f)) return;    // the reference's 0/0 marks nothing
    int left, right, bottom, top;
    if (!clip_int(floor_small((fminf(ax, bx) - umbra - fx0) * inv_dx),
                  floor_small((fmaxf(ax, bx) + umbra - fx0) * inv_dx) + 1, fncols, left, right))
        return;
    if (!clip_int(floor_small((fminf(ay, by) - umbra - fy0) * inv_dy),
                  floor_small((fmaxf(ay, by) + umbra - fy0) * inv_dy) + 1, fnrows, bottom, top))
        return;
    ntest += (unsigned)(right - left) * (unsigned)(top - bottom);
    // segment in units of dx: X from column 0 of the frame, Y from row 0
    const float aX = (ax - fx0) * inv_dx, aY = (ay - fy0) * inv_dx;
    const float bX = (bx - fx0) * inv_dx, bY = (by - fy0) * inv_dx;
    const float BAX = bX - aX, BAY = bY - aY;
    const float L2 = BAX * BAX + BAY * BAY;
    const float UL = U * sqrtf(L2);
    // band |BAY s - BAX t| < U L (t = row offset from a, s = X - aX):
    //   s in (k t - |e|, k t + |e|), k = BAX / BAY, e = U L / BAY
    // projection 0 <= BAX s + BAY t <= L^2:
    //   s in [-m t + min(0, f), -m t + max(0, f)], m = BAY / BAX, f = L^2 / BAX
    const bool bay_nz = BAY != 0.0f, bax_nz = BAX != 0.0f;
    const float iby = bay_nz ? 1.0f / BAY : 0.0f, ibx = bax_nz ? 1.0f / BAX : 0.0f;
    const float k = BAX * iby, ae = fabsf(UL * iby);
    const float m = BAY * ibx, f = L2 * ibx;
    const float flo = fminf(0.0f, f), fhi = fmaxf(0.0f, f);
    // Frame rows and columns that are grid nodes (gi = i + roff in [0, gnrows),
    // gj = j + coff in [0, gncols)), clamped once for the segment: the row
    // loop then needs no per-row range test, and clamping the interval to
    // [cl - 1, cr] yields exactly the node span that clamping it to
    // [left - 1, right] and then to the grid would.
    const int rb = max(bottom, -roff), re = min(top, gnrows - roff);
    const int cl = max(left, -coff), cr = min(right, gncols - coff);
    if (rb >= re || cl >= cr) return;
    // Node spans: the nodes strictly inside (LO, HI) are the integers from
    // nearest(LO - 1/2) + 1 to nearest(HI + 1/2) - 1 (floor(LO) + 1 and
    // ceil(HI) - 1, except at an integer LO or HI, where the tie may round
    // toward the interval: a node exactly at umbra from the segment, inside
    // the FP32 build's boundary tolerance, may then be marked).  The halves
    // are folded into the interval's ends (aXm, aXp, ... below) and the
    // column offset into the constants that take the integer out of the
    // rounded sum; these roundings move the boundary by an ulp of the
    // interval's ends, within the same tolerance.  The clamp to the columns
    // [cl, cr) is a quarter node inside cl - 1 and cr, never a tie, so it
    // gives exactly cl and cr - 1 (a clamp at cl - 1 would be the tie
    // cl - 3/2, which rounds to even and can reach column cl - 1).  An empty
    // row needs no test of its own: LO = +inf, HI = -inf give glo > ghi, and
    // so does LO >= HI up to the tie above.
    const float xlo = i2f_small(cl) - 1.25f, xhi = i2f_small(cr) + 0.25f;
    const float aXm = aX - 0.5f, aXp = aX + 0.5f, bXm = bX - 0.5f, bXp = bX + 0.5f;
    const int klo = (kMagicBits - 1) - coff, khi = (kMagicBits + 1) - coff;
    // The row loop, instantiated four times.  IN_WIN: the node box lies wholly
    // in the shared-memory window (almost every segment near the target), so
    // the marks go there without per-row or per-word window tests.  GENERAL:
    // the segment is parallel to neither axis (BAX, BAY != 0), so the band's
    // limits need no per-row case analysis.
    auto rows = [&](auto in_win, auto general) {
        float t = i2f_small(rb) * ryy - aY;             // row offset from a (units of dx)
        int base = decltype(in_win)::value ? (rb + roff - ch.r0) * ch.nw - ch.w0 : 0;
        for (int i = rb; i < re; ++i, t += ryy) {
            float LO = INFINITY, HI = -INFINITY;        // the interval's ends, less and plus 1/2
            const float tb = t - BAY;
            const float hb = U2 - tb * tb;
            if (hb > 0.0f) { const float h = sqrtf(hb); LO = fminf(LO, bXm - h); HI = fmaxf(HI, bXp + h); }
            float slo, shi;
            if (decltype(general)::value) {
                slo = fmaxf(k * t - ae, flo - m * t);
                shi = fminf(k * t + ae, fhi - m * t);
            } else {
                if (bay_nz) {
                    const float kt = k * t;
                    slo = kt - ae;
                    shi = kt + ae;
                } else {
                    const bool in = fabsf(t) < U;
                    slo = in ? -INFINITY : INFINITY;
                    shi = in ? INFINITY : -INFINITY;
                }
                if (bax_nz) {
                    const float mt = -m * t;
                    slo = fmaxf(slo, mt + flo);
                    shi = fminf(shi, mt + fhi);
                } else {
                    const float yc = BAY * t;
                    if (!(yc >= 0.0f && yc <= L2)) slo = INFINITY;
                }
            }
            if (slo < shi) { LO = fminf(LO, aXm + slo); HI = fmaxf(HI, aXp + shi); }
            const int glo = __float_as_int(__fadd_rn(fmaxf(LO, xlo), kMagic)) - klo;
            const int ghi = __float_as_int(__fadd_rn(fminf(HI, xhi), kMagic)) - khi;
            if (glo <= ghi) {
                if (decltype(in_win)::value) or_win(ch, base, glo, ghi, natom);
                else or_span(ch, i + roff, glo, ghi, natom);
            }
            if (decltype(in_win)::value) base += ch.nw;
        }
    };
    // the slot header bounds the rows that may hold marks: the segment's row range
    rlo = min(rlo, rb + roff);
    rhi = max(rhi, re - 1 + roff);
    const bool in_win = ch.win && rb + roff >= ch.r0 && re + roff <= ch.r0 + ch.nr &&
                        ((cl + coff) >> 5) >= ch.w0 && ((cr - 1 + coff) >> 5) < ch.w0 + ch.nw;
    if (bay_nz && bax_nz) {
        if (in_win) rows(std::true_type{}, std::true_type{});
        else rows(std::false_type{}, std::true_type{});
    } else {
        if (in_win) rows(std::true_type{}, std::false_type{});
        else rows(std::false_type{}, std::false_type{});
    }
}


// Chronicle the nodes strictly within umbra of the point (ax, ay) (the
// release point's disk; the same row-interval form as insert32), and return
// the rows it may have marked in [rlo, rhi].
__device__ __forceinline__ void disk32(const Chron& ch, int gnrows, int gncols, int coff, int roff, int fncols,
                                       int fnrows, float fx0, float fy0, const Raster32& g, float ax, float ay,
                                       int& rlo, int& rhi) {
    const float umbra = g.umbra, inv_dx = g.inv_dx, inv_dy = g.inv_dy, U2 = g.U2, ryy = g.ryy;
    int left, right, bottom, top;
    if (!clip_int(floor_small((ax - umbra - fx0) * inv_dx), floor_small((ax + umbra - fx0) * inv_dx) + 1, fncols,
                  left, right))
        return;
    if (!clip_int(floor_small((ay - umbra - fy0) * inv_dy), floor_small((ay + umbra - fy0) * inv_dy) + 1, fnrows,
                  bottom, top))
        return;
    const int rb = max(bottom, -roff), re = min(top, gnrows - roff);
    const int cl = max(left, -coff), cr = min(right, gncols - coff);
    if (rb >= re || cl >= cr) return;
    const float aX = (ax - fx0) * inv_dx, aY = (ay - fy0) * inv_dx;
    const float xlo = i2f_small(cl) - 1.25f, xhi = i2f_small(cr) + 0.25f;
    const float aXm = aX - 0.5f, aXp = aX + 0.5f;
    const int klo = (kMagicBits - 1) - coff, khi = (kMagicBits + 1) - coff;
    unsigned natom = 0;
    float t = i2f_small(rb) * ryy - aY;
    for (int i = rb; i < re; ++i, t += ryy) {
        const float ha = U2 - t * t;
        if (!(ha > 0.0f)) continue;
        const float h = sqrtf(ha);
        const int glo = __float_as_int(__fadd_rn(fmaxf(aXm - h, xlo), kMagic)) - klo;
        const int ghi = __float_as_int(__fadd_rn(fminf(aXp + h, xhi), kMagic)) - khi;
        if (glo <= ghi) or_span(ch, i + roff, glo, ghi, natom);
    }
    rlo = rb + roff;
    rhi = re - 1 + roff;
}

// Dormand-Prince tableau in FP32 (capturezone.py:202-209), arranged for
// running sums.  Row s = 0..5 is the stage point of k_{s+2} (row 5 is the
// 5th-order solution).  After k_{j+1} (j = 0..5) is evaluated it is added
// into every later row: P_s += dp_b(j, s) * k, where dp_b(j, s) is
// a[s][j+1] for s > j and 0 otherwise, and into the error sum with
// dp_e(j + 1) (k7 = f(xyt) carries -1/40, the reference's e[1]).  The values
// are compile-time constants, so the zero entries cost nothing.
__device__ __forceinline__ constexpr float dp_a0(int s) {
    return s == 0 ? (float)DP::a2 : s == 1 ? (float)DP::a31 : s == 2 ? (float)DP::a41
         : s == 3 ? (float)DP::a51 : s == 4 ? (float)DP::a61 : (float)DP::a71;
}
__device__ __forceinline__ constexpr float dp_b(int j, int s) {
    return j == 0 ? (s == 1 ? (float)DP::a32 : s == 2 ? (float)DP::a42 : s == 3 ? (float)DP::a52
                   : s == 4 ? (float)DP::a62 : 0.0f)
         : j == 1 ? (s == 2 ? (float)DP::a43 : s == 3 ? (float)DP::a53 : s == 4 ? (float)DP::a63
                   : s == 5 ? (float)DP::a73 : 0.0f)
         : j == 2 ? (s == 3 ? (float)DP::a54 : s == 4 ? (float)DP::a64 : s == 5 ? (float)DP::a74 : 0.0f)
         : j == 3 ? (s == 4 ? (float)DP::a65 : s == 5 ? (float)DP::a75 : 0.0f)
         : j == 4 ? (s == 5 ? (float)DP::a76 : 0.0f)
         : 0.0f;
}
__device__ __forceinline__ constexpr float dp_e(int i) {
    return i == 0 ? (float)DP::e1 : i == 1 ? 0.0f : i == 2 ? (float)DP::e3 : i == 3 ? (float)DP::e4
         : i == 4 ? (float)DP::e5 : i == 5 ? (float)DP::e6 : (float)DP::e2;
}

struct RealConst32 {
    // what every velocity evaluation reads, as three 16-byte shared-memory loads
    float4 q0;           // c0, c1, c2, c3 (A..D)
    float4 q1;           // c4, c5, ox, oy (E, F, regional origin)
    float4 q2;           // inv_hn, kh2f, inv_k, inv_kh
    float K, n, H;
    double d64[3];       // K, n, H in FP64 for the optional near-top head inversion
    float tol, maxstep;  // options, converted once
    Raster32 g;          // grid constants of the chronicle
    int skip;
    int next;            // next particle of this block's chunk
    unsigned long long counters[8];   // the block's share of OnekaTrackOut.counters
};

// float4 slots of a block's well arrays: positions [nw] float4, then
// constants [nw] float2 rounded up to whole float4s.
__host__ __device__ __forceinline__ int well_float4s(int nw) { return nw + (nw + 1) / 2; }

// Most particles one block traces (a launch splits larger realizations into
// chunks), so that its release-disk flags take at most 1 KB of shared memory.
constexpr int kMaxChunk = 8192;

// Per-lane particle state.  Everything the step loop touches is FP32: on
// GB300 the FP64 pipe runs at ~1/64 of the FP32 rate, so a handful of FP64
// operations per step would dominate it.  The time left is a float pair
// (tau_h + tau_l, error-free updates), counting down to zero.  Only what
// every attempt reads stays in registers; the rest of a particle's state
// (read or written once per accepted step at most) sits in shared memory,
// one column per lane, so more lanes fit on an SM.
struct Particle32 {
    int p;               // particle index, >= pend when the lane is out of work
    int status, att;
    float tau_h, tau_l;  // duration - t
    float dt;
    float2 ph, pl;       // position (x, y): hi and lo parts
    float2 k1;           // f at the current point (first stage, FSAL)
};

// The per-lane cold state in shared memory, four fields to a 16-byte quad:
// quad q of lane t at cold[(q * BLOCK + t) * 4] (a warp's 16-byte accesses
// are conflict-free), field f in quad f / 4 at component f % 4.  An accepted
// step reads the four quads with four 16-byte loads and writes back three.
enum ColdField { kCoff, kRoff, kNcols, kNrows,      // quad 0: the trace's frame (read only)
                 kFx0, kFy0, kRlo, kRhi,            // quad 1: frame origin; rows the trace marked
                 kNtest, kNatom, kAcc, kNv,         // quad 2: counts
                 kBx0, kBx1, kBy0, kBy1,            // quad 3: bounding box
                 kColdFields };
enum ColdQuad { kQFrame, kQWin, kQStat, kQBox };

template <int BLOCK>
struct Cold {
    uint32_t* base;
    __device__ __forceinline__ int& i(ColdField f) const {
        return reinterpret_cast<int*>(base)[(((int)f >> 2) * BLOCK + threadIdx.x) * 4 + ((int)f & 3)];
    }
    __device__ __forceinline__ float& f(ColdField fld) const {
        return reinterpret_cast<float*>(&i(fld))[0];
    }
    __device__ __forceinline__ int4& q(ColdQuad k) const {
        return reinterpret_cast<int4*>(base)[(int)k * BLOCK + threadIdx.x];
    }
};

// The realization's constants come from shared memory (block-uniform).
template <int MODE>
__device__ __forceinline__ bool feval_c(const RealConst32& rc, const float4* wp, const float2* wq, int nw,
                                        float2 ph, float2 pl, float2& k) {
    Model32 m;
    m.wp = wp;
    m.wq = wq;
    m.nw = nw;
    const float4 q0 = rc.q0, q1 = rc.q1, q2 = rc.q2;
    m.c0 = q0.x; m.c1 = q0.y; m.c2 = q0.z; m.c3 = q0.w;
    m.c4 = q1.x; m.c5 = q1.y; m.ox = q1.z; m.oy = q1.w;
    m.inv_hn = q2.x; m.kh2f = q2.y; m.inv_k = q2.z; m.inv_kh = q2.w;
    m.K = rc.K; m.n = rc.n; m.H = rc.H;
    m.d64 = rc.d64;
    return feval32<MODE>(m, ph, pl, k);
}

// Write the finished particle's outputs, and flag its release-point disk
// for marking (relmask: bit p - pbeg) when one of its segments reached the
// row loop.
template <int BLOCK>
__device__ __forceinline__ void finish32(const TrackLaunch& L, int r, const Particle32& s, const Cold<BLOCK>& c,
                                         const Chron& ch, uint32_t* relmask, int pbeg,
                                         unsigned long long* counters) {
    const long long idx = (long long)r * L.npaths + s.p;
    if (c.i(kRlo) != 0x7fffffff) atomicOr(relmask + ((s.p - pbeg) >> 5), 1u << ((s.p - pbeg) & 31));
    if (L.out.endpoint) {
        L.out.endpoint[2 * idx] = L.xt + ((double)s.ph.x + (double)s.pl.x);
        L.out.endpoint[2 * idx + 1] = L.yt + ((double)s.ph.y + (double)s.pl.y);
    }
    if (L.out.bbox) {
        L.out.bbox[4 * idx] = L.xt + (double)c.f(kBx0);
        L.out.bbox[4 * idx + 1] = L.xt + (double)c.f(kBx1);
        L.out.bbox[4 * idx + 2] = L.yt + (double)c.f(kBy0);
        L.out.bbox[4 * idx + 3] = L.yt + (double)c.f(kBy1);
    }
    if (L.out.naccept) L.out.naccept[idx] = c.i(kAcc);
    if (L.out.nattempt) L.out.nattempt[idx] = s.att;
    if (L.out.status) L.out.status[idx] = s.status;
    if (L.out.nvertices) L.out.nvertices[idx] = c.i(kNv);
    note_rows(ch.slot, L.mask_words, L.grid.nrows, c.i(kRlo), c.i(kRhi));
    if (L.out.counters)     // into the block's shared counters; flushed once per block
        add_counters((long long*)counters, s.att, c.i(kAcc), (unsigned)c.i(kNtest), (unsigned)c.i(kNatom),
                     s.status, L.grid, L.xt + (double)c.f(kBx0), L.xt + (double)c.f(kBx1), L.yt + (double)c.f(kBy0),
                     L.yt + (double)c.f(kBy1));
}

// Write the current point as vertex nv of the trace (when vertices are asked for).
__device__ __forceinline__ void push_vertex(const TrackLaunch& L, int r, const Particle32& s, int nv) {
    if (L.out.vertices && nv < L.out.max_vertices) {
        double* v = L.out.vertices + ((long long)r * L.npaths + s.p) * 2LL * L.out.max_vertices;
        v[2 * nv] = L.xt + ((double)s.ph.x + (double)s.pl.x);
        v[2 * nv + 1] = L.yt + ((double)s.ph.y + (double)s.pl.y);
    }
}

// Start particle s.p: release point, frame, first velocity (k1).  Returns
// false when the trace is already over (dry at the release point, or a zero
// duration).
template <int MODE, int BLOCK>
__device__ __forceinline__ bool start32(const TrackLaunch& L, int r, const RealConst32& rc, const float4* wp,
                                        const float2* wq, Particle32& s, const Cold<BLOCK>& c) {
    const double rx = L.release[2 * s.p] - L.xt, ry = L.release[2 * s.p + 1] - L.yt;
    s.ph = make_float2((float)rx, (float)ry);
    s.pl = make_float2((float)(rx - (double)s.ph.x), (float)(ry - (double)s.ph.y));
    const OnekaFrame f = frame_of(L, r, s.p);
    c.q(kQFrame) = make_int4(f.coff, f.roff, f.ncols, f.nrows);
    c.q(kQWin) = make_int4(__float_as_int((float)(f.xmin - L.xt)), __float_as_int((float)(f.ymin - L.yt)),
                           0x7fffffff, -1);
    s.status = ONEKA_TRACE_OK;
    s.att = 0;
    c.q(kQStat) = make_int4(0, 0, 0, 1);      // the release point is vertex 0
    const double dur = L.opts.duration;
    s.tau_h = (float)dur;
    s.tau_l = (float)(dur - (double)s.tau_h);
    s.dt = 0.1f * (dur > 0.0 ? 1.0f : (dur < 0.0 ? -1.0f : 0.0f));
    const float2 p0 = add2(s.ph, s.pl);
    c.q(kQBox) = make_int4(__float_as_int(p0.x), __float_as_int(p0.x), __float_as_int(p0.y), __float_as_int(p0.y));
    push_vertex(L, r, s, 0);
    if (!feval_c<MODE>(rc, wp, wq, L.nwells, s.ph, s.pl, s.k1)) {
        s.status = ONEKA_TRACE_DRY;
        return false;
    }
    return s.tau_h != 0.0f;
}

// One step attempt of the Dormand-Prince integrator (capturezone.py:221-247).
// Returns false when the trace is over.
template <int MODE, int BLOCK>
__device__ __forceinline__ bool attempt32(const TrackLaunch& L, const RealConst32& rc, const float4* wp,
                                          const float2* wq, const Chron& ch, Particle32& s, int r,
                                          const Cold<BLOCK>& c) {
    if (s.att >= L.max_attempts) {
        s.status = ONEKA_TRACE_STEP_LIMIT;
        return false;
    }
    ++s.att;
    // do not step past the duration (capturezone.py:223-224): |dt| > |time left|
    const float tau = s.tau_h + s.tau_l;
    bool last = false;
    if (fabsf(s.dt) > fabsf(tau)) {
        s.dt = tau;
        last = true;
    }
    const float dt = s.dt;
    const float2 DT = splat(dt);
    // running sums of the stage rows and of the error row, seeded with k1
    float2 P[6];
#pragma unroll
    for (int q = 0; q < 6; ++q) P[q] = mul2(splat(dp_a0(q)), s.k1);
    float2 E = mul2(splat(dp_e(0)), s.k1);
    float2 k = make_float2(0.0f, 0.0f);
    bool wet = true;
#pragma unroll
    for (int st = 0; st < 6; ++st) {            // evaluates k2..k7 (unrolled: stage rows are compile-time)
        // a dry stage ends the trace after the attempt (nothing of it is kept)
        wet &= feval_c<MODE>(rc, wp, wq, L.nwells, s.ph, fma2(DT, P[st], s.pl), k);
#pragma unroll
        for (int q = st + 1; q < 6; ++q)
            if (dp_b(st, q) != 0.0f) P[q] = fma2(splat(dp_b(st, q)), k, P[q]);
        E = fma2(splat(dp_e(st + 1)), k, E);
    }
    if (!wet) {
        s.status = ONEKA_TRACE_DRY;
        return false;
    }
    // k = k7 = f(xyt); the 5th-order step is dt * P_5
    const float2 S = mul2(DT, P[5]);
    const float2 Ed = mul2(DT, E);
    const float est = fmaxf(fabsf(Ed.x), fabsf(Ed.y));
    const float2 S2 = mul2(S, S);
    const float ds = sqrtf(S2.x + S2.y);
    const float tol = rc.tol, maxstep = rc.maxstep, eps = (float)DP::eps;
    if ((est < tol) && (ds < maxstep)) {
        if (last) {
            s.tau_h = s.tau_l = 0.0f;
        } else {
            float th, te;
            two_sum(s.tau_h, -dt, th, te);
            te += s.tau_l;
            two_sum(th, te, s.tau_h, s.tau_l);
        }
        const float2 a = add2(s.ph, s.pl);
        float2 q, e;
        two_sum2(s.ph, S, q, e);
        two_sum2(q, add2(s.pl, e), s.ph, s.pl);
        const float2 b = add2(s.ph, s.pl);
        int4 stat = c.q(kQStat);                 // ntest, natom, accepted steps, vertices
        if (ch.slot) {
            const int4 fr = c.q(kQFrame);        // coff, roff, ncols, nrows
            const int4 wn = c.q(kQWin);          // fx0, fy0 (float bits), rlo, rhi
            unsigned ntest = (unsigned)stat.x, natom = (unsigned)stat.y;
            int rlo = wn.z, rhi = wn.w;
            insert32(ch, L.grid.nrows, L.grid.ncols, fr.x, fr.y, fr.z, fr.w, __int_as_float(wn.x),
                     __int_as_float(wn.y), rc.g, a.x, a.y, b.x, b.y, ntest, natom, rlo, rhi);
            stat.x = (int)ntest;
            stat.y = (int)natom;
            reinterpret_cast<int2*>(&c.q(kQWin))[1] = make_int2(rlo, rhi);
        }
        int4& bq = c.q(kQBox);
        const int4 bx = bq;
        bq = make_int4(__float_as_int(fminf(__int_as_float(bx.x), b.x)), __float_as_int(fmaxf(__int_as_float(bx.y), b.x)),
                       __float_as_int(fminf(__int_as_float(bx.z), b.y)), __float_as_int(fmaxf(__int_as_float(bx.w), b.y)));
        s.k1 = k;
        push_vertex(L, r, s, stat.w);
        stat.z += 1;
        stat.w += 1;
        c.q(kQStat) = stat;
    }
    float fac = __powf(tol / (est + eps), 0.2f);
    const float fstep = maxstep / (ds + eps);
    if (fstep < fac) fac = fstep;
    if (10.0f < fac) fac = 10.0f;
    s.dt = 0.9f * fac * dt;
    return s.tau_h != 0.0f;
}

// One block: realization k of launch L (wave-local), particles of chunk `chunk`.
template <int MODE, int BLOCK>
__device__ __forceinline__ void block32(const TrackLaunch& L, int k, int chunk, int chunks) {
    extern __shared__ float4 sm32[];
    __shared__ RealConst32 rc;
    const int r = L.r0 + k;
    float4* wp = sm32;                                        // [nwells] positions (hi, lo), negated
    float2* wq = reinterpret_cast<float2*>(sm32 + L.nwells);  // [nwells] well constants
    Cold<BLOCK> cold;
    cold.base = reinterpret_cast<uint32_t*>(sm32 + well_float4s(L.nwells));
    uint32_t* slot = L.slots ? L.slots + (long long)k * L.slot_words : nullptr;
    // particles [pbeg, pend) of this block
    const int per = (L.npaths + chunks - 1) / chunks;
    uint32_t* relmask = cold.base + kColdFields * BLOCK;        // [ceil(per / 32)] release-disk flags
    const Chron ch = make_chron(L, slot, relmask + (per + 31) / 32);
    const int pbeg = chunk * per;
    const int pend = min(L.npaths, pbeg + per);
    if (threadIdx.x == 0) {
        const double* c = L.coef + 6LL * r;
        const double Kd = L.aquifer[3LL * r], nd = L.aquifer[3LL * r + 1], Hd = L.aquifer[3LL * r + 2];
        rc.q0 = make_float4((float)c[0], (float)c[1], (float)c[2], (float)c[3]);
        rc.q1 = make_float4((float)c[4], (float)c[5], (float)(L.xo - L.xt), (float)(L.yo - L.yt));
        rc.q2 = make_float4((float)(1.0 / (Hd * nd)), (float)(0.5 * Kd * (Hd * Hd)), (float)(1.0 / Kd),
                            (float)(1.0 / (Kd * Hd)));
        rc.K = (float)Kd; rc.n = (float)nd; rc.H = (float)Hd;
        rc.d64[0] = Kd; rc.d64[1] = nd; rc.d64[2] = Hd;
        rc.tol = (float)L.opts.tol;
        rc.maxstep = (float)L.opts.maxstep;
        rc.g.dx = (float)L.grid.dx;
        rc.g.dy = (float)L.grid.dy;
        rc.g.inv_dx = (float)(1.0 / L.grid.dx);
        rc.g.inv_dy = (float)(1.0 / L.grid.dy);
        rc.g.U = (float)(L.opts.umbra / L.grid.dx);
        rc.g.U2 = rc.g.U * rc.g.U;
        rc.g.ryy = (float)(L.grid.dy / L.grid.dx);
        rc.g.umbra = (float)L.opts.umbra;
        rc.skip = L.rstatus && L.rstatus[r] != ONEKA_REAL_OK;
        rc.next = pbeg + BLOCK;
        if (!rc.skip && chunk == 0 && L.registered) atomicAdd(L.registered, 1ull);
    }
    for (int i = threadIdx.x; i < L.nwells; i += BLOCK) {
        const double q = L.q[(long long)r * L.nwells + i];
        const double dx = L.wells[3 * i] - L.xt, dy = L.wells[3 * i + 1] - L.yt;
        const float xh = (float)dx, yh = (float)dy;
        wp[i] = make_float4(-xh, -yh, -(float)(dx - (double)xh), -(float)(dy - (double)yh));
        wq[i] = make_float2((float)(-q * 0.15915494309189535),
                            (float)(q * (0.07957747154594767 * 0.69314718055994531)));
    }
    window_clear(ch);
    for (int i = threadIdx.x; i < (per + 31) / 32; i += BLOCK) relmask[i] = 0u;
    if (threadIdx.x < 8) rc.counters[threadIdx.x] = 0ull;
    __syncthreads();
    if (rc.skip) {
        if (L.out.status)
            for (int p = pbeg + threadIdx.x; p < pend; p += BLOCK)
                L.out.status[(long long)r * L.npaths + p] = kTraceSkipped;
        return;   // uniform across the block: nothing was marked
    }
    Particle32 s;
    s.p = pbeg + threadIdx.x;
    bool live = false;
    // start this lane's first particle; a lane whose trace ends at once takes the next
    while (s.p < pend && !live) {
        live = start32<MODE, BLOCK>(L, r, rc, wp, wq, s, cold);
        if (!live) {
            finish32<BLOCK>(L, r, s, cold, ch, relmask, pbeg, rc.counters);
            s.p = atomicAdd(&rc.next, 1);
        }
    }
    // Warp-uniform: the vote gathers the lanes again before every attempt, so
    // a divergent chronicle insertion or refill never leaves the warp running
    // the next stage evaluations in separate groups.  BLOCK is a multiple of 32.
    while (__any_sync(0xffffffffu, live)) {
        if (!live) continue;
        live = attempt32<MODE, BLOCK>(L, rc, wp, wq, ch, s, r, cold);
        while (!live && s.p < pend) {
            finish32<BLOCK>(L, r, s, cold, ch, relmask, pbeg, rc.counters);
            s.p = atomicAdd(&rc.next, 1);
            if (s.p < pend) live = start32<MODE, BLOCK>(L, r, rc, wp, wq, s, cold);
        }
    }
    __syncthreads();
    // The release-point disks of the flagged traces, all lanes together.  (The
    // test stays outside the loop: folded into the loop condition it made
    // the compiled kernel issue 1.8 % more instructions.)
    if (ch.slot) {
        for (int p = pbeg + threadIdx.x; p < pend; p += BLOCK) {
            if (!((relmask[(p - pbeg) >> 5] >> ((p - pbeg) & 31)) & 1u)) continue;
            const double rx = L.release[2 * p] - L.xt, ry = L.release[2 * p + 1] - L.yt;
            const float2 h = make_float2((float)rx, (float)ry);
            const float2 a = add2(h, make_float2((float)(rx - (double)h.x), (float)(ry - (double)h.y)));
            const OnekaFrame f = frame_of(L, r, p);
            int rlo = 0x7fffffff, rhi = -1;
            disk32(ch, L.grid.nrows, L.grid.ncols, f.coff, f.roff, f.ncols, f.nrows, (float)(f.xmin - L.xt),
                   (float)(f.ymin - L.yt), rc.g, a.x, a.y, rlo, rhi);
            note_rows(ch.slot, L.mask_words, L.grid.nrows, rlo, rhi);
        }
    }
    __syncthreads();
    window_flush(ch);
    // the block's counters in one atomic each (per-particle global atomics on
    // eight addresses serialized in L2)
    if (L.out.counters && threadIdx.x < 8 && rc.counters[threadIdx.x])
        atomicAdd((unsigned long long*)L.out.counters + threadIdx.x, rc.counters[threadIdx.x]);
}

template <int MODE, int BLOCK, int MINB>
__global__ void __launch_bounds__(BLOCK, MINB) track32_kernel(const TrackLaunch L, int chunks) {
    block32<MODE, BLOCK>(L, blockIdx.y, blockIdx.x, chunks);
}

// Many sites in one launch: row blockIdx.x belongs to job j with
// first[j] <= row < first[j + 1]; jobs may differ in wells, paths, grid,
// duration and aquifer type.  blockIdx.y is the particle chunk.  Rows run
// along x (up to 2^31 - 1 of them) and the host packs the costliest jobs
// first, so they are dispatched first.  The table is a __grid_constant__
// parameter, so it is read in place (no copy) and a captured CUDA graph
// carries it.
template <int BLOCK, int MINB>
__global__ void __launch_bounds__(BLOCK, MINB) track32_batch_kernel(const __grid_constant__ JobTable T,
                                                                     int chunks) {
    const int row = blockIdx.x;
    int lo = 0, hi = T.njobs - 1;
    while (lo < hi) {                       // last job with first[j] <= row
        const int mid = (lo + hi + 1) >> 1;
        if (T.first[mid] <= row) lo = mid; else hi = mid - 1;
    }
    const TrackLaunch& J = T.job[lo];
    const int k = row - T.first[lo];
    if (J.opts.confined)
        block32<kConfined, BLOCK>(J, k, blockIdx.y, chunks);
    else
        block32<kGeneral, BLOCK>(J, k, blockIdx.y, chunks);
}

template <int MODE, int BLOCK, int MINB>
cudaError_t launch_variant(const TrackLaunch& L, cudaStream_t s) {
    static int sms = 0;
    if (!sms) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (sms <= 0) sms = 1;
    }
    // split realizations into particle chunks only when they cannot fill the
    // GPU, and so that no block takes more than kMaxChunk particles
    const int target = 2 * sms * MINB;
    int chunks = 1;
    if (L.nr < target) {
        chunks = (target + L.nr - 1) / L.nr;
        const int maxc = (L.npaths + BLOCK - 1) / BLOCK;
        if (chunks > maxc) chunks = maxc;
        if (chunks < 1) chunks = 1;
    }
    chunks = max(chunks, (L.npaths + kMaxChunk - 1) / kMaxChunk);
    const int per = (L.npaths + chunks - 1) / chunks;
    const size_t smem = sizeof(float4) * (size_t)well_float4s(L.nwells) + 4 * (size_t)kColdFields * BLOCK +
                        4 * (size_t)((per + 31) / 32) + 4 * (size_t)L.win_rows * L.win_words;
    auto kern = track32_kernel<MODE, BLOCK, MINB>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    kern<<<dim3((unsigned)chunks, (unsigned)L.nr), BLOCK, smem, s>>>(L, chunks);
    return cudaGetLastError();
}

template <int MODE>
cudaError_t launch_mode(const TrackLaunch& L, cudaStream_t s) {
    // (threads per block, minimum resident blocks per SM): the variants the
    // autotuner chooses between through OnekaTrackOpts.block / .occupancy
    const int block = L.opts.block > 0 ? L.opts.block : 256;
    const int occ = L.opts.occupancy;
    if (block == 64) return launch_variant<MODE, 64, 8>(L, s);
    if (block == 256) return occ >= 4 ? launch_variant<MODE, 256, 4>(L, s)
                           : occ >= 3 ? launch_variant<MODE, 256, 3>(L, s)
                                      : launch_variant<MODE, 256, 2>(L, s);
    if (block == 32) return launch_variant<MODE, 32, 16>(L, s);
    if (occ >= 8) return launch_variant<MODE, 128, 8>(L, s);
    if (occ >= 6) return launch_variant<MODE, 128, 6>(L, s);
    return launch_variant<MODE, 128, 4>(L, s);
}

template <int BLOCK, int MINB>
cudaError_t launch_batch_variant(const JobTable& T, int rows, size_t smem, cudaStream_t s) {
    static int sms = 0;
    if (!sms) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (sms <= 0) sms = 1;
    }
    int minp = 1 << 30, maxp = 0;
    for (int j = 0; j < T.njobs; ++j) {
        minp = min(minp, T.job[j].npaths);
        maxp = max(maxp, T.job[j].npaths);
    }
    const int target = 2 * sms * MINB;
    int chunks = 1;
    if (rows < target) {
        chunks = (target + rows - 1) / rows;
        const int maxc = (minp + BLOCK - 1) / BLOCK;
        if (chunks > maxc) chunks = maxc;
        if (chunks < 1) chunks = 1;
    }
    chunks = max(chunks, (maxp + kMaxChunk - 1) / kMaxChunk);
    smem += 4 * (size_t)(((maxp + chunks - 1) / chunks + 31) / 32);   // the release-disk flags
    auto kern = track32_batch_kernel<BLOCK, MINB>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    kern<<<dim3((unsigned)rows, (unsigned)chunks), BLOCK, smem, s>>>(T, chunks);
    return cudaGetLastError();
}

}  // namespace

cudaError_t launch_track32(const TrackLaunch& L, cudaStream_t s) {
    if (L.opts.confined) return launch_mode<kConfined>(L, s);
    // the FP64 near-top head inversion is compiled for the default launch shape only
    if (L.opts.head64) return launch_variant<kGeneralHead64, 256, 3>(L, s);
    return launch_mode<kGeneral>(L, s);
}

cudaError_t launch_track32_batch(const JobTable& T, int rows, cudaStream_t s) {
    if (T.njobs <= 0 || rows <= 0) return cudaSuccess;
    const int block = T.job[0].opts.block > 0 ? T.job[0].opts.block : 256;
    const int occ = T.job[0].opts.occupancy;
    size_t smem = 0;
    for (int j = 0; j < T.njobs; ++j) {
        const TrackLaunch& L = T.job[j];
        const size_t need = sizeof(float4) * (size_t)well_float4s(L.nwells) + 4 * (size_t)kColdFields * block +
                            4 * (size_t)L.win_rows * L.win_words;
        if (need > smem) smem = need;
    }
    if (block == 64) return launch_batch_variant<64, 8>(T, rows, smem, s);
    if (block == 256) return occ >= 4 ? launch_batch_variant<256, 4>(T, rows, smem, s)
                           : occ >= 3 ? launch_batch_variant<256, 3>(T, rows, smem, s)
                                      : launch_batch_variant<256, 2>(T, rows, smem, s);
    if (block == 32) return launch_batch_variant<32, 16>(T, rows, smem, s);
    if (occ >= 8) return launch_batch_variant<128, 8>(T, rows, smem, s);
    if (occ >= 6) return launch_batch_variant<128, 6>(T, rows, smem, s);
    return launch_batch_variant<128, 4>(T, rows, smem, s);
}

}  // namespace oneka
