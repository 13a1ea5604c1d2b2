// gemm_tc.cu -- the surrogate's BF16 GEMM on the 5th-generation tensor cores.
//
// C[M][N] = A[M][K] * B[N][K]^T (both operands K-major, BF16; FP32
// accumulation) for the layers of the surrogate MLP, with fused epilogues:
// bias + FP32 store (logits), bias + GELU storing the pre-activation and the
// activation in BF16 (hidden layers), bias + sigmoid summed over the rows
// (the screened capture field; C is never stored), and split-K, where each
// K slice of a tile adds its partial product into a zeroed FP32 C (the
// backward GEMMs whose K is the 65,536 outputs).
//
// A persistent, warp-specialized kernel: one CTA per SM walks work items,
// 128 x 256 output tiles (M fastest, so consecutive tiles reuse the same B
// slice from L2), times the K slices of a split-K launch.
//   * warp 0 (one lane): TMA producer.  cp.async.bulk.tensor with the 128-byte
//     swizzle stages 64-wide K slices of A (128 x 64) and B (256 x 64) into a
//     4-stage shared-memory ring; "full" mbarriers complete on the copies'
//     transaction bytes.
//   * warp 1 (one lane): MMA issuer.  tcgen05.mma (kind::f16, M = 128,
//     N = 256, K = 16) accumulates a tile in one of two 256-column FP32
//     buffers of tensor memory; tcgen05.commit releases each ring stage
//     ("empty") once its MMAs have read it, and hands a finished
//     accumulator to the epilogue ("acc_full").
//   * warps 2-17: epilogue.  Warp w reads TMEM lane quadrant w % 4 (tile rows
//     32 (w % 4) ..) and one 64-column block of the tile with tcgen05.ld,
//     applies the epilogue, and frees the buffer ("acc_empty"), so the
//     epilogue of one tile overlaps the MMAs of the next.  Sixteen warps keep
//     the epilogue's latencies (TMEM loads, the sigmoid, the column-sum
//     shuffles) hidden.
// Pairs (CL = 2): when the output has an even number of M tiles, a launch
// runs clusters of two CTAs on two SMs, which work on the M tiles 2j and
// 2j + 1 of the same N tile at once.  Each CTA loads its own A slice and one
// half of the shared B slice; the B half goes to both CTAs' shared memory by
// TMA multicast, so each SM reads 32 KB from L2 per 64-wide K step instead
// of 48 KB (the kernel is bound by L2 -> SM bandwidth).  A ring stage is
// refilled only when both CTAs' MMAs have read it: each MMA issuer's commit
// arrives on the "empty" barrier of both CTAs.
// Every mbarrier wait is bounded by the global timer: on a timeout the
// kernel records an error, waits (bounded) for its own copies and MMAs in
// flight, frees its tensor memory and returns.
//
// No counterpart in the reference (the surrogate is this project's own).
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>
#include <math.h>
#include <stdint.h>

#include <mutex>

#include "oneka_internal.cuh"

namespace oneka {

__device__ int g_tc_error;   // first failure code of a tensor-core GEMM (0: none)

namespace {

constexpr int TM = 128, TN = 256, TK = 64, STAGES = 4;
constexpr int EPI_WARPS = 16;                 // 4 per TMEM lane quadrant, 64 columns each
constexpr int THREADS = 64 + 32 * EPI_WARPS;
constexpr int A_BYTES = TM * TK * 2;          // 16 KB
constexpr int B_BYTES = TN * TK * 2;          // 32 KB
constexpr int STAGE_BYTES = A_BYTES + B_BYTES;
// Each epilogue warp's staging area for the FP32 stores: its 32 rows x 16
// columns, so that a store instruction writes 8 rows x 64 contiguous bytes
// instead of 32 rows x 16 bytes (whole 32-byte sectors, half the requests).
constexpr int EPI_STAGE_FLOATS = 32 * 16;
constexpr int SMEM_BYTES = STAGES * STAGE_BYTES + EPI_WARPS * EPI_STAGE_FLOATS * 4 + 1024;   // + alignment slack
constexpr int TMEM_COLS = 512;       // two 256-column accumulators
constexpr unsigned long long kWaitNs = 2000000000ull;      // 2 s per wait

enum TcEpilogue { kEpiF32 = 0, kEpiGelu = 1, kEpiSigsum = 2, kEpiF32Add = 3 };

struct TcArgs {
    void* C;              // kEpiF32: float [M][ldc]; kEpiGelu: bf16 H [M][ldc]
    __nv_bfloat16* Z;     // kEpiGelu: bf16 pre-activation [M][ldc]
    const float* bias;    // [N] or null
    float* sigsum;        // kEpiSigsum: out[N] += sum over rows of sigmoid
    int M, N, K, ldc;
    int ksplit;           // kEpiF32Add: K slices per output tile, each adding its partial product into C
    int kper;             // K tiles (of TK) per slice
};

// Work item w of a launch (of a CTA pair when CL = 2): output tile group
// w % groups, K slice w / groups (K tiles [kb, ke)).  A group is CL tiles
// along M of one N tile; the CTA of cluster rank `rank` takes the group's
// tile `rank`.  Groups run M fastest, so consecutive items reuse B slices.
struct TcItem {
    int m0, n0, kb, ke, slice;
};

template <int CL>
__device__ __forceinline__ TcItem tc_item(const TcArgs& g, int w, int mt, int groups, int ktiles, int rank) {
    TcItem it;
    const int t = w % groups;
    const int mg = mt / CL;
    it.slice = w / groups;
    it.m0 = ((t % mg) * CL + rank) * TM;
    it.n0 = (t / mg) * TN;
    it.kb = it.slice * g.kper;
    it.ke = min(ktiles, it.kb + g.kper);
    return it;
}

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count));
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

__device__ __forceinline__ bool mbar_try(uint32_t bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n.reg .pred p;\n"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        "selp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}

// Wait for phase `parity` of an mbarrier, at most kWaitNs; false on timeout
// or when another role of the CTA has already given up.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, volatile int* abort_flag) {
    const unsigned long long t0 = global_ns();
    for (unsigned it = 0;; ++it) {
        if (mbar_try(bar, parity)) return true;
        if ((it & 255u) == 255u) {
            if (*abort_flag) return false;
            if (global_ns() - t0 > kWaitNs) {
                *abort_flag = 1;
                atomicCAS(&g_tc_error, 0, 1);
                return false;
            }
        }
    }
}

// Teardown wait: bounded by time only (the CTA has already given up; this
// only lets its own copies and MMAs land before the memory they use goes away).
__device__ __forceinline__ void mbar_drain(uint32_t bar, uint32_t parity) {
    const unsigned long long t0 = global_ns();
    for (unsigned it = 0;; ++it) {
        if (mbar_try(bar, parity)) return;
        if ((it & 255u) == 255u && global_ns() - t0 > kWaitNs) return;
    }
}

__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap* map, int x, int y, uint32_t bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];"
        ::"r"(dst), "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(bar)
        : "memory");
}

// The same copy written to shared memory at the same offset in every CTA of
// the cluster named in `mask`, completing bytes on each one's barrier there.
__device__ __forceinline__ void tma_load_2d_mc(uint32_t dst, const CUtensorMap* map, int x, int y, uint32_t bar,
                                               uint16_t mask) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes.multicast::cluster"
        " [%0], [%1, {%2, %3}], [%4], %5;"
        ::"r"(dst), "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(bar), "h"(mask)
        : "memory");
}

__device__ __forceinline__ uint32_t cluster_rank() {
    uint32_t r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}

// Every thread of every CTA of the cluster.
__device__ __forceinline__ void cluster_sync() {
    asm volatile("barrier.cluster.arrive.release.aligned;" ::: "memory");
    asm volatile("barrier.cluster.wait.acquire.aligned;" ::: "memory");
}

// Shared-memory matrix descriptor of a K-major tile written by TMA with the
// 128-byte swizzle: rows of 128 bytes (64 BF16), 8-row swizzle atoms of
// 1024 bytes (stride-dimension offset), version 1, swizzle mode 2 (128 B).
__device__ __forceinline__ uint64_t sw128_desc(uint32_t addr) {
    uint64_t d = 0;
    d |= (uint64_t)((addr & 0x3FFFFu) >> 4);            // start address
    d |= (uint64_t)(16u >> 4) << 16;                    // leading-dimension offset (unused for swizzled K-major)
    d |= (uint64_t)(1024u >> 4) << 32;                  // stride-dimension offset
    d |= 1ull << 46;                                    // descriptor version
    d |= 2ull << 61;                                    // 128-byte swizzle
    return d;
}

// Instruction descriptor of kind::f16: FP32 accumulator, BF16 A and B, both
// K-major, N = TN, M = TM.
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(TN >> 3) << 17) |
                            ((uint32_t)(TM >> 4) << 24);

__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t accumulate) {
    asm volatile(
        "{\n.reg .pred p;\n"
        "setp.ne.b32 p, %4, 0;\n"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}"
        ::"r"(tmem_d), "l"(adesc), "l"(bdesc), "r"(kIdesc), "r"(accumulate));
}

__device__ __forceinline__ void mma_commit(uint32_t bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
                 : "memory");
}

// Arrive on the barrier at this offset in every CTA of `mask` once the MMAs
// issued so far have completed.
__device__ __forceinline__ void mma_commit_mc(uint32_t bar, uint16_t mask) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.multicast::cluster.b64 [%0], %1;"
                 ::"r"(bar), "h"(mask)
                 : "memory");
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int j = 0; j < 16; ++j) v[j] = __uint_as_float(r[j]);
}

__device__ __forceinline__ float gelu_tc(float x) { return 0.5f * x * (1.0f + erff(x * 0.70710678118654752f)); }

// Sum 16 column values over the warp's 32 lanes (rows): recursive halving,
// 16 shuffles; returns the total of column (8 b4 + 4 b3 + 2 b2 + b1) in
// every lane, b_i the lane's bits.
__device__ __forceinline__ float warp_colsum16(float (&v)[16], int lane) {
#pragma unroll
    for (int half = 8, bit = 16; half >= 1; half >>= 1, bit >>= 1) {
        const bool up = (lane & bit) != 0;
#pragma unroll
        for (int j = 0; j < half; ++j) {
            const float send = up ? v[j] : v[j + half];
            const float keep = up ? v[j + half] : v[j];
            v[j] = keep + __shfl_xor_sync(0xffffffffu, send, bit);
        }
    }
    return v[0] + __shfl_xor_sync(0xffffffffu, v[0], 1);
}

template <int EPI, int CL>
__global__ void __launch_bounds__(THREADS, 1)
    gemm_tc_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB, const TcArgs g) {
    extern __shared__ __align__(1024) unsigned char tc_smem[];
    __shared__ __align__(8) uint64_t full[STAGES], empty[STAGES], acc_full[2], acc_empty[2], drain;
    __shared__ uint32_t tmem_base;
    __shared__ int abort_flag;
    __shared__ int issued, consumed;

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int mt = (g.M + TM - 1) / TM, nt = (g.N + TN - 1) / TN, groups = (mt / CL) * nt;
    const int ktiles = g.K / TK;
    const int items = groups * g.ksplit;
    // this CTA's place: cluster `cid` of `ncl`, rank `rank` in it
    const int rank = CL > 1 ? (int)cluster_rank() : 0;
    const int cid = blockIdx.x / CL, ncl = gridDim.x / CL;
    constexpr uint16_t kPair = (uint16_t)((1u << CL) - 1u);
    unsigned char* base = tc_smem + ((1024u - (smem_addr(tc_smem) & 1023u)) & 1023u);
    const uint32_t sA = smem_addr(base), sB = sA + STAGES * A_BYTES;

    if (threadIdx.x == 0) {
        for (int s = 0; s < STAGES; ++s) {
            mbar_init(smem_addr(&full[s]), 1);
            mbar_init(smem_addr(&empty[s]), CL);       // one commit from each CTA's MMA issuer
        }
        for (int b = 0; b < 2; ++b) {
            mbar_init(smem_addr(&acc_full[b]), 1);
            mbar_init(smem_addr(&acc_empty[b]), EPI_WARPS);     // one arrival per epilogue warp
        }
        mbar_init(smem_addr(&drain), 1);
        abort_flag = 0;
        issued = consumed = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                     ::"r"(smem_addr(&tmem_base)), "r"(TMEM_COLS));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (CL > 1) cluster_sync();      // the peer's barriers are initialised before any copy reaches them
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = tmem_base;
    volatile int* abort_v = &abort_flag;

    if (warp == 0) {
        if (lane == 0) {
            // producer: TMA slices of A and B into the ring, tile after tile
            int it = 0;
            for (int w = cid; w < items && !*abort_v; w += ncl) {
                const TcItem c = tc_item<CL>(g, w, mt, groups, ktiles, rank);
                int kt = c.kb;
                for (; kt < c.ke; ++kt, ++it) {
                    const int s = it % STAGES;
                    if (it >= STAGES && !mbar_wait(smem_addr(&empty[s]), ((it / STAGES) - 1) & 1, abort_v)) break;
                    const uint32_t bar = smem_addr(&full[s]);
                    mbar_expect_tx(bar, STAGE_BYTES);      // A, and both halves of B when CL = 2
                    tma_load_2d(sA + s * A_BYTES, &tmA, kt * TK, c.m0, bar);
                    if (CL > 1)
                        tma_load_2d_mc(sB + s * B_BYTES + rank * (B_BYTES / CL), &tmB, kt * TK,
                                       c.n0 + rank * (TN / CL), bar, kPair);
                    else
                        tma_load_2d(sB + s * B_BYTES, &tmB, kt * TK, c.n0, bar);
                    issued = it + 1;
                }
                if (kt < c.ke) break;
            }
        }
    } else if (warp == 1) {
        if (lane == 0) {
            // MMA issuer: tile tl of this CTA accumulates in buffer tl & 1
            int it = 0, tl = 0;
            for (int w = cid; w < items && !*abort_v; w += ncl, ++tl) {
                const TcItem c = tc_item<CL>(g, w, mt, groups, ktiles, rank);
                const int b = tl & 1, u = tl >> 1;
                if (tl >= 2 && !mbar_wait(smem_addr(&acc_empty[b]), (u - 1) & 1, abort_v)) break;
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                const uint32_t acc = tmem + (uint32_t)(b * TN);
                int kt = c.kb;
                for (; kt < c.ke; ++kt, ++it) {
                    const int s = it % STAGES;
                    if (!mbar_wait(smem_addr(&full[s]), (it / STAGES) & 1, abort_v)) break;
                    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                    const uint64_t ad = sw128_desc(sA + s * A_BYTES), bd = sw128_desc(sB + s * B_BYTES);
#pragma unroll
                    for (int kk = 0; kk < TK / 16; ++kk)   // +32 bytes of K per MMA: +2 in the encoded address
                        mma_bf16(acc, ad + 2 * kk, bd + 2 * kk, (kt > c.kb || kk > 0) ? 1u : 0u);
                    if (CL > 1)
                        mma_commit_mc(smem_addr(&empty[s]), kPair);   // frees the stage in both CTAs
                    else
                        mma_commit(smem_addr(&empty[s]));
                    consumed = it + 1;
                }
                if (kt < c.ke) break;
                mma_commit(smem_addr(&acc_full[b]));   // fires when the tile's MMAs have completed
            }
            if (*abort_v) {                          // let every MMA issued above land
                mma_commit(smem_addr(&drain));
                mbar_drain(smem_addr(&drain), 0);
            }
        }
    } else {
        // epilogue warps 2..17: TMEM lane quadrant q = warp % 4 (tile rows
        // 32q .. 32q + 31), columns [cb, cb + 64) of the tile
        const int q = warp & 3, cb = ((warp - 2) >> 2) * 64;
        int tl = 0;
        for (int w = cid; w < items; w += ncl, ++tl) {
            const int b = tl & 1, u = tl >> 1;
            int okw = 0;
            if (lane == 0) okw = mbar_wait(smem_addr(&acc_full[b]), u & 1, abort_v) ? 1 : 0;
            okw = __shfl_sync(0xffffffffu, okw, 0);      // warp-uniform (tcgen05.ld is warp-collective)
            if (!okw) break;
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const TcItem ci = tc_item<CL>(g, w, mt, groups, ktiles, rank);
            const int m0 = ci.m0, n0 = ci.n0;
            const float* bias = ci.slice == 0 ? g.bias : nullptr;   // a split product adds the bias once
            const int row = m0 + q * 32 + lane;
            const bool rows_in = m0 + q * 32 + 32 <= g.M;          // the warp's 32 rows all exist
            const uint32_t trow = tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(b * TN);
#pragma unroll 1
            for (int c = cb; c < cb + 64; c += 16) {
                const int nc = n0 + c;
                if (nc >= g.N) break;                        // uniform across the warp
                const bool whole = nc + 16 <= g.N;
                // the bias of these columns is requested before the tensor-memory
                // load, so the two latencies overlap
                float4 bq[4];
                if (bias && whole) {
                    const float4* bp = reinterpret_cast<const float4*>(bias + nc);
#pragma unroll
                    for (int j = 0; j < 4; ++j) bq[j] = __ldg(bp + j);
                }
                float v[16];
                tmem_ld16(trow + c, v);
                if (bias) {
                    if (whole) {
#pragma unroll
                        for (int j = 0; j < 4; ++j) {
                            v[4 * j] += bq[j].x; v[4 * j + 1] += bq[j].y; v[4 * j + 2] += bq[j].z; v[4 * j + 3] += bq[j].w;
                        }
                    } else {
#pragma unroll
                        for (int j = 0; j < 16; ++j)
                            if (nc + j < g.N) v[j] += __ldg(bias + nc + j);
                    }
                }
                if (EPI == kEpiSigsum) {
                    // sigmoid with the hardware exponential and reciprocal (each
                    // within 2 ulp; a correctly rounded division here cost the
                    // epilogue most of its issue slots)
                    if (rows_in) {
#pragma unroll
                        for (int j = 0; j < 16; ++j) v[j] = __fdividef(1.0f, 1.0f + __expf(-v[j]));
                    } else {
#pragma unroll
                        for (int j = 0; j < 16; ++j) v[j] = row < g.M ? __fdividef(1.0f, 1.0f + __expf(-v[j])) : 0.0f;
                    }
                    const float sum = warp_colsum16(v, lane);
                    const int col = nc + 8 * ((lane >> 4) & 1) + 4 * ((lane >> 3) & 1) + 2 * ((lane >> 2) & 1) +
                                    ((lane >> 1) & 1);
                    if ((lane & 1) == 0 && col < g.N) atomicAdd(g.sigsum + col, sum);
                } else if ((EPI == kEpiF32 || EPI == kEpiF32Add) && whole && rows_in) {
                    // row `lane` goes to the staging area (float4 k of row r in
                    // slot k ^ ((r >> 1) & 3): conflict-free), then lanes 4i..4i+3
                    // store row 4i + t, 16 columns, for t = 0..3
                    float4* st = reinterpret_cast<float4*>(base + STAGES * STAGE_BYTES) + (warp - 2) * (EPI_STAGE_FLOATS / 4);
#pragma unroll
                    for (int k = 0; k < 4; ++k)
                        st[lane * 4 + (k ^ ((lane >> 1) & 3))] = make_float4(v[4 * k], v[4 * k + 1], v[4 * k + 2], v[4 * k + 3]);
                    __syncwarp();
                    const int j = lane & 3;
#pragma unroll
                    for (int t = 0; t < 4; ++t) {
                        const int r = (lane & ~3) + t;
                        const float4 x = st[r * 4 + (j ^ ((r >> 1) & 3))];
                        float* Cp = reinterpret_cast<float*>(g.C) + (long long)(m0 + q * 32 + r) * g.ldc + nc + 4 * j;
                        if (EPI == kEpiF32Add)
                            atomicAdd(reinterpret_cast<float4*>(Cp), x);
                        else
                            *reinterpret_cast<float4*>(Cp) = x;
                    }
                    __syncwarp();
                } else if (row < g.M) {
                    const long long off = (long long)row * g.ldc + nc;
                    if (EPI == kEpiF32Add) {
                        float* Cp = reinterpret_cast<float*>(g.C) + off;
                        if (whole) {
#pragma unroll
                            for (int j = 0; j < 16; j += 4)
                                atomicAdd(reinterpret_cast<float4*>(Cp + j), make_float4(v[j], v[j + 1], v[j + 2],
                                                                                         v[j + 3]));
                        } else {
#pragma unroll
                            for (int j = 0; j < 16; ++j)
                                if (nc + j < g.N) atomicAdd(Cp + j, v[j]);
                        }
                    } else if (EPI == kEpiF32) {
                        float* Cp = reinterpret_cast<float*>(g.C) + off;
                        if (whole) {
#pragma unroll
                            for (int j = 0; j < 16; j += 4)
                                *reinterpret_cast<float4*>(Cp + j) = make_float4(v[j], v[j + 1], v[j + 2], v[j + 3]);
                        } else {
#pragma unroll
                            for (int j = 0; j < 16; ++j)
                                if (nc + j < g.N) Cp[j] = v[j];
                        }
                    } else {
                        __nv_bfloat16* H = reinterpret_cast<__nv_bfloat16*>(g.C) + off;
                        __nv_bfloat16* Z = g.Z + off;
                        if (whole) {
                            uint32_t zp[8], hp[8];
#pragma unroll
                            for (int j = 0; j < 8; ++j) {
                                const __nv_bfloat162 z2 = __floats2bfloat162_rn(v[2 * j], v[2 * j + 1]);
                                const __nv_bfloat162 h2 =
                                    __floats2bfloat162_rn(gelu_tc(v[2 * j]), gelu_tc(v[2 * j + 1]));
                                zp[j] = *reinterpret_cast<const uint32_t*>(&z2);
                                hp[j] = *reinterpret_cast<const uint32_t*>(&h2);
                            }
                            uint4* zq = reinterpret_cast<uint4*>(Z);
                            uint4* hq = reinterpret_cast<uint4*>(H);
                            zq[0] = make_uint4(zp[0], zp[1], zp[2], zp[3]);
                            zq[1] = make_uint4(zp[4], zp[5], zp[6], zp[7]);
                            hq[0] = make_uint4(hp[0], hp[1], hp[2], hp[3]);
                            hq[1] = make_uint4(hp[4], hp[5], hp[6], hp[7]);
                        } else {
#pragma unroll
                            for (int j = 0; j < 16; ++j) {
                                if (nc + j < g.N) {
                                    Z[j] = __float2bfloat16(v[j]);
                                    H[j] = __float2bfloat16(gelu_tc(v[j]));
                                }
                            }
                        }
                    }
                }
            }
            asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
            __syncwarp();
            if (lane == 0) mbar_arrive(smem_addr(&acc_empty[b]));
        }
    }

    // teardown: nothing of ours may still be in flight when the tensor memory
    // is freed and the CTA exits
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (threadIdx.x == 0 && *abort_v) {
        for (int k = consumed; k < issued; ++k)      // copies not yet consumed by an MMA
            mbar_drain(smem_addr(&full[k % STAGES]), (k / STAGES) & 1);
    }
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS));
    // neither CTA of a pair leaves while the other's copies or commits may
    // still reach its shared memory
    if (CL > 1) cluster_sync();
}

int sm_count() {
    static int n[64] = {0};
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= 64) return 148;
    if (n[dev] == 0) {
        int v = 0;
        cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
        n[dev] = v > 0 ? v : 148;
    }
    return n[dev];
}

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    });
    return fn;
}

// 2-D K-major BF16 operand [rows][ld] with a box of `box_rows` x 64.
bool make_map(CUtensorMap* map, const void* ptr, int rows, int k, int ld, int box_rows) {
    PFN_cuTensorMapEncodeTiled_v12000 fn = encode_fn();
    if (!fn) return false;
    const cuuint64_t dims[2] = {(cuuint64_t)k, (cuuint64_t)rows};
    const cuuint64_t strides[1] = {(cuuint64_t)ld * 2u};
    const cuuint32_t box[2] = {(cuuint32_t)TK, (cuuint32_t)box_rows};
    const cuuint32_t estr[2] = {1u, 1u};
    return fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(ptr), dims, strides, box, estr,
              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

}  // namespace

// Whether the tensor-core path takes this GEMM: K-major A and B, K a
// multiple of 64, no split-K.
bool gemm_tc_eligible(int a_kmajor, int b_kmajor, int K, int splitk) {
    (void)splitk;
    return a_kmajor && b_kmajor && K % TK == 0 && K > 0 && encode_fn() != nullptr;
}

namespace {

// Clusters of CL CTAs (each alone on its SM) that can be resident at once for
// this kernel, cached per kernel; 0 when the query fails.
template <int EPI, int CL>
int resident_clusters(cudaStream_t s) {
    static int n[64] = {0};
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= 64) return 0;
    if (n[dev] == 0) {
        cudaLaunchConfig_t cfg = {};
        cudaLaunchAttribute at[1];
        at[0].id = cudaLaunchAttributeClusterDimension;
        at[0].val.clusterDim.x = CL;
        at[0].val.clusterDim.y = 1;
        at[0].val.clusterDim.z = 1;
        cfg.gridDim = dim3(CL * sm_count());
        cfg.blockDim = dim3(THREADS);
        cfg.dynamicSmemBytes = SMEM_BYTES;
        cfg.stream = s;
        cfg.attrs = at;
        cfg.numAttrs = 1;
        int v = 0;
        if (cudaOccupancyMaxActiveClusters(&v, gemm_tc_kernel<EPI, CL>, &cfg) != cudaSuccess) {
            cudaGetLastError();
            v = -1;
        }
        n[dev] = v;
    }
    return n[dev] > 0 ? n[dev] : 0;
}

template <int EPI>
cudaError_t launch_tc(const CUtensorMap& ta, const void* B, int N, int K, int ldb, const TcArgs& g, bool pairs,
                      cudaStream_t s) {
    const int mt = (g.M + TM - 1) / TM, nt = (g.N + TN - 1) / TN;
    cudaError_t e;
    if (pairs && mt % 2 == 0) {
        e = cudaFuncSetAttribute(gemm_tc_kernel<EPI, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES);
        if (e != cudaSuccess) return e;
        const int clusters = resident_clusters<EPI, 2>(s);
        if (clusters > 0) {
            CUtensorMap tb;     // B in half tiles: each CTA of a pair loads one half
            if (!make_map(&tb, B, N, K, ldb, TN / 2)) return cudaErrorInvalidValue;
            const int items = (mt / 2) * nt * g.ksplit;
            cudaLaunchConfig_t cfg = {};
            cudaLaunchAttribute at[1];
            at[0].id = cudaLaunchAttributeClusterDimension;
            at[0].val.clusterDim.x = 2;
            at[0].val.clusterDim.y = 1;
            at[0].val.clusterDim.z = 1;
            cfg.gridDim = dim3(2 * (items < clusters ? items : clusters));
            cfg.blockDim = dim3(THREADS);
            cfg.dynamicSmemBytes = SMEM_BYTES;
            cfg.stream = s;
            cfg.attrs = at;
            cfg.numAttrs = 1;
            e = cudaLaunchKernelEx(&cfg, gemm_tc_kernel<EPI, 2>, ta, tb, g);
            return e != cudaSuccess ? e : cudaGetLastError();
        }
    }
    CUtensorMap tb;
    if (!make_map(&tb, B, N, K, ldb, TN)) return cudaErrorInvalidValue;
    e = cudaFuncSetAttribute(gemm_tc_kernel<EPI, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES);
    if (e != cudaSuccess) return e;
    const int items = mt * nt * g.ksplit;
    gemm_tc_kernel<EPI, 1><<<items < sm_count() ? items : sm_count(), THREADS, SMEM_BYTES, s>>>(ta, tb, g);
    return cudaGetLastError();
}

}  // namespace

// epi: 0 FP32 C, 1 GELU (C = H bf16, Z bf16), 2 sigmoid column sums into
// sigsum; splitk > 1 (FP32 C only): K is cut into splitk slices whose partial
// products are added into C, which the caller has zeroed.  pairs: allow the
// CTA-pair form (taken when the output has an even number of M tiles).
cudaError_t launch_gemm_tc(const void* A, int lda, const void* B, int ldb, void* C, int ldc, int epi, const float* bias,
                           void* Z, float* sigsum, int M, int N, int K, int splitk, int pairs, cudaStream_t s) {
    CUtensorMap ta;
    if (!make_map(&ta, A, M, K, lda, TM)) return cudaErrorInvalidValue;
    TcArgs g;
    g.C = C;
    g.Z = (__nv_bfloat16*)Z;
    g.bias = bias;
    g.sigsum = sigsum;
    g.M = M; g.N = N; g.K = K; g.ldc = ldc;
    const int ktiles = K / TK;
    if (splitk < 1 || epi != kEpiF32) splitk = 1;
    if (splitk > ktiles) splitk = ktiles;
    g.kper = (ktiles + splitk - 1) / splitk;
    g.ksplit = (ktiles + g.kper - 1) / g.kper;        // no empty slice
    if (g.ksplit > 1) epi = kEpiF32Add;
    const bool pr = pairs != 0;
    if (epi == kEpiF32) return launch_tc<kEpiF32>(ta, B, N, K, ldb, g, pr, s);
    if (epi == kEpiF32Add) return launch_tc<kEpiF32Add>(ta, B, N, K, ldb, g, pr, s);
    if (epi == kEpiGelu) return launch_tc<kEpiGelu>(ta, B, N, K, ldb, g, pr, s);
    return launch_tc<kEpiSigsum>(ta, B, N, K, ldb, g, pr, s);
}

// Read and clear the device error flag of the tensor-core GEMM (synchronizes).
cudaError_t gemm_tc_take_error(int* code) {
    int zero = 0;
    cudaError_t e = cudaMemcpyFromSymbol(code, g_tc_error, sizeof(int));
    if (e != cudaSuccess) return e;
    return cudaMemcpyToSymbol(g_tc_error, &zero, sizeof(int));
}

}  // namespace oneka
