// mlp.cu -- kernels of the learned surrogate: a BF16 tensor-core GEMM with
// fused bias/GELU epilogues, the BCE loss against chronicle bitmasks, GELU
// backward, bias gradients and the AdamW update (FP32 master weights).
//
// The surrogate maps a realization's parameter vector (A..F, discharges, K,
// porosity) to per-cell capture logits; its training labels are the
// per-realization bitmasks the tracker chronicles (oneka_track mark-only
// mode).  It has no counterpart in the reference.
#include <cuda_bf16.h>
#include <math.h>
#include <stdint.h>

#include "oneka_internal.cuh"

namespace oneka {
namespace {

constexpr int BM = 128, BN = 128, BK = 32, STAGES = 3, THREADS = 256;
constexpr int KPAD = BK + 8;      // k-major tiles: rows of 40 bf16 (80 B)
constexpr int MPAD = BM + 8;      // m/n-major tiles: rows of 136 bf16 (272 B)

struct GemmArgs {
    const __nv_bfloat16* A;   // k-major: [M][lda]; m-major: [K][lda]
    const __nv_bfloat16* B;   // k-major: [N][ldb]; n-major: [K][ldb]
    void* C;                  // [M][ldc], bf16 or f32
    __nv_bfloat16* Z;         // pre-activation copy (bf16, ldc), or null
    const float* bias;        // [N] or null
    float* sigsum;            // non-null: out[n] += sum over rows of sigmoid(C[m][n]); C not written
    int M, N, K, lda, ldb, ldc;
    int c_f32, gelu, kper;    // kper: K range of one split
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void cp_async16(void* dst, const void* src, bool valid) {
    const int n = valid ? 16 : 0;   // 0: zero-fill, nothing read
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(smem_u32(dst)), "l"(src), "r"(n));
}

__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;\n" ::); }
template <int N>
__device__ __forceinline__ void cp_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N)); }

__device__ __forceinline__ void ldsm_x4(uint32_t& r0, uint32_t& r1, uint32_t& r2, uint32_t& r3, const void* p) {
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3) : "r"(smem_u32(p)));
}
__device__ __forceinline__ void ldsm_x4_t(uint32_t& r0, uint32_t& r1, uint32_t& r2, uint32_t& r3, const void* p) {
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3) : "r"(smem_u32(p)));
}

__device__ __forceinline__ void mma_bf16(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
    asm volatile("mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
                 "{%8,%9}, {%0,%1,%2,%3};\n"
                 : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
                 : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

__device__ __forceinline__ float gelu_f(float x) { return 0.5f * x * (1.0f + erff(x * 0.70710678118654752f)); }
__device__ __forceinline__ float gelu_grad(float x) {
    return 0.5f * (1.0f + erff(x * 0.70710678118654752f)) + x * 0.39894228040143268f * expf(-0.5f * x * x);
}

// C = A * B (+ bias, GELU) with FP32 accumulation.  Block 128 x 128, 8 warps
// of 64 x 32, three cp.async stages of BK = 32.  Rows/columns beyond M or N
// are zero-filled on load and skipped on store; K must be a multiple of 32
// and the leading dimensions multiples of 8 (16-byte rows).  gridDim.z
// splits K: each split adds its partial product into a zeroed FP32 C.
template <bool A_KMAJOR, bool B_KMAJOR>
__global__ void __launch_bounds__(THREADS) gemm_bf16_kernel(const GemmArgs g) {
    extern __shared__ __align__(16) unsigned char gsm[];
    constexpr int A_ELEMS = A_KMAJOR ? BM * KPAD : BK * MPAD;
    constexpr int B_ELEMS = B_KMAJOR ? BN * KPAD : BK * MPAD;
    __nv_bfloat16* As = reinterpret_cast<__nv_bfloat16*>(gsm);
    __nv_bfloat16* Bs = As + STAGES * A_ELEMS;

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int wm = warp >> 2, wn = warp & 3;             // 2 x 4 warps
    const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
    const int kbeg = blockIdx.z * g.kper;
    const int kend = min(g.K, kbeg + g.kper);
    const int ktiles = (kend - kbeg) / BK;

    auto load_stage = [&](int stage, int kt) {
        const int k0 = kbeg + kt * BK;
        __nv_bfloat16* as = As + stage * A_ELEMS;
        __nv_bfloat16* bs = Bs + stage * B_ELEMS;
#pragma unroll
        for (int c = tid; c < 512; c += THREADS) {
            if (A_KMAJOR) {          // 128 rows x 4 chunks
                const int row = c >> 2, ch = c & 3;
                const bool ok = m0 + row < g.M;
                cp_async16(as + row * KPAD + ch * 8, g.A + (long long)(ok ? m0 + row : 0) * g.lda + k0 + ch * 8, ok);
            } else {                 // 32 k-rows x 16 chunks
                const int row = c >> 4, ch = c & 15;
                const bool ok = m0 + ch * 8 < g.M;
                cp_async16(as + row * MPAD + ch * 8, g.A + (long long)(k0 + row) * g.lda + (ok ? m0 + ch * 8 : 0), ok);
            }
            if (B_KMAJOR) {
                const int row = c >> 2, ch = c & 3;
                const bool ok = n0 + row < g.N;
                cp_async16(bs + row * KPAD + ch * 8, g.B + (long long)(ok ? n0 + row : 0) * g.ldb + k0 + ch * 8, ok);
            } else {
                const int row = c >> 4, ch = c & 15;
                const bool ok = n0 + ch * 8 < g.N;
                cp_async16(bs + row * MPAD + ch * 8, g.B + (long long)(k0 + row) * g.ldb + (ok ? n0 + ch * 8 : 0), ok);
            }
        }
    };

    float acc[4][4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j)
#pragma unroll
            for (int r = 0; r < 4; ++r) acc[i][j][r] = 0.0f;

#pragma unroll
    for (int s = 0; s < STAGES - 1; ++s) {
        if (s < ktiles) load_stage(s, s);
        cp_commit();
    }
    for (int kt = 0; kt < ktiles; ++kt) {
        cp_wait<STAGES - 2>();
        __syncthreads();
        const int nxt = kt + STAGES - 1;
        if (nxt < ktiles) load_stage(nxt % STAGES, nxt);
        cp_commit();
        const __nv_bfloat16* as = As + (kt % STAGES) * A_ELEMS;
        const __nv_bfloat16* bs = Bs + (kt % STAGES) * B_ELEMS;
#pragma unroll
        for (int kk = 0; kk < BK; kk += 16) {
            uint32_t af[4][4], bfr[4][2];
            const int q = lane >> 3, r8 = lane & 7;
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                const int mb = wm * 64 + i * 16;
                if (A_KMAJOR)
                    ldsm_x4(af[i][0], af[i][1], af[i][2], af[i][3],
                            as + (mb + (lane & 15)) * KPAD + kk + (lane >> 4) * 8);
                else
                    ldsm_x4_t(af[i][0], af[i][1], af[i][2], af[i][3],
                              as + (kk + r8 + (q >> 1) * 8) * MPAD + mb + (q & 1) * 8);
            }
#pragma unroll
            for (int j = 0; j < 4; j += 2) {
                const int nb = wn * 32 + j * 8;
                if (B_KMAJOR)
                    ldsm_x4(bfr[j][0], bfr[j][1], bfr[j + 1][0], bfr[j + 1][1],
                            bs + (nb + r8 + (q >> 1) * 8) * KPAD + kk + (q & 1) * 8);
                else
                    ldsm_x4_t(bfr[j][0], bfr[j][1], bfr[j + 1][0], bfr[j + 1][1],
                              bs + (kk + r8 + (q & 1) * 8) * MPAD + nb + (q >> 1) * 8);
            }
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) mma_bf16(acc[i][j], af[i], bfr[j][0], bfr[j][1]);
        }
    }
    cp_wait<0>();

    if (g.sigsum) {
        // Column sums of sigmoid(logits) over this warp's 64 rows: each lane
        // holds 8 rows of 8 columns; lanes with equal (lane & 3) share
        // columns, so a butterfly over lane bits 2..4 finishes the sum.
#pragma unroll
        for (int j = 0; j < 4; ++j) {
#pragma unroll
            for (int e = 0; e < 2; ++e) {
                const int n = n0 + wn * 32 + j * 8 + (lane & 3) * 2 + e;
                const float bn = (n < g.N && g.bias) ? g.bias[n] : 0.0f;
                float s = 0.0f;
#pragma unroll
                for (int i = 0; i < 4; ++i)
#pragma unroll
                    for (int h = 0; h < 2; ++h) {
                        const int m = m0 + wm * 64 + i * 16 + (lane >> 2) + h * 8;
                        if (m < g.M) s += 1.0f / (1.0f + __expf(-(acc[i][j][h * 2 + e] + bn)));
                    }
                s += __shfl_xor_sync(0xffffffffu, s, 4);
                s += __shfl_xor_sync(0xffffffffu, s, 8);
                s += __shfl_xor_sync(0xffffffffu, s, 16);
                if (lane < 4 && n < g.N) atomicAdd(g.sigsum + n, s);
            }
        }
        return;
    }
    const bool split = gridDim.z > 1;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
#pragma unroll
        for (int j = 0; j < 4; ++j) {
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int m = m0 + wm * 64 + i * 16 + (lane >> 2) + h * 8;
                if (m >= g.M) continue;
#pragma unroll
                for (int e = 0; e < 2; ++e) {
                    const int n = n0 + wn * 32 + j * 8 + (lane & 3) * 2 + e;
                    if (n >= g.N) continue;
                    float v = acc[i][j][h * 2 + e];
                    if (g.bias && blockIdx.z == 0) v += g.bias[n];
                    const long long off = (long long)m * g.ldc + n;
                    if (split) {
                        atomicAdd(reinterpret_cast<float*>(g.C) + off, v);
                        continue;
                    }
                    if (g.Z) g.Z[off] = __float2bfloat16(v);
                    if (g.gelu) v = gelu_f(v);
                    if (g.c_f32)
                        reinterpret_cast<float*>(g.C)[off] = v;
                    else
                        reinterpret_cast<__nv_bfloat16*>(g.C)[off] = __float2bfloat16(v);
                }
            }
        }
    }
}

// Mean binary cross-entropy of logits z against the bits of a chronicle
// mask (cell i*ncols + j <-> bit j%32 of word i*wpr + j/32 of the sample's
// slot), and its gradient (sigmoid(z) - y) * scale as BF16.
__device__ __forceinline__ float bce_term(float z, float y, float scale, float& grad) {
    // max(z, 0) - z y + log(1 + e^-|z|) and d/dz = sigmoid(z) - y, with one exponential
    const float e = __expf(-fabsf(z));
    const float inv = __frcp_rn(1.0f + e);
    const float p = z >= 0.0f ? inv : e * inv;
    grad = (p - y) * scale;
    return fmaxf(z, 0.0f) - z * y + __logf(1.0f + e);
}

// Eight consecutive cells of one grid row per thread: two float4 logit loads,
// one mask word, one 16-byte store of BF16 gradients.  blockIdx.y is the
// sample.  Needs ncols % 8 == 0 (else bce_bitmask_kernel below).
__global__ void __launch_bounds__(256) bce_bitmask8_kernel(const float* __restrict__ logits,
                                                           const uint32_t* __restrict__ masks, long long slot_words,
                                                           int wpr, int ncols, int ncells, float scale,
                                                           __nv_bfloat16* __restrict__ dlogits,
                                                           float* __restrict__ loss) {
    const int b = blockIdx.y;
    const int chunk = blockIdx.x * blockDim.x + threadIdx.x;
    float part = 0.0f;
    if (chunk < ncells / 8) {
        const int cell = chunk * 8, row = cell / ncols, col = cell - row * ncols;
        const uint32_t w = masks[(long long)b * slot_words + (long long)row * wpr + (col >> 5)] >> (col & 31);
        const long long i = (long long)b * ncells + cell;
        const float4 z0 = *reinterpret_cast<const float4*>(logits + i);
        const float4 z1 = *reinterpret_cast<const float4*>(logits + i + 4);
        const float z[8] = {z0.x, z0.y, z0.z, z0.w, z1.x, z1.y, z1.z, z1.w};
        float g[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) part += bce_term(z[j], (float)((w >> j) & 1u), scale, g[j]);
        if (dlogits) {
            uint32_t q[4];
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const __nv_bfloat162 h = __floats2bfloat162_rn(g[2 * j], g[2 * j + 1]);
                q[j] = *reinterpret_cast<const uint32_t*>(&h);
            }
            *reinterpret_cast<uint4*>(dlogits + i) = make_uint4(q[0], q[1], q[2], q[3]);
        }
    }
    for (int off = 16; off > 0; off >>= 1) part += __shfl_xor_sync(0xffffffffu, part, off);
    __shared__ float wsum[8];
    if ((threadIdx.x & 31) == 0) wsum[threadIdx.x >> 5] = part;
    __syncthreads();
    if (threadIdx.x == 0 && loss) {
        float t = 0.0f;
        for (int k = 0; k < (int)(blockDim.x >> 5); ++k) t += wsum[k];
        atomicAdd(loss, t * scale);
    }
}

// BCE over a tile of 64 samples x 64 cells of one grid row, writing the
// gradient both row-major (dlogits [B][ncells]) and transposed (dlogits_t
// [ncells][ldt]), the latter through a shared-memory tile: the weight
// gradient GEMM reads it K-major, so no separate transpose pass is needed.
// Needs ncols % 64 == 0, B % 64 == 0, ldt % 8 == 0.
__global__ void __launch_bounds__(256) bce_bitmask_t_kernel(const float* __restrict__ logits,
                                                            const uint32_t* __restrict__ masks, long long slot_words,
                                                            int wpr, int ncols, int ncells, float scale,
                                                            __nv_bfloat16* __restrict__ dlogits,
                                                            __nv_bfloat16* __restrict__ dlogits_t, long long ldt,
                                                            float* __restrict__ loss) {
    __shared__ __align__(16) __nv_bfloat16 tile[64][72];
    __shared__ float wsum[8];
    const int c0 = blockIdx.x * 64, b0 = blockIdx.y * 64;
    const int grow = c0 / ncols, gcol0 = c0 - grow * ncols;
    float part = 0.0f;
    for (int i = threadIdx.x; i < 64 * 16; i += 256) {
        const int r = i >> 4, q = (i & 15) * 4;
        const int b = b0 + r, col = gcol0 + q;
        const uint32_t w = masks[(long long)b * slot_words + (long long)grow * wpr + (col >> 5)] >> (col & 31);
        const long long idx = (long long)b * ncells + c0 + q;
        const float4 z = *reinterpret_cast<const float4*>(logits + idx);
        const float zz[4] = {z.x, z.y, z.z, z.w};
        float g[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) part += bce_term(zz[j], (float)((w >> j) & 1u), scale, g[j]);
        const __nv_bfloat162 h0 = __floats2bfloat162_rn(g[0], g[1]), h1 = __floats2bfloat162_rn(g[2], g[3]);
        const uint2 packed = make_uint2(*reinterpret_cast<const uint32_t*>(&h0),
                                        *reinterpret_cast<const uint32_t*>(&h1));
        *reinterpret_cast<uint2*>(dlogits + idx) = packed;
        *reinterpret_cast<uint2*>(&tile[r][q]) = packed;
    }
    __syncthreads();
    for (int i = threadIdx.x; i < 64 * 8; i += 256) {
        const int cc = i >> 3, s8 = (i & 7) * 8;
        uint32_t e[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const __nv_bfloat162 h = __halves2bfloat162(tile[s8 + 2 * j][cc], tile[s8 + 2 * j + 1][cc]);
            e[j] = *reinterpret_cast<const uint32_t*>(&h);
        }
        *reinterpret_cast<uint4*>(dlogits_t + (long long)(c0 + cc) * ldt + b0 + s8) = make_uint4(e[0], e[1], e[2], e[3]);
    }
    for (int off = 16; off > 0; off >>= 1) part += __shfl_xor_sync(0xffffffffu, part, off);
    if ((threadIdx.x & 31) == 0) wsum[threadIdx.x >> 5] = part;
    __syncthreads();
    if (threadIdx.x == 0 && loss) {
        float t = 0.0f;
        for (int k = 0; k < 8; ++k) t += wsum[k];
        atomicAdd(loss, t * scale);
    }
}

__global__ void bce_bitmask_kernel(const float* __restrict__ logits, const uint32_t* __restrict__ masks,
                                   long long slot_words, int wpr, int ncols, int B, int ncells, float scale,
                                   __nv_bfloat16* __restrict__ dlogits, float* __restrict__ loss) {
    const long long n = (long long)B * ncells;
    float part = 0.0f;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const int b = (int)(i / ncells), c = (int)(i % ncells);
        const int row = c / ncols, col = c % ncols;
        const uint32_t w = masks[(long long)b * slot_words + (long long)row * wpr + (col >> 5)];
        float g;
        part += bce_term(logits[i], (float)((w >> (col & 31)) & 1u), scale, g);
        if (dlogits) dlogits[i] = __float2bfloat16(g);
    }
    for (int off = 16; off > 0; off >>= 1) part += __shfl_xor_sync(0xffffffffu, part, off);
    if ((threadIdx.x & 31) == 0 && loss) atomicAdd(loss, part * scale);
}

// dz = dh * gelu'(z), dh in FP32, z (pre-activation) and dz in BF16.
__global__ void gelu_backward_kernel(const float* __restrict__ dh, const __nv_bfloat16* __restrict__ z,
                                     __nv_bfloat16* __restrict__ dz, long long n) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x)
        dz[i] = __float2bfloat16(dh[i] * gelu_grad(__bfloat162float(z[i])));
}

// out[c] = sum_r x[r][c] (bias gradients), x in BF16: a block of 8 warps
// per 32 columns, each warp a strided eighth of the rows, then a
// shared-memory sum over the warps.
__global__ void __launch_bounds__(256) colsum_kernel(const __nv_bfloat16* __restrict__ x, int rows, int cols,
                                                     float* __restrict__ out) {
    __shared__ float part[8][33];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int c = blockIdx.x * 32 + lane;
    float s = 0.0f;
    if (c < cols)
        for (int r = warp; r < rows; r += 8) s += __bfloat162float(x[(long long)r * cols + c]);
    part[warp][lane] = s;
    __syncthreads();
    if (warp == 0 && c < cols) {
        float t = 0.0f;
#pragma unroll
        for (int k = 0; k < 8; ++k) t += part[k][lane];
        out[c] = t;
    }
}

// AdamW with bias correction (decoupled weight decay), FP32 master weights,
// and the BF16 copy the GEMMs read.
// hyper (optional, device [3]): lr, 1 - b1^t, 1 - b2^t of this step, read on
// the device so that a captured training step takes its schedule from memory.
__global__ void adamw_kernel(float* __restrict__ w, float* __restrict__ m, float* __restrict__ v,
                             const float* __restrict__ g, __nv_bfloat16* __restrict__ wb, long long n, float lr,
                             float b1, float b2, float eps, float wd, float c1, float c2,
                             const float* __restrict__ hyper) {
    if (hyper) {
        lr = hyper[0];
        c1 = hyper[1];
        c2 = hyper[2];
    }
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const float gi = g[i];
        const float mi = b1 * m[i] + (1.0f - b1) * gi;
        const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        const float upd = (mi / c1) / (sqrtf(vi / c2) + eps);
        const float wi = w[i] - lr * (upd + wd * w[i]);
        w[i] = wi;
        if (wb) wb[i] = __float2bfloat16(wi);
    }
}

// AdamW over a 64 x 64 tile of a [rows][cols] weight matrix (the update of
// adamw_kernel, with the schedule in hyper), writing the BF16 copy both
// row-major (wb) and transposed (wbt [cols][ldt]) through shared memory: the
// backward pass reads W^T K-major, so no separate transpose pass is needed.
// Needs cols % 64 == 0, rows % 64 == 0, ldt % 8 == 0.
__global__ void __launch_bounds__(256) adamw_t_kernel(float* __restrict__ w, float* __restrict__ m,
                                                      float* __restrict__ v, const float* __restrict__ g,
                                                      __nv_bfloat16* __restrict__ wb, __nv_bfloat16* __restrict__ wbt,
                                                      long long ldt, int cols, const float* __restrict__ hyper,
                                                      float b1, float b2, float eps, float wd) {
    __shared__ __align__(16) __nv_bfloat16 tile[64][72];
    const float lr = hyper[0], c1 = hyper[1], c2 = hyper[2];
    const int c0 = blockIdx.x * 64, r0 = blockIdx.y * 64;
    for (int i = threadIdx.x; i < 64 * 16; i += 256) {
        const int r = i >> 4, q = (i & 15) * 4;
        const long long idx = (long long)(r0 + r) * cols + c0 + q;
        float4 W = *reinterpret_cast<const float4*>(w + idx);
        float4 M = *reinterpret_cast<const float4*>(m + idx);
        float4 V = *reinterpret_cast<const float4*>(v + idx);
        const float4 G = *reinterpret_cast<const float4*>(g + idx);
        float* Wp = &W.x;
        float* Mp = &M.x;
        float* Vp = &V.x;
        const float* Gp = &G.x;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const float mi = b1 * Mp[j] + (1.0f - b1) * Gp[j];
            const float vi = b2 * Vp[j] + (1.0f - b2) * Gp[j] * Gp[j];
            Mp[j] = mi;
            Vp[j] = vi;
            const float upd = (mi / c1) / (sqrtf(vi / c2) + eps);
            Wp[j] = Wp[j] - lr * (upd + wd * Wp[j]);
        }
        *reinterpret_cast<float4*>(w + idx) = W;
        *reinterpret_cast<float4*>(m + idx) = M;
        *reinterpret_cast<float4*>(v + idx) = V;
        const __nv_bfloat162 h0 = __floats2bfloat162_rn(W.x, W.y), h1 = __floats2bfloat162_rn(W.z, W.w);
        const uint2 packed = make_uint2(*reinterpret_cast<const uint32_t*>(&h0),
                                        *reinterpret_cast<const uint32_t*>(&h1));
        *reinterpret_cast<uint2*>(wb + idx) = packed;
        *reinterpret_cast<uint2*>(&tile[r][q]) = packed;
    }
    __syncthreads();
    for (int i = threadIdx.x; i < 64 * 8; i += 256) {
        const int cc = i >> 3, s8 = (i & 7) * 8;
        uint32_t e[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const __nv_bfloat162 h = __halves2bfloat162(tile[s8 + 2 * j][cc], tile[s8 + 2 * j + 1][cc]);
            e[j] = *reinterpret_cast<const uint32_t*>(&h);
        }
        *reinterpret_cast<uint4*>(wbt + (long long)(c0 + cc) * ldt + r0 + s8) = make_uint4(e[0], e[1], e[2], e[3]);
    }
}

// Standardized features of realizations [first, first + n) as BF16 rows of
// ld columns (zero beyond nf): A..F, discharges, then K and porosity.
__global__ void features_kernel(const double* __restrict__ coef, const double* __restrict__ q,
                                const double* __restrict__ aquifer, int nwells, int n, const float* __restrict__ mean,
                                const float* __restrict__ inv_std, int nf, int ld, __nv_bfloat16* __restrict__ x) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long long)n * ld) return;
    const int r = (int)(i / ld), f = (int)(i % ld);
    float v = 0.0f;
    if (f < nf) {
        double raw;
        if (f < 6) raw = coef[6LL * r + f];
        else if (f < 6 + nwells) raw = q[(long long)r * nwells + (f - 6)];
        else raw = aquifer[3LL * r + (f - 6 - nwells)];
        v = ((float)raw - mean[f]) * inv_std[f];
    }
    x[i] = __float2bfloat16(v);
}

// out[c] += sum_r sigmoid(logits[r][c]): the surrogate's expected visits per cell.
__global__ void sigmoid_colsum_kernel(const float* __restrict__ logits, int rows, int cols, float* __restrict__ out) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= cols) return;
    float s = 0.0f;
    for (int r = 0; r < rows; ++r) s += 1.0f / (1.0f + expf(-logits[(long long)r * cols + c]));
    out[c] += s;
}

// dst[c][r] = src[r][c] for BF16 matrices: 64 x 64 tiles staged in shared
// memory (rows padded by 16 bytes), 16-byte loads and stores, 256 threads.
constexpr int TT = 64;
__global__ void __launch_bounds__(256) transpose_bf16_kernel(const uint16_t* __restrict__ src, int rows, int cols,
                                                             long long lds, uint16_t* __restrict__ dst, long long ldd) {
    __shared__ __align__(16) uint16_t tile[TT][TT + 8];
    const int r0 = blockIdx.y * TT, c0 = blockIdx.x * TT;
    const int t = threadIdx.x;
    // load: 64 rows x 8 chunks of 8 elements
    for (int i = t; i < TT * (TT / 8); i += 256) {
        const int r = i >> 3, ch = (i & 7) * 8;
        const int gr = r0 + r, gc = c0 + ch;
        uint4 v = make_uint4(0, 0, 0, 0);
        if (gr < rows) {
            if (gc + 8 <= cols && (((uintptr_t)(src + gr * lds + gc)) & 15) == 0) {
                v = *reinterpret_cast<const uint4*>(src + gr * lds + gc);
            } else {
                uint16_t e[8];
                for (int j = 0; j < 8; ++j) e[j] = gc + j < cols ? src[gr * lds + gc + j] : 0;
                v = make_uint4(e[0] | (e[1] << 16), e[2] | (e[3] << 16), e[4] | (e[5] << 16), e[6] | (e[7] << 16));
            }
        }
        *reinterpret_cast<uint4*>(&tile[r][ch]) = v;
    }
    __syncthreads();
    // store: output row c (a column of the tile), 8 chunks of 8 source rows
    for (int i = t; i < TT * (TT / 8); i += 256) {
        const int c = i >> 3, ch = (i & 7) * 8;
        const int gc = c0 + c, gr = r0 + ch;
        if (gc >= cols) continue;
        uint16_t e[8];
        for (int j = 0; j < 8; ++j) e[j] = tile[ch + j][c];
        uint16_t* out = dst + gc * ldd + gr;
        if (gr + 8 <= rows && (((uintptr_t)out) & 15) == 0) {
            *reinterpret_cast<uint4*>(out) =
                make_uint4(e[0] | (e[1] << 16), e[2] | (e[3] << 16), e[4] | (e[5] << 16), e[6] | (e[7] << 16));
        } else {
            for (int j = 0; j < 8; ++j)
                if (gr + j < rows) out[j] = e[j];
        }
    }
}

unsigned grid_for(long long n, int per) {
    long long b = (n + per - 1) / per;
    return (unsigned)(b > 4096 ? 4096 : (b < 1 ? 1 : b));
}

}  // namespace

bool gemm_tc_eligible(int a_kmajor, int b_kmajor, int K, int splitk);
cudaError_t launch_gemm_tc(const void* A, int lda, const void* B, int ldb, void* C, int ldc, int epi, const float* bias,
                           void* Z, float* sigsum, int M, int N, int K, int splitk, int pairs, cudaStream_t s);

// Which kernel a GEMM runs on: 1 the tcgen05 kernel (gemm_tc.cu), 0 the
// mma.sync kernel below.  The tcgen05 kernel takes K-major operands with K a
// multiple of 64, for the FP32 (also split-K), GELU and sigmoid-sum
// epilogues; bit 0 of `flags` forces the mma.sync kernel, bit 1 keeps the
// tcgen05 kernel to one CTA per tile (no CTA pairs).
int gemm_path(int a_kmajor, int b_kmajor, int K, int splitk, int c_f32, int gelu, void* Z, float* sigsum, int flags) {
    if (flags & 1) return 0;
    if (!gemm_tc_eligible(a_kmajor, b_kmajor, K, splitk)) return 0;
    if (sigsum) return splitk <= 1 ? 1 : 0;
    if (gelu) return (!c_f32 && Z && splitk <= 1) ? 1 : 0;
    return c_f32 ? 1 : 0;
}

cudaError_t launch_gemm_bf16(const void* A, int lda, int a_kmajor, const void* B, int ldb, int b_kmajor, void* C,
                             int ldc, int c_f32, const float* bias, int gelu, void* Z, int M, int N, int K,
                             int splitk, float* sigsum, int flags, cudaStream_t s) {
    if (gemm_path(a_kmajor, b_kmajor, K, splitk, c_f32, gelu, Z, sigsum, flags))
        return launch_gemm_tc(A, lda, B, ldb, C, ldc, sigsum ? 2 : (gelu ? 1 : 0), bias, Z, sigsum, M, N, K, splitk,
                              (flags & 2) ? 0 : 1, s);
    GemmArgs g;
    g.A = (const __nv_bfloat16*)A;
    g.B = (const __nv_bfloat16*)B;
    g.C = C;
    g.Z = (__nv_bfloat16*)Z;
    g.bias = bias;
    g.sigsum = sigsum;
    g.M = M; g.N = N; g.K = K; g.lda = lda; g.ldb = ldb; g.ldc = ldc;
    g.c_f32 = c_f32;
    g.gelu = gelu;
    if (splitk < 1) splitk = 1;
    int ktiles = K / BK;
    if (splitk > ktiles) splitk = ktiles > 0 ? ktiles : 1;
    g.kper = ((ktiles + splitk - 1) / splitk) * BK;
    dim3 grid((N + BN - 1) / BN, (M + BM - 1) / BM, splitk);
    const size_t smA = (size_t)STAGES * (a_kmajor ? BM * KPAD : BK * MPAD) * 2;
    const size_t smB = (size_t)STAGES * (b_kmajor ? BN * KPAD : BK * MPAD) * 2;
    const int smem = (int)(smA + smB);
#define ONEKA_GEMM_CASE(AK, BKM)                                                                          \
    {                                                                                                     \
        cudaError_t e = cudaFuncSetAttribute(gemm_bf16_kernel<AK, BKM>,                                   \
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, smem);          \
        if (e != cudaSuccess) return e;                                                                   \
        gemm_bf16_kernel<AK, BKM><<<grid, THREADS, smem, s>>>(g);                                         \
    }
    if (a_kmajor && b_kmajor) ONEKA_GEMM_CASE(true, true)
    else if (a_kmajor) ONEKA_GEMM_CASE(true, false)
    else if (b_kmajor) ONEKA_GEMM_CASE(false, true)
    else ONEKA_GEMM_CASE(false, false)
#undef ONEKA_GEMM_CASE
    return cudaGetLastError();
}

cudaError_t launch_bce_bitmask(const float* logits, const uint32_t* masks, long long slot_words, int wpr, int ncols,
                               int B, int ncells, float scale, void* dlogits, float* loss, cudaStream_t s) {
    const bool aligned = ((uintptr_t)logits & 15) == 0 && (!dlogits || ((uintptr_t)dlogits & 15) == 0);
    if (ncols % 8 == 0 && aligned && B <= 65535) {
        dim3 grid((unsigned)((ncells / 8 + 255) / 256), (unsigned)B);
        bce_bitmask8_kernel<<<grid, 256, 0, s>>>(logits, masks, slot_words, wpr, ncols, ncells, scale,
                                                 (__nv_bfloat16*)dlogits, loss);
    } else {
        bce_bitmask_kernel<<<grid_for((long long)B * ncells, 256), 256, 0, s>>>(
            logits, masks, slot_words, wpr, ncols, B, ncells, scale, (__nv_bfloat16*)dlogits, loss);
    }
    return cudaGetLastError();
}

cudaError_t launch_gelu_backward(const float* dh, const void* z, void* dz, long long n, cudaStream_t s) {
    gelu_backward_kernel<<<grid_for(n, 256), 256, 0, s>>>(dh, (const __nv_bfloat16*)z, (__nv_bfloat16*)dz, n);
    return cudaGetLastError();
}

cudaError_t launch_colsum(const void* x, int rows, int cols, float* out, cudaStream_t s) {
    colsum_kernel<<<(cols + 31) / 32, 256, 0, s>>>((const __nv_bfloat16*)x, rows, cols, out);
    return cudaGetLastError();
}

cudaError_t launch_adamw(float* w, float* m, float* v, const float* g, void* wb, long long n, float lr, float b1,
                         float b2, float eps, float wd, int step, cudaStream_t s) {
    const float c1 = 1.0f - powf(b1, (float)step), c2 = 1.0f - powf(b2, (float)step);
    adamw_kernel<<<grid_for(n, 256), 256, 0, s>>>(w, m, v, g, (__nv_bfloat16*)wb, n, lr, b1, b2, eps, wd, c1, c2,
                                                   nullptr);
    return cudaGetLastError();
}

cudaError_t launch_adamw_scheduled(float* w, float* m, float* v, const float* g, void* wb, long long n,
                                   const float* hyper, float b1, float b2, float eps, float wd, cudaStream_t s) {
    adamw_kernel<<<grid_for(n, 256), 256, 0, s>>>(w, m, v, g, (__nv_bfloat16*)wb, n, 0.0f, b1, b2, eps, wd, 1.0f,
                                                   1.0f, hyper);
    return cudaGetLastError();
}

cudaError_t launch_bce_bitmask_t(const float* logits, const uint32_t* masks, long long slot_words, int wpr,
                                 int ncols, int B, int ncells, float scale, void* dlogits, void* dlogits_t,
                                 long long ldt, float* loss, cudaStream_t s) {
    dim3 grid((unsigned)(ncells / 64), (unsigned)(B / 64));
    bce_bitmask_t_kernel<<<grid, 256, 0, s>>>(logits, masks, slot_words, wpr, ncols, ncells, scale,
                                              (__nv_bfloat16*)dlogits, (__nv_bfloat16*)dlogits_t, ldt, loss);
    return cudaGetLastError();
}

cudaError_t launch_adamw_t(float* w, float* m, float* v, const float* g, void* wb, void* wbt, long long ldt, int rows,
                           int cols, const float* hyper, float b1, float b2, float eps, float wd, cudaStream_t s) {
    dim3 grid((unsigned)(cols / 64), (unsigned)(rows / 64));
    adamw_t_kernel<<<grid, 256, 0, s>>>(w, m, v, g, (__nv_bfloat16*)wb, (__nv_bfloat16*)wbt, ldt, cols, hyper, b1, b2,
                                        eps, wd);
    return cudaGetLastError();
}

cudaError_t launch_transpose_bf16(const void* src, int rows, int cols, long long lds, void* dst, long long ldd,
                                  cudaStream_t s) {
    if (rows <= 0 || cols <= 0) return cudaSuccess;
    dim3 grid((unsigned)((cols + TT - 1) / TT), (unsigned)((rows + TT - 1) / TT));
    transpose_bf16_kernel<<<grid, 256, 0, s>>>((const uint16_t*)src, rows, cols, lds, (uint16_t*)dst, ldd);
    return cudaGetLastError();
}

cudaError_t launch_sigmoid_colsum(const float* logits, int rows, int cols, float* out, cudaStream_t s) {
    sigmoid_colsum_kernel<<<(cols + 255) / 256, 256, 0, s>>>(logits, rows, cols, out);
    return cudaGetLastError();
}

cudaError_t launch_features(const double* coef, const double* q, const double* aquifer, int nwells, int n,
                            const float* mean, const float* inv_std, int nf, int ld, void* x, cudaStream_t s) {
    const long long tot = (long long)n * ld;
    if (tot <= 0) return cudaSuccess;
    features_kernel<<<(unsigned)((tot + 255) / 256), 256, 0, s>>>(coef, q, aquifer, nwells, n, mean, inv_std, nf,
                                                                  ld, (__nv_bfloat16*)x);
    return cudaGetLastError();
}

}  // namespace oneka
