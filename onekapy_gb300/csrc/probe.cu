// probe.cu -- FMA throughput probe used as the roofline denominator of the
// tracker (the tracker is bound by the FP32 (fast build) or FP64 (parity
// build) FMA pipe, which the HBM/BF16 peak table does not cover).
#include "oneka_internal.cuh"

namespace oneka {
namespace {

constexpr int kChains = 8;

template <typename T>
__global__ void __launch_bounds__(256) fma_loop_kernel(T b, T c, int iters, T* sink) {
    T a[kChains];
#pragma unroll
    for (int k = 0; k < kChains; ++k) a[k] = (T)(threadIdx.x + k);
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int k = 0; k < kChains; ++k) a[k] = fma(a[k], b, c);
    }
    T s = 0;
#pragma unroll
    for (int k = 0; k < kChains; ++k) s += a[k];
    if (s == (T)-1.2345e-7) sink[threadIdx.x] = s;   // never true; keeps the loop live
}

template <typename T>
cudaError_t time_fma(double* flops_per_s, cudaStream_t s) {
    int dev = 0, sms = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
    const int block = 256, blocks = sms * 8;
    const int iters = sizeof(T) == 4 ? 1 << 16 : 1 << 12;
    T* sink = nullptr;     // the store never executes
    cudaEvent_t t0, t1;
    cudaEventCreate(&t0);
    cudaEventCreate(&t1);
    fma_loop_kernel<T><<<blocks, block, 0, s>>>((T)0.999999, (T)1e-7, iters, sink);   // warm-up
    cudaEventRecord(t0, s);
    fma_loop_kernel<T><<<blocks, block, 0, s>>>((T)0.999999, (T)1e-7, iters, sink);
    cudaEventRecord(t1, s);
    e = cudaEventSynchronize(t1);
    float ms = 0.f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, t0, t1);
    cudaEventDestroy(t0);
    cudaEventDestroy(t1);
    if (e != cudaSuccess) return e;
    *flops_per_s = 2.0 * kChains * (double)iters * block * (double)blocks / (ms * 1e-3);
    return cudaGetLastError();
}

}  // namespace

cudaError_t probe_fma(int fp64, double* flops_per_s, cudaStream_t s) {
    return fp64 ? time_fma<double>(flops_per_s, s) : time_fma<float>(flops_per_s, s);
}

}  // namespace oneka
