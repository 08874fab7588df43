// jt_peak.cu -- CUDA-core FMA throughput of this GPU, the compute roofline
// of the Double (FP64) and Float (FP32) transform paths.
//
// Every thread runs ACC independent FMA chains (acc = acc * m + a) for
// `iters` steps: enough independent chains to keep the pipe busy, no memory
// traffic in the loop.  One FMA counts as two flops.  The accumulators are
// stored at the end so the chains are not optimised away.
#include <cuda_runtime.h>

#include "../../include/jtgpu.h"

namespace jt {

template <typename T, int ACC>
__global__ void __launch_bounds__(256) fma_peak_kernel(T *out, int iters, T m, T a) {
    T acc[ACC];
#pragma unroll
    for (int k = 0; k < ACC; k++) acc[k] = (T)(threadIdx.x + k);
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int k = 0; k < ACC; k++) acc[k] = fma(acc[k], m, a);
    }
    T s = 0;
#pragma unroll
    for (int k = 0; k < ACC; k++) s += acc[k];
    out[blockIdx.x * (size_t)blockDim.x + threadIdx.x] = s;
}

template <typename T> static int measure(double *gflops) {
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        return JT_ECUDA;
    constexpr int ACC = 8, THREADS = 256;
    const int blocks = sms * 8;
    const int iters = sizeof(T) == 8 ? 1 << 14 : 1 << 16;
    T *out = nullptr;
    if (cudaMalloc(&out, sizeof(T) * (size_t)blocks * THREADS) != cudaSuccess) return JT_ENOMEM;
    cudaStream_t s = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    int st = JT_OK;
    if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess || cudaEventCreate(&e0) != cudaSuccess ||
        cudaEventCreate(&e1) != cudaSuccess)
        st = JT_ECUDA;
    float best = 1e30f;
    // m slightly below 1 keeps the values finite over the chain
    const T m = (T)0.999999, a = (T)1e-3;
    for (int r = 0; r < 6 && st == JT_OK; r++) {  // the first run warms up
        cudaEventRecord(e0, s);
        fma_peak_kernel<T, ACC><<<blocks, THREADS, 0, s>>>(out, iters, m, a);
        cudaEventRecord(e1, s);
        if (cudaEventSynchronize(e1) != cudaSuccess) {
            st = JT_ECUDA;
            break;
        }
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        if (r > 0 && ms < best) best = ms;
    }
    if (st == JT_OK && cudaGetLastError() != cudaSuccess) st = JT_ECUDA;
    if (st == JT_OK) *gflops = 2.0 * ACC * (double)iters * blocks * THREADS / (best * 1e-3) / 1e9;
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (s) cudaStreamDestroy(s);
    cudaFree(out);
    return st;
}

}  // namespace jt

extern "C" int jt_fma_peak(int prec, double *gflops) {
    if (!gflops || (prec != JT_FLOAT32 && prec != JT_FLOAT64)) return JT_EINVAL;
    return prec == JT_FLOAT64 ? jt::measure<double>(gflops) : jt::measure<float>(gflops);
}
