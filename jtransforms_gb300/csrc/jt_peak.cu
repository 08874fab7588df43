// jt_peak.cu -- CUDA-core FMA throughput of this GPU, the compute roofline
// of the Double (FP64) and Float (FP32) transform paths; and the read
// bandwidth of distributed shared memory within a thread-block cluster, the
// bound of any plan that exchanges a transform between the CTAs of a cluster.
//
// Every thread runs ACC independent FMA chains (acc = acc * m + a) for
// `iters` steps: enough independent chains to keep the pipe busy, no memory
// traffic in the loop.  One FMA counts as two flops.  The accumulators are
// stored at the end so the chains are not optimised away.
#include <cooperative_groups.h>
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

// Every CTA fills DSMEM_BYTES of its shared memory, then reads `sweeps` whole
// copies of it from a peer of its cluster (remote = 1: peer = rank + 1 +
// sweep mod (cluster - 1), never itself) or from itself (remote = 0), 16 bytes
// per thread and load, 8 loads in flight per thread.
constexpr int DSMEM_BYTES = 128 * 1024, DSMEM_THREADS = 1024;

__global__ void __launch_bounds__(DSMEM_THREADS) dsmem_peak_kernel(float *out, int sweeps, int remote) {
    extern __shared__ float4 sbuf[];
    namespace cg = cooperative_groups;
    cg::cluster_group cl = cg::this_cluster();
    const int cs = (int)cl.num_blocks(), rank = (int)cl.block_rank();
    constexpr int N4 = DSMEM_BYTES / 16;
    static_assert(N4 % (8 * DSMEM_THREADS) == 0 && (N4 & (N4 - 1)) == 0, "8 loads per thread cover the buffer");
    for (int i = threadIdx.x; i < N4; i += blockDim.x) sbuf[i] = make_float4((float)i, (float)rank, 1.f, 2.f);
    cl.sync();
    float acc = 0.f;
    for (int it = 0; it < sweeps; it++) {
        const int peer = remote ? (rank + 1 + it % (cs - 1)) % cs : rank;
        const float4 *p = cl.map_shared_rank(sbuf, peer);
        // the start rotates by 16 elements per sweep, so no sweep repeats the
        // previous one's addresses (the loads cannot be hoisted out of the loop)
        for (int i = threadIdx.x; i < N4; i += 8 * DSMEM_THREADS) {
            float4 v[8];
#pragma unroll
            for (int u = 0; u < 8; u++) v[u] = p[(i + u * DSMEM_THREADS + it * 16) & (N4 - 1)];
#pragma unroll
            for (int u = 0; u < 8; u++) acc += v[u].x + v[u].y + v[u].z + v[u].w;
        }
    }
    cl.sync();  // no CTA leaves while a peer may still read its shared memory
    if (acc == -1.f) out[blockIdx.x] = acc;
}

static int measure_dsmem(int cluster, int remote, double *gbs, int *ctas) {
    if (cudaFuncSetAttribute(dsmem_peak_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, DSMEM_BYTES) != cudaSuccess ||
        cudaFuncSetAttribute(dsmem_peak_kernel, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess)
        return JT_ECUDA;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = (unsigned)cluster;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)cluster);
    cfg.blockDim = dim3(DSMEM_THREADS);
    cfg.dynamicSmemBytes = DSMEM_BYTES;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    int nclusters = 0;
    if (cudaOccupancyMaxActiveClusters(&nclusters, dsmem_peak_kernel, &cfg) != cudaSuccess) return JT_ECUDA;
    if (nclusters <= 0) return JT_EINVAL;  // clusters of this size do not fit
    cfg.gridDim = dim3((unsigned)(nclusters * cluster));  // one wave: every cluster resident
    float *out = nullptr;
    if (cudaMalloc(&out, sizeof(float) * nclusters * cluster) != cudaSuccess) return JT_ENOMEM;
    cudaStream_t s = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    int st = JT_OK;
    if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess || cudaEventCreate(&e0) != cudaSuccess ||
        cudaEventCreate(&e1) != cudaSuccess)
        st = JT_ECUDA;
    cfg.stream = s;
    const int sweeps = 64;
    float best = 1e30f;
    for (int r = 0; r < 4 && st == JT_OK; r++) {  // the first run warms up
        cudaEventRecord(e0, s);
        if (cudaLaunchKernelEx(&cfg, dsmem_peak_kernel, out, sweeps, remote) != cudaSuccess) st = JT_ECUDA;
        cudaEventRecord(e1, s);
        if (cudaEventSynchronize(e1) != cudaSuccess) st = JT_ECUDA;
        float ms = 0;
        if (st == JT_OK) cudaEventElapsedTime(&ms, e0, e1);
        if (st == JT_OK && r > 0 && ms < best) best = ms;
    }
    if (st == JT_OK && cudaGetLastError() != cudaSuccess) st = JT_ECUDA;
    if (st == JT_OK) {
        *gbs = (double)nclusters * cluster * sweeps * DSMEM_BYTES / (best * 1e-3) / 1e9;
        if (ctas) *ctas = nclusters * cluster;
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (s) cudaStreamDestroy(s);
    cudaFree(out);
    return st;
}

}  // namespace jt

extern "C" int jt_dsmem_peak(int cluster, int remote, double *gbs, int *active_ctas) {
    if (!gbs || (cluster != 2 && cluster != 4 && cluster != 8 && cluster != 16) || (remote != 0 && remote != 1))
        return JT_EINVAL;
    return jt::measure_dsmem(cluster, remote, gbs, active_ctas);
}

extern "C" int jt_fma_peak(int prec, double *gflops) {
    if (!gflops || (prec != JT_FLOAT32 && prec != JT_FLOAT64)) return JT_EINVAL;
    return prec == JT_FLOAT64 ? jt::measure<double>(gflops) : jt::measure<float>(gflops);
}
