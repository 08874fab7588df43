// jt_tc_f32.cu -- launchers of the split-operand tensor-core kernels
// (jt_tcsplit.cuh) for Float32 row lines of length 16..2048.
#include <mutex>

#include "jt_tcsplit.cuh"

namespace jt {

// DFT-16 operand tables (heads + remainders) for sign -1 and +1, built once.
static float *g_btab[2] = {nullptr, nullptr};
static std::mutex g_btab_mu;

static const float *tc_btab(int sign) {
    const int i = sign < 0 ? 0 : 1;
    std::lock_guard<std::mutex> g(g_btab_mu);
    if (!g_btab[i]) {
        float *d = nullptr;
        if (cudaMalloc(&d, 2048 * sizeof(float)) != cudaSuccess) return nullptr;
        tc_btab_kernel<<<4, 256>>>(d, sign);
        if (cudaGetLastError() != cudaSuccess || cudaDeviceSynchronize() != cudaSuccess) {
            cudaFree(d);
            return nullptr;
        }
        g_btab[i] = d;
    }
    return g_btab[i];
}

template <int L> struct TcLaunch {
    template <int SIGN>
    static bool one(const float2 *in, float2 *out, const StockParams &p, const float2 *W, const float *B, int *err, int sms,
                    cudaStream_t s) {
        typedef TcCfg<L> K;
        static int per_sm = 0;
        if (!per_sm) {
            cudaFuncSetAttribute(tcfft_kernel<L, SIGN>, cudaFuncAttributeMaxDynamicSharedMemorySize, K::SMEM);
            // shared memory for the resident blocks (the occupancy query
            // follows the carveout preference)
            cudaFuncSetAttribute(tcfft_kernel<L, SIGN>, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, tcfft_kernel<L, SIGN>, K::NT, K::SMEM);
            // the register and shared-memory limits directly (the occupancy
            // query may not count a tensor-memory kernel's blocks)
            cudaFuncAttributes fa;
            if (cudaFuncGetAttributes(&fa, tcfft_kernel<L, SIGN>) == cudaSuccess && fa.numRegs > 0) {
                const int regs = (fa.numRegs + 7) / 8 * 8;
                const int by_regs = 65536 / (regs * K::NT);
                const int by_smem = (228 * 1024) / (K::SMEM + 1024);
                per_sm = std::max(per_sm, std::min(by_regs, by_smem));
            }
            if (per_sm < 1) per_sm = 1;
            if (per_sm > 8) per_sm = 8;  // 8 x 32 tensor-memory columns: half the SM's 512
        }
        const int64_t ntiles = (p.nlines + K::C - 1) / K::C;
        const int64_t grid = std::min<int64_t>(ntiles, (int64_t)sms * per_sm);
        tcfft_kernel<L, SIGN><<<(unsigned)grid, K::NT, K::SMEM, s>>>(in, out, p, W, B, err);
        return true;
    }
};

// Whether the tensor-core kernel exists for length L.
bool tc_split_ok(int L) {
    switch (L) {
        case 16: case 32: case 64: case 128: case 256: case 512: case 1024: case 2048: return true;
        default: return false;
    }
}

// Transforms p.nlines row lines of length L (W: the length's pass twiddle
// table); false when L has no kernel or the DFT tables could not be built.
bool tc_split_launch(int L, int sign, const float2 *in, float2 *out, const StockParams &p, const float2 *W, int *err, int sms,
                     cudaStream_t s) {
    const float *B = tc_btab(sign);
    if (!B) return false;
#define JT_TCASE(LL)                                                                                   \
    case LL:                                                                                           \
        return sign < 0 ? TcLaunch<LL>::one<-1>(in, out, p, W, B, err, sms, s)                          \
                        : TcLaunch<LL>::one<1>(in, out, p, W, B, err, sms, s);
    switch (L) {
        JT_TCASE(16) JT_TCASE(32) JT_TCASE(64) JT_TCASE(128) JT_TCASE(256) JT_TCASE(512) JT_TCASE(1024) JT_TCASE(2048)
        default: return false;
    }
#undef JT_TCASE
}

}  // namespace jt
