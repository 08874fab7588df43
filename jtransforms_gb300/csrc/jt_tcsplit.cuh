// jt_tcsplit.cuh -- split-operand tensor-core path for Float32 lines.
//
// The radix-16 Stockham passes of the register kernel (jt_stockham.cuh) run
// here as dense DFT-16 products on the tensor cores.  A CTA of 128 threads
// holds 2048 complex elements (2048 / L lines); thread i owns butterfly i of
// every pass, which is row i of the M = 128 product
//     D (128 x 32) = X (128 x 32) * F16 (32 x 32)
// with each butterfly's 16 inputs interleaved as (re, im) along K and the
// real 32 x 32 form of the DFT-16 matrix as B.  Each FP32 operand is split
// into a TF32 head (rounded to 11 significant bits) and the exact FP32
// remainder; three products hi*hi + lo*hi + hi*lo accumulate in FP32 in
// tensor memory (kind::tf32, 12 MMAs of K = 8 per pass).  The dropped lo*lo
// term and the remainders' own TF32 truncation are below 2^-21 of each
// product.  (A BF16 head + BF16 remainder keeps only 16 bits and leaves a
// 2^-17 residual per operand, too coarse for the 1e-6 bound.)
//
// Twiddles, the head/remainder split and the final short radix (L not a
// power of 16) stay on the CUDA cores in FP32.  From the first radix-16 pass
// to the second each thread twiddles its own 16 outputs (they all feed input
// k' = 16 t / (L/16) of the next pass, so their factors w_256^{k k'} are one
// row of the pass table) and writes them straight into the next pass's A
// rows; before a final short radix the outputs go through the padded
// exchange buffer (aliasing the A operands, dead once their products
// completed), as in the register kernel.
//
// Operands are K-major without swizzle: core matrices of 8 rows x 16 bytes.
// A: element (r, k) at byte (r / 8) * 1168 + (k / 4) * 144 + (r % 8) * 16 +
// (k % 4) * 4 (leading offset 144, stride offset 1168): the 16-byte skews
// put both the own-row writes and the scattered next-pass writes of a warp
// on every bank slot equally (minimum wavefronts).  B: leading offset 128,
// stride offset 1024.
#pragma once

#include "jt_stockham.cuh"
#include "jt_umma.cuh"

namespace jt {

#define JT_TC_POLL_LIMIT (1u << 22)

// head / remainder split: hi has 11 significant bits (round to nearest),
// lo = x - hi is exact
__device__ __forceinline__ void tf32_split(float x, float &hi, float &lo) {
    const uint32_t u = __float_as_uint(x);
    hi = __uint_as_float((u + 0x1000u) & 0xFFFFE000u);
    lo = x - hi;
}

// Real 32 x 32 form of the DFT-16 matrix e^{sign 2 pi i n k / 16}, stored
// transposed (row = output nn = 2n + part, column = input kk = 2k + part) in
// the operand layout above: heads at out[0..1023], remainders at
// out[1024..2047].  FP64 sincospi, rounded afterwards.
__global__ void tc_btab_kernel(float *out, int sign) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= 1024) return;
    const int nn = i / 32, kk = i % 32, n = nn >> 1, k = kk >> 1;
    double s, c;
    sincospi((double)sign * 2.0 * (double)((n * k) & 15) / 16.0, &s, &c);
    // Y_re = sum c X_re - s X_im ; Y_im = sum s X_re + c X_im
    const double val = (nn & 1) == 0 ? ((kk & 1) == 0 ? c : -s) : ((kk & 1) == 0 ? s : c);
    const float f = (float)val;
    float hi, lo;
    tf32_split(f, hi, lo);
    lo = (float)(val - (double)hi);
    const int off = (nn / 8) * 256 + (kk / 4) * 32 + (nn % 8) * 4 + (kk % 4);
    out[off] = hi;
    out[1024 + off] = lo;
}

template <int L> struct TcCfg {
    static constexpr int TL = L / 16;     // butterflies per line and pass
    static constexpr int C = 2048 / L;    // lines per tile
    static constexpr int NT = 128;
    static constexpr int LOGL = ilog2c(L);
    static constexpr int NTC = LOGL / 4;  // radix-16 passes on the tensor cores
    static constexpr int LP = L + L / 16 + 1;
    static constexpr int A_LBO = 144, A_SBO = 1168, A_BYTES = 16 * A_SBO;
    static constexpr int OFF_AHI = 0, OFF_ALO = A_BYTES, OFF_B = 2 * A_BYTES;  // B: heads 4 KB, remainders 4 KB
    static constexpr int OFF_BAR = OFF_B + 8192, OFF_TM = OFF_BAR + 8;
    static constexpr int SMEM = OFF_BAR + 64;
    // byte offset of 16-byte chunk q (K elements 4q..4q+3) of A row r
    static __device__ __forceinline__ int aoff(int r, int q) { return (r >> 3) * A_SBO + q * A_LBO + (r & 7) * 16; }
    static constexpr bool OK = L >= 16 && L <= 2048 && (size_t)C * LP * 8 <= 2 * A_BYTES;
};

template <int L, int SIGN> struct TcPass {
    typedef TcCfg<L> K;
    typedef Stockham<float, L, 0, SIGN> S;

    // Pass s: twiddle, split into the A rows, products, read back, and
    // either exchange for the next pass or store.  Returns false when the
    // product's completion wait gave up.
    template <int s, typename Store>
    static __device__ __forceinline__ bool run(float2 (&v)[16], int t, int tid, unsigned char *sm, uint32_t sbase, uint32_t tmem,
                                               uint32_t taddr, uint64_t *bar, uint32_t &phase, const PadIdx &xi,
                                               const float2 *__restrict__ W, Store &store) {
        typedef typename S::template Pass<s> PP;
        if constexpr (s == 0) {
            __syncthreads();  // the previous tile's exchange (aliasing A) has been read
#pragma unroll
            for (int q = 0; q < 8; q++) {
                float4 h, l;
                tf32_split(v[2 * q].x, h.x, l.x);
                tf32_split(v[2 * q].y, h.y, l.y);
                tf32_split(v[2 * q + 1].x, h.z, l.z);
                tf32_split(v[2 * q + 1].y, h.w, l.w);
                *reinterpret_cast<float4 *>(sm + K::OFF_AHI + K::aoff(tid, q)) = h;
                *reinterpret_cast<float4 *>(sm + K::OFF_ALO + K::aoff(tid, q)) = l;
            }
        }
        // (pass s > 0: the previous pass wrote this pass's A rows directly)
        fence_proxy_async_smem();
        tc_fence_before();
        __syncthreads();
        if (tid == 0) {
            tc_fence_after();
            constexpr uint32_t IDESC = umma_idesc_tf32(128, 32);
            const uint64_t ahi = umma_desc(sbase + K::OFF_AHI, K::A_LBO, K::A_SBO);
            const uint64_t alo = umma_desc(sbase + K::OFF_ALO, K::A_LBO, K::A_SBO);
            const uint64_t bhi = umma_desc(sbase + K::OFF_B, 128, 1024), blo = umma_desc(sbase + K::OFF_B + 4096, 128, 1024);
#pragma unroll
            for (int pr = 0; pr < 3; pr++) {
                const uint64_t a = pr == 1 ? alo : ahi;
                const uint64_t b = pr == 2 ? blo : bhi;
                // K step ks starts 2 core matrices further: 2 * LBO bytes (16-byte units)
#pragma unroll
                for (int ks = 0; ks < 4; ks++)
                    umma_tf32(tmem, a + ks * (2 * K::A_LBO / 16), b + ks * (2 * 128 / 16), IDESC, (pr | ks) != 0);
            }
            umma_commit(bar);
        }
        // one thread polls; the others wait at the barrier
        const bool mine = tid == 0 ? mbar_wait_bounded(bar, phase & 1, JT_TC_POLL_LIMIT) : true;
        phase++;
        if (!__syncthreads_and(mine)) return false;
        tc_fence_after();
        float r[32];
        tmem_ld32(taddr, r);
        // butterfly t's outputs go to idxD + k NS (self-sorting order)
        const int jm = t & (PP::NS - 1);
        const int idxD = (t - jm) * 16 + jm;
        constexpr bool LAST_TC = s == K::NTC - 1;
        if constexpr (LAST_TC && S::NPASS == K::NTC) {
#pragma unroll
            for (int k = 0; k < 16; k++) store(idxD + k * PP::NS, make_float2(r[2 * k], r[2 * k + 1]), k);
            tc_fence_before();
            return true;
        } else if constexpr (!LAST_TC) {
            // first radix-16 pass -> second: output k of butterfly t is input
            // k' = 16 t / TL of butterfly j' = (16 t + k) mod TL of the next
            // pass (s = 0: idxD = 16 t), with factor w_256^{(j' mod 16) k'} =
            // w_256^{k k'}: the pass-1 factors of jm = k' (the table is symmetric)
            static_assert(s == 0 && PP::NS == 1, "direct writes follow the first pass");
            const int kp = (16 * t) / K::TL;
            const int c = tid / K::TL;
            float2 tw[16];
            tw[0] = make_float2(1.f, 0.f);
            S::template tw_row<1>(kp, W, &tw[1]);
            const int colb = K::aoff(0, kp >> 1) + (kp & 1) * 8;  // chunk of column pair k', row 0
#pragma unroll
            for (int k = 0; k < 16; k++) {
                float2 u = make_float2(r[2 * k], r[2 * k + 1]);
                if (k > 0) u = SIGN < 0 ? cmul<float>(u, tw[k]) : cmulc<float>(u, tw[k]);
                const int rp = c * K::TL + ((16 * t + k) & (K::TL - 1));
                const int off = colb + (rp >> 3) * K::A_SBO + (rp & 7) * 16;
                float2 h, l;
                tf32_split(u.x, h.x, l.x);
                tf32_split(u.y, h.y, l.y);
                *reinterpret_cast<float2 *>(sm + K::OFF_AHI + off) = h;
                *reinterpret_cast<float2 *>(sm + K::OFF_ALO + off) = l;
            }
            tc_fence_before();
            return run<s + 1>(v, t, tid, sm, sbase, tmem, taddr, bar, phase, xi, W, store);
        } else {
            float2 *xs = reinterpret_cast<float2 *>(sm + K::OFF_AHI);
            if constexpr (PP::NS % 16 == 0 || PP::NS == 1) {
                const int pb = xi(idxD);
                constexpr int ST = PP::NS == 1 ? 1 : PP::NS + PP::NS / 16;
#pragma unroll
                for (int k = 0; k < 16; k++) xs[pb + k * ST] = make_float2(r[2 * k], r[2 * k + 1]);
            } else {
#pragma unroll
                for (int k = 0; k < 16; k++) xs[xi(idxD + k * PP::NS)] = make_float2(r[2 * k], r[2 * k + 1]);
            }
            tc_fence_before();
            __syncthreads();
            if constexpr (K::TL % 16 == 0) {
                const int pr = xi(t);
#pragma unroll
                for (int m = 0; m < 16; m++) v[m] = xs[pr + m * (K::TL + K::TL / 16)];
            } else {
#pragma unroll
                for (int m = 0; m < 16; m++) v[m] = xs[xi(t + m * K::TL)];
            }
            // final short radix on the CUDA cores (its pass reads no shared memory)
            float2 tw[S::template Tw<K::NTC>::N];
            S::template load_tw<K::NTC>(t, W, tw);
            auto nosync = [] {};
            S::template run<K::NTC>(v, tw, t, xs, xi, W, store, nosync);
            return true;
        }
    }
};

// Persistent kernel over tiles of 2048 / L contiguous lines.  Every wait is
// bounded; on timeout the kernel raises the error flag, lets outstanding
// products finish (bounded) and frees its tensor memory before returning.
template <int L, int SIGN>
__global__ void __launch_bounds__(128, 4)
    tcfft_kernel(const float2 *in, float2 *out, StockParams p, const float2 *__restrict__ W, const float *__restrict__ Btab,
                 int *err) {
    typedef TcCfg<L> K;
    static_assert(K::OK && K::C * K::TL == K::NT, "tile: 2048 elements, one butterfly per thread, exchange within A");
    extern __shared__ __align__(1024) unsigned char sm[];
    const int tid = threadIdx.x, warp = tid >> 5;
    const int c = tid / K::TL, t = tid % K::TL;
    uint64_t *bar = reinterpret_cast<uint64_t *>(sm + K::OFF_BAR);
    uint32_t *tslot = reinterpret_cast<uint32_t *>(sm + K::OFF_TM);
    // DFT-16 operand: 8 KB, 16 bytes per thread and step
    for (int i = tid; i < 512; i += K::NT)
        reinterpret_cast<float4 *>(sm + K::OFF_B)[i] = __ldg(reinterpret_cast<const float4 *>(Btab) + i);
    if (tid == 0) {
        mbar_init(bar, 1);
        fence_mbar_init();
    }
    if (warp == 0) {
        tmem_alloc(tslot, 32);
        tmem_relinquish();
    }
    fence_proxy_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tslot;
    const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16);
    const uint32_t sbase = smem_addr(sm);
    const int64_t ntiles = (p.nlines + K::C - 1) / K::C;
    const float sc = p.scalef;
    const bool do_scale = p.do_scale != 0;
    const uint64_t spol = p.stream_out ? policy_evict_first() : policy_evict_normal();
    const PadIdx xi{c * K::LP};
    uint32_t phase = 0;
    bool ok = true;
    // this thread's 16 inputs of a tile (zeros past the last line)
    auto load = [&](int64_t tl, float2 (&x)[16]) {
        const int64_t bb = tl * K::C + c;
        if (tl < ntiles && bb < p.nlines) {
            const float2 *src = in + line_off(p.lin, bb);
#pragma unroll
            for (int m = 0; m < 16; m++) x[m] = src[t + m * K::TL];
        } else {
#pragma unroll
            for (int m = 0; m < 16; m++) x[m] = make_float2(0.f, 0.f);
        }
    };
    float2 v[16];
    load(blockIdx.x, v);
    for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int64_t b = tile * K::C + c;
        const bool valid = b < p.nlines;
        // the next tile's inputs are in flight while this one is transformed
        // (its lines are disjoint from every line written meanwhile)
        float2 vn[16];
        load(tile + gridDim.x, vn);
        float2 *dst = out + (valid ? line_off(p.lout, b) : 0);
        auto store = [&](int pos, float2 val, int) {
            if (do_scale) val = cscale<float>(val, sc);
            if (valid) st_hint(&dst[pos], val, spol);
        };
        if (!TcPass<L, SIGN>::template run<0>(v, t, tid, sm, sbase, tmem, taddr, bar, phase, xi, W, store)) {
            ok = false;
            break;
        }
#pragma unroll
        for (int m = 0; m < 16; m++) v[m] = vn[m];
    }
    if (!ok) {
        if (tid == 0) {
            atomicExch(err, 1);
            mbar_wait_bounded(bar, (phase - 1) & 1, JT_TC_POLL_LIMIT);  // outstanding products
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        tmem_dealloc(tmem, 32);
    }
}

}  // namespace jt
