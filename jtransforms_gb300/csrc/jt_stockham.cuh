// jt_stockham.cuh -- power-of-two complex FFT lines held in registers.
//
// One CTA transforms C lines of compile-time length L.  Each thread owns
// E = 16 elements of one line (t, t+TL, ..., t+15*TL with TL = L/16): the
// radix-16 butterflies of a pass run in registers and shared memory is used
// only to exchange data between passes (self-sorting Stockham order, so the
// result comes out in natural order with no bit reversal).  The first pass
// reads global memory directly and the last pass writes it directly, both
// coalesced:
//   MODE 0  rows in, rows out        (contiguous lines; threads walk a line)
//   MODE 1  columns in, columns out  (lines C adjacent columns; threads walk
//           across the columns), optional four-step twiddle on the output
//   MODE 2  rows in, columns out     (the transposing row pass of the
//           four-step scheme: rows are staged through shared memory)
#pragma once

#include "jt_device.cuh"

namespace jt {

__host__ __device__ constexpr int ilog2c(int x) { return x <= 1 ? 0 : 1 + ilog2c(x >> 1); }
__host__ __device__ constexpr int ipowc(int b, int e) { return e == 0 ? 1 : b * ipowc(b, e - 1); }

struct StockParams {
    int64_t nlines;
    Layout lin, lout;
    double scale;
    int64_t tw_n, tw_inner;  // four-step output twiddle w_{tw_n}^{pos * (b % tw_inner)}; tw_n = 0: none
    int tw_lo_bits;
};

template <typename T> struct StockCfg {
    // lines per CTA for the row mode: about 256 threads
    static constexpr int rows_C(int L) { return L >= 4096 ? 1 : 4096 / L; }
    // lines per CTA for the column modes: 128-byte row segments when the
    // line is short, at least one 32-byte sector when it is long
    static constexpr int cols_C(int L) {
        return sizeof(T) == 4 ? (L <= 512 ? 16 : (8192 / L < 4 ? 4 : 8192 / L))
                              : (L <= 256 ? 8 : (4096 / L < 2 ? 2 : 4096 / L));
    }
    static constexpr int C(int L, int mode) { return mode == 0 ? rows_C(L) : cols_C(L); }
};

template <int R, int SIGN, typename T> __device__ __forceinline__ void dft_pow2(typename V2<T>::t *u) {
    if (R == 2) dft2<SIGN, T>(u);
    else if (R == 4) dft4v<SIGN, T>(u);
    else if (R == 8) dft8<SIGN, T>(u);
    else if (R == 16) dft16<SIGN, T>(u);
}

template <typename T, int L, int MODE, int SIGN> struct Stockham {
    typedef typename V2<T>::t C2;
    static constexpr int E = L >= 16 ? 16 : L;
    static constexpr int TL = L / E;
    static constexpr int C = StockCfg<T>::C(L, MODE);
    static constexpr int NT = C * TL;
    static constexpr int LP = L + L / 16 + 1;
    static constexpr int LOGL = ilog2c(L), LOGE = ilog2c(E);
    static constexpr int NFULL = LOGL / LOGE;
    static constexpr int REM = 1 << (LOGL % LOGE);
    static constexpr int NPASS = NFULL + (REM > 1 ? 1 : 0);
    static constexpr size_t SMEM = (size_t)C * LP * sizeof(C2);

    template <int P> struct Pass {
        static constexpr int R = P < NFULL ? E : REM;
        static constexpr int NS = ipowc(E, P);
        static constexpr int NB = E / R;  // butterflies per thread
        static constexpr int SHIFT = LOGL - ilog2c(NS * R);
        static constexpr bool LAST = P == NPASS - 1;
    };

    // Butterflies of pass P on the thread's registers; non-last passes write
    // their outputs to the line's shared-memory row.
    template <int P, typename Store>
    static __device__ __forceinline__ void run(C2 (&v)[E], int t, C2 *sl, const C2 *__restrict__ W, Store &store) {
        typedef Pass<P> PP;
#pragma unroll
        for (int q = 0; q < PP::NB; q++) {
            C2 u[PP::R];
#pragma unroll
            for (int k = 0; k < PP::R; k++) u[k] = v[q + k * PP::NB];
            const int j = t + q * TL;
            const int jm = j & (PP::NS - 1);
            if (PP::NS > 1) {
#pragma unroll
                for (int k = 1; k < PP::R; k++) {
                    C2 w = __ldg(&W[(jm * k) << PP::SHIFT]);
                    u[k] = SIGN < 0 ? cmul<T>(u[k], w) : cmulc<T>(u[k], w);
                }
            }
            dft_pow2<PP::R, SIGN, T>(u);
            const int idxD = (j - jm) * PP::R + jm;
#pragma unroll
            for (int k = 0; k < PP::R; k++) {
                if (PP::LAST) store(idxD + k * PP::NS, u[k]);
                else sl[pad(idxD + k * PP::NS)] = u[k];
            }
        }
        if constexpr (!PP::LAST) {
            __syncthreads();
#pragma unroll
            for (int m = 0; m < E; m++) v[m] = sl[pad(t + m * TL)];
            __syncthreads();
            run<P + 1>(v, t, sl, W, store);
        }
    }
};

template <typename T, int L, int MODE, int SIGN>
__global__ void __launch_bounds__(Stockham<T, L, MODE, SIGN>::NT)
    stockham_kernel(const typename V2<T>::t *__restrict__ in, typename V2<T>::t *__restrict__ out, StockParams p,
                    const typename V2<T>::t *__restrict__ W, const typename V2<T>::t *__restrict__ Whi,
                    const typename V2<T>::t *__restrict__ Wlo) {
    typedef Stockham<T, L, MODE, SIGN> S;
    typedef typename V2<T>::t C2;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C2 *sm = reinterpret_cast<C2 *>(smem_raw);
    const int tid = threadIdx.x;
    int c, t;
    if (MODE == 0) {
        c = tid / S::TL;
        t = tid % S::TL;
    } else {
        c = tid % S::C;
        t = tid / S::C;
    }
    const int64_t b0 = (int64_t)blockIdx.x * S::C;
    const int64_t b = b0 + c;
    const bool valid = b < p.nlines;
    C2 *sl = sm + c * S::LP;
    C2 v[S::E];

    if (MODE == 2) {
        // stage the C rows through shared memory with row-contiguous reads
#pragma unroll 4
        for (int i = tid; i < S::C * L; i += S::NT) {
            int cc = i >> S::LOGL, e = i & (L - 1);
            if (b0 + cc < p.nlines) sm[cc * S::LP + pad(e)] = in[line_off(p.lin, b0 + cc) + e];
        }
        __syncthreads();
#pragma unroll
        for (int m = 0; m < S::E; m++) v[m] = sl[pad(t + m * S::TL)];
        __syncthreads();
    } else if (valid) {
        const C2 *src = in + line_off(p.lin, b);
        const int64_t es = MODE == 0 ? 1 : p.lin.estride;
#pragma unroll
        for (int m = 0; m < S::E; m++) v[m] = src[(int64_t)(t + m * S::TL) * es];
    } else {
#pragma unroll
        for (int m = 0; m < S::E; m++) v[m] = mk<T>(0, 0);
    }

    C2 *dst = out + (valid ? line_off(p.lout, b) : 0);
    const int64_t oes = MODE == 0 ? 1 : p.lout.estride;
    const bool tw = p.tw_n != 0;
    const int64_t j2 = tw ? b % p.tw_inner : 0;
    const int64_t lo_mask = ((int64_t)1 << p.tw_lo_bits) - 1;
    const T sc = (T)p.scale;
    const bool do_scale = p.scale != 1.0;
    auto store = [&](int pos, C2 val) {
        if (tw) {
            int64_t tt = (int64_t)pos * j2;
            C2 w = cmul<T>(__ldg(&Whi[tt >> p.tw_lo_bits]), __ldg(&Wlo[tt & lo_mask]));
            val = SIGN < 0 ? cmul<T>(val, w) : cmulc<T>(val, w);
        }
        if (do_scale) val = cscale<T>(val, sc);
        if (valid) dst[(int64_t)pos * oes] = val;
    };
    S::template run<0>(v, t, sl, W, store);
}

// Host-side launcher for one (T, L): picks the instantiation by mode/sign.
template <typename T, int L> struct StockLaunch {
    template <int MODE, int SIGN> static void one(const typename V2<T>::t *in, typename V2<T>::t *out, const StockParams &p,
                                                  const typename V2<T>::t *W, const typename V2<T>::t *Whi,
                                                  const typename V2<T>::t *Wlo, cudaStream_t s) {
        typedef Stockham<T, L, MODE, SIGN> S;
        static bool attr = false;
        if (!attr) {
            cudaFuncSetAttribute(stockham_kernel<T, L, MODE, SIGN>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)S::SMEM);
            attr = true;
        }
        int64_t grid = (p.nlines + S::C - 1) / S::C;
        stockham_kernel<T, L, MODE, SIGN><<<(unsigned)grid, S::NT, S::SMEM, s>>>(in, out, p, W, Whi, Wlo);
    }
    static void go(int mode, int sign, const typename V2<T>::t *in, typename V2<T>::t *out, const StockParams &p,
                   const typename V2<T>::t *W, const typename V2<T>::t *Whi, const typename V2<T>::t *Wlo, cudaStream_t s) {
        if (mode == 0) {
            sign < 0 ? one<0, -1>(in, out, p, W, Whi, Wlo, s) : one<0, 1>(in, out, p, W, Whi, Wlo, s);
            return;
        }
        if constexpr (L <= 4096) {  // column modes: C lines of up to 4096 fit one CTA
            if (mode == 1) sign < 0 ? one<1, -1>(in, out, p, W, Whi, Wlo, s) : one<1, 1>(in, out, p, W, Whi, Wlo, s);
            else sign < 0 ? one<2, -1>(in, out, p, W, Whi, Wlo, s) : one<2, 1>(in, out, p, W, Whi, Wlo, s);
        }
    }
    static int lines_per_cta(int mode) { return StockCfg<T>::C(L, mode); }
};

}  // namespace jt
