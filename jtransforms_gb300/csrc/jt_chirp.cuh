// jt_chirp.cuh -- Bluestein (chirp-z) transforms in one CTA tile.
//
// For a length n whose padded length nB = nextPow2(2n - 1) fits a tile (the
// tile kernel's limit), a CTA runs the whole chirp-z transform of C lines in
// shared memory: the chirp premultiply and zero pad on the load, the nB-point
// forward FFT, the multiply by the transformed chirp, the nB-point inverse
// FFT, and the chirp postmultiply (times the scale) on the store.  The
// chirp tables are the FP64-built bk1 (n) and bk2 (nB) of the plan, the
// same ones the separate pre/mul/post kernels of jt_device.cuh use.
// Reference: fft/DoubleFFT_1D.java:1864-1890 (bluesteini), :1920-2107
// (bluestein_complex).
#pragma once

#include "jt_device.cuh"

namespace jt {

#define C2 typename V2<T>::t

struct BlueParams {
    int n, nB;              // transform and padded lengths
    int npass;              // passes of the nB-point FFT
    int radix[JT_MAX_PASSES];
    int C;                  // lines per CTA
    int64_t nlines;
    Layout lin, lout;       // line layouts in complex elements
    double scale;           // output multiplier (double plans)
    float scalef;           // the same for float plans
};

// Tile `blk` run by the calling CTA, any block size; shared memory at
// smem_raw holds 2 * C * padded(nB) complex.  W: e^{-2 pi i t/nB}.
template <int SIGN, typename T>
__device__ void blue_tile_body(const C2 *in, C2 *out, const BlueParams &p, const C2 *__restrict__ W,
                               const C2 *__restrict__ bk1, const C2 *__restrict__ bk2, int64_t blk, unsigned char *smem_raw) {
    const int n = p.n, nB = p.nB, Lp = padded_len(nB);
    C2 *bufA = reinterpret_cast<C2 *>(smem_raw);
    C2 *bufB = bufA + p.C * Lp;
    const int64_t b0 = blk * p.C;
    const int lines = (int)min((int64_t)p.C, p.nlines - b0);
    if (lines <= 0) return;
    T sc;
    if constexpr (sizeof(T) == 4) sc = p.scalef;
    else sc = (T)p.scale;
    const int tid = threadIdx.x, nt = blockDim.x;
    const int tot = lines * nB;
    for (int idx = tid; idx < tot; idx += nt) {
        const int c = idx / nB, i = idx - c * nB;
        C2 v = mk<T>(0, 0);
        if (i < n) {
            const C2 x = in[line_off(p.lin, b0 + c) + (int64_t)i * p.lin.estride], w = __ldg(&bk1[i]);
            v = SIGN < 0 ? cmulc<T>(x, w) : cmul<T>(x, w);
        }
        bufA[c * Lp + pad(i)] = v;
    }
    __syncthreads();
    C2 *z = tile_passes<-1, T>(bufA, bufB, lines, nB, Lp, p.npass, p.radix, W);
    for (int idx = tid; idx < tot; idx += nt) {
        const int c = idx / nB, k = idx - c * nB;
        C2 &v = z[c * Lp + pad(k)];
        const C2 w = __ldg(&bk2[k]);
        v = SIGN < 0 ? cmul<T>(v, w) : cmulc<T>(v, w);
    }
    __syncthreads();
    const C2 *y = tile_passes<1, T>(z, z == bufA ? bufB : bufA, lines, nB, Lp, p.npass, p.radix, W);
    const int tn = lines * n;
    for (int idx = tid; idx < tn; idx += nt) {
        const int c = idx / n, i = idx - c * n;
        const C2 x = y[c * Lp + pad(i)], w = __ldg(&bk1[i]);
        C2 v = SIGN < 0 ? cmulc<T>(x, w) : cmul<T>(x, w);
        if (sc != (T)1) v = cscale<T>(v, sc);
        out[line_off(p.lout, b0 + c) + (int64_t)i * p.lout.estride] = v;
    }
}

template <int SIGN, typename T>
__global__ void __launch_bounds__(512) blue_tile_kernel(const C2 *in, C2 *out, BlueParams p, const C2 *__restrict__ W,
                                                        const C2 *__restrict__ bk1, const C2 *__restrict__ bk2) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    blue_tile_body<SIGN, T>(in, out, p, W, bk1, bk2, (int64_t)blockIdx.x, smem_raw);
}

#undef C2

}  // namespace jt
