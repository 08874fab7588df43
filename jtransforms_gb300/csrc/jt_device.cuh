// jt_device.cuh -- device code of jtransforms_gb300 (sm_103a).
//
// Kernels:
//   fft_tile_kernel     batched complex FFT of one length L held in shared
//                       memory: self-sorting (Stockham) passes of radix
//                       16/8/4/2/3/5/7 and generic odd radices, strided line
//                       layouts so the same kernel serves contiguous rows,
//                       2D/3D column passes and both passes of the large-N
//                       two-pass (four-step) scheme.  Replaces the Ooura
//                       split-radix tree (utils/CommonUtils.java:708-5749),
//                       bitrv2* and the FFTPACK passes (fft/DoubleFFT_1D.java:
//                       6630-7842).
//   real_*              real-FFT pack/unpack around a half-length complex FFT
//                       (replaces rftfsub/rftbsub, utils/CommonUtils.java:5750-5830).
//   bluestein_*         chirp multiplies (fft/DoubleFFT_1D.java:1920-2107).
//   dct_* / dht_*       DCT-II/III, DST, DHT pre/post passes around a real FFT
//                       (dct/DoubleDCT_1D.java:169-440, dst/DoubleDST_1D.java,
//                       dht/DoubleDHT_1D.java).
//   rdft2d_kernel, ytransform*_kernel   2D real packing fix-up and DHT nD
//                       combine (fft/DoubleFFT_2D.java:2544, dht/DoubleDHT_3D.java:2314).
//   transpose_kernel    batched tiled transpose for axis passes.
//   table kernels       FP64 twiddle/chirp generation with sincospi.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace jt {

template <typename T> struct V2;
template <> struct V2<float> { typedef float2 t; };
template <> struct V2<double> { typedef double2 t; };

template <typename T> __host__ __device__ __forceinline__ typename V2<T>::t mk(T x, T y) {
    typename V2<T>::t r;
    r.x = x;
    r.y = y;
    return r;
}

#define C2 typename V2<T>::t

template <typename T> __device__ __forceinline__ C2 cadd(C2 a, C2 b) { return mk<T>(a.x + b.x, a.y + b.y); }
template <typename T> __device__ __forceinline__ C2 csub(C2 a, C2 b) { return mk<T>(a.x - b.x, a.y - b.y); }
template <typename T> __device__ __forceinline__ C2 cmul(C2 a, C2 b) {
    return mk<T>(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// a * conj(b)
template <typename T> __device__ __forceinline__ C2 cmulc(C2 a, C2 b) {
    return mk<T>(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y);
}
template <typename T> __device__ __forceinline__ C2 cscale(C2 a, T s) { return mk<T>(a.x * s, a.y * s); }
template <typename T> __device__ __forceinline__ C2 cconj(C2 a) { return mk<T>(a.x, -a.y); }
// a * (SIGN * i)
template <int SIGN, typename T> __device__ __forceinline__ C2 mul_si(C2 a) {
    return SIGN > 0 ? mk<T>(-a.y, a.x) : mk<T>(a.y, -a.x);
}

// Padded shared-memory index: one spare slot every 16 elements keeps the
// strided butterfly writes free of bank conflicts for 8- and 16-byte elements.
__device__ __forceinline__ int pad(int i) { return i + (i >> 4); }
__host__ __device__ __forceinline__ int padded_len(int L) { return L + (L >> 4) + 1; }

// ---------------------------------------------------------------------------
// Small DFTs in registers.  SIGN = -1: sum v_m e^{-2 pi i km/R}; +1: e^{+}.
// ---------------------------------------------------------------------------
template <int SIGN, typename T> __device__ __forceinline__ void dft2(C2 *v) {
    C2 a = v[0], b = v[1];
    v[0] = cadd<T>(a, b);
    v[1] = csub<T>(a, b);
}

template <int SIGN, typename T> __device__ __forceinline__ void dft4(C2 &v0, C2 &v1, C2 &v2, C2 &v3) {
    C2 t0 = cadd<T>(v0, v2), t1 = csub<T>(v0, v2);
    C2 t2 = cadd<T>(v1, v3), t3 = mul_si<SIGN, T>(csub<T>(v1, v3));
    v0 = cadd<T>(t0, t2);
    v2 = csub<T>(t0, t2);
    v1 = cadd<T>(t1, t3);
    v3 = csub<T>(t1, t3);
}

template <int SIGN, typename T> __device__ __forceinline__ void dft4v(C2 *v) { dft4<SIGN, T>(v[0], v[1], v[2], v[3]); }

// multiply by e^{SIGN * 2 pi i k / 8}
template <int SIGN, int K, typename T> __device__ __forceinline__ C2 w8(C2 a) {
    const T h = (T)0.70710678118654752440084436210484903928;
    if (K == 0) return a;
    if (K == 2) return mul_si<SIGN, T>(a);
    if (K == 1) return SIGN > 0 ? mk<T>(h * (a.x - a.y), h * (a.x + a.y)) : mk<T>(h * (a.x + a.y), h * (a.y - a.x));
    // K == 3: e^{SIGN 3 pi i/4} = (-h, SIGN h)
    return SIGN > 0 ? mk<T>(-h * (a.x + a.y), h * (a.x - a.y)) : mk<T>(h * (a.y - a.x), -h * (a.x + a.y));
}

template <int SIGN, typename T> __device__ __forceinline__ void dft8(C2 *v) {
    C2 e0 = v[0], e1 = v[2], e2 = v[4], e3 = v[6];
    C2 o0 = v[1], o1 = v[3], o2 = v[5], o3 = v[7];
    dft4<SIGN, T>(e0, e1, e2, e3);
    dft4<SIGN, T>(o0, o1, o2, o3);
    o1 = w8<SIGN, 1, T>(o1);
    o2 = w8<SIGN, 2, T>(o2);
    o3 = w8<SIGN, 3, T>(o3);
    v[0] = cadd<T>(e0, o0); v[4] = csub<T>(e0, o0);
    v[1] = cadd<T>(e1, o1); v[5] = csub<T>(e1, o1);
    v[2] = cadd<T>(e2, o2); v[6] = csub<T>(e2, o2);
    v[3] = cadd<T>(e3, o3); v[7] = csub<T>(e3, o3);
}

// radix 16 as 4 x 4 with internal twiddles e^{SIGN 2 pi i jk/16}
template <int SIGN, typename T> __device__ __forceinline__ void dft16(C2 *v) {
    const T c1 = (T)0.92387953251128675612818318939678828682;  // cos(pi/8)
    const T h = (T)0.70710678118654752440084436210484903928;
    // columns: DFT4 over v[j], v[j+4], v[j+8], v[j+12]
#pragma unroll
    for (int j = 0; j < 4; j++) dft4<SIGN, T>(v[j], v[j + 4], v[j + 8], v[j + 12]);
    // element (k, j) at v[j + 4k] takes w^{jk}, w = e^{SIGN i pi/8}, then the
    // rows' DFT4 over j (output index k + 4 j')
    const T s = (T)SIGN;
    // Each row's twiddles are factored so that their products fold into the
    // row butterfly's additions as FMAs (w = c1 (1 + s i tau), w^3 = c1 (tau
    // + s i), w^2 = h (1 + s i), w^6 = h (-1 + s i), w^9 = -c1 (1 + s i tau)):
    // 144 floating-point instructions for the 16 points instead of 160.
    const T tau = (T)0.41421356237309504880168872420969807857;  // tan(pi/8)
    dft4<SIGN, T>(v[0], v[1], v[2], v[3]);
    // t0, t1 = x0 +- g u; t2, t3 = f P, f M: outputs t0 +- f P, t1 +- s i f M
    auto row = [&](int o, C2 t0, C2 t1, C2 P, C2 M, T f) {
        v[o] = mk<T>(fma(f, P.x, t0.x), fma(f, P.y, t0.y));
        v[o + 2] = mk<T>(fma(-f, P.x, t0.x), fma(-f, P.y, t0.y));
        v[o + 1] = mk<T>(fma(-s * f, M.y, t1.x), fma(s * f, M.x, t1.y));
        v[o + 3] = mk<T>(fma(s * f, M.y, t1.x), fma(-s * f, M.x, t1.y));
    };
    {  // k = 1: w^2 v6 = h u, w v5 = c1 p, w^3 v7 = c1 q
        const C2 x0 = v[4], a = v[5], b = v[6], d = v[7];
        const C2 u = mk<T>(b.x - s * b.y, b.y + s * b.x);
        const C2 t0 = mk<T>(fma(h, u.x, x0.x), fma(h, u.y, x0.y)), t1 = mk<T>(fma(-h, u.x, x0.x), fma(-h, u.y, x0.y));
        const C2 p = mk<T>(fma(-s * tau, a.y, a.x), fma(s * tau, a.x, a.y));
        const C2 q = mk<T>(fma(tau, d.x, -s * d.y), fma(tau, d.y, s * d.x));
        row(4, t0, t1, cadd<T>(p, q), csub<T>(p, q), c1);
    }
    {  // k = 2: w^4 v10 = s i v10, w^2 v9 = h A, w^6 v11 = h D
        const C2 x0 = v[8], a = v[9], b = v[10], d = v[11];
        const C2 t0 = mk<T>(x0.x - s * b.y, x0.y + s * b.x), t1 = mk<T>(x0.x + s * b.y, x0.y - s * b.x);
        const C2 A = mk<T>(a.x - s * a.y, a.y + s * a.x);
        const C2 D = mk<T>(-d.x - s * d.y, s * d.x - d.y);
        row(8, t0, t1, cadd<T>(A, D), csub<T>(A, D), h);
    }
    {  // k = 3: w^6 v14 = h u, w^3 v13 = c1 p, w^9 v15 = -c1 q
        const C2 x0 = v[12], a = v[13], b = v[14], d = v[15];
        const C2 u = mk<T>(-b.x - s * b.y, s * b.x - b.y);
        const C2 t0 = mk<T>(fma(h, u.x, x0.x), fma(h, u.y, x0.y)), t1 = mk<T>(fma(-h, u.x, x0.x), fma(-h, u.y, x0.y));
        const C2 p = mk<T>(fma(tau, a.x, -s * a.y), fma(tau, a.y, s * a.x));
        const C2 q = mk<T>(fma(-s * tau, d.y, d.x), fma(s * tau, d.x, d.y));
        row(12, t0, t1, csub<T>(p, q), cadd<T>(p, q), c1);
    }
    // transpose 4x4: out[k + 4 j'] = v[4k + j']
    C2 t[16];
#pragma unroll
    for (int i = 0; i < 16; i++) t[i] = v[i];
#pragma unroll
    for (int k = 0; k < 4; k++)
#pragma unroll
        for (int j = 0; j < 4; j++) v[k + 4 * j] = t[4 * k + j];
}

template <int SIGN, typename T> __device__ __forceinline__ void dft3(C2 *v) {
    const T c = (T)-0.5, sn = (T)SIGN * (T)0.86602540378443864676372317075293618347;
    C2 t = cadd<T>(v[1], v[2]);
    C2 d = csub<T>(v[1], v[2]);
    C2 m = mk<T>(v[0].x + c * t.x, v[0].y + c * t.y);
    C2 r = mk<T>(-sn * d.y, sn * d.x);  // i*sn*d
    v[0] = cadd<T>(v[0], t);
    v[1] = cadd<T>(m, r);
    v[2] = csub<T>(m, r);
}

template <int SIGN, typename T> __device__ __forceinline__ void dft5(C2 *v) {
    const T c1 = (T)0.30901699437494742410229341718281905886, c2 = (T)-0.80901699437494742410229341718281905886;
    const T s1 = (T)SIGN * (T)0.95105651629515357211643933337938214340, s2 = (T)SIGN * (T)0.58778525229247312916870595463907276860;
    C2 a1 = cadd<T>(v[1], v[4]), b1 = csub<T>(v[1], v[4]);
    C2 a2 = cadd<T>(v[2], v[3]), b2 = csub<T>(v[2], v[3]);
    C2 x0 = v[0];
    C2 m1 = mk<T>(x0.x + c1 * a1.x + c2 * a2.x, x0.y + c1 * a1.y + c2 * a2.y);
    C2 m2 = mk<T>(x0.x + c2 * a1.x + c1 * a2.x, x0.y + c2 * a1.y + c1 * a2.y);
    // i*(s1 b1 + s2 b2), i*(s2 b1 - s1 b2)
    C2 n1 = mk<T>(-(s1 * b1.y + s2 * b2.y), s1 * b1.x + s2 * b2.x);
    C2 n2 = mk<T>(-(s2 * b1.y - s1 * b2.y), s2 * b1.x - s1 * b2.x);
    v[0] = mk<T>(x0.x + a1.x + a2.x, x0.y + a1.y + a2.y);
    v[1] = cadd<T>(m1, n1);
    v[4] = csub<T>(m1, n1);
    v[2] = cadd<T>(m2, n2);
    v[3] = csub<T>(m2, n2);
}

template <int SIGN, typename T> __device__ __forceinline__ void dft7(C2 *v) {
    const T c1 = (T)0.62348980185873353052500488400423981063, c2 = (T)-0.22252093395631440428890256449679475947,
            c3 = (T)-0.90096886790241912623610231950744505117;
    const T s1 = (T)SIGN * (T)0.78183148246802980870844452667405775023, s2 = (T)SIGN * (T)0.97492791218182360701813168299393121723,
            s3 = (T)SIGN * (T)0.43388373911755812047576833284835875461;
    C2 a1 = cadd<T>(v[1], v[6]), b1 = csub<T>(v[1], v[6]);
    C2 a2 = cadd<T>(v[2], v[5]), b2 = csub<T>(v[2], v[5]);
    C2 a3 = cadd<T>(v[3], v[4]), b3 = csub<T>(v[3], v[4]);
    C2 x0 = v[0];
    // k=1: c1 c2 c3 / s1 s2 s3; k=2: c2 c3 c1 / s2 -s3 -s1; k=3: c3 c1 c2 / s3 -s1 s2
    C2 m1 = mk<T>(x0.x + c1 * a1.x + c2 * a2.x + c3 * a3.x, x0.y + c1 * a1.y + c2 * a2.y + c3 * a3.y);
    C2 m2 = mk<T>(x0.x + c2 * a1.x + c3 * a2.x + c1 * a3.x, x0.y + c2 * a1.y + c3 * a2.y + c1 * a3.y);
    C2 m3 = mk<T>(x0.x + c3 * a1.x + c1 * a2.x + c2 * a3.x, x0.y + c3 * a1.y + c1 * a2.y + c2 * a3.y);
    T p1r = s1 * b1.x + s2 * b2.x + s3 * b3.x, p1i = s1 * b1.y + s2 * b2.y + s3 * b3.y;
    T p2r = s2 * b1.x - s3 * b2.x - s1 * b3.x, p2i = s2 * b1.y - s3 * b2.y - s1 * b3.y;
    T p3r = s3 * b1.x - s1 * b2.x + s2 * b3.x, p3i = s3 * b1.y - s1 * b2.y + s2 * b3.y;
    v[0] = mk<T>(x0.x + a1.x + a2.x + a3.x, x0.y + a1.y + a2.y + a3.y);
    v[1] = mk<T>(m1.x - p1i, m1.y + p1r);
    v[6] = mk<T>(m1.x + p1i, m1.y - p1r);
    v[2] = mk<T>(m2.x - p2i, m2.y + p2r);
    v[5] = mk<T>(m2.x + p2i, m2.y - p2r);
    v[3] = mk<T>(m3.x - p3i, m3.y + p3r);
    v[4] = mk<T>(m3.x + p3i, m3.y - p3r);
}

// ---------------------------------------------------------------------------
// fft_tile_kernel
// ---------------------------------------------------------------------------
#define JT_MAX_PASSES 24
#define JT_MAX_GENERIC_RADIX 64

// Where the elements of line b live: element i of line b is at
//   (b / inner) * outer + (b % inner) * istride + i * estride
// (complex-element units).
struct Layout {
    int64_t inner, outer, istride, estride;
};

struct TileParams {
    int L;            // line length
    int npass;
    int radix[JT_MAX_PASSES];
    int C;            // lines per tile
    int64_t nlines;
    Layout lin, lout;
    double scale;     // output multiplier (1 = none), double plans
    float scalef;     // the same for float plans (no FP64 work in float kernels)
    int do_scale;
    int64_t tw_n;     // four-step post twiddle w_{tw_n}^{sign*k*(b % tw_inner)}; 0 = none
    int64_t tw_inner;
    int tw_lo_bits;
};

// b / d and b % d for the non-negative line indices of the kernels: shift and
// mask for a power-of-two d (every power-of-two plan's layouts), 32-bit
// division when both fit, 64-bit otherwise.
__device__ __forceinline__ int64_t div_fast(int64_t b, int64_t d, int64_t *rem) {
    if ((d & (d - 1)) == 0) {
        *rem = b & (d - 1);
        return b >> (__ffsll(d) - 1);
    }
    if (b <= 0x7fffffff && d <= 0x7fffffff) {
        const uint32_t q = (uint32_t)b / (uint32_t)d;
        *rem = b - (int64_t)q * d;
        return q;
    }
    const int64_t q = b / d;
    *rem = b - q * d;
    return q;
}

__device__ __forceinline__ int64_t line_off(const Layout &l, int64_t b) {
    if (l.inner == 1) return b * l.outer;
    int64_t r;
    const int64_t q = div_fast(b, l.inner, &r);
    return q * l.outer + r * l.istride;
}

// One Stockham pass of radix R for every butterfly of the tile.
template <int R, int SIGN, typename T>
__device__ __forceinline__ void pass_r(const C2 *__restrict__ src, C2 *__restrict__ dst, int lines, int L, int Lp, int Ns,
                                       const C2 *__restrict__ W) {
    const int nb = L / R;
    const int total = lines * nb;
    const int step = L / (Ns * R);
    for (int q = threadIdx.x; q < total; q += blockDim.x) {
        int c = q / nb;
        int j = q - c * nb;
        const C2 *s = src + c * Lp;
        C2 v[R];
#pragma unroll
        for (int k = 0; k < R; k++) v[k] = s[pad(j + k * nb)];
        int jm = j % Ns;
        if (jm) {
#pragma unroll
            for (int k = 1; k < R; k++) {
                C2 w = __ldg(&W[jm * k * step]);
                v[k] = SIGN < 0 ? cmul<T>(v[k], w) : cmulc<T>(v[k], w);
            }
        }
        if (R == 2) dft2<SIGN, T>(v);
        else if (R == 3) dft3<SIGN, T>(v);
        else if (R == 4) dft4v<SIGN, T>(v);
        else if (R == 5) dft5<SIGN, T>(v);
        else if (R == 7) dft7<SIGN, T>(v);
        else if (R == 8) dft8<SIGN, T>(v);
        else if (R == 16) dft16<SIGN, T>(v);
        int idxD = (j - jm) * R + jm;
        C2 *d = dst + c * Lp;
#pragma unroll
        for (int k = 0; k < R; k++) d[pad(idxD + k * Ns)] = v[k];
    }
}

// Generic odd radix (11..63) with the line's own roots of unity: W[m * L/R].
template <int SIGN, typename T>
__device__ void pass_generic(const C2 *__restrict__ src, C2 *__restrict__ dst, int lines, int L, int Lp, int Ns, int R,
                             const C2 *__restrict__ W) {
    const int nb = L / R;
    const int total = lines * nb;
    const int step = L / (Ns * R);
    const int rstep = L / R;
    if (total < (int)blockDim.x) {
        // fewer butterflies than threads (a prime line is one butterfly): one
        // thread per output k of a butterfly, each forming its own sum in
        // the same order as below
        const int items = total * R;
        for (int idx = threadIdx.x; idx < items; idx += blockDim.x) {
            const int q = idx / R, k = idx - q * R;
            const int c = q / nb, j = q - c * nb;
            const C2 *s = src + c * Lp;
            const int jm = j % Ns;
            T sr = 0, si = 0;
            int e = 0;  // k m mod R
            for (int m = 0; m < R; m++) {
                C2 x = s[pad(j + m * nb)];
                if (jm && m) {
                    const C2 w = __ldg(&W[jm * m * step]);
                    x = SIGN < 0 ? cmul<T>(x, w) : cmulc<T>(x, w);
                }
                if (m == 0) {
                    sr = x.x;
                    si = x.y;
                } else {
                    C2 w = __ldg(&W[e * rstep]);
                    if (SIGN > 0) w.y = -w.y;
                    sr += x.x * w.x - x.y * w.y;
                    si += x.x * w.y + x.y * w.x;
                }
                e += k;
                if (e >= R) e -= R;
            }
            dst[c * Lp + pad((j - jm) * R + jm + k * Ns)] = mk<T>(sr, si);
        }
        return;
    }
    for (int q = threadIdx.x; q < total; q += blockDim.x) {
        int c = q / nb;
        int j = q - c * nb;
        const C2 *s = src + c * Lp;
        C2 v[JT_MAX_GENERIC_RADIX];
        int jm = j % Ns;
        for (int k = 0; k < R; k++) {
            C2 x = s[pad(j + k * nb)];
            if (jm && k) {
                C2 w = __ldg(&W[jm * k * step]);
                x = SIGN < 0 ? cmul<T>(x, w) : cmulc<T>(x, w);
            }
            v[k] = x;
        }
        int idxD = (j - jm) * R + jm;
        C2 *d = dst + c * Lp;
        for (int k = 0; k < R; k++) {
            T sr = v[0].x, si = v[0].y;
            int e = 0;
            for (int m = 1; m < R; m++) {
                e += k;
                if (e >= R) e -= R;
                C2 w = __ldg(&W[e * rstep]);
                if (SIGN > 0) w.y = -w.y;
                sr += v[m].x * w.x - v[m].y * w.y;
                si += v[m].x * w.y + v[m].y * w.x;
            }
            d[pad(idxD + k * Ns)] = mk<T>(sr, si);
        }
    }
}

// The Stockham passes of a tile: `lines` lines of length L at stride Lp in
// `src`, ping-ponging with `dst`; returns the buffer holding the result.
template <int SIGN, typename T>
__device__ C2 *tile_passes(C2 *src, C2 *dst, int lines, int L, int Lp, int npass, const int *radix, const C2 *__restrict__ W) {
    int Ns = 1;
    for (int ps = 0; ps < npass; ps++) {
        const int R = radix[ps];
        switch (R) {
            case 2: pass_r<2, SIGN, T>(src, dst, lines, L, Lp, Ns, W); break;
            case 3: pass_r<3, SIGN, T>(src, dst, lines, L, Lp, Ns, W); break;
            case 4: pass_r<4, SIGN, T>(src, dst, lines, L, Lp, Ns, W); break;
            case 5: pass_r<5, SIGN, T>(src, dst, lines, L, Lp, Ns, W); break;
            case 7: pass_r<7, SIGN, T>(src, dst, lines, L, Lp, Ns, W); break;
            case 8: pass_r<8, SIGN, T>(src, dst, lines, L, Lp, Ns, W); break;
            case 16: pass_r<16, SIGN, T>(src, dst, lines, L, Lp, Ns, W); break;
            default: pass_generic<SIGN, T>(src, dst, lines, L, Lp, Ns, R, W); break;
        }
        __syncthreads();
        C2 *t = src;
        src = dst;
        dst = t;
        Ns *= R;
    }
    return src;
}

// W: e^{-2 pi i t/L}, t < L.  Whi/Wlo: two-level table of the four-step post
// twiddle, e^{-2 pi i t/tw_n} = Whi[t >> lo_bits] * Wlo[t & mask].
// Tile `blk` of a generic line pass, run by the calling CTA with its shared
// memory at `smem_raw` (2 * C * padded L elements).
template <int SIGN, typename T>
__device__ void tile_fft_body(const C2 *in, C2 *out, const TileParams &p, const C2 *__restrict__ W, const C2 *__restrict__ Whi,
                              const C2 *__restrict__ Wlo, int64_t blk, unsigned char *smem_raw) {
    const int L = p.L, Lp = padded_len(L);
    C2 *bufA = reinterpret_cast<C2 *>(smem_raw);
    C2 *bufB = bufA + p.C * Lp;
    const int64_t b0 = blk * p.C;
    const int lines = (int)min((int64_t)p.C, p.nlines - b0);
    if (lines <= 0) return;
    const int tot = lines * L;

    // load: contiguous lines read element-fastest; strided lines read
    // line-fastest so neighbouring threads touch neighbouring columns.
    if (p.lin.estride == 1) {
        for (int idx = threadIdx.x; idx < tot; idx += blockDim.x) {
            int c = idx / L, i = idx - c * L;
            bufA[c * Lp + pad(i)] = in[line_off(p.lin, b0 + c) + i];
        }
    } else {
        for (int idx = threadIdx.x; idx < tot; idx += blockDim.x) {
            int i = idx / lines, c = idx - i * lines;
            bufA[c * Lp + pad(i)] = in[line_off(p.lin, b0 + c) + (int64_t)i * p.lin.estride];
        }
    }
    __syncthreads();

    const C2 *src = tile_passes<SIGN, T>(bufA, bufB, lines, L, Lp, p.npass, p.radix, W);

    T sc;
    if constexpr (sizeof(T) == 4) sc = p.scalef;
    else sc = (T)p.scale;
    const bool do_scale = p.do_scale != 0;
    const int64_t lo_mask = ((int64_t)1 << p.tw_lo_bits) - 1;
    if (p.lout.estride == 1) {
        for (int idx = threadIdx.x; idx < tot; idx += blockDim.x) {
            int c = idx / L, i = idx - c * L;
            C2 v = src[c * Lp + pad(i)];
            if (p.tw_n) {
                int64_t t = ((int64_t)i * ((b0 + c) % p.tw_inner)) % p.tw_n;
                C2 w = cmul<T>(__ldg(&Whi[t >> p.tw_lo_bits]), __ldg(&Wlo[t & lo_mask]));
                v = SIGN < 0 ? cmul<T>(v, w) : cmulc<T>(v, w);
            }
            if (do_scale) v = cscale<T>(v, sc);
            out[line_off(p.lout, b0 + c) + i] = v;
        }
    } else {
        for (int idx = threadIdx.x; idx < tot; idx += blockDim.x) {
            int i = idx / lines, c = idx - i * lines;
            C2 v = src[c * Lp + pad(i)];
            if (p.tw_n) {
                int64_t t = ((int64_t)i * ((b0 + c) % p.tw_inner)) % p.tw_n;
                C2 w = cmul<T>(__ldg(&Whi[t >> p.tw_lo_bits]), __ldg(&Wlo[t & lo_mask]));
                v = SIGN < 0 ? cmul<T>(v, w) : cmulc<T>(v, w);
            }
            if (do_scale) v = cscale<T>(v, sc);
            out[line_off(p.lout, b0 + c) + (int64_t)i * p.lout.estride] = v;
        }
    }
}

template <int SIGN, typename T>
__global__ void __launch_bounds__(512) fft_tile_kernel(const C2 *in, C2 *out, TileParams p, const C2 *__restrict__ W,
                                                        const C2 *__restrict__ Whi, const C2 *__restrict__ Wlo) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    tile_fft_body<SIGN, T>(in, out, p, W, Whi, Wlo, (int64_t)blockIdx.x, smem_raw);
}

// ---------------------------------------------------------------------------
// Table generation (FP64, sincospi), rounded to T.
// ---------------------------------------------------------------------------
// out[t] = e^{-2 pi i t * num / den} for t < count
template <typename T> __global__ void roots_kernel(C2 *out, int64_t count, int64_t num, int64_t den) {
    int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= count) return;
    // reduce t*num mod den exactly in integers, then angle = 2 * r / den (in half turns)
    int64_t r = (t * num) % den;
    double s, c;
    sincospi(-2.0 * (double)r / (double)den, &s, &c);
    out[t] = mk<T>((T)c, (T)s);
}

// Bluestein chirp bk1[i] = e^{i pi (i^2 mod 2n) / n} (fft/DoubleFFT_1D.java:1864-1879)
template <typename T> __global__ void chirp_kernel(C2 *bk1, double2 *b64, int64_t n, int64_t nB) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= nB) return;
    // symmetric, 1/nB-scaled chirp in FP64 for bk2 (fft/DoubleFFT_1D.java:1880-1889)
    double2 v = make_double2(0.0, 0.0);
    int64_t src = -1;
    if (i < n) src = i;
    else if (nB - i < n) src = nB - i;
    if (src >= 0) {
        int64_t k = (src * src) % (2 * n);
        double s, c;
        sincospi((double)k / (double)n, &s, &c);
        if (i < n) bk1[i] = mk<T>((T)c, (T)s);
        v = make_double2(c / (double)nB, s / (double)nB);
    }
    b64[i] = v;
}

template <typename T> __global__ void d2t_kernel(C2 *out, const double2 *in, int64_t count) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < count) out[i] = mk<T>((T)in[i].x, (T)in[i].y);
}

// ---------------------------------------------------------------------------
// Bluestein multiplies.  SIGN=-1 forward.
// ---------------------------------------------------------------------------
// tmp[b][i] = a[b][i] * conj(bk1[i]) (forward) or * bk1[i] (inverse), zero padded to nB.
template <int SIGN, typename T>
__device__ __forceinline__ void bluestein_pre_body(const C2 *a, int64_t dist, C2 *tmp, const C2 *__restrict__ bk1, int64_t n, int64_t nB,
                                     int64_t batch, int64_t idx) {
    if (idx >= batch * nB) return;
    int64_t b = idx / nB, i = idx - b * nB;
    C2 v = mk<T>(0, 0);
    if (i < n) {
        C2 x = a[b * dist + i], w = __ldg(&bk1[i]);
        v = SIGN < 0 ? cmulc<T>(x, w) : cmul<T>(x, w);
    }
    tmp[idx] = v;
}

template <int SIGN, typename T>
__global__ void bluestein_pre_kernel(const C2 *a, int64_t dist, C2 *tmp, const C2 *__restrict__ bk1, int64_t n, int64_t nB,
                                     int64_t batch) {
    bluestein_pre_body<SIGN, T>(a, dist, tmp, bk1, n, nB, batch, blockIdx.x * (int64_t)blockDim.x + threadIdx.x);
}

template <int SIGN, typename T>
__device__ __forceinline__ void bluestein_mul_body(C2 *tmp, const C2 *__restrict__ bk2, int64_t nB, int64_t total, int64_t idx) {
    if (idx >= total) return;
    C2 w = __ldg(&bk2[idx % nB]);
    tmp[idx] = SIGN < 0 ? cmul<T>(tmp[idx], w) : cmulc<T>(tmp[idx], w);
}

template <int SIGN, typename T>
__global__ void bluestein_mul_kernel(C2 *tmp, const C2 *__restrict__ bk2, int64_t nB, int64_t total) {
    bluestein_mul_body<SIGN, T>(tmp, bk2, nB, total, blockIdx.x * (int64_t)blockDim.x + threadIdx.x);
}

template <int SIGN, typename T>
__device__ __forceinline__ void bluestein_post_body(C2 *a, int64_t dist, const C2 *tmp, const C2 *__restrict__ bk1, int64_t n, int64_t nB,
                                      int64_t batch, T scale, int64_t idx) {
    if (idx >= batch * n) return;
    int64_t b = idx / n, i = idx - b * n;
    C2 x = tmp[b * nB + i], w = __ldg(&bk1[i]);
    C2 v = SIGN < 0 ? cmulc<T>(x, w) : cmul<T>(x, w);
    if (scale != (T)1) v = cscale<T>(v, scale);
    a[b * dist + i] = v;
}

template <int SIGN, typename T>
__global__ void bluestein_post_kernel(C2 *a, int64_t dist, const C2 *tmp, const C2 *__restrict__ bk1, int64_t n, int64_t nB,
                                      int64_t batch, T scale) {
    bluestein_post_body<SIGN, T>(a, dist, tmp, bk1, n, nB, batch, scale, blockIdx.x * (int64_t)blockDim.x + threadIdx.x);
}

// ---------------------------------------------------------------------------
// Real FFT pack / unpack (even n, h = n/2 complex points).
// Wr[k] = e^{-2 pi i k / n}, k <= n/4.
// ---------------------------------------------------------------------------
// X_k from Z (the h-point FFT of z_j = x_2j + i x_2j+1):
//   X_k = 0.5 (Z_k + conj Z_{h-k}) - 0.5 i w (Z_k - conj Z_{h-k})
// with w = e^{-2 pi i k/n} for the forward transform.  The same formula with
// w = e^{+2 pi i k/n} turns the e^{+} h-point FFT into the e^{+} n-point real
// transform (realInverseFull); only the twiddle changes.
template <typename T>
__device__ __forceinline__ void real_split(C2 zk, C2 zh, C2 w, C2 &xk) {
    C2 a = mk<T>((T)0.5 * (zk.x + zh.x), (T)0.5 * (zk.y - zh.y));
    C2 d = mk<T>((T)0.5 * (zk.x - zh.x), (T)0.5 * (zk.y + zh.y));
    C2 wd = cmul<T>(w, d);
    xk = mk<T>(a.x + wd.y, a.y - wd.x);  // a - i * wd
}

// In place: a holds Z (h complex); writes the packed realForward layout.
template <typename T>
__device__ __forceinline__ void real_post_packed_body(T *a, int64_t dist, int64_t n, int64_t batch, const C2 *__restrict__ Wr, int64_t idx) {
    const int64_t h = n / 2, q = h / 2 + 1;  // pairs k = 0..h/2
    if (idx >= batch * q) return;
    int64_t b = idx / q, k = idx - b * q;
    C2 *z = reinterpret_cast<C2 *>(a + b * dist);
    if (k == 0) {
        C2 z0 = z[0];
        z[0] = mk<T>(z0.x + z0.y, z0.x - z0.y);  // a[0] = X0, a[1] = X_{n/2}
        return;
    }
    int64_t k2 = h - k;
    C2 zk = z[k], zh = z[k2];
    C2 w = __ldg(&Wr[k]);
    C2 xk, xh;
    real_split<T>(zk, zh, w, xk);
    if (k2 != k) {
        // w_{h-k} = -conj(w_k)
        real_split<T>(zh, zk, mk<T>(-w.x, w.y), xh);
        z[k2] = xh;
    }
    z[k] = xk;
}

template <typename T>
__global__ void real_post_packed_kernel(T *a, int64_t dist, int64_t n, int64_t batch, const C2 *__restrict__ Wr) {
    real_post_packed_body<T>(a, dist, n, batch, Wr, blockIdx.x * (int64_t)blockDim.x + threadIdx.x);
}

// Out of place: z (h complex) -> full spectrum F (n complex) in out.
// SIGN=+1 writes the e^{+} transform (z must be the e^{+} FFT), times scale.
template <int SIGN, typename T>
__device__ __forceinline__ void real_post_full_body(const T *zin, int64_t zdist, T *out, int64_t odist, int64_t n, int64_t batch,
                                      const C2 *__restrict__ Wr, T scale, int64_t idx) {
    const int64_t h = n / 2, q = h / 2 + 1;
    if (idx >= batch * q) return;
    int64_t b = idx / q, k = idx - b * q;
    const C2 *z = reinterpret_cast<const C2 *>(zin + b * zdist);
    C2 *F = reinterpret_cast<C2 *>(out + b * odist);
    const T s = scale;
    if (k == 0) {
        C2 z0 = z[0];
        F[0] = mk<T>((z0.x + z0.y) * s, 0);
        F[h] = mk<T>((z0.x - z0.y) * s, 0);
        return;
    }
    int64_t k2 = h - k;
    C2 zk = z[k], zh = z[k2];
    C2 w = __ldg(&Wr[k]);
    if (SIGN > 0) w.y = -w.y;
    C2 xk, xh;
    real_split<T>(zk, zh, w, xk);
    xk = cscale<T>(xk, s);
    F[k] = xk;
    F[n - k] = cconj<T>(xk);
    if (k2 != k) {
        real_split<T>(zh, zk, mk<T>(-w.x, w.y), xh);
        xh = cscale<T>(xh, s);
        F[k2] = xh;
        F[n - k2] = cconj<T>(xh);
    }
}

template <int SIGN, typename T>
__global__ void real_post_full_kernel(const T *zin, int64_t zdist, T *out, int64_t odist, int64_t n, int64_t batch,
                                      const C2 *__restrict__ Wr, T scale) {
    real_post_full_body<SIGN, T>(zin, zdist, out, odist, n, batch, Wr, scale, blockIdx.x * (int64_t)blockDim.x + threadIdx.x);
}

// In place: packed spectrum -> Z (h complex) whose e^{+} h-point FFT is
// (n/2) * x interleaved; everything times `mult`.
template <typename T>
__device__ __forceinline__ void real_pre_inverse_body(T *a, int64_t dist, int64_t n, int64_t batch, const C2 *__restrict__ Wr, T mult, int64_t idx) {
    const int64_t h = n / 2, q = h / 2 + 1;
    if (idx >= batch * q) return;
    int64_t b = idx / q, k = idx - b * q;
    C2 *z = reinterpret_cast<C2 *>(a + b * dist);
    const T m = mult;
    if (k == 0) {
        C2 x = z[0];  // (X0, X_{n/2})
        z[0] = mk<T>((T)0.5 * (x.x + x.y) * m, (T)0.5 * (x.x - x.y) * m);
        return;
    }
    int64_t k2 = h - k;
    C2 xk = z[k], xh = z[k2];
    C2 w = __ldg(&Wr[k]);
    w.y = -w.y;  // e^{+2 pi i k/n}
    // Z_k = 0.5 (Xk + conj Xh) + 0.5 i w (Xk - conj Xh)
    auto mkz = [&](C2 p, C2 r, C2 ww) {
        C2 sa = mk<T>((T)0.5 * (p.x + r.x), (T)0.5 * (p.y - r.y));
        C2 d = mk<T>((T)0.5 * (p.x - r.x), (T)0.5 * (p.y + r.y));
        C2 wd = cmul<T>(ww, d);
        return mk<T>((sa.x - wd.y) * m, (sa.y + wd.x) * m);
    };
    C2 zk = mkz(xk, xh, w);
    if (k2 != k) {
        // e^{+2 pi i (h-k)/n} = -conj(w)
        C2 zh = mkz(xh, xk, mk<T>(-w.x, w.y));
        z[k2] = zh;
    }
    z[k] = zk;
}

template <typename T>
__global__ void real_pre_inverse_kernel(T *a, int64_t dist, int64_t n, int64_t batch, const C2 *__restrict__ Wr, T mult) {
    real_pre_inverse_body<T>(a, dist, n, batch, Wr, mult, blockIdx.x * (int64_t)blockDim.x + threadIdx.x);
}

// Odd-n (and general) helpers working through a full complex buffer.
// tmp[b][i] = (a[b][i], 0)
template <typename T>
__device__ __forceinline__ void real_to_complex_body(const T *a, int64_t dist, C2 *tmp, int64_t n, int64_t batch, int64_t idx) {
    if (idx >= batch * n) return;
    int64_t b = idx / n, i = idx - b * n;
    tmp[idx] = mk<T>(a[b * dist + i], (T)0);
}

template <typename T>
__global__ void real_to_complex_kernel(const T *a, int64_t dist, C2 *tmp, int64_t n, int64_t batch) {
    real_to_complex_body<T>(a, dist, tmp, n, batch, blockIdx.x * (int64_t)blockDim.x + threadIdx.x);
}

// full spectrum F (n complex) -> packed realForward layout (fft/DoubleFFT_1D.java:433-451)
template <typename T>
__device__ __forceinline__ void pack_from_full_body(const C2 *F, T *a, int64_t dist, int64_t n, int64_t batch, int64_t idx) {
    if (idx >= batch * n) return;
    int64_t b = idx / n, i = idx - b * n;
    const C2 *f = F + b * n;
    T v;
    if (i == 0) v = f[0].x;
    else if (i == 1) v = (n % 2 == 0) ? f[n / 2].x : f[(n - 1) / 2].y;
    else {
        int64_t k = i / 2;
        v = (i & 1) ? f[k].y : f[k].x;
    }
    a[b * dist + i] = v;
}

template <typename T>
__global__ void pack_from_full_kernel(const C2 *F, T *a, int64_t dist, int64_t n, int64_t batch) {
    pack_from_full_body<T>(F, a, dist, n, batch, blockIdx.x * (int64_t)blockDim.x + threadIdx.x);
}

// packed -> full Hermitian spectrum
template <typename T>
__device__ __forceinline__ void unpack_to_full_body(const T *a, int64_t dist, C2 *F, int64_t n, int64_t batch, int64_t idx) {
    if (idx >= batch * n) return;
    int64_t b = idx / n, k = idx - b * n;
    const T *p = a + b * dist;
    C2 v;
    int64_t kk = k <= n / 2 ? k : n - k;
    if (kk == 0) v = mk<T>(p[0], 0);
    else if (n % 2 == 0 && kk == n / 2) v = mk<T>(p[1], 0);
    else if (n % 2 == 1 && kk == (n - 1) / 2) v = mk<T>(p[2 * kk], p[1]);
    else v = mk<T>(p[2 * kk], p[2 * kk + 1]);
    if (k != kk) v.y = -v.y;
    F[idx] = v;
}

template <typename T>
__global__ void unpack_to_full_kernel(const T *a, int64_t dist, C2 *F, int64_t n, int64_t batch) {
    unpack_to_full_body<T>(a, dist, F, n, batch, blockIdx.x * (int64_t)blockDim.x + threadIdx.x);
}

// a[b][i] = Re(F[b][i]) * mult
template <typename T>
__device__ __forceinline__ void real_part_body(const C2 *F, T *a, int64_t dist, int64_t n, int64_t batch, T mult, int64_t idx) {
    if (idx >= batch * n) return;
    int64_t b = idx / n, i = idx - b * n;
    a[b * dist + i] = F[idx].x * mult;
}

template <typename T>
__global__ void real_part_kernel(const C2 *F, T *a, int64_t dist, int64_t n, int64_t batch, T mult) {
    real_part_body<T>(F, a, dist, n, batch, mult, blockIdx.x * (int64_t)blockDim.x + threadIdx.x);
}

// Copies batch*len complex (strided) with an optional scale and conjugation.
template <typename T>
__device__ __forceinline__ void copy_complex_body(const C2 *src, int64_t sdist, C2 *dst, int64_t ddist, int64_t len, int64_t batch,
                                    T scale, int conj, int64_t idx) {
    if (idx >= batch * len) return;
    int64_t b = idx / len, i = idx - b * len;
    C2 v = src[b * sdist + i];
    if (conj) v.y = -v.y;
    if (scale != (T)1) v = cscale<T>(v, scale);
    dst[b * ddist + i] = v;
}

template <typename T>
__global__ void copy_complex_kernel(const C2 *src, int64_t sdist, C2 *dst, int64_t ddist, int64_t len, int64_t batch,
                                    T scale, int conj) {
    copy_complex_body<T>(src, sdist, dst, ddist, len, batch, scale, conj, blockIdx.x * (int64_t)blockDim.x + threadIdx.x);
}

// ---------------------------------------------------------------------------
// DCT-II / DCT-III / DST / DHT passes around a real FFT of length n.
// Wd[k] = e^{-i pi k / (2n)}, k < n.
// ---------------------------------------------------------------------------
// v_j = x_2j, v_{n-1-j} = x_2j+1 (DST: odd inputs negated)
template <typename T>
__device__ __forceinline__ void dct2_pre_body(const T *a, int64_t dist, T *v, int64_t vdist, int64_t n, int64_t batch, int dst, int64_t idx) {
    if (idx >= batch * n) return;
    int64_t b = idx / n, i = idx - b * n;
    T x = a[b * dist + i];
    int64_t j = (i & 1) ? n - 1 - (i >> 1) : (i >> 1);
    if (dst && (i & 1)) x = -x;
    v[b * vdist + j] = x;
}

template <typename T>
__global__ void dct2_pre_kernel(const T *a, int64_t dist, T *v, int64_t vdist, int64_t n, int64_t batch, int dst) {
    dct2_pre_body<T>(a, dist, v, vdist, n, batch, dst, blockIdx.x * (int64_t)blockDim.x + threadIdx.x);
}

// reads V_k (k <= n/2 packed, conj-mirrored above)
template <typename T> __device__ __forceinline__ C2 packed_get(const T *p, int64_t n, int64_t k) {
    int64_t kk = k <= n / 2 ? k : n - k;
    C2 v;
    if (kk == 0) v = mk<T>(p[0], 0);
    else if (n % 2 == 0 && kk == n / 2) v = mk<T>(p[1], 0);
    else if (n % 2 == 1 && kk == (n - 1) / 2) v = mk<T>(p[2 * kk], p[1]);
    else v = mk<T>(p[2 * kk], p[2 * kk + 1]);
    if (k != kk) v.y = -v.y;
    return v;
}

// C_k = Re(e^{-i pi k/2n} V_k) * mult (k=0: * mult0); DST writes C_k to n-1-k.
template <typename T>
__device__ __forceinline__ void dct2_post_body(const T *v, int64_t vdist, T *a, int64_t dist, int64_t n, int64_t batch,
                                 const C2 *__restrict__ Wd, T mult, T mult0, int dst, int64_t idx) {
    if (idx >= batch * n) return;
    int64_t b = idx / n, k = idx - b * n;
    C2 V = packed_get<T>(v + b * vdist, n, k);
    C2 w = __ldg(&Wd[k]);
    T c = (w.x * V.x - w.y * V.y) * (k == 0 ? mult0 : mult);
    a[b * dist + (dst ? n - 1 - k : k)] = c;
}

template <typename T>
__global__ void dct2_post_kernel(const T *v, int64_t vdist, T *a, int64_t dist, int64_t n, int64_t batch,
                                 const C2 *__restrict__ Wd, T mult, T mult0, int dst) {
    dct2_post_body<T>(v, vdist, a, dist, n, batch, Wd, mult, mult0, dst, blockIdx.x * (int64_t)blockDim.x + threadIdx.x);
}

// DCT-III: from coefficients b_k (DST: read reversed) build the packed
// spectrum of V_k = e^{i pi k/2n} (C_k - i C_{n-k}), C_k = g_k * b_k with
// g_0 = mult0, g_k = mult.  Thread k <= n/2 writes V_k.
template <typename T>
__device__ __forceinline__ void dct3_pre_body(const T *a, int64_t dist, T *v, int64_t vdist, int64_t n, int64_t batch,
                                const C2 *__restrict__ Wd, T mult, T mult0, int dst, int64_t idx) {
    const int64_t q = n / 2 + 1;
    if (idx >= batch * q) return;
    int64_t b = idx / q, k = idx - b * q;
    const T *p = a + b * dist;
    T *o = v + b * vdist;
    auto coef = [&](int64_t kk) -> T {
        if (kk >= n) return (T)0;
        T x = p[dst ? n - 1 - kk : kk];
        return x * (T)(kk == 0 ? mult0 : mult);
    };
    T ck = coef(k), cnk = k == 0 ? (T)0 : coef(n - k);
    C2 w = __ldg(&Wd[k]);
    w.y = -w.y;  // e^{+i pi k/2n}
    C2 V = cmul<T>(w, mk<T>(ck, -cnk));
    if (k == 0) o[0] = V.x;
    else if (n % 2 == 0 && k == n / 2) o[1] = V.x;
    else if (n % 2 == 1 && k == (n - 1) / 2) { o[2 * k] = V.x; o[1] = V.y; }
    else { o[2 * k] = V.x; o[2 * k + 1] = V.y; }
}

template <typename T>
__global__ void dct3_pre_kernel(const T *a, int64_t dist, T *v, int64_t vdist, int64_t n, int64_t batch,
                                const C2 *__restrict__ Wd, T mult, T mult0, int dst) {
    dct3_pre_body<T>(a, dist, v, vdist, n, batch, Wd, mult, mult0, dst, blockIdx.x * (int64_t)blockDim.x + threadIdx.x);
}

// x_2j = v_j, x_2j+1 = v_{n-1-j}; DST negates the odd outputs.
template <typename T>
__device__ __forceinline__ void dct3_post_body(const T *v, int64_t vdist, T *a, int64_t dist, int64_t n, int64_t batch, int dst, int64_t idx) {
    if (idx >= batch * n) return;
    int64_t b = idx / n, i = idx - b * n;
    int64_t j = (i & 1) ? n - 1 - (i >> 1) : (i >> 1);
    T x = v[b * vdist + j];
    if (dst && (i & 1)) x = -x;
    a[b * dist + i] = x;
}

template <typename T>
__global__ void dct3_post_kernel(const T *v, int64_t vdist, T *a, int64_t dist, int64_t n, int64_t batch, int dst) {
    dct3_post_body<T>(v, vdist, a, dist, n, batch, dst, blockIdx.x * (int64_t)blockDim.x + threadIdx.x);
}

// H_k = Re X_k - Im X_k from the packed spectrum (dht/DoubleDHT_1D.java:94-159)
template <typename T>
__device__ __forceinline__ void dht_post_body(const T *v, int64_t vdist, T *a, int64_t dist, int64_t n, int64_t batch, T mult, int64_t idx) {
    if (idx >= batch * n) return;
    int64_t b = idx / n, k = idx - b * n;
    C2 X = packed_get<T>(v + b * vdist, n, k);
    a[b * dist + k] = (X.x - X.y) * mult;
}

template <typename T>
__global__ void dht_post_kernel(const T *v, int64_t vdist, T *a, int64_t dist, int64_t n, int64_t batch, T mult) {
    dht_post_body<T>(v, vdist, a, dist, n, batch, mult, blockIdx.x * (int64_t)blockDim.x + threadIdx.x);
}

// ---------------------------------------------------------------------------
// 2D / 3D helpers
// ---------------------------------------------------------------------------
// rdft2d_sub (fft/DoubleFFT_2D.java:2544-2575): isgn=+1 after the column
// pass of realForward, -1 before the column pass of realInverse.
template <typename T>
__global__ void rdft2d_kernel(T *a, int64_t dist, int64_t rows, int64_t cols, int64_t batch, int isgn) {
    const int64_t n1h = rows >> 1;
    const int64_t q = n1h > 1 ? n1h - 1 : 0;
    int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (idx >= batch * q) return;
    int64_t b = idx / q, i = idx - b * q + 1;
    T *p = a + b * dist;
    int64_t j = rows - i, i1 = i * cols, i2 = j * cols;
    if (isgn < 0) {
        T xi = p[i1] - p[i2];
        p[i1] += p[i2];
        p[i2] = xi;
        xi = p[i2 + 1] - p[i1 + 1];
        p[i1 + 1] += p[i2 + 1];
        p[i2 + 1] = xi;
    } else {
        T a2 = (T)0.5 * (p[i1] - p[i2]);
        p[i2] = a2;
        p[i1] -= a2;
        T b2 = (T)0.5 * (p[i1 + 1] + p[i2 + 1]);
        p[i2 + 1] = b2;
        p[i1 + 1] -= b2;
    }
}

// rdft3d_sub (fft/DoubleFFT_3D.java:6909-7021): the packed columns 0/1 of
// mirror (slice, row) pairs.  One thread per pair (x, y), enumerated as
// (ii < slices/2, kk < rows/2, w in {0,1}); ii = kk = 0 has no pair.  The
// pairs are disjoint, so any order gives the reference's result.
template <typename T>
__global__ void rdft3d_kernel(T *a, int64_t dist, int64_t slices, int64_t rows, int64_t cols, int64_t batch, int isgn) {
    const int64_t n1h = slices >> 1, n2h = rows >> 1, ss = rows * cols, rs = cols;
    const int64_t per = n1h * n2h * 2;
    int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (idx >= batch * per) return;
    const int64_t b = idx / per;
    int64_t r = idx - b * per;
    const int w = (int)(r & 1);
    r >>= 1;
    const int64_t ii = r / n2h, kk = r - ii * n2h;
    int64_t x, y;
    if (ii > 0) {
        const int64_t i = ii, j = slices - i;
        if (kk == 0) {
            x = i * ss + (w ? n2h * rs : 0);
            y = j * ss + (w ? n2h * rs : 0);
        } else {
            const int64_t k = kk, l = rows - k;
            x = (w ? j : i) * ss + k * rs;
            y = (w ? i : j) * ss + l * rs;
        }
    } else {
        if (kk == 0) return;
        const int64_t k = kk, l = rows - k, base = w ? n1h * ss : 0;
        x = base + k * rs;
        y = base + l * rs;
    }
    T *p = a + b * dist;
    if (isgn < 0) {
        T t = p[x] - p[y];
        p[x] += p[y];
        p[y] = t;
        t = p[y + 1] - p[x + 1];
        p[x + 1] += p[y + 1];
        p[y + 1] = t;
    } else {
        const T y0 = (T)0.5 * (p[x] - p[y]);
        p[y] = y0;
        p[x] -= y0;
        const T y1 = (T)0.5 * (p[x + 1] + p[y + 1]);
        p[y + 1] = y1;
        p[x + 1] -= y1;
    }
}

// DHT yTransform, 2D (dht/DoubleDHT_2D.java:1288-1310): each thread owns one
// (r, c) quadruple with r <= rows/2, c <= cols/2.  Quadruples that alias
// (r or c on a symmetry line) are processed by one thread in the reference's
// order; they never share elements with other quadruples.
template <typename T>
__global__ void ytransform2_kernel(T *a, int64_t rows, int64_t cols) {
    int64_t nr = rows / 2 + 1, nc = cols / 2 + 1;
    int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (idx >= nr * nc) return;
    int64_t r = idx / nc, c = idx - r * nc;
    int64_t mRow = (rows - r) % rows, i1 = r * cols, i2 = mRow * cols;
    int64_t mCol = (cols - c) % cols;
    T A = a[i1 + c], B = a[i2 + c], C = a[i1 + mCol], D = a[i2 + mCol];
    T E = ((A + D) - (B + C)) / (T)2;
    a[i1 + c] = A - E;
    a[i2 + c] = B + E;
    a[i1 + mCol] = C + E;
    a[i2 + mCol] = D - E;
}

// DHT yTransform, 3D (dht/DoubleDHT_3D.java:2314-2356)
template <typename T>
__global__ void ytransform3_kernel(T *a, int64_t slices, int64_t rows, int64_t cols) {
    int64_t ns = slices / 2 + 1, nr = rows / 2 + 1, nc = cols / 2 + 1;
    int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (idx >= ns * nr * nc) return;
    int64_t s = idx / (nr * nc), rem = idx - s * nr * nc;
    int64_t r = rem / nc, c = rem - r * nc;
    int64_t ss = rows * cols, rs = cols;
    int64_t sC = (slices - s) % slices, i9 = s * ss, i10 = sC * ss;
    int64_t rC = (rows - r) % rows, i11 = r * rs, i12 = rC * rs;
    int64_t cC = (cols - c) % cols;
    int64_t x1 = i9 + i12 + c, x2 = i9 + i11 + cC, x3 = i10 + i11 + c, x4 = i10 + i12 + cC;
    int64_t x5 = i10 + i12 + c, x6 = i10 + i11 + cC, x7 = i9 + i11 + c, x8 = i9 + i12 + cC;
    T A = a[x1], B = a[x2], C = a[x3], D = a[x4], E = a[x5], F = a[x6], G = a[x7], H = a[x8];
    // Same store order as the reference so aliased slots end with its value.
    a[x7] = (A + B + C - D) / (T)2;
    a[x3] = (E + F + G - H) / (T)2;
    a[x1] = (G + H + E - F) / (T)2;
    a[x5] = (C + D + A - B) / (T)2;
    a[x2] = (H + G + F - E) / (T)2;
    a[x6] = (D + C + B - A) / (T)2;
    a[x8] = (B + A + D - C) / (T)2;
    a[x4] = (F + E + H - G) / (T)2;
}

// out[o][c][r] = in[o][r][c] for a batch of R x C matrices of E-byte
// elements (E = 4, 8 or 16), 32x32 tiles through shared memory.
template <typename E>
__global__ void transpose_kernel(const E *in, E *out, int64_t R, int64_t C, int64_t outer) {
    __shared__ E tile[32][33];
    int64_t tilesC = (C + 31) / 32, tilesR = (R + 31) / 32;
    int64_t t = blockIdx.x;
    int64_t o = t / (tilesC * tilesR);
    int64_t rem = t - o * tilesC * tilesR;
    int64_t tr = rem / tilesC, tc = rem - tr * tilesC;
    if (o >= outer) return;
    const E *src = in + o * R * C;
    E *dstp = out + o * R * C;
    int tx = threadIdx.x, ty = threadIdx.y;  // 32 x 8
    for (int k = 0; k < 32; k += 8) {
        int64_t r = tr * 32 + ty + k, c = tc * 32 + tx;
        if (r < R && c < C) tile[ty + k][tx] = src[r * C + c];
    }
    __syncthreads();
    for (int k = 0; k < 32; k += 8) {
        int64_t c = tc * 32 + ty + k, r = tr * 32 + tx;
        if (r < R && c < C) dstp[c * R + r] = tile[tx][ty + k];
    }
}

template <typename T> __device__ __forceinline__ void scale_body(T *a, int64_t dist, int64_t len, int64_t batch, T s, int64_t idx) {
    if (idx >= batch * len) return;
    int64_t b = idx / len, i = idx - b * len;
    a[b * dist + i] *= (T)s;
}

template <typename T> __global__ void scale_kernel(T *a, int64_t dist, int64_t len, int64_t batch, T s) {
    scale_body(a, dist, len, batch, s, blockIdx.x * (int64_t)blockDim.x + threadIdx.x);
}

// a[b][i] = src[b][i] (real, strided)
template <typename T> __device__ __forceinline__ void copy_real_body(const T *src, int64_t sdist, T *dst, int64_t ddist, int64_t len, int64_t batch, int64_t idx) {
    if (idx >= batch * len) return;
    int64_t b = idx / len, i = idx - b * len;
    dst[b * ddist + i] = src[b * sdist + i];
}

template <typename T> __global__ void copy_real_kernel(const T *src, int64_t sdist, T *dst, int64_t ddist, int64_t len, int64_t batch) {
    copy_real_body(src, sdist, dst, ddist, len, batch, blockIdx.x * (int64_t)blockDim.x + threadIdx.x);
}

#undef C2

}  // namespace jt
