// jt_r2r.cuh -- DCT-II/III, DST-II/III and DHT of even-length lines in one
// kernel each: one HBM round trip per axis, on contiguous or strided lines.
//
// A CTA holds C lines of n reals as C complex lines of h = n/2 in shared
// memory and runs the h-point complex FFT on them: in registers with the
// Stockham core for power-of-two h from 16 to 4096 (r2r_reg_kernel), else
// with the tile passes of jt_device.cuh (r2r_tile_kernel, also the batch's
// one-step form).  Contiguous lines whose scalar pairs are aligned complex
// values move as pairs, the rest one scalar at a time.  Around the FFT
// (Makhoul's reordering, the standard real-FFT split and the DCT
// quarter-wave twiddle):
//   forward DCT/DST   load:  v_j = x_2j, v_{n-1-j} = x_2j+1 (DST: odd
//                            inputs negated), z_m = v_2m + i v_2m+1
//                     store: V_k from Z_k and Z_{h-k}, C_k = Re(e^{-i pi k/2n}
//                            V_k) times the scale (DST: written to n-1-k)
//   DHT               load:  z_m = x_2m + i x_2m+1;  store: H_k = Re V_k - Im V_k
//   inverse DCT/DST   load:  coefficients (DST: reversed) into the second
//                            buffer; V_k = e^{+i pi k/2n}(C_k - i C_{n-k});
//                            Z_k from V_k and V_{h-k} (inverse real split)
//                     store: x_2j = v_j, x_2j+1 = v_{n-1-j} (DST: odd
//                            outputs negated), after the e^{+} h-point FFT
//   realForward       load:  z_m = x_2m + i x_2m+1;  store: the packed layout
//                            (a_0 = X_0, a_1 = X_{n/2}, a_2k + i a_2k+1 = X_k)
//   realInverse       load:  the packed spectrum; Z_k from X_k and X_{h-k};
//                     store: x_2m + i x_2m+1 = z_m after the e^{+} FFT
// The arithmetic is the same as the separate pre/post kernels of
// jt_device.cuh, which odd lengths and half lengths the tile passes do not
// take still use.
// Reference: dct/DoubleDCT_1D.java:169-440, dst/DoubleDST_1D.java:96-328,
// dht/DoubleDHT_1D.java:94-276, fft/DoubleFFT_1D.java:524-561 (realForward,
// rftfsub) and :946-989 (realInverse, rftbsub).
#pragma once

#include "jt_device.cuh"
#include "jt_stockham.cuh"

namespace jt {

#define C2 typename V2<T>::t

enum R2rOp { R2R_DCT2 = 0, R2R_DCT3 = 1, R2R_DHT = 2, R2R_RFWD = 3, R2R_RINV = 4 };

// inverse-type ops build Z from their staged input and run the e^{+} FFT
__host__ __device__ constexpr bool r2r_inverse(int op) { return op == R2R_DCT3 || op == R2R_RINV; }

struct R2rParams {
    int n;                  // real line length (even)
    int npass;              // passes of the h = n/2 point complex FFT
    int radix[JT_MAX_PASSES];
    int C;                  // lines per CTA
    int64_t nlines;
    Layout lin, lout;       // line layouts in scalars (T units)
    int dst;                // DST: sign flips and reversal around the DCT
    double mult, mult0;     // output (forward) or coefficient (inverse DCT) scale, index 0 apart;
                            // realInverse: the multiplier of Z
    float multf, mult0f;
    int vec_in, vec_out;    // 1: contiguous lines whose scalar pairs (2j, 2j+1) are aligned
                            // complex values (the register form moves them as pairs)
};

// e^{-2 pi i k/n}, 0 < k < h, from Wr (k <= n/4)
template <typename T> __device__ __forceinline__ C2 r2r_wr(const C2 *__restrict__ Wr, int k, int h) {
    if (2 * k <= h) return __ldg(&Wr[k]);
    const C2 w = __ldg(&Wr[h - k]);
    return mk<T>(-w.x, w.y);
}

// V_k (0 <= k <= h) of the real FFT from Z (line of h complex at z)
template <typename T> __device__ __forceinline__ C2 r2r_v(const C2 *z, int k, int h, const C2 *__restrict__ Wr) {
    if (k == 0 || k == h) {
        const C2 z0 = z[0];
        return mk<T>(k == 0 ? z0.x + z0.y : z0.x - z0.y, (T)0);
    }
    C2 xk;
    real_split<T>(z[pad(k)], z[pad(h - k)], r2r_wr<T>(Wr, k, h), xk);
    return xk;
}

// Z_k (0 <= k < h) of the inverse ops from the staged input, a line of n
// reals read through get(j): the (pre-scaled) DCT coefficients, whose V_k =
// e^{+i pi k/2n}(C_k - i C_{n-k}), or the packed spectrum X (realInverse).
// Z_k = m (0.5 (X_k + conj X_{h-k}) + 0.5 i e^{+2 pi i k/n} (X_k - conj X_{h-k})),
// Z_0 = m (0.5 (X_0 + X_h), 0.5 (X_0 - X_h)).
template <int OP, typename T, typename Get>
__device__ __forceinline__ C2 r2r_inv_z(Get &get, int k, int h, const C2 *__restrict__ Wr, const C2 *__restrict__ Wd,
                                        T m) {
    const int n = 2 * h;
    auto X = [&](int kk) -> C2 {
        if (OP == R2R_DCT3) {
            const C2 w = __ldg(&Wd[kk]);  // e^{-i pi k/2n}; conjugated below
            const T a = kk >= n ? (T)0 : get(kk), b = kk == 0 ? (T)0 : get(n - kk);
            return cmul<T>(mk<T>(w.x, -w.y), mk<T>(a, -b));
        } else {
            if (kk == 0) return mk<T>(get(0), (T)0);
            if (kk == h) return mk<T>(get(1), (T)0);
            return mk<T>(get(2 * kk), get(2 * kk + 1));
        }
    };
    if (k == 0) {
        const T x0 = X(0).x, xh = X(h).x;
        return mk<T>((T)0.5 * (x0 + xh) * m, (T)0.5 * (x0 - xh) * m);
    }
    const C2 xk = X(k), xh = X(h - k);
    const C2 wr = r2r_wr<T>(Wr, k, h);
    const C2 w = mk<T>(wr.x, -wr.y);  // e^{+2 pi i k/n}
    const C2 sa = mk<T>((T)0.5 * (xk.x + xh.x), (T)0.5 * (xk.y - xh.y));
    const C2 d = mk<T>((T)0.5 * (xk.x - xh.x), (T)0.5 * (xk.y + xh.y));
    const C2 wd = cmul<T>(w, d);
    return mk<T>((sa.x - wd.y) * m, (sa.y + wd.x) * m);
}

// Tile `blk` (lines blk*C ..) run by the calling CTA, any block size, its
// shared memory at smem_raw (2 * C * padded(h) complex).
// Forward outputs (DCT-II / DST-II or DHT) that depend on the pair
// (Z_kk, Z_{h-kk}), 0 <= kk <= h/2: up to four of them, k = kk, n - kk,
// h - kk and h + kk, through put(k, value).  With a = (Z_kk + conj Z_{h-kk})
// and d = (Z_kk - conj Z_{h-kk}) (both doubled; the halves ride on the
// multipliers hm = mult / 2, hm0 = mult0 / 2) and wd = w_kk d:
// V_kk = a - i wd, V_{h-kk} = conj(a) - i conj(wd), V_{n-k} = conj(V_k).
template <int OP, typename T, typename Put>
__device__ __forceinline__ void r2r_post_pair(const C2 *zl, int kk, int h, const C2 *__restrict__ Wr,
                                              const C2 *__restrict__ Wd, T hm, T hm0, Put &put) {
    const int n = 2 * h;
    auto emit = [&](int k, T vr, T vi) {
        if (OP == R2R_DHT) {
            put(k, (vr - vi) * hm);
        } else {
            const C2 w = __ldg(&Wd[k]);
            put(k, (w.x * vr - w.y * vi) * (k == 0 ? hm0 : hm));
        }
    };
    if (kk == 0) {
        const C2 z0 = zl[0];
        emit(0, (T)2 * (z0.x + z0.y), (T)0);
        emit(h, (T)2 * (z0.x - z0.y), (T)0);
        return;
    }
    const C2 zk = zl[pad(kk)], zh = zl[pad(h - kk)];
    const C2 a = mk<T>(zk.x + zh.x, zk.y - zh.y), d = mk<T>(zk.x - zh.x, zk.y + zh.y);
    const C2 wd = cmul<T>(r2r_wr<T>(Wr, kk, h), d);
    const T xr = a.x + wd.y, xi = a.y - wd.x;  // V_kk
    emit(kk, xr, xi);
    emit(n - kk, xr, -xi);
    if (2 * kk != h) {
        const T yr = a.x - wd.y, yi = -a.y - wd.x;  // V_{h-kk}
        emit(h - kk, yr, yi);
        emit(h + kk, yr, -yi);
    }
}

// The output phase of both forms: lines [b0, b0 + lines) of the FFT result
// z (rows of stride RX complex) to out.
template <int OP, typename T>
__device__ __forceinline__ void r2r_store(const C2 *z, int RX, T *out, const R2rParams &p, int64_t b0, int lines,
                                          const C2 *__restrict__ Wr, const C2 *__restrict__ Wd, T mult, T mult0, int tid,
                                          int nt) {
    const int n = p.n, h = n >> 1;
    const bool rows_out = p.lout.estride == 1;
    if (OP == R2R_RINV) {
        const int tot = lines * n;
        for (int idx = tid; idx < tot; idx += nt) {
            int c, k;
            if (rows_out) {
                c = idx / n;
                k = idx - c * n;
            } else {
                k = idx / lines;
                c = idx - k * lines;
            }
            out[line_off(p.lout, b0 + c) + (int64_t)k * p.lout.estride] =
                reinterpret_cast<const T *>(&z[c * RX + pad(k >> 1)])[k & 1];
        }
        return;
    }
    if (OP == R2R_RFWD) {
        // packed realForward: X_kk and X_{h-kk} from the pair (the halves
        // of a and d are exact scalings, applied at the end)
        const int npair = h / 2 + 1;
        const int tot = lines * npair;
        for (int idx = tid; idx < tot; idx += nt) {
            int c, kk;
            if (rows_out) {
                c = idx / npair;
                kk = idx - c * npair;
            } else {
                kk = idx / lines;
                c = idx - kk * lines;
            }
            T *o = out + line_off(p.lout, b0 + c);
            const int64_t es = p.lout.estride;
            const C2 *zl = z + c * RX;
            if (kk == 0) {
                const C2 z0 = zl[0];
                o[0] = z0.x + z0.y;
                o[es] = z0.x - z0.y;
                continue;
            }
            const C2 zk = zl[pad(kk)], zh = zl[pad(h - kk)];
            const C2 a = mk<T>(zk.x + zh.x, zk.y - zh.y), d = mk<T>(zk.x - zh.x, zk.y + zh.y);
            const C2 wd = cmul<T>(r2r_wr<T>(Wr, kk, h), d);
            o[(int64_t)(2 * kk) * es] = (T)0.5 * (a.x + wd.y);
            o[(int64_t)(2 * kk + 1) * es] = (T)0.5 * (a.y - wd.x);
            if (2 * kk != h) {
                o[(int64_t)(2 * (h - kk)) * es] = (T)0.5 * (a.x - wd.y);
                o[(int64_t)(2 * (h - kk) + 1) * es] = (T)0.5 * (-a.y - wd.x);
            }
        }
        return;
    }
    if (OP == R2R_DCT3) {
        const int tot = lines * n;
        for (int idx = tid; idx < tot; idx += nt) {
            int c, k;
            if (rows_out) {
                c = idx / n;
                k = idx - c * n;
            } else {
                k = idx / lines;
                c = idx - k * lines;
            }
            const int j = (k & 1) ? n - 1 - (k >> 1) : (k >> 1);
            T val = reinterpret_cast<const T *>(&z[c * RX + pad(j >> 1)])[j & 1];
            if (p.dst && (k & 1)) val = -val;
            out[line_off(p.lout, b0 + c) + (int64_t)k * p.lout.estride] = val;
        }
        return;
    }
    const T hm = mult * (T)0.5, hm0 = mult0 * (T)0.5;
    const int npair = h / 2 + 1;
    const int tot = lines * npair;
    for (int idx = tid; idx < tot; idx += nt) {
        int c, kk;
        if (rows_out) {
            c = idx / npair;
            kk = idx - c * npair;
        } else {
            kk = idx / lines;
            c = idx - kk * lines;
        }
        T *o = out + line_off(p.lout, b0 + c);
        const int64_t es = p.lout.estride;
        const bool rev = OP == R2R_DCT2 && p.dst;
        auto put = [&](int k, T val) { o[(int64_t)(rev ? n - 1 - k : k) * es] = val; };
        r2r_post_pair<OP, T>(z + c * RX, kk, h, Wr, Wd, hm, hm0, put);
    }
}

template <int OP, typename T>
__device__ void r2r_tile_body(const T *in, T *out, const R2rParams &p, const C2 *__restrict__ W, const C2 *__restrict__ Wr,
                              const C2 *__restrict__ Wd, int64_t blk, unsigned char *smem_raw) {
    const int n = p.n, h = n >> 1, Lp = padded_len(h);
    C2 *bufA = reinterpret_cast<C2 *>(smem_raw);
    C2 *bufB = bufA + p.C * Lp;
    const int64_t b0 = blk * p.C;
    const int lines = (int)min((int64_t)p.C, p.nlines - b0);
    if (lines <= 0) return;
    const int tot = lines * n;
    T mult, mult0;
    if constexpr (sizeof(T) == 4) {
        mult = p.multf;
        mult0 = p.mult0f;
    } else {
        mult = (T)p.mult;
        mult0 = (T)p.mult0;
    }
    // element i of line c: contiguous lines element-fastest, strided lines
    // line-fastest (neighbouring threads on neighbouring columns)
    const bool rows_in = p.lin.estride == 1, rows_out = p.lout.estride == 1;
    auto slot = [&](C2 *buf, int c, int j) -> T & { return reinterpret_cast<T *>(&buf[c * Lp + pad(j >> 1)])[j & 1]; };

    for (int idx = threadIdx.x; idx < tot; idx += blockDim.x) {
        int c, i;
        if (rows_in) {
            c = idx / n;
            i = idx - c * n;
        } else {
            i = idx / lines;
            c = idx - i * lines;
        }
        T x = in[line_off(p.lin, b0 + c) + (int64_t)i * p.lin.estride];
        if (OP == R2R_DCT2) {
            const int j = (i & 1) ? n - 1 - (i >> 1) : (i >> 1);
            if (p.dst && (i & 1)) x = -x;
            slot(bufA, c, j) = x;
        } else if (OP == R2R_DHT || OP == R2R_RFWD) {
            slot(bufA, c, i) = x;
        } else if (OP == R2R_RINV) {
            slot(bufB, c, i) = x;
        } else {
            // coefficient k (DST: read reversed), scaled
            const int k = p.dst ? n - 1 - i : i;
            slot(bufB, c, k) = x * (k == 0 ? mult0 : mult);
        }
    }
    __syncthreads();
    if (r2r_inverse(OP)) {
        const T zm = OP == R2R_RINV ? mult : (T)1;
        const int q = lines * h;
        for (int idx = threadIdx.x; idx < q; idx += blockDim.x) {
            const int c = idx / h, k = idx - c * h;
            auto get = [&](int j) -> T { return slot(bufB, c, j); };
            bufA[c * Lp + pad(k)] = r2r_inv_z<OP, T>(get, k, h, Wr, Wd, zm);
        }
        __syncthreads();
    }
    const C2 *z = r2r_inverse(OP) ? tile_passes<1, T>(bufA, bufB, lines, h, Lp, p.npass, p.radix, W)
                                  : tile_passes<-1, T>(bufA, bufB, lines, h, Lp, p.npass, p.radix, W);
    r2r_store<OP, T>(z, Lp, out, p, b0, lines, Wr, Wd, mult, mult0, threadIdx.x, blockDim.x);
}

template <int OP, typename T>
__global__ void __launch_bounds__(512) r2r_tile_kernel(const T *in, T *out, R2rParams p, const C2 *__restrict__ W,
                                                       const C2 *__restrict__ Wr, const C2 *__restrict__ Wd) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    r2r_tile_body<OP, T>(in, out, p, W, Wr, Wd, (int64_t)blockIdx.x, smem_raw);
}

// ---------------------------------------------------------------------------
// The same three line operations with the h-point FFT in registers: the
// register Stockham passes of jt_stockham.cuh (radix 16, 16 elements per
// thread, exchange in shared memory) for power-of-two h from 16 to 4096.
// A CTA holds Stockham<T, h, 0>::C lines in one shared-memory buffer that
// serves as the load staging, the pass exchange and the output staging.
// ---------------------------------------------------------------------------
template <typename T, int H, int OP> struct R2rReg {
    static constexpr int SIGN = r2r_inverse(OP) ? 1 : -1;
    typedef Stockham<T, H, 0, SIGN> S;
    static constexpr int RX = S::LP;  // row stride of a line in the buffer (complex)
    static constexpr size_t SMEM = (size_t)S::C * RX * sizeof(typename V2<T>::t);
};

template <typename T, int H, int OP>
__global__ void __launch_bounds__(R2rReg<T, H, OP>::S::NT)
    r2r_reg_kernel(const T *in, T *out, R2rParams p, const C2 *__restrict__ Wp, const C2 *__restrict__ Wr,
                   const C2 *__restrict__ Wd) {
    typedef R2rReg<T, H, OP> G;
    typedef typename G::S S;
    constexpr int n = 2 * H, RX = G::RX;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C2 *buf = reinterpret_cast<C2 *>(smem_raw);
    // lines per CTA: p.C (at most S::C), blockDim = p.C * TL
    const int tid = threadIdx.x, NT = blockDim.x;
    const int c = tid / S::TL, t = tid % S::TL;
    const int64_t b0 = (int64_t)blockIdx.x * p.C;
    const int lines = (int)min((int64_t)p.C, p.nlines - b0);
    const int tot = lines * n;
    T mult, mult0;
    if constexpr (sizeof(T) == 4) {
        mult = p.multf;
        mult0 = p.mult0f;
    } else {
        mult = (T)p.mult;
        mult0 = (T)p.mult0;
    }
    const bool rows_in = p.lin.estride == 1, rows_out = p.lout.estride == 1;
    auto slot = [&](int cc, int j) -> T & { return reinterpret_cast<T *>(&buf[cc * RX + pad(j >> 1)])[j & 1]; };
    // element i of line cc into its staged position
    auto put_in = [&](int cc, int i, T x) {
        if (OP == R2R_DCT2) {
            const int j = (i & 1) ? n - 1 - (i >> 1) : (i >> 1);
            if (p.dst && (i & 1)) x = -x;
            slot(cc, j) = x;
        } else if (OP == R2R_DHT || OP == R2R_RFWD || OP == R2R_RINV) {
            slot(cc, i) = x;
        } else {
            const int k = p.dst ? n - 1 - i : i;
            slot(cc, k) = x * (k == 0 ? mult0 : mult);
        }
    };

    C2 v[S::E];
    // forward real and DHT lines loaded as pairs need no reordering: the
    // thread's own inputs t + m TL go straight to its registers (16 or more
    // threads per line keep those loads in 128-byte runs)
    constexpr bool DIRECT_OK = (OP == R2R_DHT || OP == R2R_RFWD) && S::TL >= 16;
    const bool paired_in = rows_in && p.vec_in;
    if (paired_in && S::TL < 16) {
        // short lines: the CTA's pairs in order (idx = tid + u NT covers
        // lines * H <= NT * E), all E loads in flight, then staged
        C2 x[S::E];
#pragma unroll
        for (int u = 0; u < S::E; u++) {
            const int idx = tid + u * NT, cc = idx / H, j = idx - cc * H;
            if (cc < lines) x[u] = reinterpret_cast<const C2 *>(in + line_off(p.lin, b0 + cc))[j];
        }
#pragma unroll
        for (int u = 0; u < S::E; u++) {
            const int idx = tid + u * NT, cc = idx / H, j = idx - cc * H;
            if (cc < lines) {
                if (OP == R2R_DHT || OP == R2R_RFWD || OP == R2R_RINV) {
                    buf[cc * RX + pad(j)] = x[u];
                } else {
                    put_in(cc, 2 * j, x[u].x);
                    put_in(cc, 2 * j + 1, x[u].y);
                }
            }
        }
    } else if (paired_in) {
        // contiguous lines: each thread loads its 16 scalar pairs t + m TL of
        // line c at once (all in flight), coalesced across t
        C2 x[S::E];
        if (c < lines) {
            const C2 *src = reinterpret_cast<const C2 *>(in + line_off(p.lin, b0 + c));
#pragma unroll
            for (int m = 0; m < S::E; m++) x[m] = src[t + m * S::TL];
        }
        if constexpr (DIRECT_OK) {
#pragma unroll
            for (int m = 0; m < S::E; m++) v[m] = x[m];
        } else if (c < lines) {
#pragma unroll
            for (int m = 0; m < S::E; m++) {
                const int j = t + m * S::TL;
                if (OP == R2R_RINV) {
                    buf[c * RX + pad(j)] = x[m];
                } else {
                    put_in(c, 2 * j, x[m].x);
                    put_in(c, 2 * j + 1, x[m].y);
                }
            }
        }
    } else {
        // four loads in flight per thread
        for (int base = tid; base < tot; base += 4 * NT) {
            T xs[4];
            int cs[4], is[4];
#pragma unroll
            for (int u = 0; u < 4; u++) {
                const int idx = base + u * NT;
                if (idx < tot) {
                    if (rows_in) {
                        cs[u] = idx / n;
                        is[u] = idx - cs[u] * n;
                    } else {
                        is[u] = idx / lines;
                        cs[u] = idx - is[u] * lines;
                    }
                    xs[u] = in[line_off(p.lin, b0 + cs[u]) + (int64_t)is[u] * p.lin.estride];
                }
            }
#pragma unroll
            for (int u = 0; u < 4; u++)
                if (base + u * NT < tot) put_in(cs[u], is[u], xs[u]);
        }
    }
    __syncthreads();
    if (DIRECT_OK && paired_in) {
        // v holds the inputs already
    } else if (r2r_inverse(OP)) {
        // this thread's inputs Z_k, k = t + m TL, from the staged line
        const T zm = OP == R2R_RINV ? mult : (T)1;
        auto get = [&](int j) -> T { return slot(c, j); };
#pragma unroll
        for (int m = 0; m < S::E; m++) v[m] = r2r_inv_z<OP, T>(get, t + m * S::TL, H, Wr, Wd, zm);
    } else {
#pragma unroll
        for (int m = 0; m < S::E; m++) v[m] = buf[c * RX + pad(t + m * S::TL)];
    }
    __syncthreads();  // the passes' exchange overwrites the buffer
    {
        PadIdx xi{c * RX};
        auto store = [&](int pos, C2 val, int) { buf[c * RX + pad(pos)] = val; };
        S::run_all(v, t, buf, xi, Wp, store);
    }
    __syncthreads();
    if ((OP == R2R_RFWD || OP == R2R_RINV) && rows_out && p.vec_out) {
        if (OP == R2R_RINV) {
            // the inverse FFT's h complex values are the n reals in order
            const int totc = lines * H;
            for (int idx = tid; idx < totc; idx += NT) {
                const int cc = idx / H, j = idx - cc * H;
                reinterpret_cast<C2 *>(out + line_off(p.lout, b0 + cc))[j] = buf[cc * RX + pad(j)];
            }
        } else {
            // packed realForward: pair kk gives X_kk and X_{h-kk}, each one
            // aligned (re, im) store
            constexpr int NPAIR = H / 2 + 1;
            const int totp = lines * NPAIR;
            for (int idx = tid; idx < totp; idx += NT) {
                const int cc = idx / NPAIR, kk = idx - cc * NPAIR;
                C2 *o = reinterpret_cast<C2 *>(out + line_off(p.lout, b0 + cc));
                const C2 *zl = buf + cc * RX;
                if (kk == 0) {
                    const C2 z0 = zl[0];
                    o[0] = mk<T>(z0.x + z0.y, z0.x - z0.y);
                    continue;
                }
                const C2 zk = zl[pad(kk)], zh = zl[pad(H - kk)];
                const C2 a = mk<T>(zk.x + zh.x, zk.y - zh.y), d = mk<T>(zk.x - zh.x, zk.y + zh.y);
                const C2 wd = cmul<T>(r2r_wr<T>(Wr, kk, H), d);
                o[kk] = mk<T>((T)0.5 * (a.x + wd.y), (T)0.5 * (a.y - wd.x));
                if (2 * kk != H) o[H - kk] = mk<T>((T)0.5 * (a.x - wd.y), (T)0.5 * (-a.y - wd.x));
            }
        }
        return;
    }
    r2r_store<OP, T>(buf, RX, out, p, b0, lines, Wr, Wd, mult, mult0, tid, NT);
}

// Launches the register form for half length H (T's instantiations live in
// jt_r2r_f32.cu / jt_r2r_f64.cu); false when H has none.
template <typename T, int H> struct R2rRegLaunch {
    template <int OP>
    static void one(const T *in, T *out, const R2rParams &p, const C2 *Wp, const C2 *Wr, const C2 *Wd, cudaStream_t s) {
        typedef R2rReg<T, H, OP> G;
        static bool attr = false;
        if (!attr) {
            cudaFuncSetAttribute(r2r_reg_kernel<T, H, OP>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)G::SMEM);
            attr = true;
        }
        // p.C lines per CTA (1 .. S::C): p.C * TL threads, p.C rows of shared memory
        const int64_t grid = (p.nlines + p.C - 1) / p.C;
        const size_t smem = (size_t)p.C * G::RX * sizeof(typename V2<T>::t);
        r2r_reg_kernel<T, H, OP><<<(unsigned)grid, p.C * G::S::TL, smem, s>>>(in, out, p, Wp, Wr, Wd);
    }
    static void go(int op, const T *in, T *out, const R2rParams &p, const C2 *Wp, const C2 *Wr, const C2 *Wd, cudaStream_t s) {
        if (op == R2R_DCT2) one<R2R_DCT2>(in, out, p, Wp, Wr, Wd, s);
        else if (op == R2R_DCT3) one<R2R_DCT3>(in, out, p, Wp, Wr, Wd, s);
        else if (op == R2R_DHT) one<R2R_DHT>(in, out, p, Wp, Wr, Wd, s);
        else if (op == R2R_RFWD) one<R2R_RFWD>(in, out, p, Wp, Wr, Wd, s);
        else one<R2R_RINV>(in, out, p, Wp, Wr, Wd, s);
    }
};

#undef C2

}  // namespace jt
