// jt_oracle.cpp -- CPU restatement of JTransforms' transform path.
//
// TEST INFRASTRUCTURE ONLY.  This file is the oracle that the GPU library is
// checked against.  Only tests/, __graft_entry__.smoke() and bench.py's CPU
// baseline leg load it; the product (jtransforms_gb300, libjtgpu.so) never
// links, imports or calls it, and has no CPU fallback.
//
// What is restated, and how faithfully (all paths relative to
// src/main/java/org/jtransforms/ in the reference):
//   * plan choice (fft/DoubleFFT_1D.java:117-188): power of two -> split
//     radix; remainder after removing 4,2,3,5 >= 211 -> Bluestein with
//     nextPow2(2n-1) padding; else mixed radix.
//   * split-radix glue step for step: realForward / realInverse /
//     realInverse2 (fft/DoubleFFT_1D.java:524-561, :946-989, :1297-1355),
//     rftfsub / rftbsub / dctsub (utils/CommonUtils.java:5750-5882), the DCT's
//     private rftfsub/rftbsub (dct/DoubleDCT_1D.java:557-660), makect
//     (utils/CommonUtils.java:502-520), cftx020 / cftxc020 (:5682, :5728).
//     The Ooura cftfsub/cftbsub tree itself (utils/CommonUtils.java:708-5749)
//     is replaced by an iterative radix-2 FFT with the same semantics
//     (cftfsub = e^{+i}, cftbsub = e^{-i}, unnormalized, natural order) and
//     twiddles computed from the same first-octant angle formula as makewt
//     (:372-500; float angles for the Float classes, :578-640).
//   * mixed radix (cffti/cfftf/passf*, fft/DoubleFFT_1D.java:1430-1517,
//     :6630-7842): FFTPACK factor order (4,2,3,5,7,9,11,... with a 2 moved to
//     the front), self-sorting passes with post-twiddles w^(i*j*l1), twiddle
//     angles fi*(ld*argh) computed in the working precision as the Float
//     class does (fft/FloatFFT_1D.java:1484-1507).  The real FFTPACK passes
//     (rfftf/radf*, :3371-6630) are restated by their output: the packed real
//     layout of the complex mixed-radix transform of the real sequence.
//   * Bluestein step for step (bluesteini :1864-1890, bluestein_complex
//     :1920-2107); its real variants (:2298-3370) are the complex chirp-z on
//     zero-imaginary input followed by the same packing.
//   * DCT-II/III (dct/DoubleDCT_1D.java:169-243, :361-440) including the
//     unscaled normalisation that differs between power-of-two and other n;
//     DST (dst/DoubleDST_1D.java:96-160, :264-328); DHT
//     (dht/DoubleDHT_1D.java:94-159, :255-276).
//   * 2D/3D drivers: row/column/slice passes, rdft2d_sub
//     (fft/DoubleFFT_2D.java:2544-2575), DHT yTransform
//     (dht/DoubleDHT_2D.java:1288-1310, dht/DoubleDHT_3D.java:2314-2356).
//
// Compile with -O2 -ffp-contract=off (no -ffast-math) so float and double
// arithmetic round like Java's.

#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#include <algorithm>
#include <stdexcept>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

typedef int64_t i64;

bool is_pow2(i64 x) { return x > 0 && (x & (x - 1)) == 0; }

// CommonUtils.nextPow2 (utils/CommonUtils.java:238-253).
i64 next_pow2(i64 x) {
    i64 p = 1;
    while (p < x) p <<= 1;
    return p;
}

// CommonUtils.getReminder with factors {4,2,3,5} (utils/CommonUtils.java:317-332).
i64 get_reminder(i64 n) {
    static const int f[4] = {4, 2, 3, 5};
    i64 r = n;
    for (int i = 0; i < 4 && r != 1; i++)
        while (r % f[i] == 0) r /= f[i];
    return r;
}

enum PlanKind { SPLIT_RADIX = 0, MIXED_RADIX = 1, BLUESTEIN = 2 };

PlanKind choose_plan(i64 n) {
    if (is_pow2(n)) return SPLIT_RADIX;
    return get_reminder(n) >= 211 ? BLUESTEIN : MIXED_RADIX;
}

// ---------------------------------------------------------------------------
// Twiddles.  T is the working precision; angles are formed in T as the
// reference does (double for Double*, float for Float*), cos/sin in double and
// rounded to T.
// ---------------------------------------------------------------------------
template <class T> struct Cx { T re, im; };

// e^{+2 pi i k / N} for power-of-two N, folded to the first octant the way the
// split-radix table only stores angles below pi/4 (utils/CommonUtils.java:372-433).
template <class T> Cx<T> split_twiddle(i64 N, i64 k) {
    k %= N;
    if (k < 0) k += N;
    // Reduce to 0 <= k < N/8 using symmetries; the stored angle is delta * 2k
    // with delta = (pi/4) / (N/4) formed in T.
    i64 q = N / 8;
    if (N < 8) {
        // N = 1, 2, 4: exact quarter-turn values
        static const double c4[4] = {1, 0, -1, 0}, s4[4] = {0, 1, 0, -1};
        i64 kk = (k * (4 / N)) & 3;
        Cx<T> r = {(T)c4[kk], (T)s4[kk]};
        return r;
    }
    i64 oct = k / q, rem = k % q;
    // angle theta = 2 pi k / N = oct * pi/4 + 2 pi rem / N
    T delta = (T)0.785398163397448278999490867136046290 / (T)(N / 4);
    T cr, ci;
    auto cs = [&](i64 m, T &c, T &s) {  // cos/sin of delta * 2m, 0 <= m <= q
        T ang = delta * (T)(2 * m);
        c = (T)std::cos((double)ang);
        s = (T)std::sin((double)ang);
    };
    // Use first-octant values: for odd octants use the complementary angle.
    T c, s;
    if (rem == 0) {
        static const double cc[8] = {1, 0.70710678118654752440, 0, -0.70710678118654752440, -1, -0.70710678118654752440, 0, 0.70710678118654752440};
        static const double ss[8] = {0, 0.70710678118654752440, 1, 0.70710678118654752440, 0, -0.70710678118654752440, -1, -0.70710678118654752440};
        Cx<T> r = {(T)cc[oct], (T)ss[oct]};
        return r;
    }
    if (oct & 1) cs(q - rem, c, s); else cs(rem, c, s);
    // base angle phi in [0, pi/4); theta = oct*pi/4 + rem-part
    switch (oct) {
        case 0: cr = c;  ci = s;  break;            // phi
        case 1: cr = s;  ci = c;  break;            // pi/2 - phi'
        case 2: cr = -s; ci = c;  break;            // pi/2 + phi
        case 3: cr = -c; ci = s;  break;            // pi - phi'
        case 4: cr = -c; ci = -s; break;            // pi + phi
        case 5: cr = -s; ci = -c; break;            // 3pi/2 - phi'
        case 6: cr = s;  ci = -c; break;            // 3pi/2 + phi
        default: cr = c; ci = -s; break;            // 2pi - phi'
    }
    Cx<T> r = {cr, ci};
    return r;
}

template <class T> struct SplitTable {
    i64 N = 0;
    std::vector<Cx<T>> w;  // w[k] = e^{+2 pi i k/N}, k < N/2
    void build(i64 n) {
        N = n;
        w.resize(std::max<i64>(n / 2, 1));
        for (i64 k = 0; k < (i64)w.size(); k++) w[k] = split_twiddle<T>(n, k);
    }
};

// In-place complex DFT of N (power of two) points stored interleaved in a:
// sign=+1 computes sum x_j e^{+2 pi i jk/N} (CommonUtils.cftfsub semantics),
// sign=-1 computes e^{-2 pi i jk/N} (CommonUtils.cftbsub semantics).
// Unnormalized, natural order in and out.  Iterative radix-2 (bit reversal,
// then butterflies), not Ooura's tree; see the header.
template <class T> void cft(T *a, i64 N, int sign, const SplitTable<T> &tb) {
    if (N <= 1) return;
    // bit reversal
    for (i64 i = 1, j = 0; i < N; i++) {
        i64 bit = N >> 1;
        for (; j & bit; bit >>= 1) j ^= bit;
        j ^= bit;
        if (i < j) {
            std::swap(a[2 * i], a[2 * j]);
            std::swap(a[2 * i + 1], a[2 * j + 1]);
        }
    }
    i64 step = tb.N / N;  // table may be built for a multiple of N
    for (i64 len = 2; len <= N; len <<= 1) {
        i64 half = len >> 1;
        i64 ts = (N / len) * step;
        for (i64 i = 0; i < N; i += len) {
            for (i64 k = 0; k < half; k++) {
                Cx<T> w = tb.w[k * ts];
                T wr = w.re, wi = sign > 0 ? w.im : -w.im;
                T *u = a + 2 * (i + k), *v = a + 2 * (i + k + half);
                T vr = v[0] * wr - v[1] * wi;
                T vi = v[0] * wi + v[1] * wr;
                v[0] = u[0] - vr;
                v[1] = u[1] - vi;
                u[0] = u[0] + vr;
                u[1] = u[1] + vi;
            }
        }
    }
}

// makect (utils/CommonUtils.java:502-520): c[j] = 0.5 cos(delta j),
// c[nc-j] = 0.5 sin(delta j), delta = (pi/4)/(nc/2), angles formed in T.
template <class T> std::vector<T> makect(i64 nc) {
    std::vector<T> c(std::max<i64>(nc, 1));
    if (nc > 1) {
        i64 nch = nc >> 1;
        T delta = (T)0.785398163397448278999490867136046290 / (T)nch;
        c[0] = (T)std::cos((double)(delta * (T)nch));
        c[nch] = (T)0.5 * c[0];
        for (i64 j = 1; j < nch; j++) {
            T dj = delta * (T)j;
            c[j] = (T)0.5 * (T)std::cos((double)dj);
            c[nc - j] = (T)0.5 * (T)std::sin((double)dj);
        }
    }
    return c;
}

// CommonUtils.rftfsub (utils/CommonUtils.java:5750-5776).
template <class T> void rftfsub(i64 n, T *a, i64 nc, const T *c) {
    i64 m = n >> 1, ks = 2 * nc / m, kk = 0;
    for (i64 j = 2; j < m; j += 2) {
        i64 k = n - j;
        kk += ks;
        T wkr = (T)0.5 - c[nc - kk], wki = c[kk];
        T xr = a[j] - a[k], xi = a[j + 1] + a[k + 1];
        T yr = wkr * xr - wki * xi, yi = wkr * xi + wki * xr;
        a[j] -= yr;
        a[j + 1] = yi - a[j + 1];
        a[k] += yr;
        a[k + 1] = yi - a[k + 1];
    }
    a[m + 1] = -a[m + 1];
}

// CommonUtils.rftbsub (utils/CommonUtils.java:5806-5830).
template <class T> void rftbsub(i64 n, T *a, i64 nc, const T *c) {
    i64 m = n >> 1, ks = 2 * nc / m, kk = 0;
    for (i64 j = 2; j < m; j += 2) {
        i64 k = n - j;
        kk += ks;
        T wkr = (T)0.5 - c[nc - kk], wki = c[kk];
        T xr = a[j] - a[k], xi = a[j + 1] + a[k + 1];
        T yr = wkr * xr - wki * xi, yi = wkr * xi + wki * xr;
        a[j] -= yr;
        a[j + 1] -= yi;
        a[k] += yr;
        a[k + 1] -= yi;
    }
}

// DoubleDCT_1D's private rftfsub (dct/DoubleDCT_1D.java:557-581): same as
// rftbsub above.  Its private rftbsub (:609-633) flips the sign of wki.
template <class T> void dct_rftbsub(i64 n, T *a, i64 nc, const T *c) {
    i64 m = n >> 1, ks = 2 * nc / m, kk = 0;
    for (i64 j = 2; j < m; j += 2) {
        i64 k = n - j;
        kk += ks;
        T wkr = (T)0.5 - c[nc - kk], wki = c[kk];
        T xr = a[j] - a[k], xi = a[j + 1] + a[k + 1];
        T yr = wkr * xr + wki * xi, yi = wkr * xi - wki * xr;
        a[j] -= yr;
        a[j + 1] -= yi;
        a[k] += yr;
        a[k + 1] -= yi;
    }
}

// CommonUtils.dctsub (utils/CommonUtils.java:5860-5882).
template <class T> void dctsub(i64 n, T *a, i64 nc, const T *c) {
    i64 m = n >> 1, ks = nc / n, kk = 0;
    for (i64 j = 1; j < m; j++) {
        i64 k = n - j;
        kk += ks;
        T wkr = c[kk] - c[nc - kk], wki = c[kk] + c[nc - kk];
        T xr = wki * a[j] - wkr * a[k];
        a[j] = wkr * a[j] + wki * a[k];
        a[k] = xr;
    }
    a[m] *= c[0];
}

// CommonUtils.scale (utils/CommonUtils.java:11108-11150).
template <class T> void scale_arr(i64 len, T m, T *a) {
    for (i64 i = 0; i < len; i++) a[i] *= m;
}

// ---------------------------------------------------------------------------
// Mixed radix (FFTPACK) complex transform.
// ---------------------------------------------------------------------------
// cffti factorisation (fft/DoubleFFT_1D.java:1430-1470).
std::vector<int> fftpack_factors(i64 n) {
    std::vector<int> f;
    i64 nl = n;
    int j = 0, ntry = 0;
    static const int first[4] = {4, 2, 3, 5};
    while (nl != 1) {
        j++;
        ntry = j <= 4 ? first[j - 1] : ntry + 2;
        while (nl % ntry == 0) {
            f.push_back(ntry);
            nl /= ntry;
            if (ntry == 2 && f.size() != 1) {
                // move the 2 to the front
                for (size_t i = f.size() - 1; i > 0; i--) f[i] = f[i - 1];
                f[0] = 2;
            }
        }
    }
    return f;
}

template <class T> struct MixedPlan {
    i64 n = 0;
    std::vector<int> fac;
    // per-pass twiddles: tw[pass][(j-1)*ido + i] = angle fi*(ld*argh), ld=j*l1
    std::vector<std::vector<Cx<T>>> tw;
    std::vector<std::vector<Cx<T>>> roots;  // p-th roots e^{+2 pi i q/p}
    void build(i64 n_) {
        n = n_;
        fac = fftpack_factors(n);
        T argh = (T)6.28318530717958623199592693708837032 / (T)n;
        i64 l1 = 1;
        for (int p : fac) {
            i64 l2 = l1 * p, ido = n / l2;
            std::vector<Cx<T>> t((size_t)(p - 1) * ido);
            for (int j = 1; j < p; j++) {
                T argld = (T)(j * l1) * argh;
                for (i64 i = 0; i < ido; i++) {
                    T arg = (T)i * argld;
                    t[(j - 1) * ido + i] = {(T)std::cos((double)arg), (T)std::sin((double)arg)};
                }
            }
            tw.push_back(t);
            std::vector<Cx<T>> r(p);
            T argp = (T)6.28318530717958623199592693708837032 / (T)p;
            for (int q = 0; q < p; q++) {
                T ang = argp * (T)q;
                r[q] = {(T)std::cos((double)ang), (T)std::sin((double)ang)};
            }
            if (p == 4) { r[0] = {1, 0}; r[1] = {0, 1}; r[2] = {-1, 0}; r[3] = {0, -1}; }
            if (p == 2) { r[0] = {1, 0}; r[1] = {-1, 0}; }
            roots.push_back(r);
            l1 = l2;
        }
    }
    // isign = -1 forward (e^{-i}), +1 backward; unnormalized.
    void run(T *a, int isign) const {
        if (n <= 1) return;
        std::vector<T> buf(2 * n);
        T *in = a, *out = buf.data();
        i64 l1 = 1;
        std::vector<T> vr(64), vi(64);
        for (size_t s = 0; s < fac.size(); s++) {
            int p = fac[s];
            i64 l2 = l1 * p, ido = n / l2;
            if ((int)vr.size() < p) { vr.resize(p); vi.resize(p); }
            const auto &t = tw[s];
            const auto &r = roots[s];
            for (i64 k = 0; k < l1; k++) {
                for (i64 i = 0; i < ido; i++) {
                    // cc(i, q, k) = in[i + ido*q + ido*p*k]
                    for (int q = 0; q < p; q++) {
                        i64 idx = i + ido * q + ido * p * k;
                        vr[q] = in[2 * idx];
                        vi[q] = in[2 * idx + 1];
                    }
                    for (int j = 0; j < p; j++) {
                        T sr = 0, si = 0;
                        for (int q = 0; q < p; q++) {
                            int e = (int)(((i64)q * j) % p);
                            T wr = r[e].re, wi = isign > 0 ? r[e].im : -r[e].im;
                            sr += vr[q] * wr - vi[q] * wi;
                            si += vr[q] * wi + vi[q] * wr;
                        }
                        if (j > 0) {
                            Cx<T> w = t[(j - 1) * ido + i];
                            T wr = w.re, wi = isign > 0 ? w.im : -w.im;
                            T xr = sr * wr - si * wi;
                            T xi = sr * wi + si * wr;
                            sr = xr;
                            si = xi;
                        }
                        // ch(i, k, j) = out[i + ido*k + ido*l1*j]
                        i64 o = i + ido * k + ido * l1 * j;
                        out[2 * o] = sr;
                        out[2 * o + 1] = si;
                    }
                }
            }
            std::swap(in, out);
            l1 = l2;
        }
        if (in != a) std::memcpy(a, in, sizeof(T) * 2 * n);
    }
};

// ---------------------------------------------------------------------------
// 1D FFT plan (DoubleFFT_1D / FloatFFT_1D).
// ---------------------------------------------------------------------------
template <class T> struct FFT1D {
    i64 n = 0;
    PlanKind kind = SPLIT_RADIX;
    SplitTable<T> tab;       // e^{+i} table of the complex (n) / Bluestein (nB) size
    std::vector<T> c;        // makect table, nc = n/4
    i64 nc = 0;
    MixedPlan<T> mixed;
    i64 nB = 0;
    std::vector<T> bk1, bk2;

    explicit FFT1D(i64 n_) : n(n_) {
        if (n < 1) throw std::invalid_argument("n must be greater than 0");
        kind = choose_plan(n);
        if (kind == SPLIT_RADIX) {
            tab.build(n);
            nc = n >> 2;
            c = makect<T>(nc);
        } else if (kind == MIXED_RADIX) {
            mixed.build(n);
        } else {
            nB = next_pow2(2 * n - 1);
            tab.build(nB);
            bluesteini();
        }
    }

    // bluesteini (fft/DoubleFFT_1D.java:1864-1890; float angles as
    // fft/FloatFFT_1D.java:1866-1890).
    void bluesteini() {
        bk1.assign(2 * n, 0);
        bk2.assign(2 * nB, 0);
        i64 k = 0;
        T pi_n = (T)3.14159265358979311599796346854418516 / (T)n;
        bk1[0] = 1;
        bk1[1] = 0;
        for (i64 i = 1; i < n; i++) {
            k += 2 * i - 1;
            if (k >= 2 * n) k -= 2 * n;
            T arg = pi_n * (T)k;
            bk1[2 * i] = (T)std::cos((double)arg);
            bk1[2 * i + 1] = (T)std::sin((double)arg);
        }
        T sc = (T)1.0 / (T)nB;
        bk2[0] = bk1[0] * sc;
        bk2[1] = bk1[1] * sc;
        for (i64 i = 2; i < 2 * n; i += 2) {
            bk2[i] = bk1[i] * sc;
            bk2[i + 1] = bk1[i + 1] * sc;
            bk2[2 * nB - i] = bk2[i];
            bk2[2 * nB - i + 1] = bk2[i + 1];
        }
        cft(bk2.data(), nB, -1, tab);
    }

    // bluestein_complex (fft/DoubleFFT_1D.java:1920-2107), serial branch.
    void bluestein_complex(T *a, int isign) const {
        std::vector<T> ak(2 * nB, 0);
        if (isign > 0) {
            for (i64 i = 0; i < n; i++) {
                ak[2 * i] = a[2 * i] * bk1[2 * i] - a[2 * i + 1] * bk1[2 * i + 1];
                ak[2 * i + 1] = a[2 * i] * bk1[2 * i + 1] + a[2 * i + 1] * bk1[2 * i];
            }
        } else {
            for (i64 i = 0; i < n; i++) {
                ak[2 * i] = a[2 * i] * bk1[2 * i] + a[2 * i + 1] * bk1[2 * i + 1];
                ak[2 * i + 1] = -a[2 * i] * bk1[2 * i + 1] + a[2 * i + 1] * bk1[2 * i];
            }
        }
        cft(ak.data(), nB, -1, tab);
        if (isign > 0) {
            for (i64 i = 0; i < nB; i++) {
                T im = -ak[2 * i] * bk2[2 * i + 1] + ak[2 * i + 1] * bk2[2 * i];
                ak[2 * i] = ak[2 * i] * bk2[2 * i] + ak[2 * i + 1] * bk2[2 * i + 1];
                ak[2 * i + 1] = im;
            }
        } else {
            for (i64 i = 0; i < nB; i++) {
                T im = ak[2 * i] * bk2[2 * i + 1] + ak[2 * i + 1] * bk2[2 * i];
                ak[2 * i] = ak[2 * i] * bk2[2 * i] - ak[2 * i + 1] * bk2[2 * i + 1];
                ak[2 * i + 1] = im;
            }
        }
        cft(ak.data(), nB, +1, tab);
        if (isign > 0) {
            for (i64 i = 0; i < n; i++) {
                a[2 * i] = bk1[2 * i] * ak[2 * i] - bk1[2 * i + 1] * ak[2 * i + 1];
                a[2 * i + 1] = bk1[2 * i + 1] * ak[2 * i] + bk1[2 * i] * ak[2 * i + 1];
            }
        } else {
            for (i64 i = 0; i < n; i++) {
                a[2 * i] = bk1[2 * i] * ak[2 * i] + bk1[2 * i + 1] * ak[2 * i + 1];
                a[2 * i + 1] = -bk1[2 * i + 1] * ak[2 * i] + bk1[2 * i] * ak[2 * i + 1];
            }
        }
    }

    // Unnormalized complex transform with the plan's algorithm, isign=-1
    // forward (e^{-i}), +1 backward.
    void complex_raw(T *a, int isign) const {
        if (n == 1) return;
        switch (kind) {
            case SPLIT_RADIX: cft(a, n, isign, tab); break;
            case MIXED_RADIX: mixed.run(a, isign); break;
            case BLUESTEIN: bluestein_complex(a, isign); break;
        }
    }

    // complexForward (fft/DoubleFFT_1D.java:243-265).
    void complexForward(T *a) const { complex_raw(a, -1); }

    // complexInverse (fft/DoubleFFT_1D.java:362-386).
    void complexInverse(T *a, bool sc) const {
        if (n == 1) return;
        complex_raw(a, +1);
        if (sc) scale_arr<T>(2 * n, (T)1.0 / (T)n, a);
    }

    // Packs a full spectrum F (2n values) into JTransforms' realForward
    // layout (fft/DoubleFFT_1D.java:433-451).
    void pack(const T *F, T *a) const {
        a[0] = F[0];
        if (n % 2 == 0) {
            a[1] = F[n];  // Re[n/2]
            for (i64 k = 1; k < n / 2; k++) { a[2 * k] = F[2 * k]; a[2 * k + 1] = F[2 * k + 1]; }
        } else {
            i64 h = (n - 1) / 2;
            a[1] = F[2 * h + 1];  // Im[(n-1)/2]
            for (i64 k = 1; k < h; k++) { a[2 * k] = F[2 * k]; a[2 * k + 1] = F[2 * k + 1]; }
            a[2 * h] = F[2 * h];
        }
    }
    // Full Hermitian spectrum from the packed layout.
    void unpack(const T *a, T *F) const {
        F[0] = a[0];
        F[1] = 0;
        i64 m = (n % 2 == 0) ? n / 2 : (n + 1) / 2;
        for (i64 k = 1; k < m; k++) {
            T re = a[2 * k], im;
            if (n % 2 == 1 && k == m - 1) im = a[1];
            else im = a[2 * k + 1];
            F[2 * k] = re; F[2 * k + 1] = im;
            F[2 * (n - k)] = re; F[2 * (n - k) + 1] = -im;
        }
        if (n % 2 == 0) { F[n] = a[1]; F[n + 1] = 0; }
    }

    // realForward (fft/DoubleFFT_1D.java:524-561).
    void realForward(T *a) const {
        if (n == 1) return;
        if (kind == SPLIT_RADIX) {
            if (n > 4) {
                cft(a, n / 2, +1, tab);
                rftfsub<T>(n, a, nc, c.data());
            } else if (n == 4) {
                // cftx020 (utils/CommonUtils.java:5682-5691)
                T x0r = a[0] - a[2], x0i = -a[1] + a[3];
                a[0] += a[2];
                a[1] += a[3];
                a[2] = x0r;
                a[3] = x0i;
            }
            T xi = a[0] - a[1];
            a[0] += a[1];
            a[1] = xi;
        } else {
            std::vector<T> F(2 * n);
            for (i64 i = 0; i < n; i++) { F[2 * i] = a[i]; F[2 * i + 1] = 0; }
            complex_raw(F.data(), -1);
            pack(F.data(), a);
        }
    }

    // realForwardFull (fft/DoubleFFT_1D.java:678-755).
    void realForwardFull(T *a) const {
        if (kind == SPLIT_RADIX) {
            realForward(a);
            i64 twon = 2 * n;
            for (i64 k = 0; k < n / 2; k++) {
                i64 i1 = 2 * k, i2 = (twon - i1) % twon;
                a[i2] = a[i1];
                a[i2 + 1] = -a[i1 + 1];
            }
            a[n] = -a[1];
            a[1] = 0;
        } else {
            std::vector<T> F(2 * n);
            for (i64 i = 0; i < n; i++) { F[2 * i] = a[i]; F[2 * i + 1] = 0; }
            complex_raw(F.data(), -1);
            std::memcpy(a, F.data(), sizeof(T) * 2 * n);
        }
    }

    // realInverse (fft/DoubleFFT_1D.java:946-989).  Unscaled output is
    // (n/2)*x on the split-radix plan and n*x otherwise.
    void realInverse(T *a, bool sc) const {
        if (n == 1) return;
        if (kind == SPLIT_RADIX) {
            a[1] = (T)0.5 * (a[0] - a[1]);
            a[0] -= a[1];
            if (n > 4) {
                rftfsub<T>(n, a, nc, c.data());
                cft(a, n / 2, -1, tab);
            } else if (n == 4) {
                // cftxc020 (utils/CommonUtils.java:5728-5737)
                T x0r = a[0] - a[2], x0i = a[1] + a[3];
                a[0] += a[2];
                a[1] -= a[3];
                a[2] = x0r;
                a[3] = x0i;
            }
            if (sc) scale_arr<T>(n, (T)1.0 / ((T)n / (T)2.0), a);
        } else {
            std::vector<T> F(2 * n);
            unpack(a, F.data());
            complex_raw(F.data(), +1);
            for (i64 i = 0; i < n; i++) a[i] = F[2 * i];
            if (sc) scale_arr<T>(n, (T)1.0 / (T)n, a);
        }
    }

    // realInverse2 (fft/DoubleFFT_1D.java:1297-1355): packed layout of
    // sum x_j e^{+2 pi i jk/n}, scaled by 1/n if sc.
    void realInverse2(T *a, bool sc) const {
        if (n == 1) return;
        if (kind == SPLIT_RADIX) {
            if (n > 4) {
                cft(a, n / 2, +1, tab);
                rftbsub<T>(n, a, nc, c.data());
            } else if (n == 4) {
                cft(a, 2, -1, tab);
            }
            T xi = a[0] - a[1];
            a[0] += a[1];
            a[1] = xi;
            if (sc) scale_arr<T>(n, (T)1.0 / (T)n, a);
        } else {
            std::vector<T> F(2 * n);
            for (i64 i = 0; i < n; i++) { F[2 * i] = a[i]; F[2 * i + 1] = 0; }
            complex_raw(F.data(), +1);
            pack(F.data(), a);
            if (sc) scale_arr<T>(n, (T)1.0 / (T)n, a);
        }
    }

    // realInverseFull (fft/DoubleFFT_1D.java:1112-1195).
    void realInverseFull(T *a, bool sc) const {
        if (kind == SPLIT_RADIX) {
            realInverse2(a, sc);
            i64 twon = 2 * n;
            for (i64 k = 0; k < n / 2; k++) {
                i64 i1 = 2 * k, i2 = (twon - i1) % twon;
                a[i2] = a[i1];
                a[i2 + 1] = -a[i1 + 1];
            }
            a[n] = -a[1];
            a[1] = 0;
        } else {
            std::vector<T> F(2 * n);
            for (i64 i = 0; i < n; i++) { F[2 * i] = a[i]; F[2 * i + 1] = 0; }
            complex_raw(F.data(), +1);
            if (sc) scale_arr<T>(2 * n, (T)1.0 / (T)n, F.data());
            std::memcpy(a, F.data(), sizeof(T) * 2 * n);
        }
    }
};

// ---------------------------------------------------------------------------
// DCT / DST / DHT 1D.
// ---------------------------------------------------------------------------
template <class T> struct DCT1D {
    i64 n;
    bool pow2;
    // power of two: makewt/makect tables with nc = n (dct/DoubleDCT_1D.java:93-107)
    SplitTable<T> tab;
    std::vector<T> c;
    i64 nc = 0;
    // otherwise: w = makect(n) (dct/DoubleDCT_1D.java:523-538), 2n real FFT
    std::vector<T> w;
    FFT1D<T> *fft = nullptr;

    explicit DCT1D(i64 n_) : n(n_) {
        if (n < 1) throw std::invalid_argument("n must be greater than 0");
        pow2 = is_pow2(n);
        if (pow2) {
            tab.build(std::max<i64>(n / 2, 1));
            nc = n;
            c = makect<T>(nc);
        } else {
            w.assign(2 * n, 0);
            T delta = (T)3.14159265358979311599796346854418516 / (T)(2 * n);
            w[0] = 1;
            for (i64 j = 1; j < n; j++) {
                T dj = delta * (T)j;
                w[2 * j] = (T)std::cos((double)dj);
                w[2 * j + 1] = -(T)std::sin((double)dj);
            }
            fft = new FFT1D<T>(2 * n);
        }
    }
    ~DCT1D() { delete fft; }
    DCT1D(const DCT1D &) = delete;

    // forward (dct/DoubleDCT_1D.java:169-243)
    void forward(T *a, bool sc) const {
        if (n == 1) return;
        if (pow2) {
            T xr = a[n - 1];
            for (i64 j = n - 2; j >= 2; j -= 2) {
                a[j + 1] = a[j] - a[j - 1];
                a[j] += a[j - 1];
            }
            a[1] = a[0] - xr;
            a[0] += xr;
            if (n > 4) {
                dct_rftbsub<T>(n, a, nc, c.data());
                cft(a, n / 2, -1, tab);
            } else if (n == 4) {
                cft(a, 2, -1, tab);
            }
            dctsub<T>(n, a, nc, c.data());
            if (sc) {
                scale_arr<T>(n, (T)std::sqrt(2.0 / (double)n), a);
                a[0] = a[0] / (T)std::sqrt(2.0);
            }
        } else {
            i64 twon = 2 * n;
            std::vector<T> t(twon);
            std::memcpy(t.data(), a, sizeof(T) * n);
            for (i64 i = n; i < twon; i++) t[i] = t[twon - i - 1];
            fft->realForward(t.data());
            for (i64 i = 0; i < n; i++) a[i] = w[2 * i] * t[2 * i] - w[2 * i + 1] * t[2 * i + 1];
            if (sc) {
                scale_arr<T>(n, (T)(1.0 / std::sqrt((double)twon)), a);
                a[0] = a[0] / (T)std::sqrt(2.0);
            }
        }
    }

    // inverse (dct/DoubleDCT_1D.java:361-440)
    void inverse(T *a, bool sc) const {
        if (n == 1) return;
        if (pow2) {
            if (sc) {
                scale_arr<T>(n, (T)std::sqrt(2.0 / (double)n), a);
                a[0] = a[0] / (T)std::sqrt(2.0);
            }
            dctsub<T>(n, a, nc, c.data());
            if (n > 4) {
                cft(a, n / 2, +1, tab);
                rftbsub<T>(n, a, nc, c.data());  // the DCT's private rftfsub
            } else if (n == 4) {
                cft(a, 2, +1, tab);
            }
            T xr = a[0] - a[1];
            a[0] += a[1];
            for (i64 j = 2; j < n; j += 2) {
                a[j - 1] = a[j] - a[j + 1];
                a[j] += a[j + 1];
            }
            a[n - 1] = xr;
        } else {
            i64 twon = 2 * n;
            if (sc) {
                scale_arr<T>(n, (T)std::sqrt((double)twon), a);
                a[0] = a[0] * (T)std::sqrt(2.0);
            }
            std::vector<T> t(twon);
            for (i64 i = 0; i < n; i++) {
                T e = a[i];
                t[2 * i] = w[2 * i] * e;
                t[2 * i + 1] = -w[2 * i + 1] * e;
            }
            fft->realInverse(t.data(), true);
            std::memcpy(a, t.data(), sizeof(T) * n);
        }
    }
};

template <class T> struct DST1D {
    i64 n;
    DCT1D<T> dct;
    explicit DST1D(i64 n_) : n(n_), dct(n_) {}
    // forward (dst/DoubleDST_1D.java:96-160)
    void forward(T *a, bool sc) const {
        if (n == 1) return;
        for (i64 i = 1; i < n; i += 2) a[i] = -a[i];
        dct.forward(a, sc);
        for (i64 i = 0; i < n / 2; i++) std::swap(a[i], a[n - 1 - i]);
    }
    // inverse (dst/DoubleDST_1D.java:264-328)
    void inverse(T *a, bool sc) const {
        if (n == 1) return;
        for (i64 i = 0; i < n / 2; i++) std::swap(a[i], a[n - 1 - i]);
        dct.inverse(a, sc);
        for (i64 i = 1; i < n; i += 2) a[i] = -a[i];
    }
};

template <class T> struct DHT1D {
    i64 n;
    FFT1D<T> fft;
    explicit DHT1D(i64 n_) : n(n_), fft(n_) {}
    // forward (dht/DoubleDHT_1D.java:94-159)
    void forward(T *a) const {
        if (n == 1) return;
        fft.realForward(a);
        std::vector<T> b(a, a + n);
        i64 nd2 = n / 2;
        for (i64 i = 1; i < nd2; i++) {
            a[i] = b[2 * i] - b[2 * i + 1];
            a[n - i] = b[2 * i] + b[2 * i + 1];
        }
        if (n % 2 == 0) {
            a[nd2] = b[1];
        } else {
            a[nd2] = b[n - 1] - b[1];
            a[nd2 + 1] = b[n - 1] + b[1];
        }
    }
    // inverse (dht/DoubleDHT_1D.java:255-276)
    void inverse(T *a, bool sc) const {
        if (n == 1) return;
        forward(a);
        if (sc) scale_arr<T>(n, (T)1.0 / (T)n, a);
    }
};

// ---------------------------------------------------------------------------
// nD drivers.  Layout: row-major, last dimension contiguous.
// ---------------------------------------------------------------------------
// Applies f to every line of a real (cw = 1) or complex (cw = 2) array
// along axis `ax` of dims[0..nd).
template <class T, class F>
void for_lines(T *a, int nd, const i64 *dims, int ax, int cw, F f) {
    i64 len = dims[ax];
    i64 inner = 1, outer = 1;
    for (int d = ax + 1; d < nd; d++) inner *= dims[d];
    for (int d = 0; d < ax; d++) outer *= dims[d];
    std::vector<T> t(cw * len);
    for (i64 o = 0; o < outer; o++)
        for (i64 in = 0; in < inner; in++) {
            T *base = a + cw * (o * len * inner + in);
            for (i64 j = 0; j < len; j++)
                for (int q = 0; q < cw; q++) t[cw * j + q] = base[cw * j * inner + q];
            f(t.data());
            for (i64 j = 0; j < len; j++)
                for (int q = 0; q < cw; q++) base[cw * j * inner + q] = t[cw * j + q];
        }
}

// complexForward / complexInverse, 2D (fft/DoubleFFT_2D.java:115-400) and
// 3D (fft/DoubleFFT_3D.java:145-540): one 1D pass per dimension.
template <class T> void fftnd_complex(T *a, int nd, const i64 *dims, int isign, bool sc) {
    for (int ax = nd - 1; ax >= 0; ax--) {
        FFT1D<T> f(dims[ax]);
        for_lines<T>(a, nd, dims, ax, 2, [&](T *t) {
            if (isign < 0) f.complexForward(t); else f.complexInverse(t, sc);
        });
    }
}

// realForward 2D, power-of-two sizes (fft/DoubleFFT_2D.java:816-841):
// row realForward, column complexForward on the packed pairs, rdft2d_sub(1).
template <class T> void fft2d_real_forward(T *a, i64 rows, i64 cols) {
    FFT1D<T> fc(cols), fr(rows);
    for (i64 r = 0; r < rows; r++) fc.realForward(a + r * cols);
    i64 dims[2] = {rows, cols / 2};
    for_lines<T>(a, 2, dims, 0, 2, [&](T *t) { fr.complexForward(t); });
    // rdft2d_sub(1, a) (fft/DoubleFFT_2D.java:2544-2575)
    i64 n1h = rows >> 1;
    for (i64 i = 1; i < n1h; i++) {
        i64 j = rows - i, i1 = i * cols, i2 = j * cols;
        a[i2] = (T)0.5f * (a[i1] - a[i2]);
        a[i1] -= a[i2];
        a[i2 + 1] = (T)0.5f * (a[i1 + 1] + a[i2 + 1]);
        a[i1 + 1] -= a[i2 + 1];
    }
}

// realInverse 2D, power-of-two sizes (fft/DoubleFFT_2D.java:1077-1095).
template <class T> void fft2d_real_inverse(T *a, i64 rows, i64 cols, bool sc) {
    FFT1D<T> fc(cols), fr(rows);
    i64 n1h = rows >> 1;
    for (i64 i = 1; i < n1h; i++) {
        i64 j = rows - i, i1 = i * cols, i2 = j * cols;
        T xi = a[i1] - a[i2];
        a[i1] += a[i2];
        a[i2] = xi;
        xi = a[i2 + 1] - a[i1 + 1];
        a[i1 + 1] += a[i2 + 1];
        a[i2 + 1] = xi;
    }
    i64 dims[2] = {rows, cols / 2};
    for_lines<T>(a, 2, dims, 0, 2, [&](T *t) { fr.complexInverse(t, sc); });
    for (i64 r = 0; r < rows; r++) fc.realInverse(a + r * cols, sc);
}

// rdft3d_sub (fft/DoubleFFT_3D.java:6909-7021): combines the (slice, row)
// mirror pairs of the packed columns 0 and 1.  Each pair is (x, y): forward
// (isgn >= 0) y = (x - y)/2, x -= y on the real part and y = (x + y)/2,
// x -= y on the imaginary part; inverse (isgn < 0) x, y = x + y, x - y and
// x', y' = x' + y', y' - x'.
template <class T> void rdft3d_sub(T *a, i64 slices, i64 rows, i64 cols, int isgn) {
    const i64 n1h = slices >> 1, n2h = rows >> 1, ss = rows * cols, rs = cols;
    auto pair = [&](i64 x, i64 y) {
        if (isgn >= 0) {
            a[y] = (T)0.5f * (a[x] - a[y]);
            a[x] -= a[y];
            a[y + 1] = (T)0.5f * (a[x + 1] + a[y + 1]);
            a[x + 1] -= a[y + 1];
        } else {
            T t = a[x] - a[y];
            a[x] += a[y];
            a[y] = t;
            t = a[y + 1] - a[x + 1];
            a[x + 1] += a[y + 1];
            a[y + 1] = t;
        }
    };
    for (i64 i = 1; i < n1h; i++) {
        const i64 j = slices - i;
        pair(i * ss, j * ss);
        pair(i * ss + n2h * rs, j * ss + n2h * rs);
        for (i64 k = 1; k < n2h; k++) {
            const i64 l = rows - k;
            pair(i * ss + k * rs, j * ss + l * rs);
            pair(j * ss + k * rs, i * ss + l * rs);
        }
    }
    for (i64 k = 1; k < n2h; k++) {
        const i64 l = rows - k;
        pair(k * rs, l * rs);
        pair(n1h * ss + k * rs, n1h * ss + l * rs);
    }
}

// realForward 3D, power-of-two sizes (fft/DoubleFFT_3D.java:1339-1356):
// row realForward, complexForward along rows then along slices on the
// packed pairs (xdft3da_sub1(1, -1), cdft3db_sub(-1)), rdft3d_sub(1).
template <class T> void fft3d_real_forward(T *a, i64 slices, i64 rows, i64 cols) {
    FFT1D<T> fc(cols), fr(rows), fs(slices);
    for (i64 r = 0; r < slices * rows; r++) fc.realForward(a + r * cols);
    i64 dims[3] = {slices, rows, cols / 2};
    for_lines<T>(a, 3, dims, 1, 2, [&](T *t) { fr.complexForward(t); });
    for_lines<T>(a, 3, dims, 0, 2, [&](T *t) { fs.complexForward(t); });
    rdft3d_sub<T>(a, slices, rows, cols, 1);
}

// realInverse 3D (fft/DoubleFFT_3D.java:1629-1645): rdft3d_sub(-1),
// complexInverse along slices then rows, row realInverse.
template <class T> void fft3d_real_inverse(T *a, i64 slices, i64 rows, i64 cols, bool sc) {
    FFT1D<T> fc(cols), fr(rows), fs(slices);
    rdft3d_sub<T>(a, slices, rows, cols, -1);
    i64 dims[3] = {slices, rows, cols / 2};
    for_lines<T>(a, 3, dims, 0, 2, [&](T *t) { fs.complexInverse(t, sc); });
    for_lines<T>(a, 3, dims, 1, 2, [&](T *t) { fr.complexInverse(t, sc); });
    for (i64 r = 0; r < slices * rows; r++) fc.realInverse(a + r * cols, sc);
}

// realForwardFull / realInverseFull nD: the full complex transform of the
// real input stored in the first N slots, result in 2N slots.
template <class T> void fftnd_real_full(T *a, int nd, const i64 *dims, int isign, bool sc) {
    i64 N = 1;
    for (int d = 0; d < nd; d++) N *= dims[d];
    std::vector<T> t(2 * N);
    for (i64 i = 0; i < N; i++) { t[2 * i] = a[i]; t[2 * i + 1] = 0; }
    fftnd_complex<T>(t.data(), nd, dims, isign, sc);
    std::memcpy(a, t.data(), sizeof(T) * 2 * N);
}

// DCT/DST nD: the 1D transform along every dimension
// (dct/DoubleDCT_2D.java:104-190, dst/DoubleDST_3D.java:132-290).
template <class T> void dctnd(T *a, int nd, const i64 *dims, int fwd, bool sc, bool sine) {
    for (int ax = nd - 1; ax >= 0; ax--) {
        if (sine) {
            DST1D<T> t1(dims[ax]);
            for_lines<T>(a, nd, dims, ax, 1, [&](T *t) { if (fwd) t1.forward(t, sc); else t1.inverse(t, sc); });
        } else {
            DCT1D<T> t1(dims[ax]);
            for_lines<T>(a, nd, dims, ax, 1, [&](T *t) { if (fwd) t1.forward(t, sc); else t1.inverse(t, sc); });
        }
    }
}

// DHT 2D: separable DHT then yTransform (dht/DoubleDHT_2D.java:102-184, :1288-1310).
template <class T> void dht_ytransform2(T *a, i64 rows, i64 cols) {
    for (i64 r = 0; r <= rows / 2; r++) {
        i64 mRow = (rows - r) % rows, i1 = r * cols, i2 = mRow * cols;
        for (i64 c = 0; c <= cols / 2; c++) {
            i64 mCol = (cols - c) % cols;
            T A = a[i1 + c], B = a[i2 + c], C = a[i1 + mCol], D = a[i2 + mCol];
            T E = ((A + D) - (B + C)) / (T)2;
            a[i1 + c] = A - E;
            a[i2 + c] = B + E;
            a[i1 + mCol] = C + E;
            a[i2 + mCol] = D - E;
        }
    }
}

// DHT 3D yTransform (dht/DoubleDHT_3D.java:2314-2356).
template <class T> void dht_ytransform3(T *a, i64 slices, i64 rows, i64 cols) {
    i64 ss = rows * cols, rs = cols;
    for (i64 s = 0; s <= slices / 2; s++) {
        i64 sC = (slices - s) % slices, i9 = s * ss, i10 = sC * ss;
        for (i64 r = 0; r <= rows / 2; r++) {
            i64 rC = (rows - r) % rows, i11 = r * rs, i12 = rC * rs;
            for (i64 c = 0; c <= cols / 2; c++) {
                i64 cC = (cols - c) % cols;
                i64 x1 = i9 + i12 + c, x2 = i9 + i11 + cC, x3 = i10 + i11 + c, x4 = i10 + i12 + cC;
                i64 x5 = i10 + i12 + c, x6 = i10 + i11 + cC, x7 = i9 + i11 + c, x8 = i9 + i12 + cC;
                T A = a[x1], B = a[x2], C = a[x3], D = a[x4], E = a[x5], F = a[x6], G = a[x7], H = a[x8];
                a[x7] = (A + B + C - D) / (T)2;
                a[x3] = (E + F + G - H) / (T)2;
                a[x1] = (G + H + E - F) / (T)2;
                a[x5] = (C + D + A - B) / (T)2;
                a[x2] = (H + G + F - E) / (T)2;
                a[x6] = (D + C + B - A) / (T)2;
                a[x8] = (B + A + D - C) / (T)2;
                a[x4] = (F + E + H - G) / (T)2;
            }
        }
    }
}

template <class T> void dhtnd(T *a, int nd, const i64 *dims, int fwd, bool sc) {
    for (int ax = nd - 1; ax >= 0; ax--) {
        DHT1D<T> t1(dims[ax]);
        for_lines<T>(a, nd, dims, ax, 1, [&](T *t) { t1.forward(t); });
    }
    if (nd == 2) dht_ytransform2<T>(a, dims[0], dims[1]);
    if (nd == 3) dht_ytransform3<T>(a, dims[0], dims[1], dims[2]);
    if (!fwd && sc) {
        i64 N = 1;
        for (int d = 0; d < nd; d++) N *= dims[d];
        scale_arr<T>(N, (T)1.0 / (T)N, a);
    }
}

// Operation codes shared with include/jtgpu.h.
enum Op {
    OP_COMPLEX_FORWARD = 0, OP_COMPLEX_INVERSE = 1, OP_REAL_FORWARD = 2,
    OP_REAL_FORWARD_FULL = 3, OP_REAL_INVERSE = 4, OP_REAL_INVERSE_FULL = 5,
    OP_FORWARD = 6, OP_INVERSE = 7
};
enum Kind { K_FFT = 0, K_DCT = 1, K_DST = 2, K_DHT = 3 };

template <class T> int run_one(int kind, int op, int nd, const i64 *dims, T *a, int sc) {
    if (nd < 1 || nd > 3) return -1;
    for (int d = 0; d < nd; d++) if (dims[d] < 1) return -1;
    bool s = sc != 0;
    if (kind == K_FFT) {
        if (nd == 1) {
            FFT1D<T> f(dims[0]);
            switch (op) {
                case OP_COMPLEX_FORWARD: f.complexForward(a); break;
                case OP_COMPLEX_INVERSE: f.complexInverse(a, s); break;
                case OP_REAL_FORWARD: f.realForward(a); break;
                case OP_REAL_FORWARD_FULL: f.realForwardFull(a); break;
                case OP_REAL_INVERSE: f.realInverse(a, s); break;
                case OP_REAL_INVERSE_FULL: f.realInverseFull(a, s); break;
                default: return -1;
            }
            return 0;
        }
        switch (op) {
            case OP_COMPLEX_FORWARD: fftnd_complex<T>(a, nd, dims, -1, false); return 0;
            case OP_COMPLEX_INVERSE: fftnd_complex<T>(a, nd, dims, +1, s); return 0;
            case OP_REAL_FORWARD_FULL: fftnd_real_full<T>(a, nd, dims, -1, false); return 0;
            case OP_REAL_INVERSE_FULL: fftnd_real_full<T>(a, nd, dims, +1, s); return 0;
            case OP_REAL_FORWARD:
            case OP_REAL_INVERSE:
                for (int d = 0; d < nd; d++)
                    if (!is_pow2(dims[d])) return -3;
                if (nd == 2) {
                    if (op == OP_REAL_FORWARD) fft2d_real_forward<T>(a, dims[0], dims[1]);
                    else fft2d_real_inverse<T>(a, dims[0], dims[1], s);
                } else {
                    if (op == OP_REAL_FORWARD) fft3d_real_forward<T>(a, dims[0], dims[1], dims[2]);
                    else fft3d_real_inverse<T>(a, dims[0], dims[1], dims[2], s);
                }
                return 0;
            default: return -1;
        }
    }
    if (op != OP_FORWARD && op != OP_INVERSE) return -1;
    int fwd = op == OP_FORWARD;
    if (kind == K_DCT) { dctnd<T>(a, nd, dims, fwd, s, false); return 0; }
    if (kind == K_DST) { dctnd<T>(a, nd, dims, fwd, s, true); return 0; }
    if (kind == K_DHT) { dhtnd<T>(a, nd, dims, fwd, s); return 0; }
    return -1;
}

// Batched driver: `batch` arrays at a stride of `stride` elements, spread
// over `threads` OpenMP threads (one transform per task), as the reference's
// benchmark runs independent transforms on a thread pool.
template <class T> int run_batch(int kind, int op, int nd, const i64 *dims, T *a, i64 batch, i64 stride, int sc, int threads) {
    int err = 0;
#ifdef _OPENMP
    if (threads < 1) threads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 1) num_threads(threads) reduction(min : err)
#endif
    for (i64 b = 0; b < batch; b++) {
        int e = run_one<T>(kind, op, nd, dims, a + b * stride, sc);
        if (e < err) err = e;
    }
    return err;
}

}  // namespace

extern "C" {

// Returns the plan kind the reference would choose for a 1D size.
int jto_plan_kind(int64_t n) { return (int)choose_plan(n); }
int64_t jto_bluestein_size(int64_t n) { return next_pow2(2 * n - 1); }
int jto_fftpack_factors(int64_t n, int *out, int cap) {
    auto f = fftpack_factors(n);
    for (size_t i = 0; i < f.size() && (int)i < cap; i++) out[i] = f[i];
    return (int)f.size();
}

int jto_run_d(int kind, int op, int nd, const int64_t *dims, double *a, int scale) {
    try { return run_one<double>(kind, op, nd, dims, a, scale); } catch (...) { return -1; }
}
int jto_run_f(int kind, int op, int nd, const int64_t *dims, float *a, int scale) {
    try { return run_one<float>(kind, op, nd, dims, a, scale); } catch (...) { return -1; }
}
int jto_batch_d(int kind, int op, int nd, const int64_t *dims, double *a, int64_t batch, int64_t stride, int scale, int threads) {
    try { return run_batch<double>(kind, op, nd, dims, a, batch, stride, scale, threads); } catch (...) { return -1; }
}
int jto_batch_f(int kind, int op, int nd, const int64_t *dims, float *a, int64_t batch, int64_t stride, int scale, int threads) {
    try { return run_batch<float>(kind, op, nd, dims, a, batch, stride, scale, threads); } catch (...) { return -1; }
}
int jto_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

}  // extern "C"
