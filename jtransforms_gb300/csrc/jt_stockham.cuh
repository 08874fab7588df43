// jt_stockham.cuh -- power-of-two complex FFT lines held in registers.
//
// One CTA transforms C lines of compile-time length L.  Each thread owns
// E = 16 elements of one line (t, t+TL, ..., t+15*TL with TL = L/16): the
// radix-16 butterflies of a pass run in registers and shared memory is used
// only to exchange data between passes (self-sorting Stockham order, so the
// result comes out in natural order with no bit reversal).  Three layouts:
//   MODE 0  rows in, rows out        (contiguous lines)
//   MODE 1  columns in, columns out  (C adjacent columns per tile), optional
//           four-step twiddle fused into the store
//   MODE 2  rows in, columns out     (the transposing row pass of the
//           four-step scheme; lines are spread across a warp, so one store
//           instruction writes C adjacent columns)
//
// stockham_pipe_kernel is the main kernel: persistent CTAs walk their tiles
// and the next tile is already in flight while the current one is computed.
// TMA brings it into a second shared-memory stage: one cp.async.bulk per
// contiguous run of rows (MODE 0/2) or cp.async.bulk.tensor boxes of
// C columns x up to 256 rows (MODE 1), completing on an mbarrier.  Every
// mbarrier wait is bounded; on timeout the kernel raises the error flag,
// drains its copies (bounded) and returns.  The passes exchange through the
// stage buffer itself, in padded rows (one spare slot per 16 elements).
// stockham_kernel is the plain (non-TMA) variant for arrays whose addresses
// or strides do not meet TMA's 16-byte rules.
#pragma once

#include "jt_device.cuh"
#include "jt_tma.cuh"

namespace jt {

__host__ __device__ constexpr int ilog2c(int x) { return x <= 1 ? 0 : 1 + ilog2c(x >> 1); }
__host__ __device__ constexpr int ipowc(int b, int e) { return e == 0 ? 1 : b * ipowc(b, e - 1); }

struct StockParams {
    int64_t nlines;
    Layout lin, lout;
    double scale;  // output multiplier (double plans)
    float scalef;  // the same for float plans: float kernels do no FP64 work
    int do_scale;
    int64_t tw_n, tw_inner;  // four-step output twiddle w_{tw_n}^{pos * (b % tw_inner)}; tw_n = 0: none
    int tw_lo_bits;
    uint32_t tw_mask;        // exponent reduction: tw_n - 1 for a power of two up to 2^32, else all ones
    int64_t tiles_per_col;   // MODE 1 pipe: column tiles per outer block (inner / C)
    int discard_in;          // MODE 2 pipe: the input is a dead intermediate (drop it from L2)
    int stream_out;          // outputs are not re-read soon: streaming stores
    int reverse;             // pipe: walk the tiles last to first (the input's freshest part is in L2)
};

// w_{tw_n}^x from the two-level table.  x is formed in 32-bit unsigned
// arithmetic: for a power-of-two tw_n up to 2^32 the wrap keeps x mod tw_n
// and the mask finishes the reduction; other lengths stay below 2^31.
template <typename T>
__device__ __forceinline__ typename V2<T>::t tw_lookup(const typename V2<T>::t *__restrict__ Whi,
                                                      const typename V2<T>::t *__restrict__ Wlo, uint32_t x,
                                                      const StockParams &p) {
    x &= p.tw_mask;
    return cmul<T>(__ldg(&Whi[x >> p.tw_lo_bits]), __ldg(&Wlo[x & ((1u << p.tw_lo_bits) - 1u)]));
}

template <typename T> __device__ __forceinline__ T param_scale(const StockParams &p) {
    if constexpr (sizeof(T) == 4) return p.scalef;
    else return (T)p.scale;
}

template <typename T> struct StockCfg {
    // lines per CTA for the row mode: about 256 threads
    static constexpr int rows_C(int L) { return L >= 4096 ? 1 : 4096 / L; }
    // lines per CTA for the column modes: 128-byte row segments when the
    // line is short, at least one 32-byte sector when it is long
    static constexpr int cols_C(int L) {
        return sizeof(T) == 4 ? (L <= 512 ? 16 : 8192 / L)
                              : (L <= 256 ? 8 : (4096 / L < 2 ? 2 : 4096 / L));
    }
    // the transposing pass (MODE 2) reads rows and stores from registers.
    // At L <= 512 it takes 8 lines: its half-warps then span two positions,
    // so the input rows are read without bank conflicts (64-byte output
    // segments).  At 1024 it takes 4 (32-byte segments, which merge in L2):
    // three CTAs per SM instead of one
    static constexpr int rows2_C(int L) {
        return sizeof(T) == 4 ? (L <= 512 ? 8 : L == 1024 ? 4 : cols_C(L)) : cols_C(L);
    }
    static constexpr int C(int L, int mode) { return mode == 0 ? rows_C(L) : mode == 2 ? rows2_C(L) : cols_C(L); }
};

// Pass twiddle table of a length-L line (one per length, built by
// passtw_kernel): pass P >= 1 of radix R after NS = 16^P owns NS * R slots
// holding w_{NS R}^{jm k} for jm < NS, k = 1..R-1, factor-major so that the
// threads of a warp (consecutive jm) read consecutive addresses.  Float
// tables: factor 1 as NS entries, then factors (2,3), (4,5), ... as NS
// 16-byte pairs each; double tables: factor k as NS entries.  Passes are
// radix 16 (E = 16 elements per thread) with a last pass of the remaining
// radix.
__host__ __device__ inline int stock_tw_count(int L) {
    const int E = L >= 16 ? 16 : L;
    int logl = 0, loge = 0;
    while ((1 << logl) < L) logl++;
    while ((1 << loge) < E) loge++;
    const int nfull = loge ? logl / loge : 0, rem = loge ? 1 << (logl % loge) : 1;
    const int npass = nfull + (rem > 1 ? 1 : 0);
    int tot = 0, ns = 1;
    for (int P = 0; P < npass; P++) {
        const int R = P < nfull ? E : rem;
        if (P >= 1) tot += ns * R;
        ns *= R;
    }
    return tot;
}

template <typename T> __global__ void passtw_kernel(typename V2<T>::t *out, int L) {
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    const int E = L >= 16 ? 16 : L;
    int logl = 0, loge = 0;
    while ((1 << logl) < L) logl++;
    while ((1 << loge) < E) loge++;
    const int nfull = loge ? logl / loge : 0, rem = loge ? 1 << (logl % loge) : 1;
    const int npass = nfull + (rem > 1 ? 1 : 0);
    int off = 0, ns = 1;
    for (int P = 0; P < npass; P++) {
        const int R = P < nfull ? E : rem;
        if (P >= 1) {
            if (idx < off + ns * R) {
                const int r = idx - off;
                int jm, k;
                if (sizeof(T) == 4) {
                    // factor 1: slots [0, ns); pair p = (2p+2, 2p+3): ns pairs after that
                    const int r2 = r - ns, pr = r2 / (2 * ns), rm = r2 - pr * 2 * ns;
                    jm = r < ns ? r : rm >> 1;
                    k = r < ns ? 1 : 2 * pr + 2 + (rm & 1);
                } else {
                    jm = r % ns;
                    k = r / ns + 1;
                }
                if (k >= R) k = 0;  // the last ns slots are unused
                const int64_t den = (int64_t)ns * R;
                const int64_t num = ((int64_t)jm * k) % den;
                double s, c;
                sincospi(-2.0 * (double)num / (double)den, &s, &c);
                out[idx] = mk<T>((T)c, (T)s);
                return;
            }
            off += ns * R;
        }
        ns *= R;
    }
}

// Exchange slot of element i of a line whose padded copy starts at `base`.
// The passes recognise this index type and address their strided shared-
// memory runs as one base plus compile-time offsets.
struct PadIdx {
    int base;
    __device__ __forceinline__ int operator()(int i) const { return base + pad(i); }
};
template <typename X> struct is_pad_idx { static constexpr bool value = false; };
template <> struct is_pad_idx<PadIdx> { static constexpr bool value = true; };

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
    // pipelined kernel: two stages of C padded lines (TMA fills the first
    // C*L elements densely; the exchange uses the padded layout) and two
    // mbarriers
    // Exchange stride of the column modes.  A 64-bit shared access is served
    // per half-warp, whose 16 threads are 16/C positions t x C lines c
    // (c fastest); they hit 16 distinct 8-byte bank slots when
    // gcd(stride, 16) = 16 / C, so every exchange access takes the minimum
    // two wavefronts.  MODE 0 keeps LP (a warp stays inside one line).
    static constexpr int col_x() {
        int r = L + L / 16;
        while (true) {
            int g = 16, a = r;
            while (a % 2 == 0 && g > 1) { a /= 2; g /= 2; }  // g = 16 / gcd(r, 16)
            if (16 / g == 16 / C) return r;
            r++;
        }
    }
    // (double lines keep LP: their 16-byte accesses are served per
    // quarter-warp, which the odd stride already spreads for C = 8)
    static constexpr int ROWX = MODE == 0 || sizeof(T) != 4 ? LP : col_x();
    // MODE 2 lands each input line in its own row of even stride (one
    // 16-byte aligned bulk copy per line), read once before the exchange:
    // the exchange stride when that is even (C <= 8: its half-warps then
    // read distinct banks), else the next even stride
    static constexpr int LPS = LP + (LP & 1);
    static constexpr int ROWIN = MODE == 2 ? (ROWX % 2 == 0 ? ROWX : LPS) : ROWX;
    static constexpr int STAGE = ((C * (ROWIN > ROWX ? ROWIN : ROWX) + 15) / 16) * 16;  // keeps stage 1 128-byte aligned
    static constexpr size_t PIPE_SMEM = 2 * (size_t)STAGE * sizeof(C2) + 16;
    static constexpr bool PIPE_OK = PIPE_SMEM <= 227 * 1024;
    // Row lines too long for two stages (stockham_big_kernel): one padded
    // exchange line plus a stage for the first BIG_MP of the E element rows
    // (m < BIG_MP of t + m*TL, a contiguous prefix of the line) of the next
    // line; the thread reads the other rows from global memory.
    static constexpr size_t BIG_X = ((size_t)LP * sizeof(C2) + 15) / 16 * 16;
    static constexpr int BIG_MP_FIT = (int)((227 * 1024 - 16 - BIG_X) / ((size_t)TL * sizeof(C2)));
    static constexpr int BIG_MP = BIG_MP_FIT > E ? E : BIG_MP_FIT;
    static constexpr size_t BIG_SMEM = BIG_X + (size_t)BIG_MP * TL * sizeof(C2) + 16;
    static constexpr bool BIG_OK = MODE == 0 && C == 1 && !PIPE_OK && BIG_MP >= E / 2;
    // blocks per SM the register budget is sized for (about 24 warps)
    // (double lines need twice the registers: no cap beyond one block at 256+)
    // (single-warp blocks of short lines get more registers per thread: 18 warps)
    static constexpr int MINB = sizeof(T) == 4 ? (NT >= 512 || NT < 32 ? 1 : NT < 64 ? 576 / NT : 768 / NT)
                                               : (NT >= 256 || NT < 64 ? 1 : 384 / NT);

    template <int P> struct Pass {
        static constexpr int R = P < NFULL ? E : REM;
        static constexpr int NS = ipowc(E, P);
        static constexpr int NB = E / R;  // butterflies per thread
        static constexpr int SHIFT = LOGL - ilog2c(NS * R);
        static constexpr bool LAST = P == NPASS - 1;
    };

    // Twiddles of pass P for this thread: NB butterflies x (R-1) factors.
    template <int P> struct Tw {
        static constexpr int N = Pass<P>::NS > 1 ? Pass<P>::NB * (Pass<P>::R - 1) : 1;
    };
    // offset of pass P's rows in the pass twiddle table (stock_tw_count)
    template <int P> static constexpr int twoff() {
        if constexpr (P <= 1) return 0;
        else return twoff<P - 1>() + Pass<P - 1>::NS * Pass<P - 1>::R;
    }
    // Factors w_{NS R}^{jm k}, k = 1..R-1, of pass P into tw[0..R-2], from
    // the pass twiddle table W of length L (float pairs by 16-byte loads).
    template <int P> static __device__ __forceinline__ void tw_row(int jm, const C2 *__restrict__ W, C2 *tw) {
        typedef Pass<P> PP;
        const C2 *base = W + twoff<P>();
        if constexpr (sizeof(T) == 4) {
            tw[0] = __ldg(base + jm);
#pragma unroll
            for (int p = 0; 2 * p + 2 < PP::R; p++) {
                const float4 x = __ldg(reinterpret_cast<const float4 *>(base + PP::NS + 2 * p * PP::NS + 2 * jm));
                tw[2 * p + 1] = make_float2(x.x, x.y);
                tw[2 * p + 2] = make_float2(x.z, x.w);
            }
        } else {
#pragma unroll
            for (int k = 1; k < PP::R; k++) tw[k - 1] = __ldg(base + (k - 1) * PP::NS + jm);
        }
    }
    template <int P> static __device__ __forceinline__ void load_tw(int t, const C2 *__restrict__ W, C2 (&tw)[Tw<P>::N]) {
        typedef Pass<P> PP;
        if constexpr (PP::NS > 1) {
#pragma unroll
            for (int q = 0; q < PP::NB; q++) tw_row<P>((t + q * TL) & (PP::NS - 1), W, &tw[q * (PP::R - 1)]);
        }
    }

    // Butterflies of pass P on the thread's registers, with its twiddles
    // already in `tw`; non-last passes write their outputs to shared memory
    // at xs[xi(index)], load the next pass's twiddles (in flight during the
    // exchange) and read the next pass's inputs back.
    template <int P, typename Store, typename XIdx, typename Sync>
    static __device__ __forceinline__ void run(C2 (&v)[E], const C2 (&tw)[Tw<P>::N], int t, C2 *xs, XIdx &xi,
                                               const C2 *__restrict__ W, Store &store, Sync &sync) {
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
                    C2 w = tw[q * (PP::R - 1) + k - 1];
                    u[k] = SIGN < 0 ? cmul<T>(u[k], w) : cmulc<T>(u[k], w);
                }
            }
            dft_pow2<PP::R, SIGN, T>(u);
            const int idxD = (j - jm) * PP::R + jm;
            if constexpr (!PP::LAST && is_pad_idx<XIdx>::value && (PP::NS % 16 == 0 || (PP::NS == 1 && PP::R == 16))) {
                // pad(idxD + k NS) = pad(idxD) + k (NS + NS/16) for NS a multiple
                // of 16; for NS = 1, R = 16: pad(16 j + k) = pad(16 j) + k
                const int pb = xi(idxD);
                constexpr int ST = PP::NS == 1 ? 1 : PP::NS + PP::NS / 16;
#pragma unroll
                for (int k = 0; k < PP::R; k++) xs[pb + k * ST] = u[k];
            } else {
#pragma unroll
                for (int k = 0; k < PP::R; k++) {
                    if (PP::LAST) store(idxD + k * PP::NS, u[k], q * PP::R + k);
                    else xs[xi(idxD + k * PP::NS)] = u[k];
                }
            }
        }
        if constexpr (!PP::LAST) {
            // the next pass's twiddles load during the exchange
            C2 tw2[Tw<P + 1>::N];
            load_tw<P + 1>(t, W, tw2);
            sync();
            if constexpr (is_pad_idx<XIdx>::value && TL % 16 == 0) {
                // pad(t + m TL) = pad(t) + m (TL + TL/16)
                const int pr = xi(t);
#pragma unroll
                for (int m = 0; m < E; m++) v[m] = xs[pr + m * (TL + TL / 16)];
            } else {
#pragma unroll
                for (int m = 0; m < E; m++) v[m] = xs[xi(t + m * TL)];
            }
            sync();
            run<P + 1>(v, tw2, t, xs, xi, W, store, sync);
        }
    }

    template <typename Store, typename XIdx>
    static __device__ __forceinline__ void run_all(C2 (&v)[E], int t, C2 *xs, XIdx &xi, const C2 *__restrict__ W, Store &store) {
        C2 tw0[Tw<0>::N];
        auto cta_sync = [] { __syncthreads(); };
        run<0>(v, tw0, t, xs, xi, W, store, cta_sync);
    }
    template <typename Store, typename XIdx, typename Sync>
    static __device__ __forceinline__ void run_all(C2 (&v)[E], int t, C2 *xs, XIdx &xi, const C2 *__restrict__ W, Store &store,
                                                   Sync &sync) {
        C2 tw0[Tw<0>::N];
        run<0>(v, tw0, t, xs, xi, W, store, sync);
    }
};

// ---------------------------------------------------------------------------
// Plain kernel (no TMA): one tile per CTA.
// ---------------------------------------------------------------------------
// Tile `blk` of the plain kernel, run by the calling CTA (its shared memory at
// smem_raw, Stockham<...>::SMEM bytes).
template <typename T, int L, int MODE, int SIGN>
__device__ void stockham_body(const typename V2<T>::t *__restrict__ in, typename V2<T>::t *__restrict__ out, const StockParams &p,
                              const typename V2<T>::t *__restrict__ W, const typename V2<T>::t *__restrict__ Whi,
                              const typename V2<T>::t *__restrict__ Wlo, int64_t blk, unsigned char *smem_raw) {
    typedef Stockham<T, L, MODE, SIGN> S;
    typedef typename V2<T>::t C2;
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
    const int64_t b0 = blk * S::C;
    const int64_t b = b0 + c;
    const bool valid = b < p.nlines;
    C2 v[S::E];

    if (MODE == 2) {
#pragma unroll 4
        for (int i = tid; i < S::C * L; i += S::NT) {
            int cc = i >> S::LOGL, e = i & (L - 1);
            if (b0 + cc < p.nlines) sm[cc * S::LP + pad(e)] = in[line_off(p.lin, b0 + cc) + e];
        }
        __syncthreads();
#pragma unroll
        for (int m = 0; m < S::E; m++) v[m] = sm[c * S::LP + pad(t + m * S::TL)];
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
    const int oes32 = MODE == 0 ? 1 : (int)p.lout.estride;
    const bool tw = p.tw_n != 0;
    const uint32_t j2 = tw ? (uint32_t)(b % p.tw_inner) : 0u;
    const T sc = param_scale<T>(p);
    const bool do_scale = p.do_scale != 0;
    auto store = [&](int pos, C2 val, int) {
        if (tw) {
            C2 w = tw_lookup<T>(Whi, Wlo, (uint32_t)pos * j2, p);
            val = SIGN < 0 ? cmul<T>(val, w) : cmulc<T>(val, w);
        }
        if (do_scale) val = cscale<T>(val, sc);
        if (valid) dst[(int64_t)pos * oes32] = val;
    };
    PadIdx xi{c * S::LP};
    S::run_all(v, t, sm, xi, W, store);
}

template <typename T, int L, int MODE, int SIGN>
__global__ void __launch_bounds__(Stockham<T, L, MODE, SIGN>::NT)
    stockham_kernel(const typename V2<T>::t *__restrict__ in, typename V2<T>::t *__restrict__ out, StockParams p,
                    const typename V2<T>::t *__restrict__ W, const typename V2<T>::t *__restrict__ Whi,
                    const typename V2<T>::t *__restrict__ Wlo) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    stockham_body<T, L, MODE, SIGN>(in, out, p, W, Whi, Wlo, (int64_t)blockIdx.x, smem_raw);
}

// ---------------------------------------------------------------------------
// Pipelined persistent kernel (TMA prefetch of the next tile).
// ---------------------------------------------------------------------------
#define JT_MBAR_POLL_LIMIT (1u << 22)

// TW: the column pass fuses the four-step output twiddle (MODE 1 only).
template <typename T, int L, int MODE, int SIGN, bool TW>
__global__ void __launch_bounds__(Stockham<T, L, MODE, SIGN>::NT, Stockham<T, L, MODE, SIGN>::MINB)
    stockham_pipe_kernel(const typename V2<T>::t *__restrict__ in, typename V2<T>::t *__restrict__ out, StockParams p,
                         const __grid_constant__ CUtensorMap tmap, const typename V2<T>::t *__restrict__ W,
                         const typename V2<T>::t *__restrict__ Whi, const typename V2<T>::t *__restrict__ Wlo, int *err) {
    typedef Stockham<T, L, MODE, SIGN> S;
    typedef typename V2<T>::t C2;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    C2 *stage0 = reinterpret_cast<C2 *>(smem_raw);
    C2 *stage1 = stage0 + S::STAGE;
    uint64_t *bar = reinterpret_cast<uint64_t *>(stage1 + S::STAGE);
    const int tid = threadIdx.x;
    // the column modes walk across lines (c fastest: a warp's stores of one
    // output position cover C adjacent columns); MODE 0 walks along rows
    int c, t;
    if (MODE != 0) {
        c = tid % S::C;
        t = tid / S::C;
    } else {
        c = tid / S::TL;
        t = tid % S::TL;
    }
    const int64_t ntiles = (p.nlines + S::C - 1) / S::C;
    constexpr uint32_t ESZ = sizeof(C2);

    // Issues the copies of tile `tl` into `st`, completing on `mb`.  Input
    // read once (the caller's array in MODE 0/1, the dead intermediate in
    // MODE 2) is marked evict-first so the two-pass intermediate keeps L2.
    const uint64_t pol = policy_evict_first();
    auto issue = [&](int64_t tl, C2 *st, uint64_t *mb) {
        const int64_t b0 = tl * S::C;
        const int lines = (int)min((int64_t)S::C, p.nlines - b0);
        if (MODE == 1) {
            // tile = C adjacent columns of one outer block
            int64_t rem_unused;
            const int64_t ob = div_fast(tl, p.tiles_per_col, &rem_unused);
            const int col0 = (int)((tl - ob * p.tiles_per_col) * S::C);
            constexpr int BR = L < 256 ? L : 256;
            constexpr int XM = sizeof(T) == 4 ? 1 : 2;  // f64 complex = two FLOAT64 in the map
            // the boxes bring exactly C * L elements (the stage is larger: padding)
            mbar_arrive_expect_tx(mb, (uint32_t)(S::C * L * ESZ));
#pragma unroll 1
            for (int r = 0; r < L; r += BR) tensor3d_g2s_hint(st + r * S::C, &tmap, col0 * XM, r, (int)ob, mb, pol);
        } else if (MODE == 2) {
            // one row of stride ROWIN per line
            mbar_arrive_expect_tx(mb, (uint32_t)(lines * L * ESZ));
#pragma unroll 1
            for (int cc = 0; cc < lines; cc++)
                bulk_g2s_hint(st + cc * S::ROWIN, in + line_off(p.lin, b0 + cc), (uint32_t)(L * ESZ), mb, pol);
        } else if (p.lin.inner == 1 && p.lin.outer == L) {
            // C consecutive contiguous rows: one copy
            mbar_arrive_expect_tx(mb, (uint32_t)(lines * L * ESZ));
            bulk_g2s_hint(st, in + b0 * L, (uint32_t)(lines * L * ESZ), mb, pol);
        } else {
            mbar_arrive_expect_tx(mb, (uint32_t)(lines * L * ESZ));
#pragma unroll 1
            for (int cc = 0; cc < lines; cc++)
                bulk_g2s_hint(st + cc * L, in + line_off(p.lin, b0 + cc), (uint32_t)(L * ESZ), mb, pol);
        }
    };

    if (tid == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        fence_mbar_init();
        if (MODE == 1) prefetch_tensormap(&tmap);
    }
    __syncthreads();
    // tile schedule index -> tile: a pass reading what the previous pass
    // just wrote starts with its last tiles, still in L2
    const bool rev = p.reverse != 0;
    auto act = [&](int64_t x) -> int64_t { return rev ? ntiles - 1 - x : x; };
    int64_t tile = blockIdx.x;
    if (tid == 0 && tile < ntiles) issue(act(tile), stage0, &bar[0]);

    // the four-step twiddle belongs to the column pass (the launcher picks
    // the TW variant from tw_n)
    constexpr bool tw = MODE == 1 && TW;
    const T sc = param_scale<T>(p);
    const bool do_scale = p.do_scale != 0;
    const int oes32 = MODE == 0 ? 1 : (int)p.lout.estride;
    const uint64_t spol = p.stream_out ? pol : policy_evict_normal();  // output stores
    uint32_t it = 0;
    bool ok = true;
    for (; tile < ntiles; tile += gridDim.x, ++it) {
        const int buf = it & 1;
        C2 *st = buf ? stage1 : stage0;
        const int64_t nxt = tile + gridDim.x;
        if (tid == 0 && nxt < ntiles) issue(act(nxt), buf ? stage0 : stage1, &bar[buf ^ 1]);
        // Four-step twiddle w^{pos*j2} of this tile's outputs: the last pass
        // writes pos = t + TL*m, so w^{pos*j2} = w^{t*j2} g^m with
        // g = w^{TL*j2}.  Lines of 256+ take three table lookups, issued
        // before the wait for the tile so their latency hides behind it
        // (powers by products below); shorter tiles compute too briefly for
        // that and look up seven factors at the store.
        constexpr bool hoist = L >= 256;
        typedef typename V2<T>::t C2T;
        C2T tw_base, tw_g1, tw_g4;
        if constexpr (tw && hoist) {
            int64_t j2l;
            div_fast(act(tile) * S::C + c, p.tw_inner, &j2l);
            const uint32_t j2 = (uint32_t)j2l;
            const uint32_t g = (uint32_t)S::TL * j2;
            tw_base = tw_lookup<T>(Whi, Wlo, (uint32_t)t * j2, p);
            tw_g1 = tw_lookup<T>(Whi, Wlo, g, p);
            tw_g4 = tw_lookup<T>(Whi, Wlo, 4u * g, p);
        }
        bool mine = mbar_wait_bounded(&bar[buf], (it >> 1) & 1, JT_MBAR_POLL_LIMIT);
        if (!__syncthreads_and(mine)) {
            ok = false;
            break;
        }
        const int64_t b0 = act(tile) * S::C;
        const int64_t b = b0 + c;
        // column tiles are whole (the launcher requires nlines % C == 0)
        const bool valid = MODE == 1 || b < p.nlines;
        if (MODE == 2 && p.discard_in) {
            // the intermediate rows are now in shared memory and dead in L2
            const int lines = (int)min((int64_t)S::C, p.nlines - b0);
            constexpr int PER_LINE = L * (int)ESZ / 128;
            for (int i = tid; i < lines * PER_LINE; i += S::NT) {
                const int cc = i / PER_LINE, k = i - cc * PER_LINE;
                discard_l2_line(reinterpret_cast<const unsigned char *>(in + line_off(p.lin, b0 + cc)) + k * 128);
            }
        }
        typename V2<T>::t v[S::E];
        if (MODE == 1) {
#pragma unroll
            for (int m = 0; m < S::E; m++) v[m] = st[(t + m * S::TL) * S::C + c];
        } else {
#pragma unroll
            for (int m = 0; m < S::E; m++) v[m] = st[c * (MODE == 2 ? S::ROWIN : L) + t + m * S::TL];
        }
        __syncthreads();  // every pass-0 read is done before the exchange writes
        PadIdx xi{c * S::ROWX};
        {
            C2 *dst = out + (valid ? line_off(p.lout, b) : 0);
            // output slot q*R + k holds pos = t + TL*m with m = q + k*NB:
            // w^{pos*j2} = (base g^{m&3}) (g^4)^{m>>2}
            typedef typename S::template Pass<S::NPASS - 1> LP_;
            int64_t j2l = 0;
            if (tw && !hoist) div_fast(b, p.tw_inner, &j2l);
            const uint32_t j2 = (uint32_t)j2l;
            C2 bl[4], gh[4];
            auto store = [&](int pos, C2 val, int slot) {
                if (tw) {
                    if (slot == 0) {
                        if constexpr (hoist) {
                            C2 base = tw_base;
                            if (do_scale) base = cscale<T>(base, sc);  // the scale rides on the twiddle
                            const C2 g2 = cmul<T>(tw_g1, tw_g1), g8 = cmul<T>(tw_g4, tw_g4);
                            bl[0] = base;
                            bl[1] = cmul<T>(base, tw_g1);
                            bl[2] = cmul<T>(base, g2);
                            bl[3] = cmul<T>(bl[2], tw_g1);
                            gh[0] = mk<T>(1, 0);
                            gh[1] = tw_g4;
                            gh[2] = g8;
                            gh[3] = cmul<T>(g8, tw_g4);
                        } else {
                            const uint32_t g = (uint32_t)S::TL * j2;
                            auto twv = [&](uint32_t x) { return tw_lookup<T>(Whi, Wlo, x, p); };
                            C2 base = twv((uint32_t)t * j2);
                            if (do_scale) base = cscale<T>(base, sc);
                            bl[0] = base;
                            bl[1] = cmul<T>(base, twv(g));
                            bl[2] = cmul<T>(base, twv(2u * g));
                            bl[3] = cmul<T>(base, twv(3u * g));
                            gh[0] = mk<T>(1, 0);
                            gh[1] = twv(4u * g);
                            gh[2] = twv(8u * g);
                            gh[3] = twv(12u * g);
                        }
                    }
                    const int m = slot / LP_::R + (slot % LP_::R) * LP_::NB;
                    C2 w = m < 4 ? bl[m & 3] : cmul<T>(bl[m & 3], gh[m >> 2]);
                    val = SIGN < 0 ? cmul<T>(val, w) : cmulc<T>(val, w);
                }
                if (do_scale && !tw) val = cscale<T>(val, sc);
                if (valid) st_hint(&dst[(int64_t)pos * oes32], val, spol);
            };
            if constexpr (MODE == 0 && S::TL <= 32) {
                // a warp holds whole lines: the exchanges need no CTA barrier
                auto warp_sync = [] { __syncwarp(); };
                S::run_all(v, t, st, xi, W, store, warp_sync);
            } else if constexpr (MODE == 0 && S::C > 1 && S::C < 16) {
                // a line spans TL / 32 warps: one named barrier per line
                auto line_sync = [c] { named_barrier(1 + c, S::TL); };
                S::run_all(v, t, st, xi, W, store, line_sync);
            } else {
                S::run_all(v, t, st, xi, W, store);
            }
        }
        // this thread's generic writes to the stage come before the TMA that
        // refills it two tiles later
        fence_proxy_async_smem();
        __syncthreads();
    }
    if (!ok) {
        if (tid == 0) {
            atomicExch(err, 1);
            // drain copies still in flight into this CTA's shared memory
            mbar_wait_bounded(&bar[it & 1], (it >> 1) & 1, JT_MBAR_POLL_LIMIT);
            if (tile + gridDim.x < ntiles) mbar_wait_bounded(&bar[(it + 1) & 1], ((it + 1) >> 1) & 1, JT_MBAR_POLL_LIMIT);
        }
        __syncthreads();
    }
}

// Persistent row kernel for lines whose two-stage pipeline does not fit
// (one line per CTA, a CTA of TL threads holds the whole line in
// registers): the prefix of the next line comes in by one TMA bulk copy
// into its own stage while the current line is computed in the exchange
// line; the rest of the next line is read from global memory at the start
// of its turn, issued before the wait for the copy.
template <typename T, int L, int SIGN>
__global__ void __launch_bounds__(Stockham<T, L, 0, SIGN>::NT, 1)
    stockham_big_kernel(const typename V2<T>::t *in, typename V2<T>::t *out, StockParams p,
                        const typename V2<T>::t *__restrict__ W, int *err) {
    typedef Stockham<T, L, 0, SIGN> S;
    typedef typename V2<T>::t C2;
    constexpr int MP = S::BIG_MP;
    constexpr uint32_t PBYTES = (uint32_t)(MP * S::TL * sizeof(C2));
    extern __shared__ __align__(128) unsigned char smem_raw[];
    C2 *xs = reinterpret_cast<C2 *>(smem_raw);
    C2 *pst = reinterpret_cast<C2 *>(smem_raw + S::BIG_X);
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem_raw + S::BIG_X + PBYTES);
    const int t = threadIdx.x;
    const int64_t ntiles = p.nlines;
    const uint64_t pol = policy_evict_first();
    const uint64_t spol = p.stream_out ? pol : policy_evict_normal();
    auto issue = [&](int64_t tl) {
        mbar_arrive_expect_tx(bar, PBYTES);
        bulk_g2s_hint(pst, in + line_off(p.lin, tl), PBYTES, bar, pol);
    };
    if (t == 0) {
        mbar_init(bar, 1);
        fence_mbar_init();
    }
    __syncthreads();
    int64_t tile = blockIdx.x;
    if (t == 0 && tile < ntiles) issue(tile);
    const T sc = param_scale<T>(p);
    const bool do_scale = p.do_scale != 0;
    uint32_t it = 0;
    bool ok = true;
    for (; tile < ntiles; tile += gridDim.x, ++it) {
        const C2 *src = in + line_off(p.lin, tile);
        C2 v[S::E];
#pragma unroll
        for (int m = MP; m < S::E; m++) v[m] = src[t + m * S::TL];
        const bool mine = mbar_wait_bounded(bar, it & 1, JT_MBAR_POLL_LIMIT);
        if (!__syncthreads_and(mine)) {
            ok = false;
            break;
        }
#pragma unroll
        for (int m = 0; m < MP; m++) v[m] = pst[t + m * S::TL];
        // the stage's reads come before the copy that refills it
        fence_proxy_async_smem();
        __syncthreads();
        if (t == 0 && tile + gridDim.x < ntiles) issue(tile + gridDim.x);
        C2 *dst = out + line_off(p.lout, tile);
        auto store = [&](int pos, C2 val, int) {
            if (do_scale) val = cscale<T>(val, sc);
            st_hint(&dst[pos], val, spol);
        };
        PadIdx xi{0};
        S::run_all(v, t, xs, xi, W, store);
    }
    if (!ok) {
        if (t == 0) {
            atomicExch(err, 1);
            mbar_wait_bounded(bar, it & 1, JT_MBAR_POLL_LIMIT);  // the copy in flight
        }
        __syncthreads();
    }
}

// Host-side launcher for one (T, L).
template <typename T, int L> struct StockLaunch {
    typedef typename V2<T>::t C2;
    template <int MODE, int SIGN, bool TW>
    static void pipe(const C2 *in, C2 *out, const StockParams &p, const CUtensorMap &tmap, const C2 *W, const C2 *Whi,
                     const C2 *Wlo, int *err, int sms, cudaStream_t s, int64_t ntiles) {
        typedef Stockham<T, L, MODE, SIGN> S;
        auto kern = stockham_pipe_kernel<T, L, MODE, SIGN, TW && MODE == 1>;
        static int per_sm = 0;
        if (!per_sm) {
            cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)S::PIPE_SMEM);
            cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, S::NT, S::PIPE_SMEM);
            if (per_sm < 1) per_sm = 1;
            // shared memory for exactly the resident blocks; the rest of
            // the SM's 256 KB stays L1, which holds the twiddle tables
            const int need = per_sm * ((int)S::PIPE_SMEM + 1024);
            const int pct = (need * 100 + 228 * 1024 - 1) / (228 * 1024);
            if (pct < 100) {
                cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, pct);
                int again = 0;
                cudaOccupancyMaxActiveBlocksPerMultiprocessor(&again, kern, S::NT, S::PIPE_SMEM);
                if (again < per_sm) cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
            }
        }
        const int64_t grid = std::min<int64_t>(ntiles, (int64_t)sms * per_sm);
        kern<<<(unsigned)grid, S::NT, S::PIPE_SMEM, s>>>(in, out, p, tmap, W, Whi, Wlo, err);
    }
    template <int MODE, int SIGN> static void one(const C2 *in, C2 *out, const StockParams &p, const CUtensorMap *tmap,
                                                  const C2 *W, const C2 *Whi, const C2 *Wlo, int *err, int sms,
                                                  cudaStream_t s) {
        typedef Stockham<T, L, MODE, SIGN> S;
        int64_t ntiles = (p.nlines + S::C - 1) / S::C;
        if constexpr (S::BIG_OK) if (tmap) {
            auto kern = stockham_big_kernel<T, L, SIGN>;
            static bool big_attr = false;
            if (!big_attr) {
                cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)S::BIG_SMEM);
                cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
                big_attr = true;
            }
            const int64_t grid = std::min<int64_t>(ntiles, (int64_t)sms);
            kern<<<(unsigned)grid, S::NT, S::BIG_SMEM, s>>>(in, out, p, W, err);
            return;
        }
        if constexpr (S::PIPE_OK) if (tmap) {
            if (MODE == 1 && p.tw_n != 0) pipe<MODE, SIGN, true>(in, out, p, *tmap, W, Whi, Wlo, err, sms, s, ntiles);
            else pipe<MODE, SIGN, false>(in, out, p, *tmap, W, Whi, Wlo, err, sms, s, ntiles);
            return;
        }
        static bool attr = false;
        if (!attr) {
            cudaFuncSetAttribute(stockham_kernel<T, L, MODE, SIGN>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)S::SMEM);
            cudaFuncSetAttribute(stockham_kernel<T, L, MODE, SIGN>, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
            attr = true;
        }
        stockham_kernel<T, L, MODE, SIGN><<<(unsigned)ntiles, S::NT, S::SMEM, s>>>(in, out, p, W, Whi, Wlo);
    }
    static void go(int mode, int sign, const C2 *in, C2 *out, const StockParams &p, const CUtensorMap *tmap, const C2 *W,
                   const C2 *Whi, const C2 *Wlo, int *err, int sms, cudaStream_t s) {
        if (mode == 0) {
            sign < 0 ? one<0, -1>(in, out, p, tmap, W, Whi, Wlo, err, sms, s) : one<0, 1>(in, out, p, tmap, W, Whi, Wlo, err, sms, s);
            return;
        }
        if constexpr (L <= 4096) {  // column modes: C lines of up to 4096 fit one CTA
            if (mode == 1)
                sign < 0 ? one<1, -1>(in, out, p, tmap, W, Whi, Wlo, err, sms, s) : one<1, 1>(in, out, p, tmap, W, Whi, Wlo, err, sms, s);
            else
                sign < 0 ? one<2, -1>(in, out, p, tmap, W, Whi, Wlo, err, sms, s) : one<2, 1>(in, out, p, tmap, W, Whi, Wlo, err, sms, s);
        }
    }
};

}  // namespace jt
