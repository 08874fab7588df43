// jt_engine.cu -- host side of jtransforms_gb300: per-size plans, algorithm
// choice, scratch management and the C ABI declared in include/jtgpu.h.
//
// Algorithm choice per complex length n (GPU-first, not the reference's
// split-radix / FFTPACK / Bluestein choice, which only fixes the results):
//   DIRECT    n <= 8192 (f32) / 4096 (f64) with prime factors <= 63: one
//             shared-memory tile kernel per batch of lines.
//   TWOPASS   n = n1 * n2 with both DIRECT: column pass with the four-step
//             twiddle fused into its store, then a row pass that writes the
//             transposed (natural-order) result.  The batch is processed in
//             chunks of up to 1 GiB: one launch per pass and chunk (long
//             launches measured faster than L2-sized chunks).
//   BLUESTEIN everything else: chirp-z with a power-of-two convolution of
//             nextPow2(2n-1) points (fft/DoubleFFT_1D.java:1864-2107), chirp
//             tables generated in FP64 on the device.
#include "jt_device.cuh"
#include "jt_stockham.cuh"
#include "jt_batch.cuh"
#include "jt_r2r.cuh"
#include "jt_chirp.cuh"
#include "jt_plan_table.h"
#include "../../include/jtgpu.h"

#include <cuda.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <new>
#include <string>
#include <tuple>
#include <thread>
#include <vector>

namespace jt {

static thread_local int g_last_cuda = 0;
static thread_local int64_t g_launches = 0;

#define JT_CU(call)                                  \
    do {                                             \
        cudaError_t e_ = (call);                     \
        if (e_ != cudaSuccess) {                     \
            g_last_cuda = (int)e_;                   \
            return e_ == cudaErrorMemoryAllocation ? JT_ENOMEM : JT_ECUDA; \
        }                                            \
    } while (0)

#define JT_TRY(call)                 \
    do {                             \
        int s_ = (call);             \
        if (s_ != JT_OK) return s_;  \
    } while (0)

static bool is_pow2(int64_t x) { return x > 0 && (x & (x - 1)) == 0; }
static int64_t next_pow2(int64_t x) {
    int64_t p = 1;
    while (p < x) p <<= 1;
    return p;
}
// smallest 2^a 3^b 5^c 7^d >= x
static int64_t next_smooth(int64_t x) {
    int64_t best = next_pow2(x);
    for (int64_t p7 = 1; p7 < best; p7 *= 7)
        for (int64_t p5 = p7; p5 < best; p5 *= 5)
            for (int64_t p3 = p5; p3 < best; p3 *= 3) {
                int64_t v = p3;
                while (v < x) v *= 2;
                if (v < best) best = v;
            }
    return best;
}

// Per-thread device workspace: a bump allocator that is sized by a dry run
// of the same call (no launches), then handed out in 256-byte aligned slices.
struct Arena {
    char *base = nullptr;
    size_t cap = 0, used = 0, peak = 0;
    void *get(size_t bytes, bool dry) {
        size_t off = (used + 255) & ~(size_t)255;
        used = off + bytes;
        if (used > peak) peak = used;
        return dry ? nullptr : (void *)(base + off);
    }
};

struct Ctx {
    cudaStream_t s = nullptr;
    bool dry = false;
    Arena *ws = nullptr;
    // batch recording: steps are appended here instead of launched, each
    // depending on the previous step of the same transform
    std::vector<BOp> *rec = nullptr;
    int rec_prev = -1;
    bool rec_sizing = false;  // the workspace-sizing pass before a recording
    // JT_MODE_TC_SPLIT: Float32 row passes of length 16..2048 run their
    // radix-16 stages on the tensor cores (jt_tcsplit.cuh)
    bool tc = false;
};

static void emit(Ctx &c, BOp &o) {
    o.dep = c.rec_prev;
    c.rec->push_back(o);
    c.rec_prev = (int)c.rec->size() - 1;
}

template <typename T> static BOp elem_op(int kind, int sign, int64_t total) {
    BOp o;
    memset(&o, 0, sizeof(o));
    o.type = BOP_ELEM;
    o.prec = sizeof(T) == 4 ? 0 : 1;
    o.kind = kind;
    o.sign = sign;
    o.total = total;
    o.ntasks = (int)((total + JT_BATCH_ELEMS_PER_TASK - 1) / JT_BATCH_ELEMS_PER_TASK);
    return o;
}

static inline int64_t cdiv(int64_t a, int64_t b) { return (a + b - 1) / b; }

// (a step with no batch-recordable form refuses to be recorded)
#define LAUNCH1D(ctx, total, kernel, ...)                                              \
    do {                                                                               \
        if ((ctx).rec) return JT_EINVAL;                                               \
        if (!(ctx).dry && (total) > 0) {                                               \
            int64_t g_ = cdiv((total), 256);                                           \
            auto kfn_ = kernel;                                                        \
            kfn_<<<(unsigned)g_, 256, 0, (ctx).s>>>(__VA_ARGS__);                      \
            g_launches++;                                                              \
        }                                                                              \
    } while (0)

static int g_smem_optin = 0;
static int g_sms = 1;
static int *g_err_dev = nullptr;  // raised by a kernel whose bounded wait gave up
typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *, const cuuint64_t *,
                                  const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave, CUtensorMapSwizzle,
                                  CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
static EncodeTiledFn g_encode_tiled = nullptr;
static std::atomic<int> g_opt_tma{1};
static std::atomic<int> g_opt_direct_max_f32{8192};
static std::atomic<int> g_opt_direct_max_f64{8192};
static std::atomic<int> g_opt_chunk_mb{1024};
static std::atomic<int> g_opt_host_piece_mb{64};
// elements per CTA of the generic tile kernel (0: the tuned table, else the
// default); the autotuner's probe
static std::atomic<int> g_opt_tile_elems{0};
static std::atomic<int> g_opt_real_fused_f32{1};
static std::atomic<int64_t> g_opt_threepass_min{(int64_t)1 << 21};
// pass-split overrides (jt_set_split), [precision][log2 n]; a < 0: none
#define JT_SPLIT_MAX_LOG2 30
static signed char g_split_override[2][JT_SPLIT_MAX_LOG2 + 1][3];
static bool g_split_override_init = [] {
    for (auto &p : g_split_override)
        for (auto &e : p) e[0] = e[1] = e[2] = -1;
    return true;
}();
static std::once_flag g_dev_once;
static int g_dev_status = JT_OK;
// Plan tables are built on one non-blocking setup stream, and a plan is
// ready once that stream has finished (a wait on the setup stream only:
// work on other streams is neither waited for nor stalled).
static cudaStream_t g_setup = nullptr;
static std::atomic<uint64_t> g_setup_seq{0};  // table builds so far
// bumped when an option that changes plan choice changes: cached tables of
// an older generation are not reused
static std::atomic<uint64_t> g_plan_gen{0};
// largest per-thread scratch arena in bytes (0: no limit)
static std::atomic<int64_t> g_opt_arena_limit{0};
// polls of a batch dependency wait before it gives up, and a test hook that
// makes the first step of every batch transform wait on a step that is never
// queued (a flag nothing sets), so the waits run out
static std::atomic<int> g_opt_batch_wait{1 << 24};
static std::atomic<int> g_opt_batch_inject{0};

static int device_init() {
    std::call_once(g_dev_once, [] {
        int n = 0;
        if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
            g_dev_status = JT_ENODEV;
            return;
        }
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&g_smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
        cudaDeviceGetAttribute(&g_sms, cudaDevAttrMultiProcessorCount, dev);
        if (cudaMalloc(&g_err_dev, sizeof(int)) != cudaSuccess || cudaMemset(g_err_dev, 0, sizeof(int)) != cudaSuccess ||
            cudaStreamCreateWithFlags(&g_setup, cudaStreamNonBlocking) != cudaSuccess) {
            g_dev_status = JT_ECUDA;
            return;
        }
        void *fn = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            g_encode_tiled = (EncodeTiledFn)fn;
        cudaFuncSetAttribute(fft_tile_kernel<-1, float>, cudaFuncAttributeMaxDynamicSharedMemorySize, g_smem_optin);
        cudaFuncSetAttribute(fft_tile_kernel<1, float>, cudaFuncAttributeMaxDynamicSharedMemorySize, g_smem_optin);
        cudaFuncSetAttribute(fft_tile_kernel<-1, double>, cudaFuncAttributeMaxDynamicSharedMemorySize, g_smem_optin);
        cudaFuncSetAttribute(fft_tile_kernel<1, double>, cudaFuncAttributeMaxDynamicSharedMemorySize, g_smem_optin);
        cudaFuncSetAttribute(r2r_tile_kernel<R2R_DCT2, float>, cudaFuncAttributeMaxDynamicSharedMemorySize, g_smem_optin);
        cudaFuncSetAttribute(r2r_tile_kernel<R2R_DCT3, float>, cudaFuncAttributeMaxDynamicSharedMemorySize, g_smem_optin);
        cudaFuncSetAttribute(r2r_tile_kernel<R2R_DHT, float>, cudaFuncAttributeMaxDynamicSharedMemorySize, g_smem_optin);
        cudaFuncSetAttribute(r2r_tile_kernel<R2R_DCT2, double>, cudaFuncAttributeMaxDynamicSharedMemorySize, g_smem_optin);
        cudaFuncSetAttribute(r2r_tile_kernel<R2R_DCT3, double>, cudaFuncAttributeMaxDynamicSharedMemorySize, g_smem_optin);
        cudaFuncSetAttribute(r2r_tile_kernel<R2R_DHT, double>, cudaFuncAttributeMaxDynamicSharedMemorySize, g_smem_optin);
        cudaFuncSetAttribute(blue_tile_kernel<-1, float>, cudaFuncAttributeMaxDynamicSharedMemorySize, g_smem_optin);
        cudaFuncSetAttribute(blue_tile_kernel<1, float>, cudaFuncAttributeMaxDynamicSharedMemorySize, g_smem_optin);
        cudaFuncSetAttribute(blue_tile_kernel<-1, double>, cudaFuncAttributeMaxDynamicSharedMemorySize, g_smem_optin);
        cudaFuncSetAttribute(blue_tile_kernel<1, double>, cudaFuncAttributeMaxDynamicSharedMemorySize, g_smem_optin);
        cudaFuncSetAttribute(r2r_tile_kernel<R2R_RFWD, float>, cudaFuncAttributeMaxDynamicSharedMemorySize, g_smem_optin);
        cudaFuncSetAttribute(r2r_tile_kernel<R2R_RINV, float>, cudaFuncAttributeMaxDynamicSharedMemorySize, g_smem_optin);
        cudaFuncSetAttribute(r2r_tile_kernel<R2R_RFWD, double>, cudaFuncAttributeMaxDynamicSharedMemorySize, g_smem_optin);
        cudaFuncSetAttribute(r2r_tile_kernel<R2R_RINV, double>, cudaFuncAttributeMaxDynamicSharedMemorySize, g_smem_optin);
        if (cudaGetLastError() != cudaSuccess) g_dev_status = JT_ECUDA;
    });
    return g_dev_status;
}

// Register-resident power-of-two kernel launchers (jt_pow2_f32.cu, jt_pow2_f64.cu).
bool stockham_launch(int L, int mode, int sign, const float2 *in, float2 *out, const StockParams &p, const CUtensorMap *tmap,
                     const float2 *W, const float2 *Whi, const float2 *Wlo, int *err, int sms, cudaStream_t s);
bool stockham_launch(int L, int mode, int sign, const double2 *in, double2 *out, const StockParams &p, const CUtensorMap *tmap,
                     const double2 *W, const double2 *Whi, const double2 *Wlo, int *err, int sms, cudaStream_t s);
bool stockham_pipe_ok(int L, int mode, const float *);
bool stockham_pipe_ok(int L, int mode, const double *);
int stockham_lines_per_cta(int L, int mode, const float *);
int stockham_lines_per_cta(int L, int mode, const double *);
bool tc_split_ok(int L);
// Register-form DCT/DST/DHT lines (jt_r2r_f32.cu, jt_r2r_f64.cu).
bool r2r_reg_launch(int H, int op, const float *in, float *out, const R2rParams &p, const float2 *Wp, const float2 *Wr,
                    const float2 *Wd, cudaStream_t s);
bool r2r_reg_launch(int H, int op, const double *in, double *out, const R2rParams &p, const double2 *Wp, const double2 *Wr,
                    const double2 *Wd, cudaStream_t s);
int r2r_reg_lines(int H, const float *);
int r2r_reg_lines(int H, const double *);
bool tc_split_launch(int L, int sign, const float2 *in, float2 *out, const StockParams &p, const float2 *W, int *err, int sms,
                     cudaStream_t s);

// Encodes a 3D tiled tensor map over complex elements of esz bytes (8 or 16,
// moved as 8-byte units): x = column (inner), y = row, z = outer block.
static bool make_col_tmap(CUtensorMap *m, const void *base, int esz, int64_t inner, int64_t rows, int64_t nblocks,
                          int64_t row_pitch, int64_t block_stride, int C, int BR) {
    if (!g_encode_tiled) return false;
    const int xm = esz / 8;
    cuuint64_t dims[3] = {(cuuint64_t)(inner * xm), (cuuint64_t)rows, (cuuint64_t)nblocks};
    cuuint64_t strides[2] = {(cuuint64_t)(row_pitch * esz), (cuuint64_t)(block_stride * esz)};
    cuuint32_t box[3] = {(cuuint32_t)(C * xm), (cuuint32_t)BR, 1};
    cuuint32_t es[3] = {1, 1, 1};
    if ((row_pitch * esz) % 16 || (block_stride * esz) % 16 || ((uintptr_t)base % 16)) return false;
    return g_encode_tiled(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 3, const_cast<void *>(base), dims, strides, box, es,
                          CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                          CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// ---------------------------------------------------------------------------
// Complex FFT of one length
// ---------------------------------------------------------------------------
enum { ALG_DIRECT = 0, ALG_TWOPASS = 1, ALG_BLUESTEIN = 2, ALG_TRIVIAL = 3, ALG_THREEPASS = 4 };
// longest power-of-two line of the multi-pass register plans: twiddle
// exponents are formed in 32 bits modulo the length (three passes of up to
// 2048 reach it)
static constexpr int64_t kPow2PassMax = (int64_t)1 << 32;

static const int kMaxThreads = 512;
// elements per task of a recorded (batch) tile step: the batch kernel's
// threads then all own a radix-16 butterfly (shared memory permitting)
static const int64_t kBatchTileElems = 16 * JT_BATCH_THREADS;
// whether one line of length L fits a batch task's shared-memory cap
template <typename T> static bool batch_line_ok(int64_t L) {
    return 2 * (size_t)padded_len((int)L) * sizeof(typename V2<T>::t) <= (size_t)JT_BATCH_SMEM_CAP;
}

template <typename T> struct Lim {
    static int64_t lmax() { return sizeof(T) == 4 ? 8192 : 4096; }
};

// Radices for a DIRECT line; empty if n has a prime factor > 63.
// Pass radices of the tile kernel for n, in the pass order `order`: bit 0
// puts the odd factors (7, 5, 3, then the other odd ones up to 63) before the
// power-of-two part instead of after it; bit 1 splits the power of two into
// 8s (then 4 or 2) instead of 16s (then 8, 4 or 2).  Empty if n has a prime
// factor > 63.  Every order computes the same DFT; the tuned order per size
// class comes from radix_order.
static std::vector<int> direct_radices(int64_t n, int order = 0) {
    std::vector<int> p2, odd;
    int64_t m = n;
    int a = 0;
    while (m % 2 == 0) { m /= 2; a++; }
    if (order & 2) {
        while (a >= 3) { p2.push_back(8); a -= 3; }
        if (a == 2) p2.push_back(4);
        else if (a == 1) p2.push_back(2);
    } else {
        while (a >= 4) { p2.push_back(16); a -= 4; }
        if (a == 3) p2.push_back(8);
        else if (a == 2) p2.push_back(4);
        else if (a == 1) p2.push_back(2);
    }
    for (int p : {7, 5, 3})
        while (m % p == 0) { odd.push_back(p); m /= p; }
    for (int p = 11; p <= 63 && m > 1; p += 2)
        while (m % p == 0) { odd.push_back(p); m /= p; }
    if (m != 1 || n == 1) return {};
    std::vector<int> r = (order & 1) ? odd : p2;
    const std::vector<int> &tail = (order & 1) ? p2 : odd;
    r.insert(r.end(), tail.begin(), tail.end());
    return r;
}

// Tuned pass order (direct_radices) for the tile kernel's length n: the
// probe option, else the table by ceil(log2 n) (jt_plan_table.h).
static std::atomic<int> g_opt_radix_order{-1};
static int radix_order(int64_t n, bool f32) {
    const int o = g_opt_radix_order.load();
    if (o >= 0) return o;
    int lg = 0;
    while (((int64_t)1 << lg) < n) lg++;
    if (lg >= 14) return 0;
    return f32 ? kRadixOrderF32[lg] : kRadixOrderF64[lg];
}

template <typename T> struct Fft1 {
    typedef typename V2<T>::t C2;
    int64_t n = 0;
    int algo = ALG_TRIVIAL;
    std::vector<int> radix;
    C2 *W = nullptr;
    C2 *Wp = nullptr;  // pass twiddle table of the register kernel (reg plans)
    int64_t n1 = 0, n2 = 0;
    std::unique_ptr<Fft1> pa, pb, pbl;
    C2 *Whi = nullptr, *Wlo = nullptr;
    int lo_bits = 0;
    // three passes: n = n1 * n2 * n3, the row length m = n2 * n3 split again
    int64_t n3 = 0;
    std::unique_ptr<Fft1> pc;
    C2 *Whi2 = nullptr, *Wlo2 = nullptr;  // four-step twiddle of length m
    int lo_bits2 = 0;
    // batch recording of a one-pass length the batch kernel cannot hold
    // (float lines of 8192+): the same transform in two passes
    std::unique_ptr<Fft1> rec_alt;
    int64_t nB = 0;
    C2 *bk1 = nullptr, *bk2 = nullptr;

    ~Fft1() {
        for (void *p : {(void *)W, (void *)Wp, (void *)Whi, (void *)Wlo, (void *)Whi2, (void *)Wlo2, (void *)bk1, (void *)bk2})
            if (p) cudaFree(p);
    }

    // two-level table of w_len^e, e < len: Whi[e >> bits] * Wlo[e & (2^bits - 1)]
    static int make_twiddle_pair(int64_t len, C2 **hi, C2 **lo, int *bits) {
        *bits = 0;
        while (((int64_t)1 << (2 * *bits)) < len) (*bits)++;
        const int64_t nlo = (int64_t)1 << *bits;
        JT_TRY(make_roots(lo, nlo, 1, len));
        return make_roots(hi, cdiv(len, nlo), nlo, len);
    }

    static bool generic_ok(int64_t n) { return n >= 2 && n <= Lim<T>::lmax() && !direct_radices(n).empty(); }
    // Elements per CTA of a generic tile pass over lines of length L (lines
    // per CTA = elements / L, threads = elements / 16): the probe option, the
    // tuned table (jt_plan_table.h, by ceil(log2 L)), or 4096 / 2048
    static int64_t tile_elems(int L) {
        const int o = g_opt_tile_elems.load();
        if (o > 0) return o;
        int lg = 0;
        while ((1 << lg) < L) lg++;
        if (lg < 14) {
            const int t = sizeof(T) == 4 ? kTileElemsF32[lg] : kTileElemsF64[lg];
            if (t > 0) return t;
        }
        return sizeof(T) == 4 ? 4096 : 2048;
    }
    // register-resident power-of-two kernel (jt_stockham.cuh): row mode up to
    // reg_rows_max, column modes up to 4096
    static int64_t reg_rows_max() { return sizeof(T) == 4 ? 16384 : 8192; }
    static int64_t one_pass_max() {
        return std::min<int64_t>(reg_rows_max(), sizeof(T) == 4 ? g_opt_direct_max_f32.load() : g_opt_direct_max_f64.load());
    }
    static bool reg_ok(int64_t n) { return is_pow2(n) && n >= 16 && n <= reg_rows_max(); }
    static bool direct_ok(int64_t n) { return reg_ok(n) || generic_ok(n); }
    bool reg = false;
    // whether a line pass with strided (column) layouts can run in one kernel
    bool cols_ok() const { return algo == ALG_DIRECT && (reg ? n <= 4096 : true); }

    static int make_roots(C2 **out, int64_t count, int64_t num, int64_t den) {
        JT_CU(cudaMalloc(out, sizeof(C2) * std::max<int64_t>(count, 1)));
        roots_kernel<T><<<(unsigned)cdiv(count, 256), 256, 0, g_setup>>>(*out, count, num, den);
        g_launches++;
        JT_CU(cudaGetLastError());
        return JT_OK;
    }

    static int make_pass_table(C2 **out, int L) {
        const int count = stock_tw_count(L);
        JT_CU(cudaMalloc(out, sizeof(C2) * std::max(count, 1)));
        if (count > 0) {
            passtw_kernel<T><<<(unsigned)cdiv(count, 256), 256, 0, g_setup>>>(*out, L);
            g_launches++;
            JT_CU(cudaGetLastError());
        }
        return JT_OK;
    }
    // register kernel plans need the pass table; sub-plans that fall back to
    // the generic kernel drop it
    int set_reg(bool on) {
        reg = on;
        if (reg && !Wp) return make_pass_table(&Wp, (int)n);
        return JT_OK;
    }

    // Pass split of a power-of-two length from jt_set_split's override or
    // the measured plan table (jt_plan_table.h): {0,0,0} one pass, {a,b,0}
    // two passes 2^a x 2^b, {a,b,c} three passes; nullptr: the rules below.
    static const signed char *table_split(int64_t n) {
        int lg = 0;
        while (((int64_t)1 << lg) < n) lg++;
        if (lg > JT_SPLIT_MAX_LOG2) return nullptr;
        const int pi = sizeof(T) == 4 ? 0 : 1;
        const signed char *o = g_split_override[pi][lg];
        if (o[0] >= 0) return o;
        const signed char *t = sizeof(T) == 4 ? kSplitF32[lg] : kSplitF64[lg];
        return t[0] >= 0 ? t : nullptr;
    }

    int init_direct() {
        algo = ALG_DIRECT;
        JT_TRY(set_reg(reg_ok(n)));
        if (!reg) radix = direct_radices(n, radix_order(n, sizeof(T) == 4));
        return make_roots(&W, n, 1, n);
    }

    // n = n1 (column pass, four-step twiddle fused) x n2 (transposing row pass)
    int init_twopass(int64_t d) {
        algo = ALG_TWOPASS;
        n1 = d;
        n2 = n / d;
        JT_TRY(create(n1, pa, false));
        JT_TRY(create(n2, pb, false));
        // pass A reads and writes columns, pass B writes columns: the
        // register kernel does that up to 4096, the generic one always
        for (Fft1 *sub : {pa.get(), pb.get()})
            if (sub->reg && sub->n > 4096) {
                sub->reg = false;
                sub->radix = direct_radices(sub->n, radix_order(sub->n, sizeof(T) == 4));
            }
        return make_twiddle_pair(n, &Whi, &Wlo, &lo_bits);
    }

    // n = n1 x (n2 x n3): column pass A, column pass B1 of each row's
    // n2 x n3 view, transposing row pass B2 (register kernel, <= 4096 each)
    int init_threepass(int64_t a, int64_t b, int64_t c) {
        algo = ALG_THREEPASS;
        n1 = a;
        n2 = b;
        n3 = c;
        JT_TRY(create(n1, pa, false));
        JT_TRY(create(n2, pb, false));
        JT_TRY(create(n3, pc, false));
        JT_TRY(make_twiddle_pair(n, &Whi, &Wlo, &lo_bits));
        return make_twiddle_pair(n2 * n3, &Whi2, &Wlo2, &lo_bits2);
    }

    // top: a transform of its own (its pass split may come from the plan
    // table); sub-plans are the line passes of a two- or three-pass plan
    static int create(int64_t n, std::unique_ptr<Fft1> &out, bool top = true) {
        std::unique_ptr<Fft1> f(new (std::nothrow) Fft1());
        if (!f) return JT_ENOMEM;
        f->n = n;
        const signed char *sp = (top && n > 16 && is_pow2(n)) ? table_split(n) : nullptr;
        if (n == 1) {
            f->algo = ALG_TRIVIAL;
        } else if (sp && sp[0] == 0 && reg_ok(n)) {
            JT_TRY(f->init_direct());
        } else if (sp && sp[0] > 0 && sp[2] == 0 && sp[0] <= 12 && sp[1] <= 12) {
            JT_TRY(f->init_twopass((int64_t)1 << sp[0]));
        } else if (sp && sp[2] > 0 && n <= kPow2PassMax && sp[0] <= 12 && sp[1] <= 12 && sp[2] <= 12) {
            JT_TRY(f->init_threepass((int64_t)1 << sp[0], (int64_t)1 << sp[1], (int64_t)1 << sp[2]));
        } else if (direct_ok(n) && (!is_pow2(n) || n <= one_pass_max())) {
            JT_TRY(f->init_direct());
        } else if (is_pow2(n) && n <= kPow2PassMax &&
                   ((sizeof(T) == 4 && g_opt_threepass_min.load() > 0 && n >= g_opt_threepass_min.load()) ||
                    n > (int64_t)4096 * 4096)) {
            // three register-kernel passes of lengths as equal as possible
            // (2^24 = 256^3): every pass runs 128-byte-wide column tiles,
            // where a 4096 x 4096 split would run 16-byte ones; beyond
            // 4096 x 4096 three passes are the only register-kernel split
            int lg = 0;
            while (((int64_t)1 << lg) < n) lg++;
            const int a = lg / 3, b = (lg - a) / 2, c = lg - a - b;
            JT_TRY(f->init_threepass((int64_t)1 << a, (int64_t)1 << b, (int64_t)1 << c));
        } else {
            // two DIRECT lengths, n = n1 (column pass) * n2 (row pass): as
            // balanced as possible, preferring lengths both passes run on
            // the register kernel (n1, n2 <= 4096 powers of two)
            int64_t best = 0;
            double bestd = 1e300;
            for (int64_t d = 2; d <= reg_rows_max() && d < n; d++) {
                if (n % d) continue;
                int64_t e = n / d;
                if (!direct_ok(d) || !direct_ok(e)) continue;
                bool fast = reg_ok(d) && reg_ok(e) && d <= 4096 && e <= 4096;
                if (!fast && (!generic_ok(d) || !generic_ok(e))) continue;
                double dd = std::fabs(std::log((double)d) - std::log((double)e)) - (fast ? 100.0 : 0.0);
                if (dd < bestd) { bestd = dd; best = d; }
            }
            if (best) {
                JT_TRY(f->init_twopass(best));
            } else {
                f->algo = ALG_BLUESTEIN;
                f->nB = next_pow2(2 * n - 1);
                if (f->nB > kPow2PassMax) return JT_ETOOBIG;
                JT_TRY(create(f->nB, f->pbl));
                JT_TRY(f->make_chirp());
            }
        }
        if (top) JT_TRY(f->make_rec_alt());
        out = std::move(f);
        return JT_OK;
    }

    int make_chirp();

    // A one-pass length whose line does not fit a batch task (the tile
    // kernel's limit or the batch's shared-memory cap) is recorded as the
    // same transform in two passes of shorter lines: the balanced split with
    // both lengths fitting, if there is one.
    // A Bluestein length records its convolution at the smallest 7-smooth
    // length >= 2n - 1 instead of the power of two: batch steps run every
    // line on the mixed-radix tile passes, so the shorter convolution is
    // less work there (up to 2x); single calls keep the power of two, whose
    // register-kernel passes are faster.  Only for convolutions up to 2^20.
    int make_rec_alt() {
        if (algo == ALG_BLUESTEIN) {
            const int64_t nS = next_smooth(2 * n - 1);
            if (nB > ((int64_t)1 << 20) || nS >= nB) return JT_OK;
            rec_alt.reset(new (std::nothrow) Fft1());
            if (!rec_alt) return JT_ENOMEM;
            rec_alt->n = n;
            rec_alt->algo = ALG_BLUESTEIN;
            rec_alt->nB = nS;
            JT_TRY(create(nS, rec_alt->pbl));
            return rec_alt->make_chirp();
        }
        if (algo != ALG_DIRECT || (generic_ok(n) && batch_line_ok<T>(n))) return JT_OK;
        int64_t best = 0;
        double bestd = 1e300;
        for (int64_t d = 2; d < n && d <= Lim<T>::lmax(); d++) {
            if (n % d) continue;
            const int64_t e = n / d;
            if (!generic_ok(d) || !generic_ok(e) || !batch_line_ok<T>(d) || !batch_line_ok<T>(e)) continue;
            const double dd = std::fabs(std::log((double)d) - std::log((double)e));
            if (dd < bestd) {
                bestd = dd;
                best = d;
            }
        }
        if (!best) return JT_OK;
        rec_alt.reset(new (std::nothrow) Fft1());
        if (!rec_alt) return JT_ENOMEM;
        rec_alt->n = n;
        return rec_alt->init_twopass(best);
    }

    // Bluestein in one CTA tile (jt_chirp.cuh) when the padded length fits
    // the tile passes: always inside batches, and for float calls (double
    // calls keep the register-kernel FFTs of the FP64-bound convolution)
    bool blue_fused_ok(const Ctx &ctx) const {
        const bool rec = ctx.rec || ctx.rec_sizing;
        return pbl && pbl->algo == ALG_DIRECT && pbl->W && generic_ok(nB) && (rec || sizeof(T) == 4) &&
               (!rec || batch_line_ok<T>(nB));
    }
    int exec_blue_fused(Ctx &ctx, const C2 *in, int64_t din, C2 *out, int64_t dout, int64_t batch, int sign,
                        double scale) const {
        BlueParams p;
        memset(&p, 0, sizeof(p));
        p.n = (int)n;
        p.nB = (int)nB;
        std::vector<int> rr = direct_radices(nB, radix_order(nB, sizeof(T) == 4));
        if (rr.empty() || (int)rr.size() > JT_MAX_PASSES) return JT_EINVAL;
        p.npass = (int)rr.size();
        for (int i = 0; i < p.npass; i++) p.radix[i] = rr[i];
        const size_t per_line = 2 * (size_t)padded_len((int)nB) * sizeof(C2);
        int C = (int)std::max<int64_t>(1, (ctx.rec ? kBatchTileElems : (sizeof(T) == 4 ? 4096 : 2048)) / nB);
        C = std::min(C, (int)std::max<size_t>(1, (size_t)g_smem_optin / per_line));
        if ((int64_t)C > batch) C = (int)batch;
        p.C = C;
        p.nlines = batch;
        p.lin = Layout{1, din, 0, 1};
        p.lout = Layout{1, dout, 0, 1};
        p.scale = scale;
        p.scalef = (float)scale;
        if (ctx.rec) {
            BOp o;
            memset(&o, 0, sizeof(o));
            o.type = BOP_BLUE;
            o.prec = sizeof(T) == 4 ? 0 : 1;
            o.sign = sign;
            o.in = in;
            o.out = out;
            o.W = pbl->W;
            o.Whi = bk1;
            o.Wlo = bk2;
            o.bp = p;
            o.ntasks = (int)cdiv(batch, C);
            o.smem = (int)(per_line * C);
            emit(ctx, o);
            return JT_OK;
        }
        if (ctx.dry) return JT_OK;  // no scratch
        const int64_t grid = cdiv(batch, C);
        if (grid > 0x7fffffff) return JT_ETOOBIG;
        const int threads = (int)std::min<int64_t>(512, std::max<int64_t>(64, cdiv((int64_t)C * nB / 16, 32) * 32));
        if (sign < 0)
            blue_tile_kernel<-1, T><<<(unsigned)grid, threads, per_line * C, ctx.s>>>(in, out, p, pbl->W, bk1, bk2);
        else
            blue_tile_kernel<1, T><<<(unsigned)grid, threads, per_line * C, ctx.s>>>(in, out, p, pbl->W, bk1, bk2);
        g_launches++;
        return JT_OK;
    }

    // Batch recording of a line pass: the generic tile kernel (any layout,
    // lengths up to the tile kernel's limit; longer one-pass lengths are
    // recorded through their two-pass alternate, make_rec_alt).
    int record_lines(Ctx &ctx, const C2 *in, C2 *out, int64_t nlines, const Layout &lin, const Layout &lout, int sign,
                     double scale, int64_t tw_n, int64_t tw_inner, const C2 *Whi_, const C2 *Wlo_, int tw_lo_bits) const {
        BOp o;
        memset(&o, 0, sizeof(o));
        o.prec = sizeof(T) == 4 ? 0 : 1;
        o.sign = sign;
        o.in = in;
        o.out = out;
        o.W = W;
        o.Whi = Whi_;
        o.Wlo = Wlo_;
        if (generic_ok(n)) {
            const int L = (int)n;
            const int Lp = padded_len(L);
            const bool strided = lin.estride != 1 || lout.estride != 1;
            int64_t target = kBatchTileElems;  // the batch CTA has 512 threads: 512 radix-16 butterflies
            int C = (int)std::max<int64_t>(1, target / L);
            if (strided) C = std::max(C, sizeof(T) == 4 ? 16 : 8);
            size_t per_line = 2 * (size_t)Lp * sizeof(C2);
            int cmax = (int)std::max<size_t>(1, std::min<size_t>(g_smem_optin, JT_BATCH_SMEM_CAP) / per_line);
            C = std::min(C, cmax);
            if ((int64_t)C > nlines) C = (int)nlines;
            std::vector<int> rr = radix.empty() ? direct_radices(n, radix_order(n, sizeof(T) == 4)) : radix;
            o.type = BOP_TILE;
            o.tp.L = L;
            o.tp.npass = (int)rr.size();
            for (int i = 0; i < o.tp.npass; i++) o.tp.radix[i] = rr[i];
            o.tp.C = C;
            o.tp.nlines = nlines;
            o.tp.lin = lin;
            o.tp.lout = lout;
            o.tp.scale = scale;
            o.tp.scalef = (float)scale;
            o.tp.do_scale = scale != 1.0;
            o.tp.tw_n = tw_n;
            o.tp.tw_inner = tw_inner;
            o.tp.tw_lo_bits = tw_lo_bits;
            o.ntasks = (int)cdiv(nlines, C);
            o.smem = (int)(per_line * C);
        } else {
            return JT_EINVAL;  // no single-CTA step for this line in a batch
        }
        emit(ctx, o);
        return JT_OK;
    }

    // DIRECT pass over `nlines` lines with arbitrary layouts.
    int exec_direct(Ctx &ctx, const C2 *in, C2 *out, int64_t nlines, const Layout &lin, const Layout &lout, int sign,
                    double scale, int64_t tw_n = 0, int64_t tw_inner = 1, const C2 *Whi_ = nullptr, const C2 *Wlo_ = nullptr,
                    int tw_lo_bits = 0, int hint_discard_in = 0, int hint_stream_out = 1, int hint_reverse = 0) const {
        if (nlines <= 0) return JT_OK;
        if (ctx.rec) return record_lines(ctx, in, out, nlines, lin, lout, sign, scale, tw_n, tw_inner, Whi_, Wlo_, tw_lo_bits);
        if (reg) {
            int mode = -1;
            if (lin.estride == 1 && lout.estride == 1) mode = 0;
            else if (lin.estride != 1 && lout.estride != 1 && n <= 4096) mode = 1;
            else if (lin.estride == 1 && lout.estride != 1 && n <= 4096) mode = 2;
            if (mode < 0 || (mode != 1 && tw_n != 0)) return JT_EINVAL;  // the four-step twiddle rides on column passes
            StockParams sp;
            memset(&sp, 0, sizeof(sp));
            sp.nlines = nlines;
            sp.lin = lin;
            sp.lout = lout;
            sp.scale = scale;
            sp.scalef = (float)scale;
            sp.do_scale = scale != 1.0;
            sp.tw_n = tw_n;
            sp.tw_inner = tw_inner;
            sp.tw_lo_bits = tw_lo_bits;
            // register kernels form twiddle exponents in 32 bits, reduced
            // modulo a power-of-two tw_n (up to 2^32); other lengths below 2^31
            if (tw_n != 0 && (is_pow2(tw_n) ? tw_n > ((int64_t)1 << 32) : tw_n >= ((int64_t)1 << 31))) return JT_ETOOBIG;
            sp.tw_mask = tw_n != 0 && is_pow2(tw_n) ? (uint32_t)(tw_n - 1) : 0xffffffffu;
            sp.discard_in = hint_discard_in;
            sp.stream_out = hint_stream_out;
            sp.reverse = hint_reverse;
            if (ctx.dry) return JT_OK;
            const int esz = (int)sizeof(C2);
            // split-operand tensor-core kernel for Float32 row passes
            if constexpr (sizeof(T) == 4) {
                if (ctx.tc && mode == 0 && tc_split_ok((int)n)) {
                    if (!tc_split_launch((int)n, sign, (const float2 *)in, (float2 *)out, sp, (const float2 *)Wp, g_err_dev,
                                         g_sms, ctx.s))
                        return JT_ECUDA;
                    g_launches++;
                    return JT_OK;
                }
            }
            // TMA pipeline when the 16-byte rules hold, else the plain kernel
            const int Cl = stockham_lines_per_cta((int)n, mode, (const T *)nullptr);
            CUtensorMap tm;
            memset(&tm, 0, sizeof(tm));
            bool pipe = g_opt_tma.load() && stockham_pipe_ok((int)n, mode, (const T *)nullptr) && ((uintptr_t)in % 16) == 0;
            if (pipe && mode == 1) {
                pipe = lin.istride == 1 && lin.inner % Cl == 0 && nlines % lin.inner == 0 &&
                       make_col_tmap(&tm, in, esz, lin.inner, n, nlines / lin.inner, lin.estride, lin.outer, Cl,
                                     (int)std::min<int64_t>(n, 256));
                sp.tiles_per_col = lin.inner / Cl;
            } else if (pipe) {
                bool contig = lin.inner == 1 && lin.outer == n;
                pipe = contig || ((lin.outer * esz) % 16 == 0 && (lin.inner == 1 || (lin.istride * esz) % 16 == 0));
                pipe = pipe && (n * esz) % 16 == 0;
            }
            if (!stockham_launch((int)n, mode, sign, in, out, sp, pipe ? &tm : nullptr, Wp, Whi_, Wlo_, g_err_dev, g_sms,
                                 ctx.s))
                return JT_EINVAL;
            g_launches++;
            return JT_OK;
        }
        const int L = (int)n;
        const int Lp = padded_len(L);
        const bool strided = lin.estride != 1 || lout.estride != 1;
        const int64_t target = tile_elems(L);
        int C = (int)std::max<int64_t>(1, target / L);
        if (strided) C = std::max(C, sizeof(T) == 4 ? 16 : 8);
        size_t per_line = 2 * (size_t)Lp * sizeof(C2);
        int cmax = (int)std::max<size_t>(1, (size_t)g_smem_optin / per_line);
        C = std::min(C, cmax);
        if ((int64_t)C > nlines) C = (int)nlines;
        size_t smem = per_line * C;
        int threads = (int)std::min<int64_t>(kMaxThreads, std::max<int64_t>(64, cdiv((int64_t)C * L / 16, 32) * 32));
        TileParams p;
        memset(&p, 0, sizeof(p));
        p.L = L;
        p.npass = (int)radix.size();
        for (int i = 0; i < p.npass; i++) p.radix[i] = radix[i];
        p.C = C;
        p.nlines = nlines;
        p.lin = lin;
        p.lout = lout;
        p.scale = scale;
        p.scalef = (float)scale;
        p.do_scale = scale != 1.0;
        p.tw_n = tw_n;
        p.tw_inner = tw_inner;
        p.tw_lo_bits = tw_lo_bits;
        if (ctx.dry) return JT_OK;
        int64_t grid = cdiv(nlines, C);
        if (grid > 0x7fffffff) return JT_ETOOBIG;
        if (sign < 0)
            fft_tile_kernel<-1, T><<<(unsigned)grid, threads, smem, ctx.s>>>(in, out, p, W, Whi_, Wlo_);
        else
            fft_tile_kernel<1, T><<<(unsigned)grid, threads, smem, ctx.s>>>(in, out, p, W, Whi_, Wlo_);
        g_launches++;
        return JT_OK;
    }

    // `batch` contiguous lines: line b at in + b*din, out + b*dout (complex units).
    int exec(Ctx &ctx, const C2 *in, int64_t din, C2 *out, int64_t dout, int64_t batch, int sign, double scale) const {
        if (batch <= 0) return JT_OK;
        switch (algo) {
            case ALG_TRIVIAL: {
                if (in == out && scale == 1.0) return JT_OK;
                if (ctx.rec) {
                    BOp o = elem_op<T>(EK_COPY_COMPLEX, 0, batch);
                    o.e.p[0] = in; o.e.p[1] = out; o.e.i[0] = din; o.e.i[1] = dout; o.e.i[2] = 1; o.e.i[3] = batch;
                    o.e.d[0] = scale; o.e.f = 0;
                    emit(ctx, o);
                    return JT_OK;
                }
                LAUNCH1D(ctx, batch, copy_complex_kernel<T>, in, din, out, dout, (int64_t)1, batch, scale, 0);
                return JT_OK;
            }
            case ALG_DIRECT: {
                if ((ctx.rec || ctx.rec_sizing) && rec_alt) return rec_alt->exec(ctx, in, din, out, dout, batch, sign, scale);
                Layout li = {1, din, 0, 1}, lo = {1, dout, 0, 1};
                return exec_direct(ctx, in, out, batch, li, lo, sign, scale);
            }
            case ALG_TWOPASS: {
                const int64_t chunk_bytes = (int64_t)g_opt_chunk_mb.load() << 20;
                int64_t chunk = std::max<int64_t>(1, std::min<int64_t>(batch, chunk_bytes / (n * (int64_t)sizeof(C2))));
                C2 *tmp = (C2 *)ctx.ws->get(sizeof(C2) * chunk * n, ctx.dry);
                for (int64_t b = 0; b < batch; b += chunk) {
                    int64_t cb = std::min(chunk, batch - b);
                    Layout lai = {n2, din, 1, n2}, lao = {n2, n, 1, n2};
                    JT_TRY(pa->exec_direct(ctx, in + b * din, tmp, cb * n2, lai, lao, sign, 1.0, n, n2, Whi, Wlo, lo_bits, 0, 0));
                    Layout lbi = {n1, n, n2, 1}, lbo = {n1, dout, 1, n1};
                    // pass B walks its tiles last to first: the transforms
                    // pass A wrote last are still in L2
                    JT_TRY(pb->exec_direct(ctx, tmp, out + b * dout, cb * n1, lbi, lbo, sign, scale, 0, 1, nullptr, nullptr, 0, 1, 1,
                                           1));
                }
                return JT_OK;
            }
            case ALG_THREEPASS: {
                if (ctx.rec) return JT_EINVAL;  // batches record lengths up to the tile kernel's
                const int64_t m = n2 * n3;
                const int64_t chunk_bytes = (int64_t)g_opt_chunk_mb.load() << 20;
                int64_t chunk = std::max<int64_t>(1, std::min<int64_t>(batch, chunk_bytes / (n * (int64_t)sizeof(C2))));
                C2 *tmp = (C2 *)ctx.ws->get(sizeof(C2) * chunk * n, ctx.dry);
                for (int64_t b = 0; b < batch; b += chunk) {
                    int64_t cb = std::min(chunk, batch - b);
                    // A: n1-point columns of the n1 x m view, twiddle w_n^{k1 c}
                    Layout lai = {m, din, 1, m}, lao = {m, n, 1, m};
                    JT_TRY(pa->exec_direct(ctx, in + b * din, tmp, cb * m, lai, lao, sign, 1.0, n, m, Whi, Wlo, lo_bits, 0, 0));
                    // B1: n2-point columns of each row's n2 x n3 view, twiddle
                    // w_m^{t u}, in place (a tile is in shared memory before
                    // any of its columns is written)
                    Layout lb = {n3, m, 1, n3};
                    JT_TRY(pb->exec_direct(ctx, tmp, tmp, cb * n1 * n3, lb, lb, sign, 1.0, m, n3, Whi2, Wlo2, lo_bits2, 0, 0));
                    // B2: n3-point rows, written to X[k1 + n1 (t + n2 v)];
                    // line k1 + n1 t of one transform per launch
                    Layout lci = {n1, n3, m, 1}, lco = {n1, n1, 1, n1 * n2};
                    for (int64_t t = 0; t < cb; t++)
                        JT_TRY(pc->exec_direct(ctx, tmp + t * n, out + (b + t) * dout, n1 * n2, lci, lco, sign, scale, 0, 1,
                                               nullptr, nullptr, 0, 1, 1));
                }
                return JT_OK;
            }
            case ALG_BLUESTEIN: {
                if ((ctx.rec || ctx.rec_sizing) && rec_alt) return rec_alt->exec(ctx, in, din, out, dout, batch, sign, scale);
                if (blue_fused_ok(ctx)) return exec_blue_fused(ctx, in, din, out, dout, batch, sign, scale);
                int64_t chunk = std::max<int64_t>(1, std::min<int64_t>(batch, (int64_t)(128ll << 20) / (nB * (int64_t)sizeof(C2))));
                C2 *tmp = (C2 *)ctx.ws->get(sizeof(C2) * chunk * nB, ctx.dry);
                for (int64_t b = 0; b < batch; b += chunk) {
                    int64_t cb = std::min(chunk, batch - b);
                    if (ctx.rec) {
                        BOp o = elem_op<T>(EK_BLUE_PRE, sign, cb * nB);
                        o.e.p[0] = in + b * din; o.e.p[1] = tmp; o.e.p[2] = bk1; o.e.i[0] = din; o.e.i[1] = n; o.e.i[2] = nB; o.e.i[3] = cb;
                        emit(ctx, o);
                    } else if (sign < 0) LAUNCH1D(ctx, cb * nB, (bluestein_pre_kernel<-1, T>), in + b * din, din, tmp, bk1, n, nB, cb);
                    else LAUNCH1D(ctx, cb * nB, (bluestein_pre_kernel<1, T>), in + b * din, din, tmp, bk1, n, nB, cb);
                    JT_TRY(pbl->exec(ctx, tmp, nB, tmp, nB, cb, -1, 1.0));
                    if (ctx.rec) {
                        BOp o = elem_op<T>(EK_BLUE_MUL, sign, cb * nB);
                        o.e.p[0] = tmp; o.e.p[1] = bk2; o.e.i[0] = nB; o.e.i[1] = cb * nB;
                        emit(ctx, o);
                    } else if (sign < 0) LAUNCH1D(ctx, cb * nB, (bluestein_mul_kernel<-1, T>), tmp, bk2, nB, cb * nB);
                    else LAUNCH1D(ctx, cb * nB, (bluestein_mul_kernel<1, T>), tmp, bk2, nB, cb * nB);
                    JT_TRY(pbl->exec(ctx, tmp, nB, tmp, nB, cb, 1, 1.0));
                    if (ctx.rec) {
                        BOp o = elem_op<T>(EK_BLUE_POST, sign, cb * n);
                        o.e.p[0] = out + b * dout; o.e.p[1] = tmp; o.e.p[2] = bk1; o.e.i[0] = dout; o.e.i[1] = n; o.e.i[2] = nB;
                        o.e.i[3] = cb; o.e.d[0] = scale;
                        emit(ctx, o);
                    } else if (sign < 0) LAUNCH1D(ctx, cb * n, (bluestein_post_kernel<-1, T>), out + b * dout, dout, tmp, bk1, n, nB, cb, scale);
                    else LAUNCH1D(ctx, cb * n, (bluestein_post_kernel<1, T>), out + b * dout, dout, tmp, bk1, n, nB, cb, scale);
                }
                return JT_OK;
            }
        }
        return JT_EINVAL;
    }
};

// bk1 (n) and bk2 = FFT_-(symmetric chirp / nB) (nB), built in FP64 on the
// device and rounded to T (fft/DoubleFFT_1D.java:1864-1890).
template <typename T> int Fft1<T>::make_chirp() {
    JT_CU(cudaMalloc(&bk1, sizeof(C2) * n));
    JT_CU(cudaMalloc(&bk2, sizeof(C2) * nB));
    double2 *b64 = nullptr;
    JT_CU(cudaMallocAsync(&b64, sizeof(double2) * nB, g_setup));
    chirp_kernel<T><<<(unsigned)cdiv(nB, 256), 256, 0, g_setup>>>(bk1, b64, n, nB);
    g_launches++;
    int st = JT_OK;
    {
        std::unique_ptr<Fft1<double>> f64;
        st = Fft1<double>::create(nB, f64);
        if (st == JT_OK) {
            Arena ar;
            Ctx c;
            c.s = g_setup;
            c.ws = &ar;
            c.dry = true;
            st = f64->exec(c, b64, nB, b64, nB, 1, -1, 1.0);
            if (st == JT_OK) {
                if (ar.peak) {
                    if (cudaMallocAsync((void **)&ar.base, ar.peak, g_setup) != cudaSuccess) st = JT_ENOMEM;
                    ar.cap = ar.peak;
                }
                ar.used = 0;
                c.dry = false;
                if (st == JT_OK) st = f64->exec(c, b64, nB, b64, nB, 1, -1, 1.0);
                if (ar.base) cudaFreeAsync(ar.base, g_setup);
            }
            // the FP64 plan's own tables are freed when it goes out of scope:
            // its kernels on the setup stream finish first
            cudaStreamSynchronize(g_setup);
        }
    }
    if (st == JT_OK) {
        d2t_kernel<T><<<(unsigned)cdiv(nB, 256), 256, 0, g_setup>>>(bk2, b64, nB);
        g_launches++;
    }
    cudaFreeAsync(b64, g_setup);
    JT_CU(cudaGetLastError());
    return st;
}

// ---------------------------------------------------------------------------
// Table cache.  The per-length objects below (complex, real, DCT/DST and DHT
// lines) and their device tables are shared by every jt_plan that needs
// them, keyed by (length, planning generation): a second DoubleFFT_1D(4096)
// builds nothing.  Entries that no plan holds any more are kept, least
// recently used first out, up to kCacheIdleMax per object type.
// ---------------------------------------------------------------------------
static std::recursive_mutex g_cache_mu;
static const int kCacheIdleMax = 32;

template <typename X> struct TableCache {
    struct Entry {
        std::shared_ptr<X> obj;
        uint64_t tick;
    };
    std::map<std::pair<int64_t, uint64_t>, Entry> m;
    uint64_t tick = 0;
    static TableCache &get() {
        static TableCache c;
        return c;
    }
};

template <typename X> static int cached(int64_t n, std::shared_ptr<X> &out) {
    std::lock_guard<std::recursive_mutex> g(g_cache_mu);
    TableCache<X> &c = TableCache<X>::get();
    const auto key = std::make_pair(n, g_plan_gen.load());
    auto it = c.m.find(key);
    if (it != c.m.end()) {
        it->second.tick = ++c.tick;
        out = it->second.obj;
        return JT_OK;
    }
    std::unique_ptr<X> u;
    JT_TRY(X::create(n, u));
    g_setup_seq++;
    std::shared_ptr<X> sp(u.release());
    c.m.emplace(key, typename TableCache<X>::Entry{sp, ++c.tick});
    out = sp;
    for (;;) {
        int idle = 0;
        auto victim = c.m.end();
        for (auto e = c.m.begin(); e != c.m.end(); ++e)
            if (e->second.obj.use_count() == 1) {
                idle++;
                if (victim == c.m.end() || e->second.tick < victim->second.tick) victim = e;
            }
        if (idle <= kCacheIdleMax) break;
        // kernels of a destroyed plan may still read the victim's tables
        JT_CU(cudaDeviceSynchronize());
        c.m.erase(victim);
    }
    return JT_OK;
}

// One-kernel line form (defined below, after the real and r2r plans)
template <typename T> struct Real1;
template <typename T> static bool r2r_fused_ok(const Ctx &, int64_t n, const Real1<T> *rf);
template <typename T> static int r2r_reg_c(int64_t h, const Real1<T> *rf);
template <typename T>
static int r2r_fused(Ctx &ctx, int op, const Real1<T> *rf, const T *in, T *out, int64_t nlines, const Layout &lin,
                     const Layout &lout, int dst, double mult, double mult0, const typename V2<T>::t *Wd);

// ---------------------------------------------------------------------------
// Real FFT of length n (packed layouts of fft/DoubleFFT_1D.java:433-451)
// ---------------------------------------------------------------------------
template <typename T> struct Real1 {
    typedef typename V2<T>::t C2;
    int64_t n = 0;
    std::shared_ptr<Fft1<T>> half, full;
    C2 *Wr = nullptr;
    ~Real1() {
        if (Wr) cudaFree(Wr);
    }
    static int create(int64_t n, std::unique_ptr<Real1> &out) {
        std::unique_ptr<Real1> r(new (std::nothrow) Real1());
        if (!r) return JT_ENOMEM;
        r->n = n;
        if (n >= 2 && n % 2 == 0) {
            JT_TRY(cached<Fft1<T>>(n / 2, r->half));
            JT_TRY(Fft1<T>::make_roots(&r->Wr, n / 4 + 1, 1, n));
        } else if (n > 1) {
            JT_TRY(cached<Fft1<T>>(n, r->full));
        }
        out = std::move(r);
        return JT_OK;
    }
    bool even() const { return n >= 2 && n % 2 == 0; }
    // One kernel for packed realForward/realInverse: the FP64-bound double
    // lines, batch steps, and float lines with a register form whose scalar
    // pairs are aligned complex values (paired loads and stores)
    bool fused_here(const Ctx &ctx, const T *a, int64_t dist) const {
        if (!r2r_fused_ok<T>(ctx, n, this)) return false;
        if (sizeof(T) == 8 || ctx.rec || ctx.rec_sizing) return true;
        return g_opt_real_fused_f32.load() != 0 && r2r_reg_c<T>(n / 2, this) > 0 && dist % 2 == 0 &&
               ((uintptr_t)a % sizeof(C2)) == 0;
    }

    // In place: n reals at a + b*dist -> packed spectrum.  dist must be even
    // for even n (the complex view).
    int fwd_packed(Ctx &ctx, T *a, int64_t dist, int64_t batch) const {
        if (n == 1 || batch <= 0) return JT_OK;
        // one kernel (the half-length FFT with the real split on its store)
        // where fused_here allows; otherwise the TMA-pipelined FFT and a
        // separate split
        if (fused_here(ctx, a, dist)) {
            const Layout l = {1, dist, 0, 1};
            return r2r_fused<T>(ctx, R2R_RFWD, this, a, a, batch, l, l, 0, 1.0, 1.0, nullptr);
        }
        if (even()) {
            JT_TRY(half->exec(ctx, (C2 *)a, dist / 2, (C2 *)a, dist / 2, batch, -1, 1.0));
            if (ctx.rec) {
                BOp o = elem_op<T>(EK_REAL_POST_PACKED, 0, batch * (n / 4 + 1));
                o.e.p[0] = a; o.e.p[1] = Wr; o.e.i[0] = dist; o.e.i[1] = n; o.e.i[2] = batch;
                emit(ctx, o);
            } else LAUNCH1D(ctx, batch * (n / 4 + 1), real_post_packed_kernel<T>, a, dist, n, batch, Wr);
            return JT_OK;
        }
        C2 *tmp = (C2 *)ctx.ws->get(sizeof(C2) * batch * n, ctx.dry);
        if (ctx.rec) {
            BOp o = elem_op<T>(EK_R2C, 0, batch * n);
            o.e.p[0] = a; o.e.p[1] = tmp; o.e.i[0] = dist; o.e.i[1] = n; o.e.i[2] = batch;
            emit(ctx, o);
        } else LAUNCH1D(ctx, batch * n, real_to_complex_kernel<T>, a, dist, tmp, n, batch);
        JT_TRY(full->exec(ctx, tmp, n, tmp, n, batch, -1, 1.0));
        if (ctx.rec) {
            BOp o = elem_op<T>(EK_PACK_FULL, 0, batch * n);
            o.e.p[0] = tmp; o.e.p[1] = a; o.e.i[0] = dist; o.e.i[1] = n; o.e.i[2] = batch;
            emit(ctx, o);
        } else LAUNCH1D(ctx, batch * n, pack_from_full_kernel<T>, tmp, a, dist, n, batch);
        return JT_OK;
    }

    // n reals at a + b*dist -> 2n (full complex spectrum) at the same place;
    // sign=+1 gives the e^{+} transform (realInverseFull), times scale.
    int fwd_full(Ctx &ctx, T *a, int64_t dist, int64_t batch, int sign, double scale) const {
        if (batch <= 0) return JT_OK;
        if (n == 1) {
            if (ctx.rec) {
                BOp o = elem_op<T>(EK_SCALE, 0, batch);
                o.e.p[0] = a; o.e.i[0] = dist; o.e.i[1] = 1; o.e.i[2] = batch; o.e.d[0] = scale;
                emit(ctx, o);
                BOp o2 = elem_op<T>(EK_SCALE, 0, batch);
                o2.e.p[0] = a + 1; o2.e.i[0] = dist; o2.e.i[1] = 1; o2.e.i[2] = batch; o2.e.d[0] = 0.0;
                emit(ctx, o2);
                return JT_OK;
            }
            LAUNCH1D(ctx, batch, scale_kernel<T>, a, dist, (int64_t)1, batch, scale);
            LAUNCH1D(ctx, batch, scale_kernel<T>, a + 1, dist, (int64_t)1, batch, 0.0);
            return JT_OK;
        }
        if (even()) {
            const int64_t h = n / 2;
            C2 *tmp = (C2 *)ctx.ws->get(sizeof(C2) * batch * h, ctx.dry);
            JT_TRY(half->exec(ctx, (const C2 *)a, dist / 2, tmp, h, batch, sign, 1.0));
            if (ctx.rec) {
                BOp o = elem_op<T>(EK_REAL_POST_FULL, sign, batch * (h / 2 + 1));
                o.e.p[0] = tmp; o.e.p[1] = a; o.e.p[2] = Wr; o.e.i[0] = 2 * h; o.e.i[1] = dist; o.e.i[2] = n; o.e.i[3] = batch;
                o.e.d[0] = scale;
                emit(ctx, o);
            } else if (sign < 0)
                LAUNCH1D(ctx, batch * (h / 2 + 1), (real_post_full_kernel<-1, T>), (const T *)tmp, 2 * h, a, dist, n, batch, Wr, scale);
            else
                LAUNCH1D(ctx, batch * (h / 2 + 1), (real_post_full_kernel<1, T>), (const T *)tmp, 2 * h, a, dist, n, batch, Wr, scale);
            return JT_OK;
        }
        C2 *tmp = (C2 *)ctx.ws->get(sizeof(C2) * batch * n, ctx.dry);
        if (ctx.rec) {
            BOp o = elem_op<T>(EK_R2C, 0, batch * n);
            o.e.p[0] = a; o.e.p[1] = tmp; o.e.i[0] = dist; o.e.i[1] = n; o.e.i[2] = batch;
            emit(ctx, o);
        } else LAUNCH1D(ctx, batch * n, real_to_complex_kernel<T>, a, dist, tmp, n, batch);
        JT_TRY(full->exec(ctx, tmp, n, tmp, n, batch, sign, scale));
        if (ctx.rec) {
            BOp o = elem_op<T>(EK_COPY_COMPLEX, 0, batch * n);
            o.e.p[0] = tmp; o.e.p[1] = a; o.e.i[0] = n; o.e.i[1] = dist / 2; o.e.i[2] = n; o.e.i[3] = batch; o.e.d[0] = 1.0;
            emit(ctx, o);
        } else LAUNCH1D(ctx, batch * n, copy_complex_kernel<T>, tmp, n, (C2 *)a, dist / 2, n, batch, 1.0, 0);
        return JT_OK;
    }

    // In place: packed spectrum -> factor * x, x the 1/n-normalised inverse.
    int inv_packed(Ctx &ctx, T *a, int64_t dist, int64_t batch, double factor) const {
        if (batch <= 0) return JT_OK;
        if (n == 1) {
            if (factor != 1.0) {
                if (ctx.rec) {
                    BOp o = elem_op<T>(EK_SCALE, 0, batch);
                    o.e.p[0] = a; o.e.i[0] = dist; o.e.i[1] = 1; o.e.i[2] = batch; o.e.d[0] = factor;
                    emit(ctx, o);
                } else LAUNCH1D(ctx, batch, scale_kernel<T>, a, dist, (int64_t)1, batch, factor);
            }
            return JT_OK;
        }
        if (fused_here(ctx, a, dist)) {
            const Layout l = {1, dist, 0, 1};
            return r2r_fused<T>(ctx, R2R_RINV, this, a, a, batch, l, l, 0, factor * 2.0 / (double)n, 1.0, nullptr);
        }
        if (even()) {
            if (ctx.rec) {
                BOp o = elem_op<T>(EK_REAL_PRE_INV, 0, batch * (n / 4 + 1));
                o.e.p[0] = a; o.e.p[1] = Wr; o.e.i[0] = dist; o.e.i[1] = n; o.e.i[2] = batch; o.e.d[0] = factor * 2.0 / (double)n;
                emit(ctx, o);
            } else LAUNCH1D(ctx, batch * (n / 4 + 1), real_pre_inverse_kernel<T>, a, dist, n, batch, Wr, factor * 2.0 / (double)n);
            JT_TRY(half->exec(ctx, (C2 *)a, dist / 2, (C2 *)a, dist / 2, batch, 1, 1.0));
            return JT_OK;
        }
        C2 *tmp = (C2 *)ctx.ws->get(sizeof(C2) * batch * n, ctx.dry);
        if (ctx.rec) {
            BOp o = elem_op<T>(EK_UNPACK_FULL, 0, batch * n);
            o.e.p[0] = a; o.e.p[1] = tmp; o.e.i[0] = dist; o.e.i[1] = n; o.e.i[2] = batch;
            emit(ctx, o);
        } else LAUNCH1D(ctx, batch * n, unpack_to_full_kernel<T>, a, dist, tmp, n, batch);
        JT_TRY(full->exec(ctx, tmp, n, tmp, n, batch, 1, 1.0));
        if (ctx.rec) {
            BOp o = elem_op<T>(EK_REAL_PART, 0, batch * n);
            o.e.p[0] = tmp; o.e.p[1] = a; o.e.i[0] = dist; o.e.i[1] = n; o.e.i[2] = batch; o.e.d[0] = factor / (double)n;
            emit(ctx, o);
        } else LAUNCH1D(ctx, batch * n, real_part_kernel<T>, tmp, a, dist, n, batch, factor / (double)n);
        return JT_OK;
    }
};

// ---------------------------------------------------------------------------
// One-kernel DCT/DST/DHT lines (jt_r2r.cuh): even n whose half length the
// tile passes run (h = n/2 up to the tile kernel's limit, prime factors <= 63),
// any line layout.  Batch recordings keep the separate pre/post steps.
// ---------------------------------------------------------------------------
template <typename T> static bool r2r_fused_ok(const Ctx &ctx, int64_t n, const Real1<T> *rf) {
    return n >= 4 && n % 2 == 0 && rf && rf->half && rf->half->algo == ALG_DIRECT && rf->half->W && rf->Wr &&
           Fft1<T>::generic_ok(n / 2) && (!(ctx.rec || ctx.rec_sizing) || batch_line_ok<T>(n / 2));
}

// Lines per CTA of the register form for half length h (0: none): power-of-
// two h from 16 to 4096 whose plan holds the pass table
template <typename T> static int r2r_reg_c(int64_t h, const Real1<T> *rf) {
    if (!is_pow2(h) || h < 16 || h > 4096 || !rf->half->reg || !rf->half->Wp) return 0;
    return r2r_reg_lines((int)h, (const T *)nullptr);
}

// Whether strided (column) lines run in one kernel with coalesced enough
// access: at least 32-byte runs of adjacent lines per CTA
template <typename T> static bool r2r_strided_ok(const Ctx &ctx, int64_t n, const Real1<T> *rf) {
    if (!r2r_fused_ok<T>(ctx, n, rf)) return false;
    const int64_t h = n / 2;
    const int need = (int)(32 / sizeof(T));
    if (r2r_reg_c<T>(h, rf) >= need) return true;
    const size_t per_line = 2 * (size_t)padded_len((int)h) * sizeof(typename V2<T>::t);
    return (size_t)g_smem_optin / per_line >= (size_t)need;
}

template <typename T>
static int r2r_fused(Ctx &ctx, int op, const Real1<T> *rf, const T *in, T *out, int64_t nlines, const Layout &lin,
                     const Layout &lout, int dst, double mult, double mult0, const typename V2<T>::t *Wd) {
    typedef typename V2<T>::t C2;
    if (nlines <= 0) return JT_OK;
    const int64_t n = rf->n, h = n / 2;
    std::vector<int> rr = direct_radices(h, radix_order(h, sizeof(T) == 4));
    if (rr.empty() || (int)rr.size() > JT_MAX_PASSES) return JT_EINVAL;
    R2rParams p;
    memset(&p, 0, sizeof(p));
    p.n = (int)n;
    p.npass = (int)rr.size();
    for (int i = 0; i < p.npass; i++) p.radix[i] = rr[i];
    const int Lp = padded_len((int)h);
    const bool strided = lin.estride != 1 || lout.estride != 1;
    int C = (int)std::max<int64_t>(1, (ctx.rec ? kBatchTileElems : (sizeof(T) == 4 ? 4096 : 2048)) / h);
    if (strided) C = std::max(C, sizeof(T) == 4 ? 16 : 8);
    const size_t per_line = 2 * (size_t)Lp * sizeof(C2);
    C = std::min(C, (int)std::max<size_t>(1, (size_t)g_smem_optin / per_line));
    if ((int64_t)C > nlines) C = (int)nlines;
    p.C = C;
    p.nlines = nlines;
    p.lin = lin;
    p.lout = lout;
    p.dst = dst;
    p.mult = mult;
    p.mult0 = mult0;
    p.multf = (float)mult;
    p.mult0f = (float)mult0;
    // scalar pairs as aligned complex values: contiguous lines at even
    // offsets from an aligned base
    auto paired = [](const T *ptr, const Layout &l) {
        return l.estride == 1 && ((uintptr_t)ptr % sizeof(C2)) == 0 && l.outer % 2 == 0 && (l.inner == 1 || l.istride % 2 == 0);
    };
    p.vec_in = paired(in, lin) ? 1 : 0;
    p.vec_out = paired(out, lout) ? 1 : 0;
    if (ctx.rec) {
        // a batch step: the tile form, run by the batch kernel's CTAs
        BOp o;
        memset(&o, 0, sizeof(o));
        o.type = BOP_R2R;
        o.prec = sizeof(T) == 4 ? 0 : 1;
        o.kind = op;
        o.in = in;
        o.out = out;
        o.W = rf->half->W;
        o.Whi = rf->Wr;
        o.Wlo = Wd;
        o.rp = p;
        o.ntasks = (int)cdiv(nlines, C);
        o.smem = (int)(per_line * C);
        emit(ctx, o);
        return JT_OK;
    }
    // the register form when h has one and the runs stay coalesced; lines
    // per CTA from its maximum down so that the grid covers the SMs twice
    // (at least 32-byte runs on strided lines, at least one warp per CTA)
    const int creg = r2r_reg_c<T>(h, rf);
    if (creg > 0 && (!strided || creg >= (int)(32 / sizeof(T)))) {
        int cr = creg;
        const int cmin = std::max<int>(strided ? (int)(32 / sizeof(T)) : 1, (int)std::max<int64_t>(1, 32 / (h / 16)));
        while (cr > cmin && cdiv(nlines, cr) < 2 * (int64_t)g_sms) cr /= 2;
        p.C = std::max(cr, 1);
        if (ctx.dry) return JT_OK;
        if (cdiv(nlines, creg) > 0x7fffffff) return JT_ETOOBIG;
        if (!r2r_reg_launch((int)h, op, in, out, p, rf->half->Wp, rf->Wr, Wd, ctx.s)) return JT_EINVAL;
        g_launches++;
        return JT_OK;
    }
    if (ctx.dry) return JT_OK;
    const int64_t grid = cdiv(nlines, C);
    if (grid > 0x7fffffff) return JT_ETOOBIG;
    const int threads = (int)std::min<int64_t>(512, std::max<int64_t>(64, cdiv((int64_t)C * h / 8, 32) * 32));
    const size_t smem = per_line * C;
    const C2 *W = rf->half->W;
    if (op == R2R_DCT2) r2r_tile_kernel<R2R_DCT2, T><<<(unsigned)grid, threads, smem, ctx.s>>>(in, out, p, W, rf->Wr, Wd);
    else if (op == R2R_DCT3) r2r_tile_kernel<R2R_DCT3, T><<<(unsigned)grid, threads, smem, ctx.s>>>(in, out, p, W, rf->Wr, Wd);
    else if (op == R2R_DHT) r2r_tile_kernel<R2R_DHT, T><<<(unsigned)grid, threads, smem, ctx.s>>>(in, out, p, W, rf->Wr, Wd);
    else if (op == R2R_RFWD) r2r_tile_kernel<R2R_RFWD, T><<<(unsigned)grid, threads, smem, ctx.s>>>(in, out, p, W, rf->Wr, Wd);
    else r2r_tile_kernel<R2R_RINV, T><<<(unsigned)grid, threads, smem, ctx.s>>>(in, out, p, W, rf->Wr, Wd);
    g_launches++;
    return JT_OK;
}

// ---------------------------------------------------------------------------
// DCT-II/III and DST-II/III (dct/DoubleDCT_1D.java:169-440, dst/DoubleDST_1D.java)
// ---------------------------------------------------------------------------
template <typename T> struct Dct1 {
    typedef typename V2<T>::t C2;
    int64_t n = 0;
    std::shared_ptr<Real1<T>> rf;
    C2 *Wd = nullptr;
    ~Dct1() {
        if (Wd) cudaFree(Wd);
    }
    static int create(int64_t n, std::unique_ptr<Dct1> &out) {
        std::unique_ptr<Dct1> d(new (std::nothrow) Dct1());
        if (!d) return JT_ENOMEM;
        d->n = n;
        if (n > 1) {
            JT_TRY(cached<Real1<T>>(n, d->rf));
            JT_TRY(Fft1<T>::make_roots(&d->Wd, n, 1, 4 * n));  // e^{-i pi k/(2n)}
        }
        out = std::move(d);
        return JT_OK;
    }
    int64_t vdist() const { return (n + 1) & ~(int64_t)1; }

    bool strided_ok(const Ctx &ctx) const { return r2r_strided_ok<T>(ctx, n, rf.get()); }

    // `nlines` lines in place with layout l (scalar units): one kernel when
    // the length allows it, else (contiguous lines only) the separate steps
    int lines(Ctx &ctx, bool fwd, T *a, int64_t nlines, const Layout &l, bool scale, bool dst) const {
        if (n == 1 || nlines <= 0) return JT_OK;
        if (r2r_fused_ok<T>(ctx, n, rf.get())) {
            double m, m0;
            if (fwd) {
                if (scale) {
                    m = std::sqrt(2.0 / (double)n);
                    m0 = 1.0 / std::sqrt((double)n);
                } else {
                    m = m0 = is_pow2(n) ? 1.0 : 2.0;
                }
                return r2r_fused<T>(ctx, R2R_DCT2, rf.get(), a, a, nlines, l, l, dst, m, m0, Wd);
            }
            // coefficient scales of the inverse: q for k >= 1, 2 q0 for k = 0
            if (scale) {
                m = std::sqrt(2.0 / (double)n);
                m0 = 2.0 / std::sqrt((double)n);
            } else if (is_pow2(n)) {
                m = 1.0;
                m0 = 2.0;
            } else {
                m = 1.0 / (double)n;
                m0 = 1.0 / (double)n;
            }
            return r2r_fused<T>(ctx, R2R_DCT3, rf.get(), a, a, nlines, l, l, dst, m, m0, Wd);
        }
        if (l.estride != 1 || (l.inner != 1 && nlines > 1)) return JT_EINVAL;
        return fwd ? forward(ctx, a, l.outer, nlines, scale, dst) : inverse(ctx, a, l.outer, nlines, scale, dst);
    }

    int forward(Ctx &ctx, T *a, int64_t dist, int64_t batch, bool scale, bool dst) const {
        if (n == 1 || batch <= 0) return JT_OK;
        const int64_t vd = vdist();
        T *v = (T *)ctx.ws->get(sizeof(T) * batch * vd, ctx.dry);
        if (ctx.rec) {
            BOp o = elem_op<T>(EK_DCT2_PRE, 0, batch * n);
            o.e.p[0] = a; o.e.p[1] = v; o.e.i[0] = dist; o.e.i[1] = vd; o.e.i[2] = n; o.e.i[3] = batch; o.e.f = (int)dst;
            emit(ctx, o);
        } else LAUNCH1D(ctx, batch * n, dct2_pre_kernel<T>, a, dist, v, vd, n, batch, (int)dst);
        JT_TRY(rf->fwd_packed(ctx, v, vd, batch));
        double mult, mult0;
        if (scale) {
            mult = std::sqrt(2.0 / (double)n);
            mult0 = 1.0 / std::sqrt((double)n);
        } else {
            mult = mult0 = is_pow2(n) ? 1.0 : 2.0;
        }
        if (ctx.rec) {
            BOp o = elem_op<T>(EK_DCT2_POST, 0, batch * n);
            o.e.p[0] = v; o.e.p[1] = a; o.e.p[2] = Wd; o.e.i[0] = vd; o.e.i[1] = dist; o.e.i[2] = n; o.e.i[3] = batch;
            o.e.d[0] = mult; o.e.d[1] = mult0; o.e.f = (int)dst;
            emit(ctx, o);
        } else LAUNCH1D(ctx, batch * n, dct2_post_kernel<T>, v, vd, a, dist, n, batch, Wd, mult, mult0, (int)dst);
        return JT_OK;
    }

    int inverse(Ctx &ctx, T *a, int64_t dist, int64_t batch, bool scale, bool dst) const {
        if (n == 1 || batch <= 0) return JT_OK;
        const int64_t vd = vdist();
        T *v = (T *)ctx.ws->get(sizeof(T) * batch * vd, ctx.dry);
        double q, q0;
        if (scale) {
            q = std::sqrt(2.0 / (double)n);
            q0 = 1.0 / std::sqrt((double)n);
        } else if (is_pow2(n)) {
            q = q0 = 1.0;
        } else {
            q = 1.0 / (double)n;
            q0 = 0.5 / (double)n;
        }
        if (ctx.rec) {
            BOp o = elem_op<T>(EK_DCT3_PRE, 0, batch * (n / 2 + 1));
            o.e.p[0] = a; o.e.p[1] = v; o.e.p[2] = Wd; o.e.i[0] = dist; o.e.i[1] = vd; o.e.i[2] = n; o.e.i[3] = batch;
            o.e.d[0] = q * (double)n / 2.0; o.e.d[1] = q0 * (double)n; o.e.f = (int)dst;
            emit(ctx, o);
        } else LAUNCH1D(ctx, batch * (n / 2 + 1), dct3_pre_kernel<T>, a, dist, v, vd, n, batch, Wd, q * (double)n / 2.0,
                 q0 * (double)n, (int)dst);
        JT_TRY(rf->inv_packed(ctx, v, vd, batch, 1.0));
        if (ctx.rec) {
            BOp o = elem_op<T>(EK_DCT3_POST, 0, batch * n);
            o.e.p[0] = v; o.e.p[1] = a; o.e.i[0] = vd; o.e.i[1] = dist; o.e.i[2] = n; o.e.i[3] = batch; o.e.f = (int)dst;
            emit(ctx, o);
        } else LAUNCH1D(ctx, batch * n, dct3_post_kernel<T>, v, vd, a, dist, n, batch, (int)dst);
        return JT_OK;
    }
};

// DHT (dht/DoubleDHT_1D.java:94-159, :255-276)
template <typename T> struct Dht1 {
    int64_t n = 0;
    std::shared_ptr<Real1<T>> rf;
    static int create(int64_t n, std::unique_ptr<Dht1> &out) {
        std::unique_ptr<Dht1> d(new (std::nothrow) Dht1());
        if (!d) return JT_ENOMEM;
        d->n = n;
        if (n > 1) JT_TRY(cached<Real1<T>>(n, d->rf));
        out = std::move(d);
        return JT_OK;
    }
    bool strided_ok(const Ctx &ctx) const { return r2r_strided_ok<T>(ctx, n, rf.get()); }

    // `nlines` lines in place with layout l (scalar units)
    int lines(Ctx &ctx, T *a, int64_t nlines, const Layout &l, double mult) const {
        if (n == 1 || nlines <= 0) return JT_OK;
        if (r2r_fused_ok<T>(ctx, n, rf.get())) return r2r_fused<T>(ctx, R2R_DHT, rf.get(), a, a, nlines, l, l, 0, mult, mult, nullptr);
        if (l.estride != 1 || (l.inner != 1 && nlines > 1)) return JT_EINVAL;
        return forward(ctx, a, l.outer, nlines, mult);
    }

    int forward(Ctx &ctx, T *a, int64_t dist, int64_t batch, double mult) const {
        if (n == 1 || batch <= 0) return JT_OK;
        const int64_t vd = (n + 1) & ~(int64_t)1;
        T *v = (T *)ctx.ws->get(sizeof(T) * batch * vd, ctx.dry);
        if (ctx.rec) {
            BOp o = elem_op<T>(EK_COPY_REAL, 0, batch * n);
            o.e.p[0] = a; o.e.p[1] = v; o.e.i[0] = dist; o.e.i[1] = vd; o.e.i[2] = n; o.e.i[3] = batch;
            emit(ctx, o);
        } else LAUNCH1D(ctx, batch * n, copy_real_kernel<T>, a, dist, v, vd, n, batch);
        JT_TRY(rf->fwd_packed(ctx, v, vd, batch));
        if (ctx.rec) {
            BOp o = elem_op<T>(EK_DHT_POST, 0, batch * n);
            o.e.p[0] = v; o.e.p[1] = a; o.e.i[0] = vd; o.e.i[1] = dist; o.e.i[2] = n; o.e.i[3] = batch; o.e.d[0] = mult;
            emit(ctx, o);
        } else LAUNCH1D(ctx, batch * n, dht_post_kernel<T>, v, vd, a, dist, n, batch, mult);
        return JT_OK;
    }
};

// ---------------------------------------------------------------------------
// Plan: one transform kind/precision over 1..3 dimensions.
// ---------------------------------------------------------------------------
template <typename T> struct PlanImpl {
    typedef typename V2<T>::t C2;
    int kind = JT_FFT, nd = 1;
    int64_t dims[3] = {1, 1, 1};
    int64_t N = 1;
    std::mutex mu;
    // per axis length, from the table cache (shared with other plans)
    std::map<int64_t, std::shared_ptr<Fft1<T>>> fft;
    std::map<int64_t, std::shared_ptr<Real1<T>>> real;
    std::map<int64_t, std::shared_ptr<Dct1<T>>> dct;
    std::map<int64_t, std::shared_ptr<Dht1<T>>> dht;
    template <typename X> static int get(std::map<int64_t, std::shared_ptr<X>> &m, int64_t n, X **out) {
        auto it = m.find(n);
        if (it == m.end()) {
            std::shared_ptr<X> f;
            JT_TRY(cached<X>(n, f));
            it = m.emplace(n, std::move(f)).first;
        }
        *out = it->second.get();
        return JT_OK;
    }
    int get_fft(int64_t n, Fft1<T> **out) { return get(fft, n, out); }
    int get_real(int64_t n, Real1<T> **out) { return get(real, n, out); }
    int get_dct(int64_t n, Dct1<T> **out) { return get(dct, n, out); }
    int get_dht(int64_t n, Dht1<T> **out) { return get(dht, n, out); }

    // Builds (or takes from the cache) every table `op` needs, under the
    // mutex; when anything was built, waits for the setup stream.
    int prepare(int op) {
        const uint64_t seq0 = g_setup_seq.load();
        int st = prepare_locked(op);
        if (st == JT_OK && g_setup_seq.load() != seq0) {
            JT_CU(cudaStreamSynchronize(g_setup));
            JT_CU(cudaGetLastError());
        }
        return st;
    }
    int prepare_locked(int op) {
        std::lock_guard<std::mutex> g(mu);
        Fft1<T> *f;
        Real1<T> *r;
        Dct1<T> *d;
        Dht1<T> *h;
        if (kind == JT_FFT) {
            if (nd == 1 && (op == JT_REAL_FORWARD || op == JT_REAL_INVERSE || op == JT_REAL_FORWARD_FULL || op == JT_REAL_INVERSE_FULL))
                return get_real(dims[0], &r);
            if (nd == 2 && (op == JT_REAL_FORWARD || op == JT_REAL_INVERSE)) {
                JT_TRY(get_real(dims[1], &r));
                return get_fft(dims[0], &f);
            }
            if (nd == 3 && (op == JT_REAL_FORWARD || op == JT_REAL_INVERSE)) {
                JT_TRY(get_real(dims[2], &r));
                JT_TRY(get_fft(dims[1], &f));
                return get_fft(dims[0], &f);
            }
            for (int a = 0; a < nd; a++) JT_TRY(get_fft(dims[a], &f));
            return JT_OK;
        }
        for (int a = 0; a < nd; a++) {
            if (kind == JT_DCT || kind == JT_DST) JT_TRY(get_dct(dims[a], &d));
            else JT_TRY(get_dht(dims[a], &h));
        }
        return JT_OK;
    }

    // Moves axis `ax` of [outer][len][inner] (elements of E bytes) between
    // the array and a contiguous-line copy.
    template <typename E> void transpose(Ctx &ctx, const E *in, E *out, int64_t outer, int64_t R, int64_t Cc) const {
        if (ctx.dry || outer * R * Cc == 0) return;
        int64_t blocks = outer * cdiv(R, 32) * cdiv(Cc, 32);
        transpose_kernel<E><<<(unsigned)blocks, dim3(32, 8), 0, ctx.s>>>(in, out, R, Cc, outer);
        g_launches++;
    }

    void axis_shape(int ax, int64_t batch, int64_t &outer, int64_t &len, int64_t &inner) const {
        len = dims[ax];
        inner = 1;
        outer = batch;
        for (int d = ax + 1; d < nd; d++) inner *= dims[d];
        for (int d = 0; d < ax; d++) outer *= dims[d];
    }

    // Complex nD transform of `batch` contiguous arrays.
    int complex_nd(Ctx &ctx, C2 *a, int64_t batch, int sign, bool scale) {
        for (int ax = nd - 1; ax >= 0; ax--) {
            int64_t outer, len, inner;
            axis_shape(ax, batch, outer, len, inner);
            Fft1<T> *f = fft.at(len).get();
            double s = (sign > 0 && scale) ? 1.0 / (double)len : 1.0;
            if (inner == 1) {
                JT_TRY(f->exec(ctx, a, len, a, len, outer, sign, s));
            } else if (f->cols_ok()) {
                Layout l = {inner, len * inner, 1, inner};
                JT_TRY(f->exec_direct(ctx, a, a, outer * inner, l, l, sign, s));
            } else if (f->algo == ALG_TRIVIAL) {
                continue;
            } else {
                C2 *tmp = (C2 *)ctx.ws->get(sizeof(C2) * outer * len * inner, ctx.dry);
                transpose<C2>(ctx, a, tmp, outer, len, inner);
                JT_TRY(f->exec(ctx, tmp, len, tmp, len, outer * inner, sign, s));
                transpose<C2>(ctx, tmp, a, outer, inner, len);
            }
        }
        return JT_OK;
    }

    // Applies a real 1D line operation along every axis (DCT/DST/DHT):
    // line_op(ctx, len, array, nlines, layout).  Strided axes run in place
    // when the length has the one-kernel form (strided_ok(len)), else
    // through a transposed copy.
    template <typename F, typename G> int real_axes(Ctx &ctx, T *a, int64_t batch, F line_op, G strided_ok) {
        for (int ax = nd - 1; ax >= 0; ax--) {
            int64_t outer, len, inner;
            axis_shape(ax, batch, outer, len, inner);
            if (inner == 1) {
                JT_TRY(line_op(ctx, len, a, outer, Layout{1, len, 0, 1}));
            } else if (strided_ok(len)) {
                JT_TRY(line_op(ctx, len, a, outer * inner, Layout{inner, len * inner, 1, inner}));
            } else {
                T *tmp = (T *)ctx.ws->get(sizeof(T) * outer * len * inner, ctx.dry);
                transpose<T>(ctx, a, tmp, outer, len, inner);
                JT_TRY(line_op(ctx, len, tmp, outer * inner, Layout{1, len, 0, 1}));
                transpose<T>(ctx, tmp, a, outer, inner, len);
            }
        }
        return JT_OK;
    }

    int64_t extent(int op) const {
        if (kind == JT_FFT) {
            if (op == JT_REAL_FORWARD || op == JT_REAL_INVERSE) return N;
            return 2 * N;
        }
        return N;
    }

    // Runs `op` on `batch` arrays at a + b*dist (dist == extent for nD).
    int run(Ctx &ctx, int op, T *a, int64_t batch, int64_t dist, bool scale) {
        if (kind == JT_FFT) {
            if (nd == 1) {
                const int64_t n = dims[0];
                if (op == JT_COMPLEX_FORWARD || op == JT_COMPLEX_INVERSE) {
                    Fft1<T> *f = fft.at(n).get();
                    int sign = op == JT_COMPLEX_FORWARD ? -1 : 1;
                    double s = (op == JT_COMPLEX_INVERSE && scale) ? 1.0 / (double)n : 1.0;
                    return f->exec(ctx, (C2 *)a, dist / 2, (C2 *)a, dist / 2, batch, sign, s);
                }
                Real1<T> *r = real.at(n).get();
                switch (op) {
                    case JT_REAL_FORWARD: return r->fwd_packed(ctx, a, dist, batch);
                    case JT_REAL_FORWARD_FULL: return r->fwd_full(ctx, a, dist, batch, -1, 1.0);
                    case JT_REAL_INVERSE_FULL: return r->fwd_full(ctx, a, dist, batch, 1, scale ? 1.0 / (double)n : 1.0);
                    case JT_REAL_INVERSE: {
                        double factor = scale ? 1.0 : ((is_pow2(n) && n > 1) ? (double)n / 2.0 : (double)n);
                        return r->inv_packed(ctx, a, dist, batch, factor);
                    }
                }
                return JT_EINVAL;
            }
            if (dist != extent(op)) return JT_EINVAL;
            switch (op) {
                case JT_COMPLEX_FORWARD: return complex_nd(ctx, (C2 *)a, batch, -1, false);
                case JT_COMPLEX_INVERSE: return complex_nd(ctx, (C2 *)a, batch, 1, scale);
                case JT_REAL_FORWARD_FULL:
                case JT_REAL_INVERSE_FULL: {
                    T *tmp = (T *)ctx.ws->get(sizeof(T) * batch * N, ctx.dry);
                    LAUNCH1D(ctx, batch * N, copy_real_kernel<T>, a, dist, tmp, N, N, batch);
                    LAUNCH1D(ctx, batch * N, real_to_complex_kernel<T>, tmp, N, (C2 *)a, N, batch);
                    int sign = op == JT_REAL_FORWARD_FULL ? -1 : 1;
                    return complex_nd(ctx, (C2 *)a, batch, sign, op == JT_REAL_INVERSE_FULL && scale);
                }
                case JT_REAL_FORWARD:
                case JT_REAL_INVERSE: {
                    if (nd == 3) {
                        // fft/DoubleFFT_3D.java:1339-1356, :1629-1645: rows' real
                        // FFT, complex passes along rows then slices on the
                        // packed pairs, rdft3d_sub (inverse: the reverse order)
                        const int64_t S = dims[0], R = dims[1], Cc = dims[2], H = Cc / 2;
                        Real1<T> *r = real.at(Cc).get();
                        Fft1<T> *fr = fft.at(R).get();
                        Fft1<T> *fs = fft.at(S).get();
                        Layout lr = {H, R * H, 1, H};
                        Layout ls = {R * H, S * R * H, 1, R * H};
                        const int64_t pairs = batch * (S / 2) * (R / 2) * 2;
                        if (op == JT_REAL_FORWARD) {
                            JT_TRY(r->fwd_packed(ctx, a, Cc, batch * S * R));
                            JT_TRY(column_fft(ctx, fr, (C2 *)a, batch * S, R, H, lr, -1, 1.0));
                            JT_TRY(column_fft(ctx, fs, (C2 *)a, batch, S, R * H, ls, -1, 1.0));
                            LAUNCH1D(ctx, pairs, rdft3d_kernel<T>, a, dist, S, R, Cc, batch, 1);
                            return JT_OK;
                        }
                        LAUNCH1D(ctx, pairs, rdft3d_kernel<T>, a, dist, S, R, Cc, batch, -1);
                        JT_TRY(column_fft(ctx, fs, (C2 *)a, batch, S, R * H, ls, 1, scale ? 1.0 / (double)S : 1.0));
                        JT_TRY(column_fft(ctx, fr, (C2 *)a, batch * S, R, H, lr, 1, scale ? 1.0 / (double)R : 1.0));
                        double factor = scale ? 1.0 : (double)Cc / 2.0;
                        return r->inv_packed(ctx, a, Cc, batch * S * R, factor);
                    }
                    if (nd != 2) return JT_EINVAL;
                    const int64_t rows = dims[0], cols = dims[1];
                    Real1<T> *r = real.at(cols).get();
                    Fft1<T> *fr = fft.at(rows).get();
                    Layout l = {cols / 2, rows * cols / 2, 1, cols / 2};
                    if (op == JT_REAL_FORWARD) {
                        JT_TRY(r->fwd_packed(ctx, a, cols, batch * rows));
                        JT_TRY(column_fft(ctx, fr, (C2 *)a, batch, rows, cols / 2, l, -1, 1.0));
                        LAUNCH1D(ctx, batch * std::max<int64_t>(rows / 2 - 1, 0), rdft2d_kernel<T>, a, dist, rows, cols, batch, 1);
                        return JT_OK;
                    }
                    LAUNCH1D(ctx, batch * std::max<int64_t>(rows / 2 - 1, 0), rdft2d_kernel<T>, a, dist, rows, cols, batch, -1);
                    JT_TRY(column_fft(ctx, fr, (C2 *)a, batch, rows, cols / 2, l, 1, scale ? 1.0 / (double)rows : 1.0));
                    double factor = scale ? 1.0 : (double)cols / 2.0;
                    return r->inv_packed(ctx, a, cols, batch * rows, factor);
                }
            }
            return JT_EINVAL;
        }
        if (op != JT_FORWARD && op != JT_INVERSE) return JT_EINVAL;
        if (nd > 1 && dist != N) return JT_EINVAL;
        const bool fwd = op == JT_FORWARD;
        if (kind == JT_DCT || kind == JT_DST) {
            const bool dst = kind == JT_DST;
            if (nd == 1) {
                Dct1<T> *d = dct.at(dims[0]).get();
                return d->lines(ctx, fwd, a, batch, Layout{1, dist, 0, 1}, scale, dst);
            }
            return real_axes(
                ctx, a, batch,
                [&](Ctx &c, int64_t len, T *x, int64_t nb, const Layout &l) {
                    return dct.at(len)->lines(c, fwd, x, nb, l, scale, dst);
                },
                [&](int64_t len) { return dct.at(len)->strided_ok(ctx); });
        }
        // DHT
        if (nd == 1) {
            Dht1<T> *h = dht.at(dims[0]).get();
            double mult = (!fwd && scale) ? 1.0 / (double)dims[0] : 1.0;
            return h->lines(ctx, a, batch, Layout{1, dist, 0, 1}, mult);
        }
        JT_TRY(real_axes(
            ctx, a, batch,
            [&](Ctx &c, int64_t len, T *x, int64_t nb, const Layout &l) { return dht.at(len)->lines(c, x, nb, l, 1.0); },
            [&](int64_t len) { return dht.at(len)->strided_ok(ctx); }));
        for (int64_t b = 0; b < batch; b++) {
            T *p = a + b * dist;
            if (nd == 2) LAUNCH1D(ctx, (dims[0] / 2 + 1) * (dims[1] / 2 + 1), ytransform2_kernel<T>, p, dims[0], dims[1]);
            else LAUNCH1D(ctx, (dims[0] / 2 + 1) * (dims[1] / 2 + 1) * (dims[2] / 2 + 1), ytransform3_kernel<T>, p, dims[0], dims[1], dims[2]);
        }
        if (!fwd && scale) LAUNCH1D(ctx, batch * N, scale_kernel<T>, a, dist, N, batch, 1.0 / (double)N);
        return JT_OK;
    }

    // Column pass over `cols` complex columns of `rows` rows, batch arrays.
    int column_fft(Ctx &ctx, Fft1<T> *f, C2 *a, int64_t batch, int64_t rows, int64_t cols, const Layout &l, int sign, double s) {
        if (f->cols_ok()) return f->exec_direct(ctx, a, a, batch * cols, l, l, sign, s);
        if (f->algo == ALG_TRIVIAL) return JT_OK;
        C2 *tmp = (C2 *)ctx.ws->get(sizeof(C2) * batch * rows * cols, ctx.dry);
        transpose<C2>(ctx, a, tmp, batch, rows, cols);
        JT_TRY(f->exec(ctx, tmp, rows, tmp, rows, batch * cols, sign, s));
        transpose<C2>(ctx, tmp, a, batch, cols, rows);
        return JT_OK;
    }
};

}  // namespace jt

// ===========================================================================
// C ABI
// ===========================================================================
using namespace jt;

struct jt_plan {
    int kind, prec, nd;
    int64_t dims[3];
    int mode;
    int device;  // the device current at jt_plan_create: its tables live there
    void *impl;
};

namespace {

// host-array calls move pieces of the batch through a ring of device
// buffers: copy in (stream h2d), transform (stream), copy out (stream d2h)
#define JT_HOST_RING 3

struct ThreadState {
    cudaStream_t stream = nullptr;
    cudaStream_t h2d = nullptr, d2h = nullptr;
    cudaEvent_t in_done[JT_HOST_RING] = {}, run_done[JT_HOST_RING] = {}, out_done[JT_HOST_RING] = {};
    Arena arena;
    cudaEvent_t done = nullptr;
    cudaStream_t last = nullptr;
    ~ThreadState() {
        // device resources are reclaimed at process exit
    }
};
thread_local ThreadState t_state;

int ensure_stream() {
    if (!t_state.stream) {
        JT_CU(cudaStreamCreateWithFlags(&t_state.stream, cudaStreamNonBlocking));
        JT_CU(cudaEventCreateWithFlags(&t_state.done, cudaEventDisableTiming));
    }
    return JT_OK;
}

int ensure_copy_streams() {
    if (!t_state.h2d) {
        JT_CU(cudaStreamCreateWithFlags(&t_state.h2d, cudaStreamNonBlocking));
        JT_CU(cudaStreamCreateWithFlags(&t_state.d2h, cudaStreamNonBlocking));
        for (int r = 0; r < JT_HOST_RING; r++) {
            JT_CU(cudaEventCreateWithFlags(&t_state.in_done[r], cudaEventDisableTiming));
            JT_CU(cudaEventCreateWithFlags(&t_state.run_done[r], cudaEventDisableTiming));
            JT_CU(cudaEventCreateWithFlags(&t_state.out_done[r], cudaEventDisableTiming));
        }
    }
    return JT_OK;
}

int ensure_arena(size_t bytes) {
    Arena &a = t_state.arena;
    // a call needing more scratch than the limit fails, whatever the arena holds
    const int64_t lim = g_opt_arena_limit.load();
    if (lim > 0 && (int64_t)bytes > lim) {
        g_last_cuda = (int)cudaErrorMemoryAllocation;
        return JT_ENOMEM;
    }
    if (bytes <= a.cap) return JT_OK;
    if (a.base) {
        cudaStreamSynchronize(t_state.stream);
        if (t_state.last && t_state.last != t_state.stream) cudaStreamSynchronize(t_state.last);
        cudaFree(a.base);
        a.base = nullptr;
        a.cap = 0;
    }
    size_t cap = std::max(bytes, (size_t)(a.cap * 3 / 2));
    JT_CU(cudaMalloc(&a.base, cap));
    a.cap = cap;
    return JT_OK;
}

template <typename T> PlanImpl<T> *impl_of(jt_plan *p) { return (PlanImpl<T> *)p->impl; }

// After a synchronize: JT_ETIMEOUT if a kernel's bounded wait gave up.
int check_err_flag() {
    int h = 0;
    JT_CU(cudaMemcpy(&h, g_err_dev, sizeof(int), cudaMemcpyDeviceToHost));
    if (h) {
        JT_CU(cudaMemset(g_err_dev, 0, sizeof(int)));
        return JT_ETIMEOUT;
    }
    return JT_OK;
}

// Runs op on device memory: dry run to size the scratch, then the launches.
template <typename T>
int run_device(jt_plan *p, int op, T *a, int64_t batch, int64_t dist, bool scale, cudaStream_t s) {
    PlanImpl<T> *im = impl_of<T>(p);
    JT_TRY(im->prepare(op));
    Ctx c;
    c.s = s;
    c.tc = p->mode == JT_MODE_TC_SPLIT;
    c.ws = &t_state.arena;
    c.dry = true;
    t_state.arena.used = 0;
    t_state.arena.peak = 0;
    std::lock_guard<std::mutex> g(im->mu);
    JT_TRY(im->run(c, op, a, batch, dist, scale));
    size_t need = t_state.arena.peak;
    JT_TRY(ensure_arena(need));
    // the arena is shared by this thread's calls: order this call after the
    // previous one when it ran on another stream
    if (t_state.last && t_state.last != s) {
        JT_CU(cudaEventRecord(t_state.done, t_state.last));
        JT_CU(cudaStreamWaitEvent(s, t_state.done, 0));
    }
    t_state.arena.used = 0;
    c.dry = false;
    JT_TRY(im->run(c, op, a, batch, dist, scale));
    t_state.last = s;
    JT_CU(cudaGetLastError());
    return JT_OK;
}

bool valid_op(const jt_plan *p, int op) {
    if (p->kind == JT_FFT) return op >= JT_COMPLEX_FORWARD && op <= JT_REAL_INVERSE_FULL;
    return op == JT_FORWARD || op == JT_INVERSE;
}

int check_op(const jt_plan *p, int op) {
    if (!valid_op(p, op)) return JT_EINVAL;
    if (p->kind == JT_FFT && p->nd > 1 && (op == JT_REAL_FORWARD || op == JT_REAL_INVERSE)) {
        for (int d = 0; d < p->nd; d++)
            if (!is_pow2(p->dims[d])) return JT_ENOTPOW2;
    }
    return JT_OK;
}

// ---------------------------------------------------------------------------
// Host-staged four-step: one complex 1D transform whose device working set
// does not fit the device budget (the free device memory, or
// JT_OPT_ARENA_LIMIT_MB) runs as n = n1 x m over host pieces, the way the
// reference's LargeArray path works through its array in parts
// (fft/DoubleFFT_1D.java:280-304):
//   pass A  blocks of w columns of the n1 x m view: copied in as n1 x w
//           (one 2D copy), n1-point column FFTs, the four-step twiddle
//           w_n^{k1 (b0 + c)}, copied back in place;
//   pass B  blocks of h rows: copied in, m-point row FFTs (scaled for the
//           inverse), transposed on the device and written to
//           X[k1 + n1 k2] of a host copy, which replaces the array at the end.
// Device memory: two block buffers and the row plan's scratch.
// ---------------------------------------------------------------------------
template <int SIGN, typename T>
__global__ void block_twiddle_kernel(typename V2<T>::t *y, int64_t n1, int64_t w, int64_t b0, int64_t n,
                                     const typename V2<T>::t *__restrict__ Whi, const typename V2<T>::t *__restrict__ Wlo,
                                     int lo_bits) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n1 * w) return;
    const int64_t k1 = i / w, c = i - k1 * w;
    const uint64_t e = ((uint64_t)k1 * (uint64_t)(b0 + c)) % (uint64_t)n;
    const typename V2<T>::t t = cmul<T>(Whi[e >> lo_bits], Wlo[e & ((1ull << lo_bits) - 1)]);
    y[i] = SIGN < 0 ? cmul<T>(y[i], t) : cmulc<T>(y[i], t);
}

static int64_t device_budget() {
    const int64_t lim = g_opt_arena_limit.load();
    if (lim > 0) return lim;
    size_t fr = 0, tot = 0;
    if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) return INT64_MAX;
    // the arena itself can be given back and regrown
    return (int64_t)fr + (int64_t)t_state.arena.cap - ((int64_t)256 << 20);
}

template <typename T>
int stream_fourstep(PlanImpl<T> *im, Fft1<T> *f, void *host, int sign, double scale, int64_t budget) {
    typedef typename V2<T>::t C2;
    const int64_t n = f->n, n1 = f->n1, m = n / n1;
    const int64_t esz = (int64_t)sizeof(C2);
    if (!f->Whi || !f->pa) return JT_ENOMEM;
    // the caller's array holds pairs of T at any T-aligned address: host
    // addresses are formed in bytes
    char *h = (char *)host;
    // the m-point row plan: pass B of a two-pass plan, or (three passes) a
    // plan of its own
    std::shared_ptr<Fft1<T>> fm_own;
    Fft1<T> *fm = f->algo == ALG_TWOPASS ? f->pb.get() : nullptr;
    if (!fm) {
        const uint64_t seq0 = g_setup_seq.load();
        JT_TRY(cached<Fft1<T>>(m, fm_own));
        if (g_setup_seq.load() != seq0) JT_CU(cudaStreamSynchronize(g_setup));
        fm = fm_own.get();
    }
    cudaStream_t s = t_state.stream;
    Ctx c;
    c.s = s;
    c.ws = &t_state.arena;
    // block size: the largest (down to one row of m) whose working set fits
    int64_t blk = std::min<int64_t>(budget / 3, (int64_t)256 << 20), w = 0, hr = 0;
    for (;; blk /= 2) {
        if (blk < m * esz) return JT_ENOMEM;  // not even one row fits
        w = std::max<int64_t>(1, std::min<int64_t>(m, blk / (n1 * esz)));
        hr = std::max<int64_t>(1, std::min<int64_t>(n1, blk / (m * esz)));
        c.dry = true;
        t_state.arena.used = t_state.arena.peak = 0;
        t_state.arena.get(blk, true);
        t_state.arena.get(blk, true);
        Layout la = {w, n1 * w, 1, w};
        JT_TRY(f->pa->exec_direct(c, nullptr, nullptr, w, la, la, sign, 1.0));
        JT_TRY(fm->exec(c, nullptr, m, nullptr, m, hr, sign, scale));
        if ((int64_t)t_state.arena.peak <= budget) break;
    }
    JT_TRY(ensure_arena(t_state.arena.peak));
    std::unique_ptr<C2[]> out(new (std::nothrow) C2[n]);
    if (!out) return JT_ENOMEM;
    c.dry = false;
    t_state.arena.used = 0;
    C2 *d0 = (C2 *)t_state.arena.get(blk, false), *d1 = (C2 *)t_state.arena.get(blk, false);
    const size_t mark = t_state.arena.used;
    // pass A: column blocks, in place in the host array
    for (int64_t b0 = 0; b0 < m; b0 += w) {
        const int64_t wb = std::min(w, m - b0);
        JT_CU(cudaMemcpy2DAsync(d0, wb * esz, h + b0 * esz, m * esz, wb * esz, n1, cudaMemcpyHostToDevice, s));
        Layout la = {wb, n1 * wb, 1, wb};
        t_state.arena.used = mark;
        JT_TRY(f->pa->exec_direct(c, d0, d0, wb, la, la, sign, 1.0));
        const int64_t tot = n1 * wb;
        if (sign < 0)
            block_twiddle_kernel<-1, T><<<(unsigned)cdiv(tot, 256), 256, 0, s>>>(d0, n1, wb, b0, n, f->Whi, f->Wlo, f->lo_bits);
        else
            block_twiddle_kernel<1, T><<<(unsigned)cdiv(tot, 256), 256, 0, s>>>(d0, n1, wb, b0, n, f->Whi, f->Wlo, f->lo_bits);
        g_launches++;
        JT_CU(cudaMemcpy2DAsync(h + b0 * esz, m * esz, d0, wb * esz, wb * esz, n1, cudaMemcpyDeviceToHost, s));
    }
    // pass B: row blocks, transposed into the host copy
    for (int64_t r0 = 0; r0 < n1; r0 += hr) {
        const int64_t hb = std::min(hr, n1 - r0);
        JT_CU(cudaMemcpyAsync(d0, h + r0 * m * esz, hb * m * esz, cudaMemcpyHostToDevice, s));
        t_state.arena.used = mark;
        JT_TRY(fm->exec(c, d0, m, d0, m, hb, sign, scale));
        im->template transpose<C2>(c, d0, d1, 1, hb, m);
        JT_CU(cudaMemcpy2DAsync(out.get() + r0, n1 * esz, d1, hb * esz, hb * esz, m, cudaMemcpyDeviceToHost, s));
    }
    JT_CU(cudaStreamSynchronize(s));
    JT_CU(cudaGetLastError());
    JT_TRY(check_err_flag());
    // the result replaces the array (a few threads: the copy is host-bound)
    const int nt = (int)std::max<int64_t>(1, std::min<int64_t>(8, n / ((int64_t)1 << 22)));
    std::vector<std::thread> th;
    for (int t = 0; t < nt; t++)
        th.emplace_back([&, t] {
            const int64_t a = n * t / nt, b = n * (t + 1) / nt;
            std::memcpy(h + a * esz, out.get() + a, (size_t)(b - a) * esz);
        });
    for (auto &x : th) x.join();
    return JT_OK;
}

template <typename T>
int exec_host(jt_plan *p, int op, void *host, int64_t len, int64_t off, int64_t batch, int64_t dist, int scale) {
    int64_t ext = 0;
    JT_TRY(jt_plan_extent(p, op, &ext));
    if (!host || batch < 0 || off < 0) return JT_EINVAL;
    if (batch == 0) return JT_OK;
    if (batch > 1 && dist < ext) return JT_EINVAL;
    if (off + (batch - 1) * dist + ext > len) return JT_ESHORTBUF;
    JT_TRY(device_init());
    JT_TRY(ensure_stream());
    JT_TRY(ensure_copy_streams());
    cudaStream_t s = t_state.stream;
    // device copy laid out densely at distance ext (even, for complex views)
    int64_t dd = (ext + 1) & ~(int64_t)1;
    if (p->nd > 1) dd = ext;
    PlanImpl<T> *im = impl_of<T>(p);
    JT_TRY(im->prepare(op));
    // pieces of about JT_OPT_HOST_PIECE_MB, up to JT_HOST_RING of them in
    // flight: the copy in of piece i+1 and the copy out of piece i-1 overlap
    // the transform of piece i
    const int64_t per = (int64_t)sizeof(T) * dd;
    const int64_t piece_bytes = (int64_t)g_opt_host_piece_mb.load() << 20;
    const int64_t piece = std::max<int64_t>(1, std::min<int64_t>(batch, piece_bytes / per));
    const int64_t npieces = (batch + piece - 1) / piece;
    const int ring = (int)std::min<int64_t>(JT_HOST_RING, npieces);
    // size: ring buffers + one piece's scratch (dry run)
    Ctx c;
    c.s = s;
    c.tc = p->mode == JT_MODE_TC_SPLIT;
    c.ws = &t_state.arena;
    c.dry = true;
    t_state.arena.used = 0;
    t_state.arena.peak = 0;
    for (int r = 0; r < ring; r++) t_state.arena.get(per * piece, true);
    std::lock_guard<std::mutex> g(im->mu);
    JT_TRY(im->run(c, op, (T *)nullptr, piece, dd, scale != 0));
    const int64_t budget = device_budget();
    if ((int64_t)t_state.arena.peak > budget) {
        // one transform's working set exceeds the device: complex 1D
        // multi-pass lengths stream through host pieces, the rest fail
        Fft1<T> *f = nullptr;
        if (p->kind == JT_FFT && p->nd == 1 && (op == JT_COMPLEX_FORWARD || op == JT_COMPLEX_INVERSE)) {
            auto it = im->fft.find(p->dims[0]);
            if (it != im->fft.end() && (it->second->algo == ALG_TWOPASS || it->second->algo == ALG_THREEPASS))
                f = it->second.get();
        }
        if (!f) {
            g_last_cuda = (int)cudaErrorMemoryAllocation;
            return JT_ENOMEM;
        }
        if (t_state.last && t_state.last != s) {
            JT_CU(cudaEventRecord(t_state.done, t_state.last));
            JT_CU(cudaStreamWaitEvent(s, t_state.done, 0));
        }
        const int sign = op == JT_COMPLEX_FORWARD ? -1 : 1;
        const double sc = (op == JT_COMPLEX_INVERSE && scale) ? 1.0 / (double)p->dims[0] : 1.0;
        for (int64_t b = 0; b < batch; b++)
            JT_TRY(stream_fourstep<T>(im, f, (T *)host + off + b * dist, sign, sc, budget));
        t_state.last = s;
        return JT_OK;
    }
    JT_TRY(ensure_arena(t_state.arena.peak));
    if (t_state.last && t_state.last != s) {
        JT_CU(cudaEventRecord(t_state.done, t_state.last));
        JT_CU(cudaStreamWaitEvent(s, t_state.done, 0));
    }
    // the copy streams start after earlier work on this thread's arena
    JT_CU(cudaEventRecord(t_state.done, s));
    JT_CU(cudaStreamWaitEvent(t_state.h2d, t_state.done, 0));
    JT_CU(cudaStreamWaitEvent(t_state.d2h, t_state.done, 0));
    t_state.arena.used = 0;
    c.dry = false;
    T *buf[JT_HOST_RING];
    for (int r = 0; r < ring; r++) buf[r] = (T *)t_state.arena.get(per * piece, false);
    const size_t mark = t_state.arena.used;
    T *h = (T *)host + off;
    auto copy = [&](T *dst, const T *src, int64_t nb, cudaMemcpyKind kind, cudaStream_t st) -> int {
        const bool to_dev = kind == cudaMemcpyHostToDevice;
        if (dist == dd || nb == 1) {
            JT_CU(cudaMemcpyAsync(dst, src, sizeof(T) * ((nb - 1) * dd + ext), kind, st));
        } else {
            JT_CU(cudaMemcpy2DAsync(dst, sizeof(T) * (to_dev ? dd : dist), src, sizeof(T) * (to_dev ? dist : dd),
                                    sizeof(T) * ext, nb, kind, st));
        }
        return JT_OK;
    };
    for (int64_t i = 0; i < npieces; i++) {
        const int r = (int)(i % ring);
        const int64_t b0 = i * piece, nb = std::min(piece, batch - b0);
        // buffer r is free once the copy out of piece i - ring finished
        if (i >= ring) JT_CU(cudaStreamWaitEvent(t_state.h2d, t_state.out_done[r], 0));
        JT_TRY(copy(buf[r], h + b0 * dist, nb, cudaMemcpyHostToDevice, t_state.h2d));
        JT_CU(cudaEventRecord(t_state.in_done[r], t_state.h2d));
        JT_CU(cudaStreamWaitEvent(s, t_state.in_done[r], 0));
        t_state.arena.used = mark;  // the pieces run in order on one stream: one scratch region
        JT_TRY(im->run(c, op, buf[r], nb, dd, scale != 0));
        JT_CU(cudaEventRecord(t_state.run_done[r], s));
        JT_CU(cudaStreamWaitEvent(t_state.d2h, t_state.run_done[r], 0));
        JT_TRY(copy(h + b0 * dist, buf[r], nb, cudaMemcpyDeviceToHost, t_state.d2h));
        JT_CU(cudaEventRecord(t_state.out_done[r], t_state.d2h));
    }
    // later work on this thread's arena (on any stream) follows the copies out
    JT_CU(cudaEventRecord(t_state.done, t_state.d2h));
    JT_CU(cudaStreamWaitEvent(s, t_state.done, 0));
    t_state.last = s;
    JT_CU(cudaStreamSynchronize(t_state.d2h));
    JT_CU(cudaStreamSynchronize(s));
    JT_CU(cudaGetLastError());
    return check_err_flag();
}

}  // namespace

extern "C" {

int jt_plan_create(int kind, int prec, int ndim, const int64_t *dims, jt_plan **out) {
    if (!out || !dims) return JT_EINVAL;
    *out = nullptr;
    if (kind < JT_FFT || kind > JT_DHT || (prec != JT_FLOAT32 && prec != JT_FLOAT64) || ndim < 1 || ndim > 3) return JT_EINVAL;
    for (int d = 0; d < ndim; d++) {
        if (ndim == 1 && dims[d] < 1) return JT_EBADSIZE;
        if (ndim > 1 && dims[d] <= 1) return JT_EBADSIZE;
    }
    JT_TRY(device_init());
    jt_plan *p = new (std::nothrow) jt_plan();
    if (!p) return JT_ENOMEM;
    p->kind = kind;
    p->prec = prec;
    p->nd = ndim;
    p->mode = JT_MODE_FP32;
    p->device = 0;
    cudaGetDevice(&p->device);
    int64_t N = 1;
    for (int d = 0; d < 3; d++) p->dims[d] = d < ndim ? dims[d] : 1;
    for (int d = 0; d < ndim; d++) N *= dims[d];
    auto fill = [&](auto *im) {
        im->kind = kind;
        im->nd = ndim;
        for (int d = 0; d < 3; d++) im->dims[d] = p->dims[d];
        im->N = N;
    };
    if (prec == JT_FLOAT32) {
        auto *im = new (std::nothrow) PlanImpl<float>();
        if (!im) { delete p; return JT_ENOMEM; }
        fill(im);
        p->impl = im;
    } else {
        auto *im = new (std::nothrow) PlanImpl<double>();
        if (!im) { delete p; return JT_ENOMEM; }
        fill(im);
        p->impl = im;
    }
    // Build the tables the transform's main ops use now, as the reference
    // constructors do, so execution does no setup work.
    int st = JT_OK;
    int main_op = kind == JT_FFT ? JT_COMPLEX_FORWARD : JT_FORWARD;
    if (prec == JT_FLOAT32) st = impl_of<float>(p)->prepare(main_op);
    else st = impl_of<double>(p)->prepare(main_op);
    if (st != JT_OK) {
        jt_plan_destroy(p);
        return st;
    }
    *out = p;
    return JT_OK;
}

int jt_plan_destroy(jt_plan *p) {
    if (!p) return JT_EINVAL;
    // the plan's tables stay in the table cache: nothing is freed here, so
    // kernels still running with them are unaffected and nothing waits
    if (p->prec == JT_FLOAT32) delete (PlanImpl<float> *)p->impl;
    else delete (PlanImpl<double> *)p->impl;
    delete p;
    return JT_OK;
}

int jt_plan_extent(const jt_plan *p, int op, int64_t *out_len) {
    if (!p || !out_len) return JT_EINVAL;
    JT_TRY(check_op(p, op));
    *out_len = p->prec == JT_FLOAT32 ? ((PlanImpl<float> *)p->impl)->extent(op) : ((PlanImpl<double> *)p->impl)->extent(op);
    return JT_OK;
}

int jt_plan_set_mode(jt_plan *p, int mode) {
    if (!p) return JT_EINVAL;
    if (mode == JT_MODE_FP32 || (mode == JT_MODE_TC_SPLIT && p->prec == JT_FLOAT32)) {
        p->mode = mode;
        return JT_OK;
    }
    return JT_EINVAL;
}

int jt_plan_algorithm(const jt_plan *p, int axis) {
    if (!p || axis < 0 || axis >= p->nd) return JT_EINVAL;
    const int64_t n = p->dims[axis];
    if (p->prec == JT_FLOAT32) {
        PlanImpl<float> *im = (PlanImpl<float> *)p->impl;
        std::lock_guard<std::mutex> g(im->mu);
        auto it = im->fft.find(n);
        if (it != im->fft.end()) return it->second->algo;
    } else {
        PlanImpl<double> *im = (PlanImpl<double> *)p->impl;
        std::lock_guard<std::mutex> g(im->mu);
        auto it = im->fft.find(n);
        if (it != im->fft.end()) return it->second->algo;
    }
    return JT_EINVAL;
}

int jt_execute(jt_plan *p, int op, void *host, int64_t len, int64_t off, int scale) {
    return jt_execute_batch(p, op, host, len, off, 1, 0, scale);
}

int jt_execute_batch(jt_plan *p, int op, void *host, int64_t len, int64_t off, int64_t batch, int64_t dist, int scale) {
    if (!p) return JT_EINVAL;
    JT_TRY(check_op(p, op));
    if (p->prec == JT_FLOAT32) return exec_host<float>(p, op, host, len, off, batch, dist, scale);
    return exec_host<double>(p, op, host, len, off, batch, dist, scale);
}

int jt_execute_device(jt_plan *p, int op, void *dev, int64_t batch, int64_t dist, int scale, void *stream) {
    if (!p || !dev || batch < 0) return JT_EINVAL;
    JT_TRY(check_op(p, op));
    if (batch == 0) return JT_OK;
    int64_t ext = 0;
    JT_TRY(jt_plan_extent(p, op, &ext));
    if (batch > 1 && dist < ext) return JT_EINVAL;
    if (batch == 1 && dist < ext) dist = (ext + 1) & ~(int64_t)1;
    size_t esz = p->prec == JT_FLOAT32 ? 4 : 8;
    // FFT ops view the array as complex pairs: every array must start on a
    // pair boundary
    if (p->kind == JT_FFT && (((uintptr_t)dev % (2 * esz)) != 0 || (batch > 1 && (dist % 2) != 0))) return JT_EINVAL;
    JT_TRY(device_init());
    JT_TRY(ensure_stream());
    cudaStream_t s = (cudaStream_t)stream;
    if (p->prec == JT_FLOAT32) return run_device<float>(p, op, (float *)dev, batch, dist, scale != 0, s);
    return run_device<double>(p, op, (double *)dev, batch, dist, scale != 0, s);
}

int jt_synchronize(void) {
    JT_TRY(ensure_stream());
    JT_CU(cudaStreamSynchronize(t_state.stream));
    if (t_state.last && t_state.last != t_state.stream) JT_CU(cudaStreamSynchronize(t_state.last));
    JT_CU(cudaDeviceSynchronize());
    JT_CU(cudaGetLastError());
    return check_err_flag();
}

int jt_check_error(void) {
    JT_TRY(device_init());
    return check_err_flag();
}

const char *jt_strerror(int s) {
    switch (s) {
        case JT_OK: return "ok";
        case JT_EBADSIZE: return "size must be >= 1 (1D) or > 1 (2D/3D)";
        case JT_ESHORTBUF: return "array too short for offset and transform extent";
        case JT_ENOTPOW2: return "rows and columns must be power of two numbers";
        case JT_ECUDA: return "CUDA error";
        case JT_ETIMEOUT: return "device wait timed out";
        case JT_EINVAL: return "invalid argument";
        case JT_ENOMEM: return "device out of memory";
        case JT_ENODEV: return "no CUDA device";
        case JT_ETOOBIG: return "size beyond this build's single-GPU limit";
        case JT_ESCRATCH: return "transform needs more scratch than the fixed 32 MiB no-allocation buffer (or is a Bluestein length)";
    }
    return "unknown status";
}

int jt_last_cuda_error(void) { return g_last_cuda; }

int jt_set_split(int prec, int log2n, int a, int b, int c) {
    if ((prec != JT_FLOAT32 && prec != JT_FLOAT64) || log2n < 4 || log2n > JT_SPLIT_MAX_LOG2) return JT_EINVAL;
    signed char *e = g_split_override[prec == JT_FLOAT32 ? 0 : 1][log2n];
    if (a < 0) {
        if (e[0] >= 0) g_plan_gen++;
        e[0] = e[1] = e[2] = -1;
        return JT_OK;
    }
    const bool one = a == 0 && b == 0 && c == 0;
    const bool two = a >= 1 && b >= 1 && c == 0 && a <= 12 && b <= 12 && a + b == log2n;
    const bool three = a >= 1 && b >= 1 && c >= 1 && a <= 12 && b <= 12 && c <= 12 && a + b + c == log2n;
    if (!one && !two && !three) return JT_EINVAL;
    e[0] = (signed char)a;
    e[1] = (signed char)b;
    e[2] = (signed char)c;
    g_plan_gen++;
    return JT_OK;
}

int jt_set_option(int option, int value) {
    if (option == JT_OPT_TMA_PIPELINE) return g_opt_tma.exchange(value ? 1 : 0);
    if (option == JT_OPT_DIRECT_MAX_F32 || option == JT_OPT_DIRECT_MAX_F64) {
        const int prev = (option == JT_OPT_DIRECT_MAX_F32 ? g_opt_direct_max_f32 : g_opt_direct_max_f64).exchange(value);
        if (prev != value) g_plan_gen++;  // plans created from now on choose again
        return prev;
    }
    if (option == JT_OPT_COLUMN_KERNEL) return value == 0 ? 0 : JT_EINVAL;
    if (option == JT_OPT_ARENA_LIMIT_MB) {
        if (value < 0) return JT_EINVAL;
        return (int)(g_opt_arena_limit.exchange((int64_t)value << 20) >> 20);
    }
    if (option == JT_OPT_BATCH_WAIT_POLLS) {
        if (value < 1) return JT_EINVAL;
        return g_opt_batch_wait.exchange(value);
    }
    if (option == JT_OPT_BATCH_STALL_TEST) return g_opt_batch_inject.exchange(value ? 1 : 0);
    if (option == JT_OPT_TILE_ELEMS) {
        if (value < 0 || value > (1 << 16)) return JT_EINVAL;
        return g_opt_tile_elems.exchange(value);
    }
    if (option == JT_OPT_REAL_FUSED_F32) return g_opt_real_fused_f32.exchange(value ? 1 : 0);
    if (option == JT_OPT_RADIX_ORDER) {
        if (value < -1 || value > 3) return JT_EINVAL;
        const int prev = g_opt_radix_order.exchange(value);
        if (prev != value) g_plan_gen++;  // plans fix their radices at creation
        return prev;
    }
    if (option == JT_OPT_THREEPASS_MIN_LOG2) {
        if (value < 0 || value > 30) return JT_EINVAL;
        const int64_t nv = value ? (int64_t)1 << value : 0;
        const int64_t prev = g_opt_threepass_min.exchange(nv);
        if (prev != nv) g_plan_gen++;
        int lg = 0;
        while (prev && ((int64_t)1 << lg) < prev) lg++;
        return prev ? lg : 0;
    }
    if (option == JT_OPT_HOST_PIECE_MB) {
        if (value < 1 || value > 16384) return JT_EINVAL;
        return g_opt_host_piece_mb.exchange(value);
    }
    if (option == JT_OPT_TWOPASS_CHUNK_MB) {
        if (value < 1 || value > 16384) return JT_EINVAL;
        return g_opt_chunk_mb.exchange(value);
    }
    return JT_EINVAL;
}

int64_t jt_launch_count(int reset) {
    int64_t v = g_launches;
    if (reset) g_launches = 0;
    return v;
}

}  // extern "C"

// ===========================================================================
// Mixed-size batch: many 1D transforms of different plans in one launch
// (jt_batch.cuh describes the recording and the interpreter kernel)
// ===========================================================================
struct jt_batch {
    std::vector<jt_plan *> plans;
    std::vector<int> ops, scales;
    std::vector<void *> ptrs;
    // recorded steps, on the device
    int nops = 0, ntasks = 0, smem = 0, grid = 0;
    BOp *d_ops = nullptr;
    BTask *d_tasks = nullptr;
    int *d_done = nullptr;  // completed tasks per step
    int *d_head = nullptr;  // queue head
    char *scratch = nullptr;    // float transforms' scratch
    char *scratch_d = nullptr;  // double transforms' scratch
    cudaGraphExec_t graph = nullptr;
    cudaStream_t graph_stream = nullptr;
    int wait_polls = 1 << 24;  // polls of a dependency wait before it gives up
    ~jt_batch() {
        if (graph) cudaGraphExecDestroy(graph);
        for (void *p : {(void *)d_ops, (void *)d_tasks, (void *)d_done, (void *)d_head, (void *)scratch, (void *)scratch_d})
            if (p) cudaFree(p);
    }
};

namespace {

template <typename T>
int batch_record(jt_batch *bt, std::vector<BOp> &ops, std::vector<std::vector<int>> &chains) {
    // size each transform's scratch with a dry run, then record its steps
    const size_t n = bt->plans.size();
    std::vector<size_t> need(n, 0), off(n, 0);
    size_t total = 0;
    for (size_t i = 0; i < n; i++) {
        jt_plan *p = bt->plans[i];
        if (p->prec != (sizeof(T) == 4 ? JT_FLOAT32 : JT_FLOAT64)) continue;
        PlanImpl<T> *im = (PlanImpl<T> *)p->impl;
        JT_TRY(im->prepare(bt->ops[i]));
        int64_t ext = im->extent(bt->ops[i]);
        Arena ar;
        Ctx c;
        c.dry = true;
        c.rec_sizing = true;
        c.ws = &ar;
        std::lock_guard<std::mutex> g(im->mu);
        JT_TRY(im->run(c, bt->ops[i], (T *)bt->ptrs[i], 1, (ext + 1) & ~(int64_t)1, bt->scales[i] != 0));
        need[i] = (ar.peak + 255) & ~(size_t)255;
        off[i] = total;
        total += need[i];
    }
    if (total) {
        char *arena = nullptr;
        JT_CU(cudaMalloc(&arena, total));
        (sizeof(T) == 4 ? bt->scratch : bt->scratch_d) = arena;
        for (size_t i = 0; i < n; i++) off[i] += (size_t)arena;
    }
    for (size_t i = 0; i < n; i++) {
        jt_plan *p = bt->plans[i];
        if (p->prec != (sizeof(T) == 4 ? JT_FLOAT32 : JT_FLOAT64)) continue;
        PlanImpl<T> *im = (PlanImpl<T> *)p->impl;
        int64_t ext = im->extent(bt->ops[i]);
        Arena ar;
        ar.base = (char *)off[i];
        ar.cap = need[i];
        Ctx c;
        c.dry = false;
        c.ws = &ar;
        c.rec = &ops;
        c.rec_prev = -1;
        size_t first = ops.size();
        std::lock_guard<std::mutex> g(im->mu);
        int st = im->run(c, bt->ops[i], (T *)bt->ptrs[i], 1, (ext + 1) & ~(int64_t)1, bt->scales[i] != 0);
        if (st != JT_OK) return st;
        for (size_t k = first; k < ops.size(); k++) chains[i].push_back((int)k);
    }
    return JT_OK;
}

}  // namespace

extern "C" {

int jt_batch_create(int count, jt_plan *const *plans, const int *ops, void *const *dev_ptrs, const int *scales, jt_batch **out) {
    if (!out || count < 0 || (count > 0 && (!plans || !ops || !dev_ptrs || !scales))) return JT_EINVAL;
    *out = nullptr;
    JT_TRY(device_init());
    std::unique_ptr<jt_batch> b(new (std::nothrow) jt_batch());
    if (!b) return JT_ENOMEM;
    for (int i = 0; i < count; i++) {
        if (!plans[i] || plans[i]->nd != 1 || !dev_ptrs[i]) return JT_EINVAL;
        JT_TRY(check_op(plans[i], ops[i]));
        const size_t esz = plans[i]->prec == JT_FLOAT32 ? 4 : 8;
        if (plans[i]->kind == JT_FFT && ((uintptr_t)dev_ptrs[i] % (2 * esz))) return JT_EINVAL;
        b->plans.push_back(plans[i]);
        b->ops.push_back(ops[i]);
        b->ptrs.push_back(dev_ptrs[i]);
        b->scales.push_back(scales[i]);
    }
    std::vector<BOp> rec;
    std::vector<std::vector<int>> chains(count);
    JT_TRY(batch_record<float>(b.get(), rec, chains));
    JT_TRY(batch_record<double>(b.get(), rec, chains));
    b->wait_polls = g_opt_batch_wait.load();
    if (g_opt_batch_inject.load() && !rec.empty()) {
        // failure-path test: a step no task ever runs, made the dependency
        // of every transform's first step, so their waits run out
        BOp never = elem_op<float>(EK_SCALE, 0, 0);
        never.ntasks = 1;
        never.dep = -1;
        rec.push_back(never);
        const int phantom = (int)rec.size() - 1;
        for (auto &c : chains)
            if (!c.empty()) rec[c[0]].dep = phantom;
    }
    // tasks, stage by stage: every transform's first step, then the second...
    std::vector<BTask> tasks;
    size_t maxlen = 0;
    for (auto &c : chains) maxlen = std::max(maxlen, c.size());
    int smem = 0;
    for (size_t s = 0; s < maxlen; s++)
        for (auto &c : chains)
            if (s < c.size()) {
                const BOp &o = rec[c[s]];
                smem = std::max(smem, o.smem);
                for (int k = 0; k < o.ntasks; k++) tasks.push_back(BTask{c[s], k});
            }
    b->nops = (int)rec.size();
    b->ntasks = (int)tasks.size();
    b->smem = smem;
    if (b->nops) {
        JT_CU(cudaMalloc(&b->d_ops, sizeof(BOp) * rec.size()));
        JT_CU(cudaMemcpy(b->d_ops, rec.data(), sizeof(BOp) * rec.size(), cudaMemcpyHostToDevice));
        JT_CU(cudaMalloc(&b->d_done, sizeof(int) * rec.size()));
    }
    if (b->ntasks) {
        JT_CU(cudaMalloc(&b->d_tasks, sizeof(BTask) * tasks.size()));
        JT_CU(cudaMemcpy(b->d_tasks, tasks.data(), sizeof(BTask) * tasks.size(), cudaMemcpyHostToDevice));
    }
    JT_CU(cudaMalloc(&b->d_head, sizeof(int)));
    JT_CU(cudaFuncSetAttribute(batch_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, std::max(smem, 1)));
    JT_CU(cudaFuncSetAttribute(batch_kernel, cudaFuncAttributePreferredSharedMemoryCarveout, 100));
    int per_sm = 0;
    JT_CU(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, batch_kernel, JT_BATCH_THREADS, std::max(smem, 1)));
    b->grid = std::max(1, per_sm) * g_sms;
    *out = b.release();
    return JT_OK;
}

int jt_batch_run(jt_batch *b, void *stream) {
    if (!b) return JT_EINVAL;
    if (!b->ntasks) return JT_OK;
    cudaStream_t s = (cudaStream_t)stream;
    JT_CU(cudaMemsetAsync(b->d_done, 0, sizeof(int) * b->nops, s));
    JT_CU(cudaMemsetAsync(b->d_head, 0, sizeof(int), s));
    batch_kernel<<<b->grid, JT_BATCH_THREADS, std::max(b->smem, 1), s>>>(b->d_ops, b->d_tasks, b->ntasks, b->d_head, b->d_done,
                                                                          g_err_dev, b->wait_polls);
    g_launches++;
    JT_CU(cudaGetLastError());
    return JT_OK;
}

int jt_batch_run_per_transform(jt_batch *b, void *stream) {
    if (!b) return JT_EINVAL;
    for (size_t i = 0; i < b->plans.size(); i++) {
        int64_t ext = 0;
        JT_TRY(jt_plan_extent(b->plans[i], b->ops[i], &ext));
        JT_TRY(jt_execute_device(b->plans[i], b->ops[i], b->ptrs[i], 1, (ext + 1) & ~(int64_t)1, b->scales[i], stream));
    }
    return JT_OK;
}

int jt_batch_run_graph(jt_batch *b, void *stream) {
    if (!b) return JT_EINVAL;
    cudaStream_t s = (cudaStream_t)stream;
    if (!b->graph || b->graph_stream != s) {
        if (b->graph) cudaGraphExecDestroy(b->graph);
        b->graph = nullptr;
        cudaStream_t cap = s;
        bool own = false;
        if (!cap) {  // the legacy default stream cannot be captured
            JT_CU(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
            own = true;
        }
        cudaGraph_t g = nullptr;
        JT_CU(cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal));
        int st = jt_batch_run(b, cap);
        cudaError_t e = cudaStreamEndCapture(cap, &g);
        if (own) cudaStreamDestroy(cap);
        if (st != JT_OK) {
            if (g) cudaGraphDestroy(g);
            return st;
        }
        if (e != cudaSuccess) {
            g_last_cuda = (int)e;
            return JT_ECUDA;
        }
        e = cudaGraphInstantiate(&b->graph, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) {
            g_last_cuda = (int)e;
            return JT_ECUDA;
        }
        b->graph_stream = s;
    }
    JT_CU(cudaGraphLaunch(b->graph, s));
    g_launches++;
    return JT_OK;
}

int jt_batch_destroy(jt_batch *b) {
    if (!b) return JT_EINVAL;
    cudaDeviceSynchronize();
    delete b;
    return JT_OK;
}

}  // extern "C"

// ===========================================================================
// Complex 1D FFT without any allocation
//
// For callers that cannot allocate device memory when they transform: code
// running while a CUDA stream is being captured into a graph (cudaMalloc is
// not allowed there), real-time loops with a fixed memory budget, and hosts
// whose allocator is owned by another framework.  The regular entry points
// grow a per-thread scratch arena with cudaMalloc on first use of a size;
// this one takes its scratch from a fixed file-scope device array instead.
// Each GPU that loads the library holds that array until the process exits.
//
// Limit: the scratch is JT_NOALLOC_SCRATCH_BYTES (32 MiB).  Lengths that
// need the two- or three-pass scheme need one length's worth of complex
// scratch per transform in flight: n * 8 bytes (float) or n * 16 bytes
// (double) must fit, so n <= 2^22 (float) / 2^21 (double) there.  Lengths
// done in one pass need none.  Bluestein lengths are rejected: their scratch
// would not be bounded by one transform.
//
// The plan must be used on the device that was current when it was created
// (its tables live there); another current device gives JT_EINVAL.  A plan in
// JT_MODE_TC_SPLIT runs the same tensor-core kernels as jt_execute_device.
//
// Errors: a kernel whose bounded wait gave up raises the library's device
// error flag; the caller learns of it from jt_check_error (after its own
// synchronisation) or jt_synchronize.
//
// Sharing: every call uses the same array.  Nothing in it has to start at
// zero (each transform writes its scratch before reading it), but two calls
// whose kernels overlap on the GPU (different streams, or different host
// threads on one device) race on it: order them on one stream.
//
// Set-up: the first call on a device looks up the array's device address
// there (cudaGetSymbolAddress, with that device current) and keeps it.  Make
// that first call before any stream capture begins.
// ===========================================================================
#define JT_NOALLOC_SCRATCH_BYTES (32u << 20)
static __device__ __align__(256) unsigned char g_noalloc_scratch[JT_NOALLOC_SCRATCH_BYTES];
static void *g_noalloc_addr[64];
static std::mutex g_noalloc_mu;

static int noalloc_scratch(void **out) {
    int dev = 0;
    JT_CU(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) return JT_EINVAL;
    std::lock_guard<std::mutex> g(g_noalloc_mu);
    if (!g_noalloc_addr[dev]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            g_last_cuda = (int)e;
            return JT_ECUDA;
        }
        g_noalloc_addr[dev] = p;
    }
    *out = g_noalloc_addr[dev];
    return JT_OK;
}

template <typename T>
static int noalloc_run(jt_plan *p, int op, const void *in, void *out, int64_t batch, int scale, cudaStream_t s) {
    typedef typename V2<T>::t C2;
    PlanImpl<T> *im = (PlanImpl<T> *)p->impl;
    const int64_t n = p->dims[0];
    std::lock_guard<std::mutex> g(im->mu);
    auto it = im->fft.find(n);
    if (it == im->fft.end()) return JT_EINVAL;  // tables are built by jt_plan_create
    Fft1<T> *f = it->second.get();
    if (f->algo == ALG_BLUESTEIN) return JT_ESCRATCH;
    const int64_t per = (f->algo == ALG_TWOPASS || f->algo == ALG_THREEPASS) ? n * (int64_t)sizeof(C2) : 0;
    if (per > (int64_t)JT_NOALLOC_SCRATCH_BYTES) return JT_ESCRATCH;
    void *scratch = nullptr;
    JT_TRY(noalloc_scratch(&scratch));
    const int64_t sub = per ? std::max<int64_t>(1, (int64_t)JT_NOALLOC_SCRATCH_BYTES / per) : batch;
    const int sign = op == JT_COMPLEX_FORWARD ? -1 : 1;
    const double sc = (op == JT_COMPLEX_INVERSE && scale) ? 1.0 / (double)n : 1.0;
    const C2 *src = (const C2 *)in;
    C2 *dst = (C2 *)out;
    for (int64_t b = 0; b < batch; b += sub) {
        const int64_t cb = std::min(sub, batch - b);
        Arena ar;
        ar.base = (char *)scratch;
        ar.cap = JT_NOALLOC_SCRATCH_BYTES;
        Ctx c;
        c.s = s;
        c.tc = p->mode == JT_MODE_TC_SPLIT;  // the same kernels as jt_execute_device
        c.ws = &ar;
        c.dry = true;  // size check first: nothing may spill past the array
        JT_TRY(f->exec(c, src + b * n, n, dst + b * n, n, cb, sign, sc));
        if (ar.peak > ar.cap) return JT_ESCRATCH;
        ar.used = ar.peak = 0;
        c.dry = false;
        JT_TRY(f->exec(c, src + b * n, n, dst + b * n, n, cb, sign, sc));
    }
    JT_CU(cudaGetLastError());
    return JT_OK;
}

extern "C" int jt_execute_device_noalloc(jt_plan *p, int op, const void *dev_in, void *dev_out, int64_t batch, int scale,
                                         void *stream) {
    if (!p || !dev_in || !dev_out || batch < 0) return JT_EINVAL;
    if (p->kind != JT_FFT || p->nd != 1 || (op != JT_COMPLEX_FORWARD && op != JT_COMPLEX_INVERSE)) return JT_EINVAL;
    if (batch == 0) return JT_OK;
    const size_t esz = p->prec == JT_FLOAT32 ? 8 : 16;
    if (((uintptr_t)dev_in % esz) || ((uintptr_t)dev_out % esz)) return JT_EINVAL;
    // the plan's tables live on the device it was created on
    int dev = 0;
    JT_CU(cudaGetDevice(&dev));
    if (dev != p->device) return JT_EINVAL;
    if (p->prec == JT_FLOAT32) return noalloc_run<float>(p, op, dev_in, dev_out, batch, scale, (cudaStream_t)stream);
    return noalloc_run<double>(p, op, dev_in, dev_out, batch, scale, (cudaStream_t)stream);
}
