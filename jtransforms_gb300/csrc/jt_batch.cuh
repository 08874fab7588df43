// jt_batch.cuh -- one persistent launch for a batch of transforms of mixed
// sizes and kinds.
//
// The host records each transform as the chain of steps the single-transform
// path would launch (generic tile FFT passes and elementwise pre/post steps),
// into a table of ops.  Each op is split into tasks of one CTA's work; the
// task queue holds every transform's first step, then every second step, and
// so on.  batch_kernel's CTAs pull tasks with an atomic counter, wait
// (bounded) until the task's previous step in the same transform has
// finished, run it and count it done.  Because a step's tasks are all queued
// before any task of the next step, every awaited task is already held by a
// running CTA and the waits end.  Producer CTAs publish with a gpu-scope
// fence before the counter update; consumers read the counter with acquire
// semantics before their threads touch the data.
#pragma once

#include "jt_device.cuh"
#include "jt_stockham.cuh"
#include "jt_r2r.cuh"
#include "jt_chirp.cuh"

namespace jt {

enum BOpType { BOP_TILE = 0, BOP_ELEM = 2, BOP_R2R = 3, BOP_BLUE = 4 };

enum ElemKind {
    EK_COPY_COMPLEX = 0,
    EK_BLUE_PRE,
    EK_BLUE_MUL,
    EK_BLUE_POST,
    EK_REAL_POST_PACKED,
    EK_REAL_POST_FULL,
    EK_REAL_PRE_INV,
    EK_R2C,
    EK_PACK_FULL,
    EK_UNPACK_FULL,
    EK_REAL_PART,
    EK_DCT2_PRE,
    EK_DCT2_POST,
    EK_DCT3_PRE,
    EK_DCT3_POST,
    EK_DHT_POST,
    EK_SCALE,
    EK_COPY_REAL,
};

struct EArgs {
    const void *p[4];
    int64_t i[6];
    double d[3];
    int f;
};

struct BOp {
    int type, prec, sign, kind;
    int dep;     // op this one waits for (-1: none)
    int ntasks;  // CTA work units
    int64_t total;  // elementwise: number of indices
    // tile / stock
    union {
        TileParams tp;
        R2rParams rp;   // DCT/DST/DHT and packed real lines in one step (kind: the R2rOp)
        BlueParams bp;  // a Bluestein transform in one step (W, Whi, Wlo: roots, bk1, bk2)
    };
    const void *in;
    void *out;
    const void *W, *Whi, *Wlo;
    int smem;  // shared memory the step needs (bytes)
    // elementwise
    EArgs e;
};

struct BTask {
    int op;
    int idx;
};

// A batch CTA has 256 threads and at most JT_BATCH_SMEM_CAP bytes of shared
// memory per task, so that three CTAs share an SM and their loads overlap one
// another's arithmetic (lines whose tile would need more are recorded as two
// passes of shorter lines).  Measured on the 10,000-transform workload: two
// CTAs per SM (110 KB) 12.1 ms, three (72 KB, 80 registers) 9.4 ms, four
// (54 KB, 64 registers, heavy spilling) 10.6 ms.
#define JT_BATCH_THREADS 256
#define JT_BATCH_ELEMS_PER_TASK (JT_BATCH_THREADS * 4)
#define JT_BATCH_SMEM_CAP (72 * 1024)

template <typename T> __device__ void elem_dispatch(const BOp &o, int64_t idx) {
    typedef typename V2<T>::t C2;
    const EArgs &e = o.e;
    switch (o.kind) {
        case EK_COPY_COMPLEX:
            copy_complex_body<T>((const C2 *)e.p[0], e.i[0], (C2 *)e.p[1], e.i[1], e.i[2], e.i[3], (T)e.d[0], e.f, idx);
            break;
        case EK_BLUE_PRE:
            if (o.sign < 0)
                bluestein_pre_body<-1, T>((const C2 *)e.p[0], e.i[0], (C2 *)e.p[1], (const C2 *)e.p[2], e.i[1], e.i[2], e.i[3], idx);
            else
                bluestein_pre_body<1, T>((const C2 *)e.p[0], e.i[0], (C2 *)e.p[1], (const C2 *)e.p[2], e.i[1], e.i[2], e.i[3], idx);
            break;
        case EK_BLUE_MUL:
            if (o.sign < 0) bluestein_mul_body<-1, T>((C2 *)e.p[0], (const C2 *)e.p[1], e.i[0], e.i[1], idx);
            else bluestein_mul_body<1, T>((C2 *)e.p[0], (const C2 *)e.p[1], e.i[0], e.i[1], idx);
            break;
        case EK_BLUE_POST:
            if (o.sign < 0)
                bluestein_post_body<-1, T>((C2 *)e.p[0], e.i[0], (const C2 *)e.p[1], (const C2 *)e.p[2], e.i[1], e.i[2], e.i[3],
                                           (T)e.d[0], idx);
            else
                bluestein_post_body<1, T>((C2 *)e.p[0], e.i[0], (const C2 *)e.p[1], (const C2 *)e.p[2], e.i[1], e.i[2], e.i[3],
                                          (T)e.d[0], idx);
            break;
        case EK_REAL_POST_PACKED:
            real_post_packed_body<T>((T *)e.p[0], e.i[0], e.i[1], e.i[2], (const C2 *)e.p[1], idx);
            break;
        case EK_REAL_POST_FULL:
            if (o.sign < 0)
                real_post_full_body<-1, T>((const T *)e.p[0], e.i[0], (T *)e.p[1], e.i[1], e.i[2], e.i[3], (const C2 *)e.p[2],
                                           (T)e.d[0], idx);
            else
                real_post_full_body<1, T>((const T *)e.p[0], e.i[0], (T *)e.p[1], e.i[1], e.i[2], e.i[3], (const C2 *)e.p[2],
                                          (T)e.d[0], idx);
            break;
        case EK_REAL_PRE_INV:
            real_pre_inverse_body<T>((T *)e.p[0], e.i[0], e.i[1], e.i[2], (const C2 *)e.p[1], (T)e.d[0], idx);
            break;
        case EK_R2C: real_to_complex_body<T>((const T *)e.p[0], e.i[0], (C2 *)e.p[1], e.i[1], e.i[2], idx); break;
        case EK_PACK_FULL: pack_from_full_body<T>((const C2 *)e.p[0], (T *)e.p[1], e.i[0], e.i[1], e.i[2], idx); break;
        case EK_UNPACK_FULL: unpack_to_full_body<T>((const T *)e.p[0], e.i[0], (C2 *)e.p[1], e.i[1], e.i[2], idx); break;
        case EK_REAL_PART: real_part_body<T>((const C2 *)e.p[0], (T *)e.p[1], e.i[0], e.i[1], e.i[2], (T)e.d[0], idx); break;
        case EK_DCT2_PRE:
            dct2_pre_body<T>((const T *)e.p[0], e.i[0], (T *)e.p[1], e.i[1], e.i[2], e.i[3], e.f, idx);
            break;
        case EK_DCT2_POST:
            dct2_post_body<T>((const T *)e.p[0], e.i[0], (T *)e.p[1], e.i[1], e.i[2], e.i[3], (const C2 *)e.p[2], (T)e.d[0],
                              (T)e.d[1], e.f, idx);
            break;
        case EK_DCT3_PRE:
            dct3_pre_body<T>((const T *)e.p[0], e.i[0], (T *)e.p[1], e.i[1], e.i[2], e.i[3], (const C2 *)e.p[2], (T)e.d[0],
                             (T)e.d[1], e.f, idx);
            break;
        case EK_DCT3_POST:
            dct3_post_body<T>((const T *)e.p[0], e.i[0], (T *)e.p[1], e.i[1], e.i[2], e.i[3], e.f, idx);
            break;
        case EK_DHT_POST:
            dht_post_body<T>((const T *)e.p[0], e.i[0], (T *)e.p[1], e.i[1], e.i[2], e.i[3], (T)e.d[0], idx);
            break;
        case EK_SCALE: scale_body<T>((T *)e.p[0], e.i[0], e.i[1], e.i[2], (T)e.d[0], idx); break;
        case EK_COPY_REAL: copy_real_body<T>((const T *)e.p[0], e.i[0], (T *)e.p[1], e.i[1], e.i[2], e.i[3], idx); break;
    }
}

template <typename T> __device__ void r2r_dispatch(const BOp &o, int idx, unsigned char *smem) {
    typedef typename V2<T>::t C2;
    const T *in = (const T *)o.in;
    T *out = (T *)o.out;
    const C2 *W = (const C2 *)o.W, *Wr = (const C2 *)o.Whi, *Wd = (const C2 *)o.Wlo;
    if (o.kind == R2R_DCT2) r2r_tile_body<R2R_DCT2, T>(in, out, o.rp, W, Wr, Wd, idx, smem);
    else if (o.kind == R2R_DCT3) r2r_tile_body<R2R_DCT3, T>(in, out, o.rp, W, Wr, Wd, idx, smem);
    else if (o.kind == R2R_DHT) r2r_tile_body<R2R_DHT, T>(in, out, o.rp, W, Wr, Wd, idx, smem);
    else if (o.kind == R2R_RFWD) r2r_tile_body<R2R_RFWD, T>(in, out, o.rp, W, Wr, Wd, idx, smem);
    else r2r_tile_body<R2R_RINV, T>(in, out, o.rp, W, Wr, Wd, idx, smem);
}

__device__ __forceinline__ int ld_acquire_gpu(const int *p) {
    int v;
    asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// wait_polls: polls of a dependency wait (64 ns apart) before it gives up;
// the library's default, 2^24, is about a second
__global__ void __launch_bounds__(JT_BATCH_THREADS, 3)
    batch_kernel(const BOp *__restrict__ ops, const BTask *__restrict__ tasks, int ntasks, int *head, int *done, int *err,
                 int wait_polls) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ int s_task;
    __shared__ int s_ok;
    const int tid = threadIdx.x;
    for (;;) {
        if (tid == 0) s_task = atomicAdd(head, 1);
        __syncthreads();
        const int ti = s_task;
        if (ti >= ntasks) break;
        const BTask tk = tasks[ti];
        const BOp &o = ops[tk.op];
        if (tid == 0) {
            int ok = 1;
            if (o.dep >= 0) {
                const int need = ops[o.dep].ntasks;
                int it = 0;
                while (ld_acquire_gpu(&done[o.dep]) < need) {
                    if (++it > wait_polls) {
                        ok = 0;
                        atomicExch(err, 1);
                        break;
                    }
                    __nanosleep(64);
                }
            }
            s_ok = ok;
        }
        __syncthreads();
        if (s_ok) {
            if (o.type == BOP_TILE) {
                if (o.prec == 0) {
                    if (o.sign < 0) tile_fft_body<-1, float>((const float2 *)o.in, (float2 *)o.out, o.tp, (const float2 *)o.W, (const float2 *)o.Whi, (const float2 *)o.Wlo, tk.idx, smem_raw);
                    else tile_fft_body<1, float>((const float2 *)o.in, (float2 *)o.out, o.tp, (const float2 *)o.W, (const float2 *)o.Whi, (const float2 *)o.Wlo, tk.idx, smem_raw);
                } else {
                    if (o.sign < 0) tile_fft_body<-1, double>((const double2 *)o.in, (double2 *)o.out, o.tp, (const double2 *)o.W, (const double2 *)o.Whi, (const double2 *)o.Wlo, tk.idx, smem_raw);
                    else tile_fft_body<1, double>((const double2 *)o.in, (double2 *)o.out, o.tp, (const double2 *)o.W, (const double2 *)o.Whi, (const double2 *)o.Wlo, tk.idx, smem_raw);
                }
            } else if (o.type == BOP_BLUE) {
                if (o.prec == 0) {
                    if (o.sign < 0) blue_tile_body<-1, float>((const float2 *)o.in, (float2 *)o.out, o.bp, (const float2 *)o.W, (const float2 *)o.Whi, (const float2 *)o.Wlo, tk.idx, smem_raw);
                    else blue_tile_body<1, float>((const float2 *)o.in, (float2 *)o.out, o.bp, (const float2 *)o.W, (const float2 *)o.Whi, (const float2 *)o.Wlo, tk.idx, smem_raw);
                } else {
                    if (o.sign < 0) blue_tile_body<-1, double>((const double2 *)o.in, (double2 *)o.out, o.bp, (const double2 *)o.W, (const double2 *)o.Whi, (const double2 *)o.Wlo, tk.idx, smem_raw);
                    else blue_tile_body<1, double>((const double2 *)o.in, (double2 *)o.out, o.bp, (const double2 *)o.W, (const double2 *)o.Whi, (const double2 *)o.Wlo, tk.idx, smem_raw);
                }
            } else if (o.type == BOP_R2R) {
                if (o.prec == 0) r2r_dispatch<float>(o, tk.idx, smem_raw);
                else r2r_dispatch<double>(o, tk.idx, smem_raw);
            } else {
                const int64_t base = (int64_t)tk.idx * JT_BATCH_ELEMS_PER_TASK;
                for (int k = tid; k < JT_BATCH_ELEMS_PER_TASK; k += JT_BATCH_THREADS) {
                    const int64_t idx = base + k;
                    if (idx < o.total) {
                        if (o.prec == 0) elem_dispatch<float>(o, idx);
                        else elem_dispatch<double>(o, idx);
                    }
                }
            }
        }
        __syncthreads();
        if (tid == 0) {
            __threadfence();
            atomicAdd(&done[tk.op], 1);
        }
    }
}

}  // namespace jt
