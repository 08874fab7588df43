/*
 * jtgpu.h -- C ABI of jtransforms_gb300, the GB300 (sm_103a) implementation
 * of JTransforms' transform path.
 *
 * Every entry point takes plain pointers and sizes and returns an int status
 * (JT_OK or a negative JT_E* code).  Arrays keep JTransforms' in-place layouts:
 * interleaved complex a[2k]=Re, a[2k+1]=Im; the packed real layouts of
 * realForward; row-major 2D/3D.  Element counts and offsets are in units of
 * the precision's scalar (float or double), as JTransforms' `offa` is.
 *
 * Reference interfaces replaced (paths relative to
 * src/main/java/org/jtransforms/ in JTransforms):
 *   jt_plan_create   <- the constructors DoubleFFT_1D(long) fft/DoubleFFT_1D.java:117,
 *                       FloatFFT_1D(long) fft/FloatFFT_1D.java:117,
 *                       DoubleFFT_2D(long,long) fft/DoubleFFT_2D.java:75,
 *                       DoubleFFT_3D(long,long,long) fft/DoubleFFT_3D.java:88,
 *                       DoubleDCT_1D dct/DoubleDCT_1D.java:84, DoubleDCT_2D
 *                       dct/DoubleDCT_2D.java:73, DoubleDST_1D dst/DoubleDST_1D.java:55,
 *                       DoubleDST_3D dst/DoubleDST_3D.java:84, DoubleDHT_1D
 *                       dht/DoubleDHT_1D.java:55, DoubleDHT_3D dht/DoubleDHT_3D.java:84
 *                       and their Float* twins.
 *   jt_execute       <- the in-place methods on double[]/float[] with offa:
 *                       complexForward fft/DoubleFFT_1D.java:243,
 *                       complexInverse :362, realForward :524,
 *                       realForwardFull :678, realInverse :946,
 *                       realInverseFull :1112; DoubleFFT_2D/3D's versions
 *                       (fft/DoubleFFT_2D.java:115-1289, fft/DoubleFFT_3D.java:145-1846);
 *                       forward/inverse(a, offa, scale) of DCT
 *                       (dct/DoubleDCT_1D.java:169, :361), DST
 *                       (dst/DoubleDST_1D.java:96, :264), DHT
 *                       (dht/DoubleDHT_1D.java:94, :255) and their nD classes.
 *   jt_execute_batch <- a loop of the above over equally spaced arrays (the
 *                       reference has no batch call; its benchmarks loop).
 *   jt_execute_device<- the same on arrays already in device memory.
 *   jt_plan_destroy  <- object finalisation (Cleaner) of the Java classes.
 */
#ifndef JTGPU_H
#define JTGPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define JT_OK 0
#define JT_EBADSIZE (-1)   /* n < 1, or nD size <= 1: IllegalArgumentException (fft/DoubleFFT_1D.java:119, fft/DoubleFFT_2D.java:77) */
#define JT_ESHORTBUF (-2)  /* array shorter than offset + the op's extent: ArrayIndexOutOfBoundsException */
#define JT_ENOTPOW2 (-3)   /* 2D/3D realForward/realInverse on non-power-of-two sizes (fft/DoubleFFT_2D.java:820-823) */
#define JT_ECUDA (-4)      /* a CUDA call failed; jt_last_cuda_error() has the code */
#define JT_ETIMEOUT (-5)   /* a bounded device-side wait gave up */
#define JT_EINVAL (-6)     /* bad enum value, null pointer, or op not defined for the kind */
#define JT_ENOMEM (-7)     /* device allocation failed */
#define JT_ENODEV (-8)     /* no CUDA device */
#define JT_ETOOBIG (-9)    /* size beyond what this build supports on one GPU */
#define JT_ESCRATCH (-10)  /* jt_execute_device_noalloc: the transform needs more than the fixed scratch */

/* transform kinds */
#define JT_FFT 0
#define JT_DCT 1
#define JT_DST 2
#define JT_DHT 3

/* precisions */
#define JT_FLOAT32 0
#define JT_FLOAT64 1

/* operations */
#define JT_COMPLEX_FORWARD 0
#define JT_COMPLEX_INVERSE 1
#define JT_REAL_FORWARD 2
#define JT_REAL_FORWARD_FULL 3
#define JT_REAL_INVERSE 4
#define JT_REAL_INVERSE_FULL 5
#define JT_FORWARD 6 /* DCT/DST/DHT forward */
#define JT_INVERSE 7 /* DCT/DST/DHT inverse */

/* Float32 FFT arithmetic modes (jt_plan_set_mode) */
#define JT_MODE_FP32 0       /* plain FP32 on the CUDA cores (default) */
#define JT_MODE_TC_SPLIT 1   /* radix-16 stages as split-operand tensor-core products */

typedef struct jt_plan jt_plan;

/* Creates a plan for `kind` in `prec` over ndim (1..3) dimensions dims[0..ndim)
 * (row-major: dims[0] slowest).  Sizes follow the reference constructors:
 * 1D n >= 1; 2D/3D each size > 1.  Device tables are built here. */
int jt_plan_create(int kind, int prec, int ndim, const int64_t *dims, jt_plan **out);

/* Releases the plan and its device tables. */
int jt_plan_destroy(jt_plan *plan);

/* Number of scalars `op` reads/writes starting at the offset (2n for complex
 * and *Full ops, n for packed real ops and DCT/DST/DHT). */
int jt_plan_extent(const jt_plan *plan, int op, int64_t *out_len);

/* Selects the FP32 arithmetic mode of a Float32 FFT plan (JT_MODE_*). */
int jt_plan_set_mode(jt_plan *plan, int mode);

/* One transform in place on a HOST array of array_len scalars, starting at
 * `offset`.  Copies to the device, runs the kernels, copies back. */
int jt_execute(jt_plan *plan, int op, void *host_array, int64_t array_len,
               int64_t offset, int scale);

/* `batch` transforms on a host array, transform b starting at
 * offset + b*dist.  Transfers are pipelined with the kernels. */
int jt_execute_batch(jt_plan *plan, int op, void *host_array, int64_t array_len,
                     int64_t offset, int64_t batch, int64_t dist, int scale);

/* `batch` transforms in place on DEVICE memory, transform b at
 * dev_array + b*dist scalars, on `stream` (a cudaStream_t; NULL = CUDA's
 * default stream).  Asynchronous: returns after the launches. */
int jt_execute_device(jt_plan *plan, int op, void *dev_array, int64_t batch,
                      int64_t dist, int scale, void *stream);

/* Complex 1D FFT (JT_COMPLEX_FORWARD / JT_COMPLEX_INVERSE) of `batch`
 * contiguous transforms from dev_in to dev_out (device memory; they may be the
 * same array) that allocates nothing.  No counterpart in the reference: it is
 * for callers that cannot allocate device memory when they transform, such as
 * code inside CUDA stream capture (cudaMalloc is not allowed there) or with a
 * fixed memory budget.  Scratch comes from one fixed 32 MiB device array per
 * GPU: two- and three-pass lengths need n*8 (float) / n*16 (double) bytes of
 * it, so n <= 2^22 / 2^21 there; Bluestein lengths are refused with
 * JT_ESCRATCH.  Calls share the array, so calls that overlap on the GPU race.
 * The first call on a device looks up the array's address: make it before any
 * stream capture.  The plan must be used on the device it was created on
 * (JT_EINVAL otherwise).  Asynchronous on `stream` (NULL = the default
 * stream); a timed-out device wait is reported by jt_check_error after the
 * caller's own synchronisation. */
int jt_execute_device_noalloc(jt_plan *plan, int op, const void *dev_in, void *dev_out, int64_t batch, int scale,
                              void *stream);

/* Waits for the calling thread's stream; returns JT_ECUDA on a device error. */
int jt_synchronize(void);

/* Reads and clears the device error flag that a kernel raises when one of
 * its bounded waits gives up: JT_ETIMEOUT if it was raised, else JT_OK.
 * For callers that synchronise their own streams or graphs (after
 * jt_execute_device or jt_execute_device_noalloc); jt_synchronize and the
 * host-array calls check it themselves.  No counterpart in the reference
 * (worker failures are logged there, fft/DoubleFFT_1D.java:711-715). */
int jt_check_error(void);

/* Mixed-size batch (work descriptors of several plans) -------------------- */
typedef struct jt_batch jt_batch;

/* Builds a batch of `count` descriptors: plans[i] (1D plans), op ops[i],
 * device array dev_ptrs[i], scale flags scales[i].  All descriptors are
 * validated here; jt_batch_run executes them as one persistent launch per
 * precision class, replayable from a CUDA graph. */
int jt_batch_create(int count, jt_plan *const *plans, const int *ops,
                    void *const *dev_ptrs, const int *scales, jt_batch **out);
int jt_batch_run(jt_batch *batch, void *stream);
/* Runs the same work as one launch sequence per descriptor (the baseline). */
int jt_batch_run_per_transform(jt_batch *batch, void *stream);
/* Captures jt_batch_run into a CUDA graph and replays it on each later call. */
int jt_batch_run_graph(jt_batch *batch, void *stream);
int jt_batch_destroy(jt_batch *batch);

/* Global options --------------------------------------------------------- */
#define JT_OPT_TMA_PIPELINE 0 /* 1 (default): power-of-two lines use the TMA-pipelined kernel when
                                 the arrays meet its 16-byte rules; 0: the plain kernel */
#define JT_OPT_DIRECT_MAX_F32 1 /* longest power-of-two float length done in one pass (default 8192);
                                   longer lengths use two passes.  Read when a plan is created. */
#define JT_OPT_DIRECT_MAX_F64 2 /* the same for double (default 8192) */
#define JT_OPT_COLUMN_KERNEL 3  /* 0 only: column passes use the tile-pipelined kernel (other values
                                   return JT_EINVAL) */
#define JT_OPT_TWOPASS_CHUNK_MB 4 /* MiB of transforms per two-pass chunk and launch (default 1024,
                                     1..16384); the intermediate scratch is one chunk */
#define JT_OPT_HOST_PIECE_MB 6   /* MiB per piece of a host-array batch (default 64, 1..16384):
                                    pieces are copied in, transformed and copied out overlapped */
#define JT_OPT_THREEPASS_MIN_LOG2 5 /* float powers of two from 2^value use three passes of
                                       near-equal lengths (default 21; 0: only beyond 2^24, where
                                       every power of two up to 2^32 takes three).  Read when a
                                       plan is created. */
#define JT_OPT_ARENA_LIMIT_MB 7   /* device scratch budget per call in MiB (default 0: no limit): a call
                                     whose scratch (host-array ring buffers included) needs more
                                     returns JT_ENOMEM before it launches anything */
#define JT_OPT_BATCH_WAIT_POLLS 8 /* polls (64 ns apart) of a batch kernel's dependency wait before it gives
                                     up with JT_ETIMEOUT (default 2^24, about a second); read by
                                     jt_batch_create */
#define JT_OPT_BATCH_STALL_TEST 9 /* failure-path test hook (default 0): 1 makes jt_batch_create add a step
                                     that never runs as the dependency of every transform's first step,
                                     so the waits run out and the run reports JT_ETIMEOUT */
#define JT_OPT_TILE_ELEMS 10     /* elements per CTA of the mixed-radix tile kernel, which sets lines and
                                     threads per CTA (default 0: the tuned table of jt_plan_table.h);
                                     the autotuner's probe */
#define JT_OPT_REAL_FUSED_F32 11 /* 1 (default): Float packed realForward/realInverse lines with a
                                     power-of-two half length of 16..4096 run as one kernel (FFT and
                                     real split together); 0: the pipelined FFT and a separate split */
#define JT_OPT_RADIX_ORDER 12   /* pass order of the mixed-radix tile kernel: -1 (default) the tuned
                                     table of jt_plan_table.h; 0 power-of-two radices (16s) first,
                                     1 odd radices first, 2 power-of-two radices as 8s first, 3 odd
                                     first then 8s; plans created afterwards; the autotuner's probe */
/* Sets a global option; returns the previous value, or JT_EINVAL. */
int jt_set_option(int option, int value);

/* Pass split of power-of-two length 2^log2n in `prec` for plans created from
 * now on, overriding the compiled plan table (the autotuner's probe):
 * (0,0,0) one pass; (a,b,0) two passes 2^a x 2^b, a + b = log2n, each <= 12;
 * (a,b,c) three passes, a + b + c = log2n; a < 0 clears the
 * override.  No counterpart in the reference. */
int jt_set_split(int prec, int log2n, int a, int b, int c);

/* Diagnostics ------------------------------------------------------------ */
const char *jt_strerror(int status);
int jt_last_cuda_error(void);
/* Number of kernel launches this thread issued since the last reset. */
int64_t jt_launch_count(int reset);
/* Algorithm the plan uses along axis `axis` for length-n complex work:
 * 0 direct in-CTA, 1 two-pass, 2 Bluestein, 3 trivial, 4 three-pass. */
int jt_plan_algorithm(const jt_plan *plan, int axis);
/* Measured CUDA-core FMA throughput of the current GPU in GFLOP/s (one FMA =
 * two flops) for `prec`: the compute roofline of the Double (FP64) and Float
 * paths.  No counterpart in the reference. */
int jt_fma_peak(int prec, double *gflops);
/* Measured aggregate read bandwidth in GB/s of shared memory within thread-block
 * clusters of `cluster` CTAs (2, 4, 8 or 16; 128 KiB and 1024 threads per CTA,
 * as many clusters as fit at once): remote = 1 reads peers' shared memory
 * (distributed shared memory), remote = 0 the CTA's own.  `active_ctas`
 * (may be NULL) receives the number of CTAs resident in that launch.  The
 * bound of a plan that exchanges one transform between the CTAs of a
 * cluster.  No counterpart in the reference. */
int jt_dsmem_peak(int cluster, int remote, double *gbs, int *active_ctas);

#ifdef __cplusplus
}
#endif

#endif /* JTGPU_H */
