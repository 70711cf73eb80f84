/*
 * lofgb.h — C ABI of liblofgb.so, the GB300 (sm_103a) kernels behind the
 * LoFloat emulation ops.
 *
 * Every entry point:
 *   - takes plain device pointers, element counts and a cudaStream_t passed as
 *     `void*` (NULL = legacy default stream); no torch types cross this line;
 *   - launches asynchronously on that stream and never synchronises the device;
 *   - returns LOFGB_OK (0) or a negative LOFGB_ERR_* code, never exits/aborts;
 *     lofgb_strerror() turns a code into text, lofgb_last_error_detail() gives
 *     the message of the last failing call on the calling host thread;
 *   - writes out-of-place; `in == out` (fully aliased) is allowed for the
 *     elementwise and MX entry points;
 *   - leaves all memory to the caller (inputs borrowed, outputs preallocated).
 *
 * Each declaration names the reference interface it replaces
 * (SudhanvaKulkarni123/LoFloat, path:line).
 */
#ifndef LOFGB_H
#define LOFGB_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- enums: integer values follow the reference's X-macro order ---------
 * src/fp_tools.hpp:13-28 (rounding_modes), :30-32 (signednesses),
 * :34-36 (inf_behaviors), :44-46 (nan_behaviors). The Python enums of the
 * reference binding (src/LoPy_bind.cpp:284-313) expose the same integers. */
enum lofgb_rounding_mode {
    LOFGB_RNE = 0,              /* RoundToNearestEven */
    LOFGB_RTZ = 1,              /* RoundTowardsZero */
    LOFGB_RAFZ = 2,             /* RoundAwayFromZero */
    LOFGB_SR_A = 3,             /* StochasticRoundingA */
    LOFGB_RNO = 4,              /* RoundToNearestOdd */
    LOFGB_RD = 5,               /* RoundDown */
    LOFGB_RU = 6,               /* RoundUp */
    LOFGB_RTA = 7,              /* RoundTiesToAway */
    LOFGB_SR_B = 8,             /* StochasticRoundingB */
    LOFGB_SR_C = 9,             /* StochasticRoundingC */
    LOFGB_TRUE_SR = 10,         /* True_StochasticRounding */
    LOFGB_PROB = 11,            /* ProbabilisticRounding */
    LOFGB_RTO = 12,             /* RoundToOdd */
    LOFGB_RTTZ = 13,            /* RoundTiesTowardsZero */
    LOFGB_SR_D = 14,            /* StochasticRoundingD */
    LOFGB_NUM_MODES = 15
};
enum lofgb_inf_behavior { LOFGB_INF_EXTENDED = 0, LOFGB_INF_SATURATING = 1 };
enum lofgb_nan_behavior { LOFGB_NAN_3109 = 0, LOFGB_NAN_754 = 1 };
enum lofgb_signedness { LOFGB_SIGNED = 0, LOFGB_UNSIGNED = 1 };

/* Runtime float format. Mirrors the fields of FloatingPointParams that the
 * rounding path reads (src/fp_tools.hpp:187-252) and of the Python
 * FloatFormatDescriptor (src/LoPy_bind.cpp:45-68). The inf/NaN checker
 * functors are not carried: virtual_round never calls them
 * (src/lo_float.h:2843-2939). */
typedef struct lofgb_format {
    int32_t bitwidth;       /* total bits incl. sign (if signed)            */
    int32_t mantissa_bits;  /* fraction bits                                 */
    int32_t bias;           /* exponent bias                                 */
    uint8_t inf_behavior;   /* lofgb_inf_behavior                            */
    uint8_t nan_behavior;   /* lofgb_nan_behavior (carried, not used)        */
    uint8_t signedness;     /* lofgb_signedness                              */
    uint8_t reserved;       /* must be 0                                     */
} lofgb_format;

/* ---- status codes -------------------------------------------------------- */
enum lofgb_status {
    LOFGB_OK = 0,
    LOFGB_ERR_NULL = -1,          /* NULL pointer where data is required     */
    LOFGB_ERR_SIZE = -2,          /* negative / inconsistent sizes            */
    LOFGB_ERR_FORMAT = -3,        /* format fields out of supported range     */
    LOFGB_ERR_MODE = -4,          /* unknown rounding mode / bad stoch_len    */
    LOFGB_ERR_BLOCK = -5,         /* unsupported MX block size                */
    LOFGB_ERR_ALIAS = -6,         /* partially overlapping in/out             */
    LOFGB_ERR_UNSUPPORTED = -7,   /* valid request the kernel does not cover  */
    LOFGB_ERR_CUDA = -8,          /* CUDA runtime error (see detail string)   */
    LOFGB_ERR_WORKSPACE = -9,     /* caller workspace too small               */
    LOFGB_ERR_TIMEOUT = -10       /* a bounded device-side wait expired       */
};

const char* lofgb_strerror(int status);
/* Message of the last failing call made by this host thread ("" if none). */
const char* lofgb_last_error_detail(void);
/* Library version as MAJOR*10000 + MINOR*100 + PATCH. */
int lofgb_version(void);

/* ---- (a) virtual rounding to a runtime format ----------------------------
 * Replaces the CUDA branch of virtual_round_params (src/LoPy_bind.cpp:122-139)
 * → round_fp_params / round_fp_params_kernel (src/Lof_kernel.cu:49-60), scalar
 * semantics lo_float::virtual_round(x, FloatingPointParams, ProjSpec)
 * (src/lo_float.h:2843-2939, public wrapper :4271-4274).
 * out[i] = virtual_round(scale * in[i], fmt, {mode, OvfInf, stoch_len}).
 * `scale` is applied in the source type, as the reference kernel does
 * (src/Lof_kernel.cu:52); scale == 1 skips the multiply.
 * Stochastic modes: element g = offset + i reads lane g mod 2^lg (from the
 * low end, 64 >> lg bits) of SplitMix64 output g >> lg of the stream `seed`,
 * lanes the narrowest of 8/16/32/64 bits holding what the mode reads
 * (SR-A/B/C: stoch_len bits, SR-D: stoch_len + 1, Prob: 1, True SR: 64), so
 * a stream split at any offset reproduces the single call.
 * f16 data is IEEE binary16 bit patterns (uint16_t). */
int lofgb_round_f32(const float* in, float* out, int64_t n, const lofgb_format* fmt,
                    int mode, int stoch_len, float scale, uint64_t seed,
                    uint64_t offset, void* stream);
int lofgb_round_f64(const double* in, double* out, int64_t n, const lofgb_format* fmt,
                    int mode, int stoch_len, double scale, uint64_t seed,
                    uint64_t offset, void* stream);
int lofgb_round_f16(const uint16_t* in, uint16_t* out, int64_t n, const lofgb_format* fmt,
                    int mode, int stoch_len, float scale, uint64_t seed,
                    uint64_t offset, void* stream);

/* ---- (a') mantissa-only rounding -----------------------------------------
 * Replaces virtual_round_mantissa (src/LoPy_bind.cpp:80-120) → round_mantissa /
 * round_mantissa_kernel (src/Lof_kernel.cu:37-48), scalar semantics
 * lo_float::virtual_round(x, int ToMantissaBits, ProjSpec)
 * (src/lo_float.h:2715-2756, wrapper :4258-4261). */
int lofgb_round_mantissa_f32(const float* in, float* out, int64_t n, int mantissa_bits,
                             int mode, int stoch_len, float scale, uint64_t seed,
                             uint64_t offset, void* stream);
int lofgb_round_mantissa_f64(const double* in, double* out, int64_t n, int mantissa_bits,
                             int mode, int stoch_len, double scale, uint64_t seed,
                             uint64_t offset, void* stream);
int lofgb_round_mantissa_f16(const uint16_t* in, uint16_t* out, int64_t n,
                             int mantissa_bits, int mode, int stoch_len, float scale,
                             uint64_t seed, uint64_t offset, void* stream);

/* ---- (b) MX block rounding -----------------------------------------------
 * Replaces virtual_mx_round (src/LoPy_bind.cpp:165-217) → run_virtual_mx_round
 * (src/Lof_kernel.cu:70-94) → virtual_mx_round<float,256,MX,NX>
 * (src/mx_round.cuh:27-214). Contiguous blocks of `block_size` elements; the
 * trailing partial block is masked. block_size ∈ {8,16,32,64,128,256}
 * (the reference launcher accepts 16..256). Element SR draws use counter
 * offset + i; scale rounding never uses stochastic bits (stoch_len 0, as
 * src/mx_round.cuh:58-65). */
int lofgb_mx_round_f32(const float* in, float* out, int64_t n, int block_size,
                       const lofgb_format* elem_fmt, const lofgb_format* scale_fmt,
                       int mode, int scale_mode, int stoch_len, uint64_t seed,
                       uint64_t offset, void* stream);

/* The same MX rounding of a BF16 tensor (bit patterns, uint16_t), written as
 * FP32: equal to lofgb_mx_round_f32 on the tensor widened to FP32 (widening
 * is exact), without that copy. No counterpart in the reference, whose MX op
 * takes FP32 only (src/LoPy_bind.cpp:172); it serves BF16 master weights and
 * activations (the linear-layer workload). Input and output may not overlap. */
int lofgb_mx_round_bf16(const uint16_t* in, float* out, int64_t n, int block_size,
                        const lofgb_format* elem_fmt, const lofgb_format* scale_fmt,
                        int mode, int scale_mode, int stoch_len, uint64_t seed,
                        uint64_t offset, void* stream);

/* ---- (c) emulated-accumulation GEMM --------------------------------------
 * Replaces LoF_gemm (src/Lof_kernel.cu:96-154) → lo_float::Gemm::run_scaled
 * (src/cutlass_gemms.cuh:1777-1787) with the OpLoFMultiplyAdd leaf
 * (src/cutlass_gemms.cuh:97-168).
 *
 * D[i,j] = alpha * acc_K(i,j), acc_0 = +0,
 * acc_{k+1} = RNE_m(rto_fma(A[i,k], B[k,j], acc_k))  for k = 0..K-1 in order.
 * A is M×K (trans_a = 0: row-major with leading dim lda ≥ K; trans_a = 1:
 * stored K×M row-major, lda ≥ M). B is K×N (trans_b = 0: row-major, ldb ≥ N;
 * trans_b = 1: stored N×K, ldb ≥ K). D is M×N row-major, ldd ≥ N.
 * The reference leaf ignores the rounding mode and always uses RNE
 * (src/cutlass_gemms.cuh:122); `mode` must be LOFGB_RNE.
 * alpha: the caller passes 1/(scale_a*scale_b) (1 if the product is 0), as
 * run_scaled computes it (src/cutlass_gemms.cuh:1784-1786).
 *
 * variant LOFGB_GEMM_PLAIN: CUDA cores, bit-exact, needs no workspace.
 * variant LOFGB_GEMM_TC: tcgen05 tensor cores; each k-chunk of `chunk`
 * (multiple of 16) is summed in FP32 in TMEM and then rounded into the
 * emulated accumulator: acc = RNE_m(rto(acc + chunk_sum)). Operands are split
 * into BF16 hi+lo pairs (3 MMAs per k-step; the lo·lo term is dropped; an
 * operand whose values are all exact in BF16 skips its lo MMAs). Not
 * bit-exact; error is stated against lofgb_gemm_f64_ref. Needs `workspace` of
 * lofgb_gemm_tc_workspace_size(M,N,K) bytes (256-byte aligned). The output
 * tile is 128 x 128 or 128 x 256 by the launch's wave count (bit-identical
 * results); the environment variable LOFGB_TC_TILE_N=128|256 overrides the
 * choice for the mantissa accumulator. */
enum lofgb_gemm_variant { LOFGB_GEMM_PLAIN = 0, LOFGB_GEMM_TC = 1 };

int lofgb_gemm_f32(const float* A, int64_t lda, int trans_a, const float* B, int64_t ldb,
                   int trans_b, float* D, int64_t ldd, int M, int N, int K,
                   int accum_mant_bits, int mode, float alpha, int variant, int chunk,
                   void* workspace, size_t workspace_bytes, void* stream);
size_t lofgb_gemm_tc_workspace_size(int M, int N, int K);

/* Strided-batched form: `batch` independent products, GEMM b reading
 * A + b*stride_a and B + b*stride_b and writing D + b*stride_d (element
 * strides; 0 broadcasts an operand; D matrices may not overlap), each exactly
 * as lofgb_gemm_f32 computes it. Replaces the per-matrix Python loop of
 * _lof_gemm_2d (LoFloat/layers.py:136-150) through which
 * LoF_MultiHeadAttention's score and context products run (:1331-1345).
 * LOFGB_GEMM_TC needs lofgb_gemm_batched_tc_workspace_size(M, N, K, batch)
 * bytes. */
int lofgb_gemm_batched_f32(const float* A, int64_t lda, int64_t stride_a, int trans_a,
                           const float* B, int64_t ldb, int64_t stride_b, int trans_b, float* D,
                           int64_t ldd, int64_t stride_d, int M, int N, int K, int batch,
                           int accum_mant_bits, int mode, float alpha, int variant, int chunk,
                           void* workspace, size_t workspace_bytes, void* stream);
size_t lofgb_gemm_batched_tc_workspace_size(int M, int N, int K, int batch);

/* Emulated GEMM whose accumulator lives in a whole floating-point format:
 * after every multiply-add (plain) or every chunk (tensor cores)
 *   acc = virtual_round(rto(acc + ...), accum_fmt, RNE)
 * — the format's exponent range, subnormals and overflow rule included, as
 * lofgb_round_f32 applies them. No counterpart in the reference, whose leaf
 * rounds only the mantissa (src/cutlass_gemms.cuh:162-163); it gives the
 * FP16-like (5 exponent, 10 mantissa bits) accumulator of the linear-layer
 * workload. Arguments and workspace as lofgb_gemm_f32. */
int lofgb_gemm_accfmt_f32(const float* A, int64_t lda, int trans_a, const float* B, int64_t ldb,
                          int trans_b, float* D, int64_t ldd, int M, int N, int K,
                          const lofgb_format* accum_fmt, float alpha, int variant, int chunk,
                          void* workspace, size_t workspace_bytes, void* stream);

/* Tensor-core GEMM for callers that cannot allocate device memory.
 * No counterpart in the reference.
 *
 * Some callers may not call cudaMalloc at the point where they run a GEMM.
 * Examples are a plugin whose host framework owns every byte of device
 * memory and forbids allocation inside its execute callback, and a serving
 * loop that allocates once at start-up. The usual tensor-core entry point
 * (lofgb_gemm_f32 with LOFGB_GEMM_TC) needs a caller-provided workspace for
 * the BF16 split operands, so these callers could not use it.
 *
 * This entry point computes exactly what lofgb_gemm_f32(..., mode = RNE,
 * variant = LOFGB_GEMM_TC, chunk, ...) computes, same arguments and layouts.
 * Its scratch is a fixed 64 MiB device array inside liblofgb.so. Every GPU
 * that loads the library keeps that array until the process exits. The call
 * itself allocates nothing: no cudaMalloc, no cudaFree, no allocating
 * library routine.
 *
 * Limits and sharing:
 *   - the split operands need lofgb_gemm_tc_workspace_size(M, N, K) bytes;
 *     above 64 MiB (for example M = N = K = 2048 fits, 4096 does not) the
 *     call returns LOFGB_ERR_WORKSPACE and does nothing;
 *   - arguments are checked first and give the codes lofgb_gemm_f32 gives;
 *     only a valid request is compared with the 64 MiB limit;
 *   - the first call on each device looks up the array's device address
 *     (cudaGetSymbolAddress) with that device current. With lazy module
 *     loading (the CUDA default) that lookup can load this library's kernel
 *     module on the device, which commits the 64 MiB array and the module
 *     code at that moment. So make the first call on each device at set-up,
 *     outside any region where allocation is forbidden, and before any
 *     stream capture; later calls on that device allocate nothing;
 *   - all calls share the one array, which keeps the last call's contents
 *     (every call rewrites the parts it reads, so nothing leaks into the
 *     result); calls that overlap on the GPU (different streams, or
 *     different host threads, without ordering between them) race on it;
 *   - device-side timeouts are not reported: the tensor-core kernel bounds
 *     its waits (about 2 s) and, when one runs out, leaves D incomplete and
 *     records LOFGB_ERR_TIMEOUT in a status word inside the private array,
 *     which no entry point reads back. lofgb_gemm_f32 with a caller
 *     workspace exposes that word (the workspace's first 4 bytes). */
int lofgb_gemm_tc_noalloc_f32(const float* A, int64_t lda, int trans_a, const float* B,
                              int64_t ldb, int trans_b, float* D, int64_t ldd, int M, int N,
                              int K, int accum_mant_bits, float alpha, int chunk,
                              void* stream);

/* Self-test of the tensor-core kernel's bounded waits. No counterpart in the
 * reference, whose CUTLASS runner exits the process on an error
 * (src/cutlass_gemms.cuh:45-50). Runs the tensor-core GEMM (A M x K, B K x N,
 * D M x N, all row-major, 10-bit accumulator, chunk 32; workspace as
 * lofgb_gemm_f32) with every wait limited to wait_limit_us microseconds
 * (100..100000) while the copy producer of every CTA withholds its first
 * pipeline stage: no copy is issued for it and nothing faults, but the MMA
 * warp's wait for it runs out. Every CTA then takes the abort path a real
 * stall would take: it records LOFGB_ERR_TIMEOUT in the workspace status word
 * (its first 4 bytes), drains its own copies and MMAs, frees its tensor memory
 * and exits; D is left incomplete. Returns the launch status; the caller reads
 * the status word after synchronising. */
int lofgb_gemm_tc_wait_selftest(const float* A, const float* B, float* D, int M, int N, int K,
                                void* workspace, size_t workspace_bytes, uint32_t wait_limit_us,
                                void* stream);

/* FP64 GPU oracle GEMM used only to state the error of the tensor-core form:
 * D[i,j] = sum_k (double)A[i,k]*(double)B[k,j] in FP64, same layouts as above.
 * No counterpart in the reference (its harness compares against cuBLAS SGEMM,
 * test/gemm_test.cu:114). */
int lofgb_gemm_f64_ref(const float* A, int64_t lda, int trans_a, const float* B,
                       int64_t ldb, int trans_b, double* D, int64_t ldd, int M, int N,
                       int K, void* stream);

/* ---- grouped tensor-core GEMM: many GEMMs of different sizes, one launch ----
 * Batched form of the tensor-core GEMM (the reference loops over a batch in
 * Python, LoFloat/layers.py:136-150). Two phases so that the launches can be
 * captured in a CUDA graph:
 *   1. lofgb_gemm_grouped_prepare() validates the tasks on the host, lays the
 *      split operands of every task out in the caller's device `workspace`
 *      (lofgb_gemm_grouped_workspace_size bytes, 256-byte aligned; only its
 *      address is used here) and writes a table of
 *      lofgb_gemm_grouped_table_size bytes into the caller's HOST buffer:
 *      per-task rows with their TMA descriptors, and the list of output
 *      tiles in the order given by `schedule`:
 *        0 = task by task, 1 = longest K first, dealt round-robin to the
 *        `grid` CTAs, 2 = longest K first, dealt boustrophedon;
 *      tiles are 128 x 128, or 128 x 64 with LOFGB_GROUPED_TILE_N64 or-ed
 *      into `schedule` (twice the tiles: finer load balance over uneven
 *      GEMMs, more operand traffic per product), or 128 x 256 with
 *      LOFGB_GROUPED_TILE_N256 (half the tiles, one MMA per 256 columns);
 *   2. the caller copies the table to device memory (256-byte aligned) and
 *      calls lofgb_gemm_grouped_launch(): one operand-split launch and one
 *      persistent tensor-core launch of `grid` CTAs (0 = one per SM).
 * Each task computes what lofgb_gemm_f32(..., LOFGB_RNE, ..., LOFGB_GEMM_TC,
 * chunk, ...) computes for it. The first 4 bytes of the workspace receive the
 * device status (0, or LOFGB_ERR_TIMEOUT). */
enum { LOFGB_GROUPED_TILE_N64 = 16, LOFGB_GROUPED_TILE_N256 = 32 };
typedef struct lofgb_gemm_task {
    const float* A;
    int64_t lda;
    const float* B;
    int64_t ldb;
    float* D;
    int64_t ldd;
    int32_t trans_a;
    int32_t trans_b;
    int32_t M, N, K;
    int32_t accum_mant_bits;
    float alpha;
    int32_t chunk;
} lofgb_gemm_task;

size_t lofgb_gemm_grouped_workspace_size(const lofgb_gemm_task* tasks, int ntasks);
size_t lofgb_gemm_grouped_table_size(const lofgb_gemm_task* tasks, int ntasks);
int lofgb_gemm_grouped_prepare(const lofgb_gemm_task* tasks, int ntasks, void* workspace,
                               size_t workspace_bytes, int schedule, int grid, void* table,
                               size_t table_bytes, int64_t* num_tiles, int64_t* split_items);
int lofgb_gemm_grouped_launch(const void* device_table, int64_t num_tiles, int64_t split_items,
                              int grid, void* stream);
/* lofgb_gemm_grouped_launch for a table prepared with tile width `tile_n`
 * (64, 128 or 256 output columns; the LOFGB_GROUPED_TILE_* flag given to
 * prepare): launches the kernel compiled for that width alone. A table
 * prepared for another width is refused on the device (status word
 * LOFGB_ERR_UNSUPPORTED, nothing computed). */
int lofgb_gemm_grouped_launch_w(const void* device_table, int64_t num_tiles, int64_t split_items,
                                int grid, int tile_n, void* stream);

/* ---- grouped rounding: many tensors, each with its own format, one launch --
 * Batched form of lofgb_round_f32 (the reference rounds one tensor per call,
 * src/LoPy_bind.cpp:122-139). Two phases so that the launch can be captured
 * in a CUDA graph:
 *   1. lofgb_round_grouped_prepare() validates the tasks on the host and writes
 *      a task table of lofgb_round_grouped_table_size(ntasks) bytes into the
 *      caller's HOST buffer `table` (no device work, no allocation);
 *   2. the caller copies that table to device memory (any 256-byte aligned
 *      buffer) and calls lofgb_round_grouped_f32() with it as often as it likes
 *      — one kernel launch, nothing else, so it can be captured.
 * Each task rounds `n` floats from `in` to `out` exactly as lofgb_round_f32
 * would with the same arguments. */
typedef struct lofgb_round_task {
    const float* in;
    float* out;
    int64_t n;
    lofgb_format fmt;
    int32_t mode;
    int32_t stoch_len;
    float scale;
    int32_t reserved;
    uint64_t seed;
    uint64_t offset;
} lofgb_round_task;

size_t lofgb_round_grouped_table_size(int ntasks);
/* Returns LOFGB_OK and stores the number of work items in *num_items. */
int lofgb_round_grouped_prepare(const lofgb_round_task* tasks, int ntasks, void* table,
                                size_t table_bytes, int64_t* num_items);
/* The same with work items of `item_elems` elements (a power of two in
 * [2^10, 2^24]; the entry above uses 2^16). Smaller items balance uneven task
 * sizes better, larger ones cost fewer task look-ups; GroupedRound's
 * item="auto" picks one by timing. */
int lofgb_round_grouped_prepare_items(const lofgb_round_task* tasks, int ntasks, void* table,
                                      size_t table_bytes, int64_t item_elems, int64_t* num_items);
int lofgb_round_grouped_f32(const void* device_table, int ntasks, int64_t num_items,
                            void* stream);

/* ---- emulated-accumulation conv2d -----------------------------------------
 * Replaces LoF_conv2d (src/Lof_kernel.cu:156-227) → lo_float::Conv2d
 * (src/cutlass_conv.cuh:57-184), and the im2col + lof_gemm path of
 * LoF_Conv2d.forward (LoFloat/layers.py:684-713). Cross-correlation,
 * groups = 1, FP32. input N×C×H×W, weight K×C×R×S (OIHW), output N×K×P×Q
 * (NCHW) with P = (H + 2·pad_h − dil_h·(R−1) − 1)/stride_h + 1 and Q alike.
 *
 * Each output is one emulated-accumulator dot product over the reduction
 * index t ↔ (c, r, s), with the per-MAC leaf of lofgb_gemm_f32:
 *   acc_0 = +0, acc_{t+1} = RNE_m(rto_fma(w[k,c,r,s], x[n,c,h,w], acc_t)),
 *   y = alpha·acc,  h = p·stride_h − pad_h + r·dil_h, w = q·stride_w − pad_w + s·dil_w,
 * where x outside the input is +0 (zero padding). The order of t:
 *   LOFGB_CONV_CRS     c outer, then r, then s — the row order of
 *                      F.unfold's columns, so lof_gemm(w.view(K,−1),
 *                      unfold(x)[n]) (layers.py:690-705) gives the same bits;
 *   LOFGB_CONV_TILED8  channel tiles of 8 outer, then r, then s, then the 8
 *                      channels of the tile — CUTLASS's analytic implicit-GEMM
 *                      fprop iterators with a k-tile of 8 (Conv2d<> default
 *                      TbK = 8, src/cutlass_conv.cuh:57-65); channels past C in
 *                      the last tile are (0, 0) products, which leave the
 *                      accumulator unchanged.
 * mode must be LOFGB_RNE (the leaf ignores it). alpha: lof_conv2d passes
 * (float)(1.0 / (weight_scale·input_scale)) computed in double, or 1 when the
 * product is 0 (src/Lof_kernel.cu:203-206); the im2col path passes lof_gemm's
 * float alpha. variant LOFGB_GEMM_PLAIN: bit-exact, no workspace.
 * LOFGB_GEMM_TC: the chunked tensor-core form of lofgb_gemm_f32 over the same
 * t order, workspace of lofgb_conv2d_workspace_size() bytes (256-byte
 * aligned). No counterpart for TC in the reference. */
typedef struct lofgb_conv2d_shape {
    int32_t n, c, h, w;  /* input N×C×H×W */
    int32_t k, r, s;     /* weight K×C×R×S */
    int32_t pad_h, pad_w;
    int32_t stride_h, stride_w;
    int32_t dil_h, dil_w;
} lofgb_conv2d_shape;

enum lofgb_conv_order { LOFGB_CONV_CRS = 0, LOFGB_CONV_TILED8 = 1 };

/* Output spatial size; LOFGB_ERR_SIZE for an invalid shape or P, Q <= 0. */
int lofgb_conv2d_out_size(const lofgb_conv2d_shape* shape, int32_t* p, int32_t* q);
size_t lofgb_conv2d_workspace_size(const lofgb_conv2d_shape* shape, int order, int variant);
int lofgb_conv2d_f32(const float* input, const float* weight, float* output,
                     const lofgb_conv2d_shape* shape, int accum_mant_bits, int mode,
                     float alpha, int order, int variant, int chunk, void* workspace,
                     size_t workspace_bytes, void* stream);

/* ---- piecewise-linear SiLU -------------------------------------------------
 * Replaces pwl_silu / pwl_silu_kernel (src/LoPy_bind.cpp:228-272,
 * src/Lof_kernel.cu:240-264). `lut` (device, FP32) holds segments + 1 knots of
 * SiLU over [-R, R]; segments is a power of two in [2, 4096]. Per element, in
 * FP32: xc = clamp(x, -R, R); u = (xc + R)·(segments / (2R)); i = min((int)u,
 * segments − 1); y = fma(u − i, lut[i+1] − lut[i], lut[i]); y = x > 0 ? x : 0
 * when |x| > R. Half / double inputs are widened to FP32 and the result
 * narrowed back, as the reference's static_cast does. */
int lofgb_pwl_silu_f32(const float* in, float* out, int64_t n, const float* lut,
                       int segments, float R, void* stream);
int lofgb_pwl_silu_f64(const double* in, double* out, int64_t n, const float* lut,
                       int segments, float R, void* stream);
int lofgb_pwl_silu_f16(const uint16_t* in, uint16_t* out, int64_t n, const float* lut,
                       int segments, float R, void* stream);

/* ---- BatchNorm approximations ------------------------------------------------
 * Replace the torch compositions of L1BatchNorm, LinfBatchNorm, FISRBatchNorm
 * and PWLBatchNorm (LoFloat/layers.py:805-1047). x is [n, c, inner]
 * contiguous FP32 (NCHW: inner = H*W; (N, C): inner = 1); channel ch holds the
 * n rows of inner values at (nn*c + ch)*inner.
 *
 * lofgb_bn_stats_f32 computes per channel the FP32 mean and one deviation
 * statistic:
 *   LOFGB_BN_MEAN_ABS_DEV  mean |x - mean| (L1BatchNorm's mad),
 *   LOFGB_BN_MAX_ABS_DEV   max |x - mean| (LinfBatchNorm's maxdev; NaN if any),
 *   LOFGB_BN_VARIANCE      the biased variance (FISR / PWL),
 * with the centring x - mean done in FP32 with the FP32 mean, as the
 * reference does, and the sums in double. running_mean / running_dev (NULL:
 * skipped) are updated to r (1 - momentum) + momentum s in FP32. Needs
 * lofgb_bn_workspace_size(n, c, inner) bytes of 16-byte aligned workspace.
 *
 * lofgb_bn_apply_f32 writes, per element, in FP32 and the reference's order,
 *   LOFGB_BN_DIVIDE  y = ((x - mean) / (dev + eps)) * scale   (scale NULL: no multiply)
 *   LOFGB_BN_FISR    y = (x - mean) * fisr(dev + eps)
 *   LOFGB_BN_PWL     y = (x - mean) * pwl(dev + eps)
 * then y = y * weight + bias when weight is not NULL. fisr is the bit-trick
 * seed 0x5F3759DF - (bits >> 1) with two Newton steps y (1.5 - (v/2) y y);
 * pwl interpolates `lut` (segments + 1 knots of 1/sqrt over [1, 2]) at the
 * mantissa m in [1, 2) of v = m 2^e and multiplies by 2^-floor(e/2), and by
 * 1/sqrt(2) in FP32 for odd e. x == y is allowed. */
enum lofgb_bn_stat { LOFGB_BN_MEAN_ABS_DEV = 0, LOFGB_BN_MAX_ABS_DEV = 1, LOFGB_BN_VARIANCE = 2 };
enum lofgb_bn_norm { LOFGB_BN_DIVIDE = 0, LOFGB_BN_FISR = 1, LOFGB_BN_PWL = 2 };
size_t lofgb_bn_workspace_size(int64_t n, int64_t c, int64_t inner);
int lofgb_bn_stats_f32(const float* x, int64_t n, int64_t c, int64_t inner, int stat, float* mean,
                       float* dev, float* running_mean, float* running_dev, float momentum,
                       void* workspace, size_t workspace_bytes, void* stream);
int lofgb_bn_apply_f32(const float* x, float* y, int64_t n, int64_t c, int64_t inner,
                       const float* mean, const float* dev, float eps, int norm, const float* scale,
                       const float* weight, const float* bias, const float* lut, int segments,
                       void* stream);

/* ---- low-precision storage codec -------------------------------------------
 * Replaces LoF_encode_cuda / LoF_decode_cuda and their CPU twins
 * (src/lo_pack.hpp:109-532): FP32 values are converted to n-bit codes of a
 * runtime format (n in [1, 16]) and packed without waste, and back.
 *
 * Codes: convert_float_to_rep (src/lo_pack.hpp:109-287), the runtime twin of
 * the typed float -> Templated_Float conversion: NaN -> the quiet-NaN code;
 * ±inf -> the infinity code, or the largest finite code under SatFinite or
 * without infinities; negative inputs of unsigned formats -> 0 or NaN
 * (neg_to_nan); target-subnormal and normal ranges rounded with the
 * reference's RoundMantissa (its RoundUp / RoundDown see a positive-sign flag
 * of false, as there); overflow -> infinity under OvfInf with infinities,
 * else the largest finite code; -0 of a format whose sign-only code is NaN
 * encodes as +0. Stochastic modes draw element i's random lane from
 * (seed, offset + i) as the rounding entry points do. Values: convert_rep_to_float
 * (:293-320): infinity and NaN codes by the format's predicates, else the
 * exact value (in double) narrowed to float.
 *
 * Packing: a group of lcm(n, 8) bits (n <= 8) or lcm(n, 16) bits (n > 8)
 * holds lcm / n codes; element i of a group sits at bit slot*n, slot = i
 * (forward) or group_count - 1 - i (reverse), LSB-first within each byte;
 * groups follow one another; the last group is zero padded.
 *
 * The special-value predicates of the reference's checker functors
 * (P3109, IEEE-style, OCP, E8M0, trivial) all take one of these forms:
 *   IsInf(rep) <=> (rep | inf_or) == inf_match   (inf_match 0xFFFFFFFF: never)
 *   IsNaN(rep) <=> LOFGB_NAN_PATTERN: rep == qnan;
 *                  LOFGB_NAN_IEEE:    rep without its sign bit > the code with
 *                                     all exponent bits set and mantissa 0;
 *                  LOFGB_NAN_NONE:    never.                                  */
enum lofgb_sat_mode { LOFGB_OVF_INF = 0, LOFGB_SAT_FINITE = 1, LOFGB_SAT_PROPAGATE = 2 };
enum lofgb_nan_kind { LOFGB_NAN_PATTERN = 0, LOFGB_NAN_IEEE = 1, LOFGB_NAN_NONE = 2 };

typedef struct lofgb_codec_format {
    lofgb_format fmt;            /* bitwidth 1..16 */
    uint32_t inf_or, inf_match;  /* IsInf predicate, see above */
    uint32_t pos_inf, neg_inf;   /* IsInf.minPosInf(), minNegInf() */
    uint32_t qnan, snan;         /* IsNaN.qNanBitPattern(), sNanBitPattern() */
    uint8_t nan_kind;            /* IsNaN form, lofgb_nan_kind */
    uint8_t neg_to_nan;          /* unsigned formats: Unsigned_behavior NegtoNaN */
    uint8_t reserved[2];
} lofgb_codec_format;

/* Bytes that `count` codes of `bitwidth` bits occupy (whole groups). */
size_t lofgb_packed_size(int bitwidth, int64_t count);
int lofgb_encode_f32(uint8_t* dst, const float* src, int64_t count, const lofgb_codec_format* fmt,
                     int mode, int sat_mode, int stoch_len, int reverse, uint64_t seed,
                     uint64_t offset, void* stream);
int lofgb_decode_f32(float* dst, const uint8_t* src, int64_t count, const lofgb_codec_format* fmt,
                     int reverse, void* stream);

/* MX storage in one pass: MX block rounding (as lofgb_mx_round_f32, blocks of
 * 32) whose outputs are stored as codes instead of rescaled values. Per block
 * of 32 values: the scale s = virtual_round(amax * (1/pmn), scale format,
 * scale_mode) and the rounded quotients q_i = virtual_round(x_i / s, element
 * format, mode) (+0 when s is not positive); `codes` receives the q_i as
 * element codes and `scales` one code per block for s, both encoded as
 * lofgb_encode_f32 encodes (RNE, sat_mode; forward groups, so the element
 * codes are lofgb_packed_size(bits, count) bytes and the scale codes
 * ceil(count / 32) bytes). decode(code_i) * decode(scale code) is the MX
 * rounding's output wherever q_i is a value of the element format (every q_i
 * but the saturating pass-through of an overflowing quotient, which the
 * codec's sat_mode maps to the largest finite code or infinity). Element
 * codes of 4, 6 or 8 bits, 8-bit scale codes (E8M0). No counterpart in the
 * reference, which rounds MX in FP32 (src/mx_round.cuh:27-214) and packs
 * per-element formats only (src/lo_pack.hpp:474-500); this writes the two
 * together as MX storage, one HBM read and (bits + 1/4) / 8 bytes written per
 * value. */
int lofgb_mx_encode_f32(const float* src, uint8_t* codes, uint8_t* scales, int64_t count,
                        int block_size, const lofgb_codec_format* elem_fmt,
                        const lofgb_codec_format* scale_fmt, int mode, int scale_mode,
                        int sat_mode, int stoch_len, uint64_t seed, uint64_t offset, void* stream);

/* Values of MX storage in one pass: dst[i] = decode(element code i) *
 * decode(scale code of block i / 32) in FP32 (round to nearest), the
 * composition of lofgb_decode_f32 on both streams and the product. Blocks of
 * 32; element codes of 4, 6 or 8 bits (forward groups, as lofgb_mx_encode_f32
 * writes them), 8-bit scale codes. `codes` 4-byte aligned, `dst` 16-byte
 * aligned (LOFGB_ERR_SIZE otherwise), no overlap between output and inputs.
 * No counterpart in the reference. */
int lofgb_mx_decode_f32(const uint8_t* codes, const uint8_t* scales, float* dst, int64_t count,
                        int block_size, const lofgb_codec_format* elem_fmt,
                        const lofgb_codec_format* scale_fmt, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* LOFGB_H */
