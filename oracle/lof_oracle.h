/*
 * lof_oracle.h — TEST INFRASTRUCTURE ONLY.
 *
 * CPU restatement of the reference's rounding, MX and emulated-accumulation
 * GEMM arithmetic (SudhanvaKulkarni123/LoFloat). It is the checker for the
 * CUDA kernels in liblofgb.so and the CPU baseline timed by bench.py. Only
 * tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load it;
 * the product path never calls it.
 *
 * Pinning: tests/golden/ holds vectors produced by the reference's own scalar
 * functions (src/lo_float.h compiled from the reference sources by
 * oracle/ref_shim.cpp); tests/test_oracle_golden.py checks this oracle
 * against them bit for bit.
 */
#ifndef LOF_ORACLE_H
#define LOF_ORACLE_H
#include <stdint.h>
#include "../include/lofgb.h"

#ifdef __cplusplus
extern "C" {
#endif

/* SplitMix64 (Steele, Lea, Flood 2014) as a counter-based generator: the
 * idx-th output of a SplitMix64 stream whose state starts at `seed`. */
uint64_t orc_rng(uint64_t seed, uint64_t idx);

/* Per-element random words: element g reads lane g mod 2^lg (from the low
 * end) of output g >> lg, lanes 64 >> lg bits wide; lg is the log2 of the
 * lanes per output for (mode, stoch_len), the narrowest of 8/16/32/64 bits
 * covering what the mode reads (SR-A/B/C: len, SR-D: len + 1, Prob: 1,
 * True SR: 53). The MX block-scale stream keeps one output per block. */
int orc_rng_lanes_log2(int mode, int len);
uint64_t orc_rng_elem(uint64_t seed, uint64_t g, int lg);

/* Scalar cores. `rbits` is the random word for stochastic modes; `usamp` is
 * the uniform [0,1) sample used by True_StochasticRounding (pass a negative
 * value to derive it from rbits as (rbits >> 11) * 2^-53). */
float orc_vr_f32(float x, const lofgb_format* f, int mode, int len, uint64_t rbits,
                 double usamp);
double orc_vr_f64(double x, const lofgb_format* f, int mode, int len, uint64_t rbits,
                  double usamp);
uint16_t orc_vr_f16(uint16_t x, const lofgb_format* f, int mode, int len,
                    uint64_t rbits, double usamp);
float orc_vm_f32(float x, int mbits, int mode, int len, uint64_t rbits, double usamp);
double orc_vm_f64(double x, int mbits, int mode, int len, uint64_t rbits, double usamp);
uint16_t orc_vm_f16(uint16_t x, int mbits, int mode, int len, uint64_t rbits,
                    double usamp);

/* Array forms with the library's (seed, offset) RNG contract. Return 0 or a
 * LOFGB_ERR_* code (same validation as the library). nthreads <= 0 → all. */
int orc_round_f32(const float* in, float* out, int64_t n, const lofgb_format* f,
                  int mode, int len, float scale, uint64_t seed, uint64_t offset,
                  int nthreads);
int orc_round_f64(const double* in, double* out, int64_t n, const lofgb_format* f,
                  int mode, int len, double scale, uint64_t seed, uint64_t offset,
                  int nthreads);
int orc_round_f16(const uint16_t* in, uint16_t* out, int64_t n, const lofgb_format* f,
                  int mode, int len, float scale, uint64_t seed, uint64_t offset,
                  int nthreads);
int orc_round_mantissa_f32(const float* in, float* out, int64_t n, int mbits, int mode,
                           int len, float scale, uint64_t seed, uint64_t offset,
                           int nthreads);
int orc_round_mantissa_f64(const double* in, double* out, int64_t n, int mbits,
                           int mode, int len, double scale, uint64_t seed,
                           uint64_t offset, int nthreads);
int orc_round_mantissa_f16(const uint16_t* in, uint16_t* out, int64_t n, int mbits,
                           int mode, int len, float scale, uint64_t seed,
                           uint64_t offset, int nthreads);

/* Array forms with explicit per-element random words (golden pinning). */
int orc_round_f32_bits(const float* in, float* out, int64_t n, const lofgb_format* f,
                       int mode, int len, const uint64_t* rbits, const double* usamp);
int orc_round_f64_bits(const double* in, double* out, int64_t n, const lofgb_format* f,
                       int mode, int len, const uint64_t* rbits, const double* usamp);
int orc_round_f16_bits(const uint16_t* in, uint16_t* out, int64_t n,
                       const lofgb_format* f, int mode, int len, const uint64_t* rbits,
                       const double* usamp);
int orc_round_mantissa_f32_bits(const float* in, float* out, int64_t n, int mbits,
                                int mode, int len, const uint64_t* rbits,
                                const double* usamp);
int orc_round_mantissa_f64_bits(const double* in, double* out, int64_t n, int mbits,
                                int mode, int len, const uint64_t* rbits,
                                const double* usamp);
int orc_round_mantissa_f16_bits(const uint16_t* in, uint16_t* out, int64_t n, int mbits,
                                int mode, int len, const uint64_t* rbits,
                                const double* usamp);

/* MX block rounding. scale_formula 0 = GPU form amax*(1/pmn)
 * (src/mx_round.cuh:59), 1 = CPU form amax/pmn (src/LoPy_bind.cpp:208). */
int orc_mx_round_f32(const float* in, float* out, int64_t n, int block,
                     const lofgb_format* ef, const lofgb_format* sf, int mode,
                     int scale_mode, int len, uint64_t seed, uint64_t offset,
                     int scale_formula, int nthreads);

/* MX storage (lofgb_mx_encode_f32 semantics): the block scales and rounded
 * quotients of orc_mx_round_f32 encoded with the storage codec (RNE, `sat`). */
int orc_mx_encode_f32(const float* in, int64_t n, int block, const lofgb_codec_format* ef,
                      const lofgb_codec_format* sf, int mode, int scale_mode, int len, int sat,
                      uint64_t seed, uint64_t offset, uint8_t* codes, uint8_t* scales);

/* Emulated-accumulation GEMM, sequential k, device round-to-odd FMA.
 * Same layout arguments as lofgb_gemm_f32. */
int orc_gemm_f32(const float* A, int64_t lda, int trans_a, const float* B, int64_t ldb,
                 int trans_b, float* D, int64_t ldd, int M, int N, int K, int mbits,
                 float alpha, int nthreads);
/* Only rows [row0, row0+rows) of D are computed (bounded CPU samples). */
int orc_gemm_f32_rows(const float* A, int64_t lda, int trans_a, const float* B,
                      int64_t ldb, int trans_b, float* D, int64_t ldd, int M, int N,
                      int K, int mbits, float alpha, int row0, int rows, int nthreads);
/* The same with the accumulator rounded into a whole format after every MAC:
 * acc = vr(rto_fma(A[i,k], B[k,j], acc), fmt, RNE) (lofgb_gemm_accfmt_f32). */
int orc_gemm_accfmt_f32(const float* A, int64_t lda, int trans_a, const float* B, int64_t ldb,
                        int trans_b, float* D, int64_t ldd, int M, int N, int K,
                        const lofgb_format* fmt, float alpha, int nthreads);
/* The device leaf's round-to-odd FMA (src/cutlass_gemms.cuh:73-88). */
float orc_rto_fma(float a, float b, float c);
/* Chunked accumulation model of the tensor-core form with exact chunk sums:
 * acc = RNE_m(rto(acc + RN_fp32(sum of chunk products in FP64))). Used only to
 * sanity-check the error statistics on the CPU. */
int orc_gemm_chunked_f32(const float* A, int64_t lda, int trans_a, const float* B,
                         int64_t ldb, int trans_b, float* D, int64_t ldd, int M, int N,
                         int K, int mbits, int chunk, float alpha, int nthreads);

/* Emulated-accumulation conv2d (lofgb_conv2d_f32 semantics): NCHW input,
 * KCRS weight, NKPQ output, per-MAC leaf in the t order `order`
 * (LOFGB_CONV_CRS: the im2col + lof_gemm path, LoFloat/layers.py:684-705;
 * LOFGB_CONV_TILED8: CUTLASS analytic fprop with 8-channel k-tiles,
 * src/cutlass_conv.cuh:57-184). Only output columns (n, p, q) with flat index
 * in [col0, col0 + ncols) are written (ncols < 0: all). */
int orc_conv2d_f32(const float* x, const float* w, float* y, const lofgb_conv2d_shape* s,
                   int mbits, float alpha, int order, int64_t col0, int64_t ncols,
                   int nthreads);
/* Piecewise-linear SiLU on FP32 values (src/LoPy_bind.cpp:258-269). */
int orc_pwl_silu_f32(const float* in, float* out, int64_t n, const float* lut, int segments,
                     float R);

/* Storage codec (lofgb_encode_f32 / lofgb_decode_f32 semantics):
 * convert_float_to_rep / convert_rep_to_float and the group packing of
 * src/lo_pack.hpp:56-420. `rbits` / `usamp` feed the stochastic modes. */
uint32_t orc_codec_encode_rep(float x, const lofgb_codec_format* f, int mode, int sat_mode,
                              int len, uint64_t rbits, double usamp);
float orc_codec_decode_rep(uint32_t rep, const lofgb_codec_format* f);
int64_t orc_packed_size(int bitwidth, int64_t count);
int orc_encode_f32(uint8_t* dst, const float* src, int64_t count, const lofgb_codec_format* f,
                   int mode, int sat_mode, int len, int reverse, uint64_t seed, uint64_t offset);
int orc_decode_f32(float* dst, const uint8_t* src, int64_t count, const lofgb_codec_format* f,
                   int reverse);

int orc_validate_format(const lofgb_format* f, int src_mant_bits);
int orc_max_threads(void);

#ifdef __cplusplus
}
#endif
#endif
