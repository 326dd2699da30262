/*
 * fsk.h - C ABI of the GB300 (sm_103a) Flash-SD-KDE hot path.
 *
 * Every entry point takes plain device pointers, element counts, a bandwidth,
 * option flags, a caller-owned device workspace and a CUDA stream (passed as
 * void*, i.e. a cudaStream_t / CUstream; NULL means the legacy default
 * stream).  Nothing here allocates device memory except where stated, nothing
 * synchronises the stream, and nothing falls back to the CPU.  Each call
 * returns an fsk_status code; FSK_ERR_INVALID_ARGUMENT corresponds to the
 * reference's ValueError, every other non-zero code to its RuntimeError.
 *
 * Layouts: 16-D point sets are row-major (n, 16) float32 with a 64-byte row
 * stride, contiguous, 16-byte aligned; 1-D sets are contiguous float32.
 *
 * Reference interfaces replaced (paths inside the Flash-SD-KDE project):
 *   fsk_kde16        kernels/kde_eval_16d_stream_splitk.py:263 (kde_eval_16d_splitk),
 *                    :373 (kde_eval_16d_atomic), kernels/flash_sd_kde/kde.py:242
 *                    (gaussian_kde_triton_nd) and the normalisation in
 *                    flash_sd_kde/kde.py:119-122
 *   fsk_empscore16   kernels/flash_sd_kde/empirical.py:134 (emp_score_16d_flash_sd_kde),
 *                    kernels/emp_score_16d_ordered_splitk.py:162,
 *                    kernels/emp_score_16d_symmetric_atomic.py:163, with the
 *                    partial reduction of kernels/reduce_partials.py:61-108
 *   fsk_debias16     flash_sd_kde/kde.py:319-322 and
 *                    kernels/flash_sd_kde/empirical.py:280-283
 *   fsk_kde1d        kernels/kde_eval_1d_splitk.py:141 (kde_eval_1d_splitk), :222
 *                    (kde_eval_1d_atomic), kernels/flash_sd_kde/kde.py:147
 *                    (gaussian_kde_triton) and flash_sd_kde/kde.py:93-94
 *   fsk_kde1d_score  kernels/flash_sd_kde/kde.py:348 (gaussian_kde_score_triton)
 *   fsk_silverman    flash_sd_kde/reference.py:171-184 (silverman_bandwidth_nd),
 *                    :24-36 (silverman_bandwidth), and the 1-D SD-KDE rule of
 *                    kernels/flash_sd_kde/empirical.py:328-333
 */
#ifndef FSK_H_
#define FSK_H_

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define FSK_API __attribute__((visibility("default")))
#else
#define FSK_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
enum fsk_status {
  FSK_OK = 0,
  FSK_ERR_INVALID_ARGUMENT = 1,   /* bad size, pointer, bandwidth or flag   */
  FSK_ERR_WORKSPACE_TOO_SMALL = 2,
  FSK_ERR_CUDA = 3,               /* a CUDA runtime call failed             */
  FSK_ERR_DEVICE_TIMEOUT = 4,     /* a bounded in-kernel wait gave up       */
  FSK_ERR_UNSUPPORTED_DEVICE = 5, /* not an sm_103 device                   */
  FSK_ERR_SCRATCH_LIMIT = 6,      /* request exceeds a fixed scratch limit  */
  FSK_ERR_DEVICE_BOUNDS = 7       /* bounds-check build only: a kernel index
                                     fell outside its buffer (write skipped) */
};

/* ---- option flags ------------------------------------------------------ */
/* precision_mode "fast_tf32" of the reference: tensor-core split-precision
 * distance products (centred, scaled coordinates as three fp16 parts
 * hi + mid + lo, seven products, FP32 accumulation, norms folded into bias
 * columns of the operands) and an exact FP32 direct-difference recompute of
 * the largest pair of every 32-pair chunk that carries more than 1/8 of its
 * query's running sum.  This is the default (value 0). */
#define FSK_PREC_TENSOR 0x0
/* precision_mode "fp32_ieee": every pair by FP32 direct differences on the
 * CUDA cores, no tensor cores. */
#define FSK_PREC_IEEE 0x1
/* fsk_kde16 only, no counterpart in the reference: the lowest rung of the
 * precision ladder - the cross product as one fp16 product per feature
 * (FP32 accumulation; the norms keep their three-part precision), no exact
 * near-pair recompute.  For precision studies; not an exact mode. */
#define FSK_PREC_FP16_SINGLE 0x40
/* fsk_kde16 tensor precision only: a quarter of the exps on the FP32 FMA pipe
 * (degree-5 Remez polynomial for 2^r with exponent-field insertion, about
 * the error of ex2.approx.f32) instead of the exp pipe. */
#define FSK_EXP_OFFLOAD 0x80
/* Laplace-corrected ("linearized") kernel phi * (1 + d/2 - dist/(2 h^2)),
 * kernels/kde_eval_16d_stream_splitk.py:75-76. */
#define FSK_LAPLACE 0x2
/* Write out = log(out_scale * sum + out_eps) instead of out_scale * sum. */
#define FSK_OUT_LOG 0x4
/* fsk_kde16 with FSK_OUT_LOG and out_eps = 0 (m < 2^32): out = log(out_scale
 * * sum) without underflow.  No counterpart in the reference, whose estimator
 * floors at log(density + 1e-12) (flash_sd_kde/estimator.py:114).  Queries
 * whose sum is below n 2^-100 (where the terms FP32 flushes to zero could
 * matter: farther than ~11 h from every data point) are recomputed by FP32
 * direct differences with a running-minimum shift,
 * sum_j exp(-(dist_j - dmin) / (2 h^2)), and get
 * log(that) - dmin / (2 h^2) + log(out_scale) in FP64. */
#define FSK_OUT_LOG_EXACT 0x20
/* Reduce splits with FP64 atomics instead of the ordered partial buffer
 * (kde_backend="atomic" / emp_score_backend="symmetric_atomic"). */
#define FSK_ATOMIC 0x8
/* fsk_empscore16: write weighted_sum as a (16, n) buffer, the layout of the
 * reference's flash backend (kernels/flash_sd_kde/empirical.py:180,223). */
#define FSK_WEIGHTED_FEATURE_MAJOR 0x10

/* empirical-score accumulation variants */
#define FSK_SCORE_ORDERED 0   /* deterministic split-K, fixed-order FP64 reduce */
#define FSK_SCORE_SYMMETRIC 1 /* triangle tiles, phi_ij = phi_ji, half the exps */

/* Silverman rules */
#define FSK_RULE_SILVERMAN 0  /* 0.9 * mean_k min(std_k, IQR_k/1.34) * n^(-1/(d+4)) */
#define FSK_RULE_SDKDE_1D 1   /* 0.4 * min(std, IQR/1.34) * n^(-1/9), 1-D only     */

/* ---- 16-D Gaussian KDE ------------------------------------------------- */
/* out[i] = out_scale * sum_j phi(q_i, x_j), phi = exp(-||q_i - x_j||^2 / (2 h^2))
 * (times the Laplace factor with FSK_LAPLACE); the sum is accumulated per
 * split with compensated FP32 and reduced across splits in FP64, and the
 * scale (and log) is applied in FP64.  m, n >= 1. */
FSK_API size_t fsk_kde16_workspace_bytes(int64_t m, int64_t n, int flags);
FSK_API int fsk_kde16(const float* queries, int64_t m, const float* data, int64_t n,
              double bandwidth, int flags, double out_scale, double out_eps,
              float* out, void* workspace, size_t workspace_bytes, void* stream);

/* ---- 16-D Gaussian KDE without a caller workspace ------------------------ */
/* No counterpart in the reference.  For callers that cannot allocate device
 * memory (C-ABI/FFI hosts without a device allocator of their own, processes
 * whose GPU memory another allocator owns, loops where cudaMalloc/cudaFree
 * would synchronise the device): same arguments and result as fsk_kde16,
 * with the scratch in a fixed device array of FSK_NOALLOC_SCRATCH_BYTES held
 * by every GPU that loads the library.  Requests needing more
 * (fsk_kde16_workspace_bytes) fail with FSK_ERR_SCRATCH_LIMIT.  All calls
 * share the array: calls whose GPU work overlaps race and must be
 * serialised.  Argument errors are reported as by fsk_kde16
 * (FSK_ERR_INVALID_ARGUMENT) before the size check.  Every call looks up
 * the array's address in the current CUDA context (so context switches and
 * cudaDeviceReset are safe); the first call in a context loads the
 * library's device code, so make it before any stream capture in that
 * context.  Allocates nothing. */
#define FSK_NOALLOC_SCRATCH_BYTES (32u << 20)
FSK_API int fsk_kde16_noalloc(const float* queries, int64_t m, const float* data, int64_t n,
                              double bandwidth, int flags, double out_scale, double out_eps,
                              float* out, void* stream);

/* ---- any feature count 1 <= d <= FSK_ND_MAX (CUDA cores) ---------------- */
/* No counterpart in the reference snapshot, which fixes d = 16
 * (ND_FEATURES, globals.py:25; its paper's review answers describe padding
 * to a multiple of 16).  Rows (n, d) / (m, d) row-major FP32 with stride d;
 * the "fp32_ieee" arithmetic of the 16-D CUDA-core kernels: FP32 direct
 * differences, compensated FP32 sums per split, fixed-order FP64 reduction.
 * fsk_kde_nd: out as fsk_kde16 (flags FSK_LAPLACE with the factor
 * 1 + d/2 - dist/(2 h^2), FSK_OUT_LOG; FSK_PREC_IEEE and FSK_ATOMIC are
 * accepted and change nothing).  fsk_empscore_nd: pdf_sum (n) and
 * weighted_sum (n, d) row-major, self pair included.  fsk_debias_nd: the
 * shift of fsk_debias16 for (n, d) rows; score may be NULL. */
#define FSK_ND_MAX 64
FSK_API size_t fsk_kde_nd_workspace_bytes(int64_t m, int64_t n, int d, int flags);
FSK_API int fsk_kde_nd(const float* queries, int64_t m, const float* data, int64_t n, int d,
                       double bandwidth, int flags, double out_scale, double out_eps, float* out,
                       void* workspace, size_t workspace_bytes, void* stream);
FSK_API size_t fsk_empscore_nd_workspace_bytes(int64_t n, int d);
FSK_API int fsk_empscore_nd(const float* data, int64_t n, int d, double bandwidth, float* pdf_sum,
                            float* weighted_sum, void* workspace, size_t workspace_bytes, void* stream);
FSK_API int fsk_debias_nd(const float* data, int64_t n, int d, const float* pdf_sum,
                          const float* weighted_sum, double bandwidth, double eps, float* debiased,
                          float* score, void* stream);

/* ---- 16-D empirical-score accumulators --------------------------------- */
/* pdf_sum[i] = sum_j phi_ij, weighted_sum[i,:] = sum_j phi_ij x_j, the
 * self-pair included (flash_sd_kde/reference.py:263-284). */
FSK_API size_t fsk_empscore16_workspace_bytes(int64_t n, int variant, int flags);
FSK_API int fsk_empscore16(const float* data, int64_t n, double bandwidth, int variant,
                   int flags, float* pdf_sum, float* weighted_sum,
                   void* workspace, size_t workspace_bytes, void* stream);

/* ---- SD-KDE in one call: score -> debias -> KDE ----------------------- */
/* The pipeline the reference runs as empirical_sd_kde_triton_nd followed by
 * gaussian_kde_triton_nd (experiments/runtime/benchmark_triton_kde.py:344-388,
 * kernels/flash_sd_kde/empirical.py:226, kernels/flash_sd_kde/kde.py:242) or
 * emp_sd_kde_fit_transform followed by kde_eval (flash_sd_kde/kde.py:258, :49),
 * enqueued by one call on one workspace: the ordered empirical score of the
 * data, the debias shift (eps on the unnormalised pdf_sum, as fsk_debias16)
 * and the 16-D KDE of the debiased set at the queries (out as fsk_kde16).
 * flags: FSK_PREC_IEEE (both stages), FSK_ATOMIC, FSK_OUT_LOG,
 * FSK_OUT_LOG_EXACT (KDE stage).  debiased (n, 16) may be NULL.  No
 * allocation and no synchronisation, so the call can be captured into a
 * CUDA graph and replayed as one launch. */
FSK_API size_t fsk_sdkde16_workspace_bytes(int64_t n, int64_t m, int flags);
FSK_API int fsk_sdkde16(const float* data, int64_t n, const float* queries, int64_t m, double bandwidth,
                        int flags, double eps, double out_scale, double out_eps, float* debiased, float* out,
                        void* workspace, size_t workspace_bytes, void* stream);

/* ---- one-step SD-KDE debias shift -------------------------------------- */
/* score = (W / (pdf + eps) - x) / h^2, debiased = x + h^2/2 * score, in FP64.
 * weighted_sum element (i, k) is read at weighted_sum[i*w_row_stride + k*w_col_stride].
 * score may be NULL. */
FSK_API int fsk_debias16(const float* data, int64_t n, const float* pdf_sum,
                 const float* weighted_sum, int64_t w_row_stride,
                 int64_t w_col_stride, double bandwidth, double eps,
                 float* debiased, float* score, void* stream);

/* ---- 1-D Gaussian KDE and KDE score ------------------------------------ */
FSK_API size_t fsk_kde1d_workspace_bytes(int64_t m, int64_t n, int flags);
FSK_API int fsk_kde1d(const float* queries, int64_t m, const float* data, int64_t n,
              double bandwidth, int flags, double out_scale, double out_eps,
              float* out, void* workspace, size_t workspace_bytes, void* stream);
/* pdf[i] = sum_j phi(z)/(n h sqrt(2 pi)), deriv[i] = sum_j -z phi(z)/(n h^2 sqrt(2 pi)),
 * score[i] = deriv[i] / (pdf[i] + 1e-12), z = (q_i - x_j)/h.  Any output may be NULL. */
FSK_API int fsk_kde1d_score(const float* queries, int64_t m, const float* data, int64_t n,
                    double bandwidth, float* score, float* pdf, float* deriv,
                    void* workspace, size_t workspace_bytes, void* stream);

/* ---- bandwidth rules ----------------------------------------------------- */
/* Writes the bandwidth (FP64) to the device scalar h_out.  Per-axis mean,
 * standard deviation and the 25th/75th percentiles (linear interpolation,
 * as numpy.percentile) are computed on the GPU in FP64 / exact selection. */
FSK_API size_t fsk_silverman_workspace_bytes(int64_t n, int d);
FSK_API int fsk_silverman(const float* data, int64_t n, int d, int rule, double* h_out,
                  void* workspace, size_t workspace_bytes, void* stream);

/* ---- split reduction ------------------------------------------------------ */
/* out[i] = sum_s partials[s * count + i] over a (splits, count) FP32 buffer,
 * accumulated in FP64 in split order.  Replaces reduce_pdf_partials and
 * reduce_weighted_partials (kernels/reduce_partials.py:61-108), which sum in
 * FP32. */
FSK_API int fsk_reduce_partials(const float* partials, int64_t splits, int64_t count,
                                float* out, void* stream);

/* ---- learned surrogate (no counterpart in the reference) ------------------ */
/* An ensemble of `members` (1..8) MLPs 16 -> 256 -> 256 -> 256 -> 1 with SiLU,
 * bf16 weights and activations, FP32 accumulation:
 *   a0 = bf16((x - in_mean) * in_inv_std)
 *   a_l = bf16(silu(bf16(W_l) a_{l-1} + b_l)), l = 1..3;  y = bf16(w4) . a3 + b4
 * FP32 parameters of a member, contiguous (FSK_MLP_PARAMS floats):
 *   W1[256][16] b1[256] W2[256][256] b2[256] W3[256][256] b3[256] w4[256] b4
 * Members are stored back to back.  in_mean / in_inv_std are 16-float device
 * arrays.  Training: fsk_mlp_fwd keeps the activations in the workspace for
 * fsk_mlp_bwd (same members, batch and workspace), which overwrites `grads`
 * with d(sum dy*y)/d(params), straight-through for the bf16 roundings. */
#define FSK_MLP_IN 16
#define FSK_MLP_HIDDEN 256
#define FSK_MLP_PARAMS 136193
FSK_API size_t fsk_mlp_train_workspace_bytes(int members, int64_t batch);
FSK_API int fsk_mlp_fwd(const float* params, int members, const float* x, int64_t batch,
                        const float* in_mean, const float* in_inv_std, float* y /* [members][batch] */,
                        void* workspace, size_t workspace_bytes, void* stream);
FSK_API int fsk_mlp_bwd(const float* params, int members, int64_t batch, const float* dy /* [members][batch] */,
                        float* grads, void* workspace, size_t workspace_bytes, void* stream);
/* dy = 2 (y - target) / batch per member; *loss (device FP64, may be NULL) +=
 * sum over members of mean squared error. */
FSK_API int fsk_mlp_mse(const float* y, const float* target, int64_t batch, int members, float* dy,
                        double* loss, void* stream);
/* AdamW step `step` (from 1) over `count` parameters, bias-corrected. */
FSK_API int fsk_mlp_adam(float* params, const float* grads, float* m, float* v, int64_t count, float lr,
                         float beta1, float beta2, float eps, float weight_decay, int step, void* stream);
/* Inference image (bf16 weights in the tensor-core kernel's layouts, the input
 * normalisation and an output affine y' = y * out_scale + out_shift). */
FSK_API size_t fsk_mlp_packed_bytes(int members);
FSK_API int fsk_mlp_pack(const float* params, int members, const float* in_mean, const float* in_inv_std,
                         float out_scale, float out_shift, void* packed, void* stream);
/* Tensor-core inference: y[member][b] for all members (x 16-byte aligned). */
FSK_API int fsk_mlp_infer(const void* packed, int members, const float* x, int64_t batch, float* y,
                          void* stream);
/* Ensemble statistics and serving gate per query b (outputs may be NULL):
 *   r2 = |(x_b - in_mean) * in_inv_std|^2 when x is given, else 0
 *   mean[b] = average_m y[m][b] + base_a + base_b * r2
 *   spread[b] = max_m y[m][b] - min_m y[m][b]
 *   served[b] = spread <= spread_tol && r2 <= r2_max */
FSK_API int fsk_mlp_combine(const float* y, int members, int64_t batch, const float* x, const float* in_mean,
                            const float* in_inv_std, float base_a, float base_b, float spread_tol, float r2_max,
                            float* mean, float* spread, uint8_t* served, void* stream);

/* ---- diagnostics --------------------------------------------------------- */
/* Synchronises the stream, reads and clears the library's device error word.
 * Returns FSK_OK, FSK_ERR_DEVICE_TIMEOUT or FSK_ERR_CUDA. */
FSK_API int fsk_device_status(void* stream);
FSK_API const char* fsk_strerror(int status);
FSK_API int fsk_version(void);
/* Number of this library's kernel launches since load (monotonic counter). */
FSK_API int64_t fsk_launch_count(void);

/* Tensor-core layout probe, no counterpart in the reference: two K=16
 * tcgen05.mma steps (fp16 inputs, FP32 accumulate, M=128, N=64) of
 * a (128,32) by b (64,32)^T over the 64-byte-row operand images the KDE
 * kernel uses; inputs are FP32 rounded to fp16, d is (128,64) FP32
 * row-major.  The tests compare it with a host dot product. */
FSK_API int fsk_diag_mma_probe(const float* a, const float* b, float* d, void* stream);
/* Tensor-memory operand probe, no counterpart in the reference: four K=16
 * tcgen05.mma steps (fp16, FP32 accumulate, M=128, N=16) with the A operand
 * a (128,64) stored to tensor memory (two fp16 per column) and b (16,64) in
 * the score kernel's transposed-feature image layout; d is (128,16) FP32
 * row-major, a . b^T of the fp16-rounded inputs. */
FSK_API int fsk_diag_mma_ts_probe(const float* a, const float* b, float* d, void* stream);
/* Tensor-memory copy probe, no counterpart in the reference: a (128,32) is
 * rounded to fp16 into the query operand image layout in shared memory,
 * copied to tensor memory with two tcgen05.cp 128x256b and read back; out is
 * (128,16) 32-bit words, word c of row r holding elements 2c (low half) and
 * 2c+1 (high half) of row r. */
FSK_API int fsk_diag_tmem_cp_probe(const float* a, uint32_t* out, void* stream);
/* Failure-path probe, no counterpart in the reference: a kernel waits on an
 * mbarrier nothing arrives on; its bounded wait gives up after about 2 s,
 * writes 0 to *out (device int) and records FSK_ERR_DEVICE_TIMEOUT, which the
 * next fsk_device_status returns (and clears). */
FSK_API int fsk_diag_wait_timeout_probe(int* out, void* stream);
/* Roofline inputs, no counterpart in the reference: sustained device rates
 * (operations / s) of ex2.approx.f32 (SFU), fma.rn.f32 and fma.rn.f32x2
 * (counted as two FMAs), written to the host array rates_out[3].  Allocates
 * a small device buffer and synchronises the stream (diagnostics only). */
FSK_API int fsk_diag_pipe_rates(double* rates_out, void* stream);

/* ---- measurement hooks (no counterpart in the reference) ------------------ */
/* Kernel ids: 1 tensor-core 16-D KDE, 2 CUDA-core 16-D KDE, 3 CUDA-core
 * ordered score, 4 CUDA-core symmetric score, 5 1-D KDE, 6 1-D KDE score,
 * 7 tensor-core score, 9 surrogate inference (unit: one query x member). */
/* When enabled, each hot-path kernel launch is bracketed by CUDA events on
 * its own stream. */
FSK_API void fsk_timer_enable(int on);
/* Per kernel id since the last call: launches, device ms and pair
 * evaluations, into host arrays of `cap` rows; returns the row count (or a
 * negated status).  Waits for the recorded events. */
FSK_API int fsk_timer_collect(int* ids, int64_t* launches, double* ms, double* work, int cap);

#ifdef __cplusplus
}
#endif
#endif /* FSK_H_ */
