// fsk_kernels.cuh - host-side launcher declarations shared by the .cu files.
#pragma once
#include "fsk_common.cuh"

namespace fsk {

// ---- device error words (see fsk_common.cuh) --------------------------------
unsigned int kde16_take_device_error();    // fsk_tc_kde16.cu
unsigned int score16_take_device_error();  // fsk_tc_score16.cu
unsigned int mlp_tc_take_device_error();   // fsk_mlp_tc.cu
unsigned int simt_take_device_error();     // fsk_simt.cu      (bounds checks only)
unsigned int reduce_take_device_error();   // fsk_reduce.cu    (bounds checks only)
unsigned int logspace_take_device_error(); // fsk_logspace.cu  (bounds checks only)

// ---- fsk_api.cu -------------------------------------------------------------
// Argument checks of fsk_kde16 (pointers, sizes, bandwidth, flags and the
// FSK_OUT_LOG_EXACT constraints): FSK_OK or FSK_ERR_INVALID_ARGUMENT.
int validate_kde16_args(const float* q, int64_t m, const float* x, int64_t n, double h, int flags,
                        double out_eps, const float* out);

// ---- fsk_simt.cu ------------------------------------------------------------
void launch_kde16_simt(const float* q, int64_t m, const float* x, int64_t n, double h, bool laplace,
                       int splits, double* partials, double* atomic_acc, cudaStream_t s);
int simt_kde16_splits(int64_t m, int64_t n);
void launch_score16_simt(const float* x, int64_t n, const float* mu, double h, int splits,
                         double* ppdf, double* pw, cudaStream_t s);
int simt_score16_splits(int64_t n);
void launch_score16_sym_simt(const float* x, int64_t n, const float* mu, double h, double* acc_pdf,
                             double* acc_w, cudaStream_t s);
int64_t sym_simt_pairs(int64_t n);
int kde1d_splits(int64_t m, int64_t n);
void launch_kde1d(const float* q, int64_t m, const float* x, int64_t n, double h, bool laplace,
                  int splits, double* partials, double* atomic_acc, cudaStream_t s);
void launch_kde1d_score(const float* q, int64_t m, const float* x, int64_t n, double h, int splits,
                        double* p0, double* p1, cudaStream_t s);

// ---- fsk_reduce.cu ------------------------------------------------------------
// Column means of an (n, 16) FP32 matrix in FP64, deterministic; writes mu
// (rounded to FP32) and mu64.  `scratch` holds mean_scratch_doubles(n) doubles.
size_t mean_scratch_doubles(int64_t n);
void launch_mean16(const float* x, int64_t n, double* scratch, float* mu, double* mu64,
                   cudaStream_t s);
// out[i] = g(scale * sum_s partials[s*m + i]), g = identity or log(. + eps).
void launch_reduce_rows(const double* partials, int splits, int64_t m, double scale, double eps,
                        bool log_out, float* out, cudaStream_t s);
// pdf[i] = sum_s ppdf[s][i]; w[i][k] = sum_s pw[s][i][k] + mu64[k] * pdf[i]
// (pass splits = 1 with atomic accumulators).  w written at w[i*ws_row + k*ws_col].
// pdf partials [pdf_splits][n], weighted partials [w_splits][n][16] (centred);
// self_x: the data when the partials leave out the self pair, else nullptr.
// scratch: reduce_score_scratch_doubles(n) doubles.
size_t reduce_score_scratch_doubles(int64_t n);
void launch_reduce_score(const double* ppdf, const double* pw, int pdf_splits, int w_splits, int64_t n,
                         const double* mu64, const float* self_x, float* pdf, float* w, int64_t ws_row,
                         int64_t ws_col, double* scratch, cudaStream_t s);
void launch_debias16(const float* x, int64_t n, const float* pdf, const float* w, int64_t ws_row,
                     int64_t ws_col, double h, double eps, float* debiased, float* score,
                     cudaStream_t s);
// 1-D score epilogue from the two partial sums.
void launch_reduce_kde1d_score(const double* p0, const double* p1, int splits, int64_t m,
                               int64_t n, double h, float* score, float* pdf, float* deriv,
                               cudaStream_t s);
void launch_zero(double* p, int64_t count, cudaStream_t s);

// ---- fsk_logspace.cu ------------------------------------------------------------
// FSK_OUT_LOG_EXACT: log(scale * sum) per query from the split partials; the
// queries whose sum underflows are recomputed with a running-minimum shift.
#define FSK_LS_PARTS 8   // data parts per recomputed query (partial rows)
struct LogExactBufs {
  uint32_t* count;   // listed queries
  uint32_t* list;    // [m] query indices
  float* pd;         // [FSK_LS_PARTS][m] smallest squared distance per part
  double* ps;        // [FSK_LS_PARTS][m] shifted sums per part
};
void take_logexact(WsCarver& c, int64_t m, LogExactBufs* b);
void launch_reduce_logexact(const float* q, int64_t m, const float* x, int64_t n, double h, bool laplace,
                            const double* partials, int splits, double scale, const LogExactBufs& b, float* out,
                            cudaStream_t s);

// ---- fsk_nd.cu ------------------------------------------------------------------
// any 1 <= d <= FSK_ND_MAX features, rows with stride d (CUDA cores)
int kde_nd_splits(int64_t m, int64_t n, int d);
int score_nd_splits(int64_t n);
void launch_kde_nd(const float* q, int64_t m, const float* x, int64_t n, int d, double h, bool laplace, int splits,
                   double* partials, cudaStream_t s);
// mu64/mu: FSK_ND_MAX entries; ppdf [splits][n], pw [splits][n][d]; writes pdf (n) and w (n, d)
void launch_score_nd(const float* x, int64_t n, int d, double h, int splits, double* mu64, float* mu, double* ppdf,
                     double* pw, float* pdf, float* w, cudaStream_t s);
void launch_debias_nd(const float* x, int64_t n, int d, const float* pdf, const float* w, double h, double eps,
                      float* deb, float* score, cudaStream_t s);

// ---- fsk_silverman.cu -----------------------------------------------------------
size_t silverman_ws_bytes(int64_t n, int d);
int run_silverman(const float* x, int64_t n, int d, int rule, double* h_out, void* ws, size_t ws_bytes,
                  cudaStream_t s);
void launch_reduce_f32_partials(const float* partials, int64_t splits, int64_t count, float* out,
                                cudaStream_t s);

}  // namespace fsk
