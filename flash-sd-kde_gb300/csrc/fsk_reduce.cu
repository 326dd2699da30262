// fsk_reduce.cu - O(n) FP64 kernels: column means for centering, the fixed-
// order cross-split reduction of partial sums with the FP64 normalisation
// (and optional log), the empirical-score reduction, and the SD-KDE debias
// shift.  The split reduction replaces kernels/reduce_partials.py:6-58 (which
// sums splits in FP32); normalisation follows flash_sd_kde/kde.py:93-94,
// :119-122; the debias shift follows flash_sd_kde/kde.py:319-322.
#include "fsk_kernels.cuh"

namespace fsk {

namespace {
constexpr int MEAN_THREADS = 256;
constexpr int MEAN_MAX_BLOCKS = 512;
}  // namespace

size_t mean_scratch_doubles(int64_t n) {
  (void)n;
  return (size_t)MEAN_MAX_BLOCKS * FSK_D;
}

__global__ void __launch_bounds__(MEAN_THREADS) mean16_partial_kernel(const float* __restrict__ x,
                                                                      int64_t n, double* __restrict__ part) {
  // thread layout: 16 features x 16 row lanes
  const int k = threadIdx.x % FSK_D;
  const int lane = threadIdx.x / FSK_D;
  double acc = 0.0;
  for (int64_t r = (int64_t)blockIdx.x * (MEAN_THREADS / FSK_D) + lane; r < n;
       r += (int64_t)gridDim.x * (MEAN_THREADS / FSK_D))
    acc += (double)x[r * FSK_D + k];
  __shared__ double sh[MEAN_THREADS];
  sh[threadIdx.x] = acc;
  __syncthreads();
  if (threadIdx.x < FSK_D) {
    double s = 0.0;
    for (int l = 0; l < MEAN_THREADS / FSK_D; ++l) s += sh[l * FSK_D + threadIdx.x];
    part[(int64_t)blockIdx.x * FSK_D + threadIdx.x] = s;
  }
}

// One block of MEAN_THREADS: thread t sums the partials b = t/16, t/16 + 16, ...
// of feature t%16, then each feature's 16 strided sums are added in a fixed
// order (deterministic).
__global__ void __launch_bounds__(MEAN_THREADS) mean16_final_kernel(const double* __restrict__ part, int blocks,
                                                                    int64_t n, float* __restrict__ mu,
                                                                    double* __restrict__ mu64) {
  const int k = threadIdx.x % FSK_D;
  const int l = threadIdx.x / FSK_D;
  constexpr int L = MEAN_THREADS / FSK_D;
  double s = 0.0;
  for (int b = l; b < blocks; b += L) s += part[b * FSK_D + k];
  __shared__ double sh[MEAN_THREADS];
  sh[threadIdx.x] = s;
  __syncthreads();
  if (threadIdx.x < FSK_D) {
    double t = 0.0;
    for (int j = 0; j < L; ++j) t += sh[j * FSK_D + threadIdx.x];
    const float mf = (float)(t / (double)n);
    mu[threadIdx.x] = mf;
    if (mu64) mu64[threadIdx.x] = (double)mf;  // the shift actually applied (exactly representable)
  }
}

void launch_mean16(const float* x, int64_t n, double* scratch, float* mu, double* mu64,
                   cudaStream_t s) {
  int blocks = (int)imin<int64_t>(MEAN_MAX_BLOCKS, (n + 255) / 256);
  blocks = imax(blocks, 1);
  mean16_partial_kernel<<<blocks, MEAN_THREADS, 0, s>>>(x, n, scratch);
  count_launch();
  mean16_final_kernel<<<1, MEAN_THREADS, 0, s>>>(scratch, blocks, n, mu, mu64);
  count_launch();
}

__global__ void reduce_rows_kernel(const double* __restrict__ partials, int splits, int64_t m,
                                   double scale, double eps, int log_out, float* __restrict__ out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m) return;
  double s = 0.0;
  for (int k = 0; k < splits; ++k) s += partials[(int64_t)k * m + i];
  double v = s * scale;
  if (log_out) v = log(v + eps);
  out[i] = (float)v;
}

void launch_reduce_rows(const double* partials, int splits, int64_t m, double scale, double eps,
                        bool log_out, float* out, cudaStream_t s) {
  const int T = 256;
  reduce_rows_kernel<<<(unsigned)((m + T - 1) / T), T, 0, s>>>(partials, splits, m, scale, eps,
                                                              log_out ? 1 : 0, out);
  count_launch();
}

// pdf = sum of pdf partials (thread per row; the FP64 sum of the partials,
// without the self pair, is kept for the weighted pass), then weighted =
// sum of centred partials + mu * pdf (thread per element, coalesced over the
// [split][row][16] partials).  self_x != nullptr: the partials leave the self
// pair out; it is added here exactly (phi_ii = 1, weight x_i).
__global__ void reduce_score_pdf_kernel(const double* __restrict__ ppdf, int pdf_splits, int64_t n,
                                        int add_self, float* __restrict__ pdf, double* __restrict__ p_other) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double p = 0.0;
  for (int s = 0; s < pdf_splits; ++s) p += ppdf[(int64_t)s * n + i];
  p_other[i] = p;
  pdf[i] = (float)(add_self ? p + 1.0 : p);
}

__global__ void reduce_score_w_kernel(const double* __restrict__ pw, int w_splits, int64_t n,
                                      const double* __restrict__ mu64, const double* __restrict__ p_other,
                                      const float* __restrict__ self_x, float* __restrict__ w, int64_t ws_row,
                                      int64_t ws_col) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n * FSK_D) return;
  const int64_t i = e / FSK_D;
  const int k = (int)(e % FSK_D);
  double a = 0.0;
  for (int s = 0; s < w_splits; ++s) a += pw[(int64_t)s * n * FSK_D + e];
  const double po = p_other[i];
  const double v = self_x ? a + mu64[k] * po + (double)self_x[e] : a + mu64[k] * po;
  const int64_t o = i * ws_row + k * ws_col;
  if (in_bounds(o, n * FSK_D, 53)) w[o] = (float)v;
}

size_t reduce_score_scratch_doubles(int64_t n) { return (size_t)n; }

void launch_reduce_score(const double* ppdf, const double* pw, int pdf_splits, int w_splits, int64_t n,
                         const double* mu64, const float* self_x, float* pdf, float* w, int64_t ws_row,
                         int64_t ws_col, double* scratch, cudaStream_t s) {
  const int T = 256;
  reduce_score_pdf_kernel<<<(unsigned)((n + T - 1) / T), T, 0, s>>>(ppdf, pdf_splits, n, self_x != nullptr, pdf,
                                                                   scratch);
  count_launch();
  reduce_score_w_kernel<<<(unsigned)((n * FSK_D + T - 1) / T), T, 0, s>>>(pw, w_splits, n, mu64, scratch, self_x,
                                                                         w, ws_row, ws_col);
  count_launch();
}

// Thread per row, FP64: one reciprocal of (pdf + eps) per row; then per
// feature score = (w / (pdf + eps) - x) / h^2 and x + h^2/2 * score, which is
// (x + w / (pdf + eps)) / 2.
__global__ void debias16_kernel(const float* __restrict__ x, int64_t n, const float* __restrict__ pdf,
                                const float* __restrict__ w, int64_t ws_row, int64_t ws_col, double inv_h2,
                                double eps, float* __restrict__ deb, float* __restrict__ score) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double inv = 1.0 / ((double)pdf[i] + eps);
#pragma unroll
  for (int k = 0; k < FSK_D; ++k) {
    const double xi = (double)x[i * FSK_D + k];
    const int64_t o = i * ws_row + k * ws_col;
    const double m = in_bounds(o, n * FSK_D, 54) ? (double)w[o] * inv : 0.0;
    deb[i * FSK_D + k] = (float)(0.5 * (xi + m));
    if (score) score[i * FSK_D + k] = (float)((m - xi) * inv_h2);
  }
}

void launch_debias16(const float* x, int64_t n, const float* pdf, const float* w, int64_t ws_row,
                     int64_t ws_col, double h, double eps, float* debiased, float* score,
                     cudaStream_t s) {
  const int T = 128;
  debias16_kernel<<<(unsigned)((n + T - 1) / T), T, 0, s>>>(x, n, pdf, w, ws_row, ws_col, 1.0 / (h * h), eps,
                                                           debiased, score);
  count_launch();
}

__global__ void reduce_kde1d_score_kernel(const double* __restrict__ p0, const double* __restrict__ p1,
                                          int splits, int64_t m, double inv_norm, double h,
                                          float* __restrict__ score, float* __restrict__ pdf,
                                          float* __restrict__ deriv) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m) return;
  double s0 = 0.0, s1 = 0.0;
  for (int s = 0; s < splits; ++s) {
    s0 += p0[(int64_t)s * m + i];
    s1 += p1[(int64_t)s * m + i];
  }
  // p1 holds sum (x - q) phi = -h * sum z phi
  const double pd = s0 * inv_norm;
  const double dv = s1 * inv_norm / (h * h);
  const float pdf_f = (float)pd, dv_f = (float)dv;
  if (pdf) pdf[i] = pdf_f;
  if (deriv) deriv[i] = dv_f;
  if (score) score[i] = dv_f / (pdf_f + 1e-12f);
}

void launch_reduce_kde1d_score(const double* p0, const double* p1, int splits, int64_t m,
                               int64_t n, double h, float* score, float* pdf, float* deriv,
                               cudaStream_t s) {
  const int T = 256;
  const double inv_norm = 1.0 / (sqrt(2.0 * 3.14159265358979323846) * (double)n * h);
  reduce_kde1d_score_kernel<<<(unsigned)((m + T - 1) / T), T, 0, s>>>(p0, p1, splits, m, inv_norm, h,
                                                                     score, pdf, deriv);
  count_launch();
}

__global__ void reduce_f32_partials_kernel(const float* __restrict__ partials, int64_t splits,
                                           int64_t count, float* __restrict__ out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  double s = 0.0;
  for (int64_t k = 0; k < splits; ++k) s += (double)partials[k * count + i];
  out[i] = (float)s;
}

void launch_reduce_f32_partials(const float* partials, int64_t splits, int64_t count, float* out,
                                cudaStream_t s) {
  const int T = 256;
  reduce_f32_partials_kernel<<<(unsigned)((count + T - 1) / T), T, 0, s>>>(partials, splits, count, out);
  count_launch();
}

__global__ void zero_kernel(double* p, int64_t count) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count;
       i += (int64_t)gridDim.x * blockDim.x)
    p[i] = 0.0;
}

void launch_zero(double* p, int64_t count, cudaStream_t s) {
  if (count <= 0) return;
  int blocks = (int)imin<int64_t>(4096, (count + 255) / 256);
  zero_kernel<<<blocks, 256, 0, s>>>(p, count);
  count_launch();
}

unsigned int reduce_take_device_error() { return take_unit_device_error(); }

}  // namespace fsk
