// fsk_silverman.cu - Silverman bandwidth rules on the GPU.
//
// h = 0.9 * mean_k min(std_k, IQR_k / 1.34) * n^(-1/(d+4))   (FSK_RULE_SILVERMAN)
//   flash_sd_kde/reference.py:171-184 (d-D) and :24-36 (1-D, same formula, d=1)
// h = 0.4 * min(std, IQR / 1.34) * n^(-1/9)                   (FSK_RULE_SDKDE_1D)
//   kernels/flash_sd_kde/empirical.py:328-333
//
// std is the population standard deviation (ddof=0) in FP64.  The 25th/75th
// percentiles use numpy's default linear interpolation between the order
// statistics floor(p(n-1)) and floor(p(n-1))+1, which are found exactly by a
// 4-pass, 8-bit radix selection on order-preserving integer keys.
#include "fsk_kernels.cuh"

namespace fsk {

namespace {
constexpr int SV_MAXD = 64;
constexpr int SV_TARGETS = 4;        // ranks: lo25, hi25, lo75, hi75
constexpr int SV_THREADS = 256;
constexpr int SV_BLOCKS = 256;

struct SvState {
  uint32_t prefix[SV_MAXD][SV_TARGETS];
  int64_t rank[SV_MAXD][SV_TARGETS];   // rank still to find inside the prefix bucket
  double mean[SV_MAXD];
  double m2[SV_MAXD];
};
}  // namespace

__device__ __forceinline__ uint32_t sortable_key(float f) {
  uint32_t u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float key_to_float(uint32_t k) {
  uint32_t u = (k & 0x80000000u) ? (k & 0x7FFFFFFFu) : ~k;
  return __uint_as_float(u);
}

// per-block FP64 column sums (pass 0) or centred sums of squares (pass 1)
__global__ void __launch_bounds__(SV_THREADS) sv_moment_kernel(const float* __restrict__ x, int64_t n, int d,
                                                               int pass, const SvState* __restrict__ st,
                                                               double* __restrict__ part) {
  __shared__ double sh[SV_MAXD];
  for (int k = threadIdx.x; k < d; k += blockDim.x) sh[k] = 0.0;
  __syncthreads();
  // thread t owns column t % d of rows (t / d), (t / d) + rows_per_iter, ...
  const int rows_per_iter = blockDim.x / d;
  const int k = threadIdx.x % d;
  const int lane_row = threadIdx.x / d;
  if (lane_row < rows_per_iter) {
    const double mk = pass == 1 ? st->mean[k] : 0.0;
    double acc = 0.0;
    for (int64_t r = (int64_t)blockIdx.x * rows_per_iter + lane_row; r < n;
         r += (int64_t)gridDim.x * rows_per_iter) {
      double v = (double)x[r * d + k];
      if (pass == 1) {
        v -= mk;
        v *= v;
      }
      acc += v;
    }
    atomicAdd(&sh[k], acc);
  }
  __syncthreads();
  for (int k = threadIdx.x; k < d; k += blockDim.x) part[(int64_t)blockIdx.x * d + k] = sh[k];
}

__global__ void sv_moment_final(const double* __restrict__ part, int blocks, int64_t n, int d, int pass,
                                SvState* __restrict__ st) {
  const int k = threadIdx.x;
  if (k >= d) return;
  double s = 0.0;
  for (int b = 0; b < blocks; ++b) s += part[(int64_t)b * d + k];
  if (pass == 0) st->mean[k] = s / (double)n;
  else st->m2[k] = s / (double)n;
}

__global__ void sv_init_kernel(SvState* st, int64_t n, int d) {
  const int k = threadIdx.x;
  if (k >= d) return;
  const double v25 = 0.25 * (double)(n - 1), v75 = 0.75 * (double)(n - 1);
  const int64_t i25 = (int64_t)floor(v25), i75 = (int64_t)floor(v75);
  const int64_t r[SV_TARGETS] = {i25, min(i25 + 1, n - 1), i75, min(i75 + 1, n - 1)};
  for (int t = 0; t < SV_TARGETS; ++t) {
    st->prefix[k][t] = 0u;
    st->rank[k][t] = r[t];
  }
}

// histogram of digit `pass` (bits [24-8*pass, 32-8*pass)) for elements whose
// higher digits match each target's prefix.  hist: [d][SV_TARGETS][256] uint32.
__global__ void __launch_bounds__(SV_THREADS) sv_hist_kernel(const float* __restrict__ x, int64_t n, int d,
                                                             int pass, const SvState* __restrict__ st,
                                                             unsigned int* __restrict__ hist) {
  extern __shared__ unsigned int sh_hist[];  // d * SV_TARGETS * 256
  const int nb = d * SV_TARGETS * 256;
  for (int i = threadIdx.x; i < nb; i += blockDim.x) sh_hist[i] = 0u;
  __syncthreads();
  const int shift = 24 - 8 * pass;
  const int64_t total = n * d;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int k = (int)(e % d);
    const uint32_t key = sortable_key(x[e]);
    const uint32_t digit = (key >> shift) & 255u;
#pragma unroll
    for (int t = 0; t < SV_TARGETS; ++t) {
      const bool match = pass == 0 ? true : ((key >> (shift + 8)) == st->prefix[k][t]);
      if (match) atomicAdd(&sh_hist[(k * SV_TARGETS + t) * 256 + digit], 1u);
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < nb; i += blockDim.x)
    if (sh_hist[i]) atomicAdd(&hist[i], sh_hist[i]);
}

__global__ void sv_select_kernel(int d, SvState* __restrict__ st, unsigned int* __restrict__ hist) {
  const int idx = threadIdx.x;  // one thread per (k, t)
  if (idx >= d * SV_TARGETS) return;
  const int k = idx / SV_TARGETS, t = idx % SV_TARGETS;
  unsigned int* h = hist + (int64_t)idx * 256;
  int64_t r = st->rank[k][t];
  int b = 0;
  for (; b < 256; ++b) {
    if (r < (int64_t)h[b]) break;
    r -= h[b];
  }
  if (b > 255) b = 255;  // unreachable for consistent counts
  st->prefix[k][t] = (st->prefix[k][t] << 8) | (uint32_t)b;
  st->rank[k][t] = r;
  for (int i = 0; i < 256; ++i) h[i] = 0u;  // ready for the next pass
}

__global__ void sv_finish_kernel(int64_t n, int d, int rule, const SvState* __restrict__ st,
                                 double* __restrict__ h_out) {
  if (threadIdx.x != 0) return;
  const double v25 = 0.25 * (double)(n - 1), v75 = 0.75 * (double)(n - 1);
  const double g25 = v25 - floor(v25), g75 = v75 - floor(v75);
  auto lerp = [](double a, double b, double t) {
    const double diff = b - a;
    return t >= 0.5 ? b - diff * (1.0 - t) : a + diff * t;
  };
  double sig_sum = 0.0;
  for (int k = 0; k < d; ++k) {
    const double a25 = key_to_float(st->prefix[k][0]), b25 = key_to_float(st->prefix[k][1]);
    const double a75 = key_to_float(st->prefix[k][2]), b75 = key_to_float(st->prefix[k][3]);
    const double iqr = lerp(a75, b75, g75) - lerp(a25, b25, g25);
    const double sd = sqrt(st->m2[k]);
    sig_sum += fmin(sd, iqr / 1.34);
  }
  double sigma = sig_sum / (double)d;
  double h;
  if (rule == FSK_RULE_SDKDE_1D) {
    h = 0.4 * sigma * pow((double)n, -1.0 / 9.0);
  } else {
    if (sigma <= 0.0) sigma = 1.0;
    h = 0.9 * sigma * pow((double)n, -1.0 / (double)(d + 4));
  }
  *h_out = h;
}

size_t silverman_ws_bytes(int64_t n, int d) {
  (void)n;
  size_t b = align_up(sizeof(SvState), 256);
  b += align_up((size_t)SV_BLOCKS * SV_MAXD * sizeof(double), 256);
  b += align_up((size_t)d * SV_TARGETS * 256 * sizeof(unsigned int), 256);
  return b;
}

int run_silverman(const float* x, int64_t n, int d, int rule, double* h_out, void* ws, size_t ws_bytes,
                  cudaStream_t s) {
  WsCarver c(ws, ws_bytes);
  SvState* st = c.take<SvState>(1);
  double* part = c.take<double>((size_t)SV_BLOCKS * SV_MAXD);
  unsigned int* hist = c.take<unsigned int>((size_t)d * SV_TARGETS * 256);
  if (!c.fits()) return FSK_ERR_WORKSPACE_TOO_SMALL;
  if (d < 1 || d > SV_MAXD) return FSK_ERR_INVALID_ARGUMENT;
  const int blocks = (int)imax<int64_t>(1, imin<int64_t>(SV_BLOCKS, (n * d + SV_THREADS - 1) / SV_THREADS));
  cudaError_t e = cudaMemsetAsync(hist, 0, (size_t)d * SV_TARGETS * 256 * sizeof(unsigned int), s);
  if (e != cudaSuccess) return cuda_status(e);
  sv_init_kernel<<<1, SV_MAXD, 0, s>>>(st, n, d);
  count_launch();
  for (int pass = 0; pass < 2; ++pass) {
    sv_moment_kernel<<<blocks, SV_THREADS, 0, s>>>(x, n, d, pass, st, part);
    count_launch();
    sv_moment_final<<<1, SV_MAXD, 0, s>>>(part, blocks, n, d, pass, st);
    count_launch();
  }
  const size_t hsm = (size_t)d * SV_TARGETS * 256 * sizeof(unsigned int);
  if (hsm > 48 * 1024) {
    e = cudaFuncSetAttribute(sv_hist_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)hsm);
    if (e != cudaSuccess) return cuda_status(e);
  }
  for (int pass = 0; pass < 4; ++pass) {
    sv_hist_kernel<<<blocks, SV_THREADS, hsm, s>>>(x, n, d, pass, st, hist);
    count_launch();
    sv_select_kernel<<<1, SV_MAXD * SV_TARGETS, 0, s>>>(d, st, hist);
    count_launch();
  }
  sv_finish_kernel<<<1, 32, 0, s>>>(n, d, rule, st, h_out);
  count_launch();
  return cuda_status(cudaGetLastError());
}

}  // namespace fsk
