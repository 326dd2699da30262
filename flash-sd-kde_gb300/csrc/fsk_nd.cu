// fsk_nd.cu - Gaussian KDE, empirical score accumulators and the debias
// shift for 1 <= d <= 64 features on the CUDA cores (no counterpart in the
// reference snapshot, which fixes d = 16: ND_FEATURES, globals.py:25; its
// paper's review answers describe padding to a multiple of 16).
//
// The math is that of the 16-D "fp32_ieee" kernels (fsk_simt.cu): squared
// distances from direct FP32 differences of the original coordinates (four
// FMA chains joined pairwise), exp2 of the double-float scaled exponent,
// compensated FP32 sums per split written as FP64 partials, fixed-order FP64
// reduction.  Rows are read with their own stride d and zero-padded to
// DP = 16 ceil(d / 16) in registers and shared memory, which changes no
// squared distance.  The weighted sums are accumulated centred on the FP64
// column means (added back in the reduction), FC features per launch slice.
// With two queries per thread (d <= 32) the KDE packs them into f32x2
// instructions, with the roundings of the scalar code.
#include "fsk_common.cuh"
#include "fsk_kernels.cuh"

namespace fsk {

namespace {
constexpr int ND_THREADS = 128;
constexpr int ND_TN = 32;   // data points per shared-memory tile
constexpr int ND_FC = 16;   // weighted-sum features per score slice (grid.z)

template <int DP>
__device__ __forceinline__ float sqdist_nd(const float (&a)[DP], const float* b) {
  float s0 = 0.f, s1 = 0.f, s2 = 0.f, s3 = 0.f;
#pragma unroll
  for (int k = 0; k < DP; k += 4) {
    const float4 v = *reinterpret_cast<const float4*>(b + k);
    const float d0 = a[k] - v.x, d1 = a[k + 1] - v.y, d2 = a[k + 2] - v.z, d3 = a[k + 3] - v.w;
    s0 = fmaf(d0, d0, s0);
    s1 = fmaf(d1, d1, s1);
    s2 = fmaf(d2, d2, s2);
    s3 = fmaf(d3, d3, s3);
  }
  return (s0 + s1) + (s2 + s3);
}

// rows [j0, j0 + valid) of an (., d) matrix into xs[ND_TN][DP], zero-padded
template <int DP>
__device__ __forceinline__ void stage_rows(float (*xs)[DP], const float* __restrict__ x, int64_t j0, int valid,
                                           int d) {
  for (int e = threadIdx.x; e < ND_TN * DP; e += ND_THREADS) {
    const int r = e / DP, k = e % DP;
    xs[r][k] = (r < valid && k < d) ? x[(j0 + r) * d + k] : 0.f;
  }
}

template <int DP, int QPT, bool LAPLACE>
__global__ void __launch_bounds__(ND_THREADS) kde_nd_kernel(const float* __restrict__ q, int64_t m,
                                                            const float* __restrict__ x, int64_t n, int d, float c2,
                                                            float c2_lo, float c1, float lap0, int64_t tps,
                                                            double* __restrict__ partials) {
  __shared__ __align__(16) float xs[ND_TN][DP];
  const int64_t q0 = (int64_t)blockIdx.x * (ND_THREADS * QPT);
  float qr[QPT][DP];
#pragma unroll
  for (int u = 0; u < QPT; ++u) {
    const int64_t qi = q0 + threadIdx.x + u * ND_THREADS;
#pragma unroll
    for (int k = 0; k < DP; ++k) qr[u][k] = (qi < m && k < d) ? q[qi * d + k] : 0.f;
  }
  Comp acc[QPT];
#pragma unroll
  for (int u = 0; u < QPT; ++u) acc[u] = Comp{0.f, 0.f};
  const int64_t n_tiles = (n + ND_TN - 1) / ND_TN;
  const int64_t t0 = (int64_t)blockIdx.y * tps;
  const int64_t t1 = min(n_tiles, t0 + tps);
  for (int64_t t = t0; t < t1; ++t) {
    const int64_t j0 = t * ND_TN;
    const int valid = (int)imin<int64_t>(ND_TN, n - j0);
    __syncthreads();
    stage_rows<DP>(xs, x, j0, valid, d);
    __syncthreads();
    if constexpr (QPT == 2) {
      // both queries in every f32x2 instruction: the roundings of the scalar
      // code below, half the issue slots
      float2 part = make_float2(0.f, 0.f);
      for (int r = 0; r < valid; ++r) {
        float2 s0 = make_float2(0.f, 0.f), s1 = s0, s2 = s0, s3 = s0;
#pragma unroll
        for (int k = 0; k < DP; k += 4) {
          const float4 v = *reinterpret_cast<const float4*>(&xs[r][k]);
          const float2 d0 = __fadd2_rn(make_float2(qr[0][k], qr[1][k]), make_float2(-v.x, -v.x));
          const float2 d1 = __fadd2_rn(make_float2(qr[0][k + 1], qr[1][k + 1]), make_float2(-v.y, -v.y));
          const float2 d2 = __fadd2_rn(make_float2(qr[0][k + 2], qr[1][k + 2]), make_float2(-v.z, -v.z));
          const float2 d3 = __fadd2_rn(make_float2(qr[0][k + 3], qr[1][k + 3]), make_float2(-v.w, -v.w));
          s0 = __ffma2_rn(d0, d0, s0);
          s1 = __ffma2_rn(d1, d1, s1);
          s2 = __ffma2_rn(d2, d2, s2);
          s3 = __ffma2_rn(d3, d3, s3);
        }
        const float2 dist = __fadd2_rn(__fadd2_rn(s0, s1), __fadd2_rn(s2, s3));
        float2 e = exp2_neg_scaled2(dist, c2, c2_lo);
        if (LAPLACE) e = __fmul2_rn(e, __ffma2_rn(make_float2(-c1, -c1), dist, make_float2(lap0, lap0)));
        part = __fadd2_rn(part, e);
      }
      acc[0].add(part.x);
      acc[1].add(part.y);
    } else {
      float part[QPT];
#pragma unroll
      for (int u = 0; u < QPT; ++u) part[u] = 0.f;
      for (int r = 0; r < valid; ++r) {
#pragma unroll
        for (int u = 0; u < QPT; ++u) {
          const float dist = sqdist_nd<DP>(qr[u], xs[r]);
          float e = exp2_neg_scaled(dist, c2, c2_lo);
          if (LAPLACE) e *= fmaf(-c1, dist, lap0);
          part[u] += e;
        }
      }
#pragma unroll
      for (int u = 0; u < QPT; ++u) acc[u].add(part[u]);
    }
  }
#pragma unroll
  for (int u = 0; u < QPT; ++u) {
    const int64_t qi = q0 + threadIdx.x + u * ND_THREADS;
    if (qi < m) partials[(int64_t)blockIdx.y * m + qi] = (double)acc[u].s + (double)acc[u].c;
  }
}

// One row i per thread; slice z accumulates features [16 z, 16 z + 16) of the
// centred weighted sum (slice 0 also the pdf sum).
template <int DP>
__global__ void __launch_bounds__(ND_THREADS) score_nd_kernel(const float* __restrict__ x, int64_t n, int d,
                                                              const float* __restrict__ mu, float c2, float c2_lo,
                                                              int64_t tps, double* __restrict__ ppdf,
                                                              double* __restrict__ pw) {
  __shared__ __align__(16) float xs[ND_TN][DP];
  __shared__ __align__(16) float xcs[ND_TN][ND_FC];
  const int f0 = blockIdx.z * ND_FC;
  const int64_t i = (int64_t)blockIdx.x * ND_THREADS + threadIdx.x;
  const bool valid_i = i < n;
  float xi[DP];
#pragma unroll
  for (int k = 0; k < DP; ++k) xi[k] = (valid_i && k < d) ? x[i * d + k] : 0.f;
  Comp pdf{0.f, 0.f};
  Comp w[ND_FC];
#pragma unroll
  for (int k = 0; k < ND_FC; ++k) w[k] = Comp{0.f, 0.f};
  const int64_t n_tiles = (n + ND_TN - 1) / ND_TN;
  const int64_t t0 = (int64_t)blockIdx.y * tps;
  const int64_t t1 = min(n_tiles, t0 + tps);
  for (int64_t t = t0; t < t1; ++t) {
    const int64_t j0 = t * ND_TN;
    const int valid = (int)imin<int64_t>(ND_TN, n - j0);
    __syncthreads();
    stage_rows<DP>(xs, x, j0, valid, d);
    for (int e = threadIdx.x; e < ND_TN * ND_FC; e += ND_THREADS) {
      const int r = e / ND_FC, k = e % ND_FC;
      xcs[r][k] = (r < valid && f0 + k < d) ? x[(j0 + r) * d + f0 + k] - mu[f0 + k] : 0.f;
    }
    __syncthreads();
    float ps = 0.f;
    float wp[ND_FC];
#pragma unroll
    for (int k = 0; k < ND_FC; ++k) wp[k] = 0.f;
    for (int r = 0; r < valid; ++r) {
      const float e = exp2_neg_scaled(sqdist_nd<DP>(xi, xs[r]), c2, c2_lo);
      ps += e;
#pragma unroll
      for (int k = 0; k < ND_FC; k += 4) {
        const float4 c = *reinterpret_cast<const float4*>(&xcs[r][k]);
        wp[k] = fmaf(e, c.x, wp[k]);
        wp[k + 1] = fmaf(e, c.y, wp[k + 1]);
        wp[k + 2] = fmaf(e, c.z, wp[k + 2]);
        wp[k + 3] = fmaf(e, c.w, wp[k + 3]);
      }
    }
    pdf.add(ps);
#pragma unroll
    for (int k = 0; k < ND_FC; ++k) w[k].add(wp[k]);
  }
  if (!valid_i) return;
  if (blockIdx.z == 0) ppdf[(int64_t)blockIdx.y * n + i] = (double)pdf.s + (double)pdf.c;
  double* wo = pw + ((int64_t)blockIdx.y * n + i) * d;
#pragma unroll
  for (int k = 0; k < ND_FC; ++k)
    if (f0 + k < d) wo[f0 + k] = (double)w[k].s + (double)w[k].c;
}

// FP64 column means, one block per feature, fixed-order tree: deterministic.
__global__ void mean_nd_kernel(const float* __restrict__ x, int64_t n, int d, double* __restrict__ mu64,
                               float* __restrict__ mu) {
  __shared__ double red[256];
  const int k = blockIdx.x;
  double s = 0.0;
  for (int64_t i = threadIdx.x; i < n; i += 256) s += (double)x[i * d + k];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    mu64[k] = red[0] / (double)n;
    mu[k] = (float)mu64[k];
  }
}

// pdf[i] = sum_s ppdf[s][i]; w[i][k] = sum_s pw[s][i][k] + mu_k pdf[i] (mu the
// FP32 centring vector the kernel subtracted, widened exactly)
__global__ void reduce_score_nd_kernel(const double* __restrict__ ppdf, const double* __restrict__ pw, int splits,
                                       int64_t n, int d, const float* __restrict__ mu, float* __restrict__ pdf,
                                       float* __restrict__ w) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n * d) return;
  const int64_t i = e / d;
  const int k = (int)(e % d);
  double p = 0.0, a = 0.0;
  for (int s = 0; s < splits; ++s) {
    p += ppdf[(int64_t)s * n + i];
    a += pw[(int64_t)s * n * d + e];
  }
  w[e] = (float)(a + (double)mu[k] * p);
  if (k == 0) pdf[i] = (float)p;
}

__global__ void debias_nd_kernel(const float* __restrict__ x, int64_t n, int d, const float* __restrict__ pdf,
                                 const float* __restrict__ w, double inv_h2, double eps, float* __restrict__ deb,
                                 float* __restrict__ score) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n * d) return;
  const int64_t i = e / d;
  const double xi = (double)x[e];
  const double mi = (double)w[e] / ((double)pdf[i] + eps);
  deb[e] = (float)(0.5 * (xi + mi));
  if (score) score[e] = (float)((mi - xi) * inv_h2);
}

int nd_splits(int64_t row_blocks, int64_t n) {
  const int64_t n_tiles = (n + ND_TN - 1) / ND_TN;
  const int64_t target = 4LL * sm_count() * 4;
  int64_t splits = (target + row_blocks - 1) / row_blocks;
  splits = imax<int64_t>(1, imin<int64_t>(splits, imax<int64_t>(1, n_tiles / 4)));
  splits = imin<int64_t>(splits, 65535);
  const int64_t tps = (n_tiles + splits - 1) / splits;
  return (int)((n_tiles + tps - 1) / tps);   // non-empty splits only
}

template <int DP, int QPT>
void launch_kde_nd_dp(const float* q, int64_t m, const float* x, int64_t n, int d, double h, bool laplace,
                      int splits, double* partials, cudaStream_t s) {
  const int64_t n_tiles = (n + ND_TN - 1) / ND_TN;
  const int64_t tps = (n_tiles + splits - 1) / splits;
  const dim3 grid((unsigned)((m + ND_THREADS * QPT - 1) / (ND_THREADS * QPT)), (unsigned)splits);
  const double c2d = FSK_LOG2E / (2.0 * h * h);
  const float c2 = (float)c2d, c2_lo = (float)(c2d - (double)c2);
  const float c1 = (float)(1.0 / (2.0 * h * h));
  const float lap0 = 1.0f + 0.5f * (float)d;
  if (laplace)
    kde_nd_kernel<DP, QPT, true><<<grid, ND_THREADS, 0, s>>>(q, m, x, n, d, c2, c2_lo, c1, lap0, tps, partials);
  else
    kde_nd_kernel<DP, QPT, false><<<grid, ND_THREADS, 0, s>>>(q, m, x, n, d, c2, c2_lo, c1, lap0, tps, partials);
}

template <int DP>
void launch_score_nd_dp(const float* x, int64_t n, int d, const float* mu, double h, int splits, double* ppdf,
                        double* pw, cudaStream_t s) {
  const int64_t n_tiles = (n + ND_TN - 1) / ND_TN;
  const int64_t tps = (n_tiles + splits - 1) / splits;
  const dim3 grid((unsigned)((n + ND_THREADS - 1) / ND_THREADS), (unsigned)splits, (unsigned)((d + ND_FC - 1) / ND_FC));
  const double c2d = FSK_LOG2E / (2.0 * h * h);
  const float c2 = (float)c2d, c2_lo = (float)(c2d - (double)c2);
  score_nd_kernel<DP><<<grid, ND_THREADS, 0, s>>>(x, n, d, mu, c2, c2_lo, tps, ppdf, pw);
}
}  // namespace

int kde_nd_splits(int64_t m, int64_t n, int d) {
  const int qpt = d <= 32 ? 2 : 1;
  return nd_splits((m + ND_THREADS * qpt - 1) / (ND_THREADS * qpt), n);
}

int score_nd_splits(int64_t n) { return nd_splits((n + ND_THREADS - 1) / ND_THREADS, n); }

void launch_kde_nd(const float* q, int64_t m, const float* x, int64_t n, int d, double h, bool laplace, int splits,
                   double* partials, cudaStream_t s) {
  TimerScope ts(K_KDE_ND, (double)m * (double)n, s);
  if (d <= 16) launch_kde_nd_dp<16, 2>(q, m, x, n, d, h, laplace, splits, partials, s);
  else if (d <= 32) launch_kde_nd_dp<32, 2>(q, m, x, n, d, h, laplace, splits, partials, s);
  else if (d <= 48) launch_kde_nd_dp<48, 1>(q, m, x, n, d, h, laplace, splits, partials, s);
  else launch_kde_nd_dp<64, 1>(q, m, x, n, d, h, laplace, splits, partials, s);
  count_launch();
}

void launch_score_nd(const float* x, int64_t n, int d, double h, int splits, double* mu64, float* mu, double* ppdf,
                     double* pw, float* pdf, float* w, cudaStream_t s) {
  mean_nd_kernel<<<d, 256, 0, s>>>(x, n, d, mu64, mu);
  count_launch();
  {
    TimerScope ts(K_SCORE_ND, (double)n * (double)n, s);
    if (d <= 16) launch_score_nd_dp<16>(x, n, d, mu, h, splits, ppdf, pw, s);
    else if (d <= 32) launch_score_nd_dp<32>(x, n, d, mu, h, splits, ppdf, pw, s);
    else if (d <= 48) launch_score_nd_dp<48>(x, n, d, mu, h, splits, ppdf, pw, s);
    else launch_score_nd_dp<64>(x, n, d, mu, h, splits, ppdf, pw, s);
    count_launch();
  }
  const int64_t total = n * d;
  reduce_score_nd_kernel<<<(unsigned)((total + 255) / 256), 256, 0, s>>>(ppdf, pw, splits, n, d, mu, pdf, w);
  count_launch();
}

void launch_debias_nd(const float* x, int64_t n, int d, const float* pdf, const float* w, double h, double eps,
                      float* deb, float* score, cudaStream_t s) {
  const int64_t total = n * d;
  debias_nd_kernel<<<(unsigned)((total + 255) / 256), 256, 0, s>>>(x, n, d, pdf, w, 1.0 / (h * h), eps, deb, score);
  count_launch();
}

}  // namespace fsk
