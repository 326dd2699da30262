// fsk_logspace.cu - exact log-densities for queries whose Gaussian sum
// underflows (fsk_kde16 with FSK_OUT_LOG_EXACT).
//
// The estimator of the reference returns log(kde + 1e-12)
// (flash_sd_kde/estimator.py:114), and every FP32 path flushes terms below
// 2^-126, so a query farther than ~13 h from all data gets the floor (or
// -inf without it) instead of its log-density.  With FSK_OUT_LOG_EXACT:
//  1. the split partials of the main pass are reduced as usual; a query whose
//     FP64 sum is at least n 2^-100 gets log(scale * sum) (the terms flushed
//     to zero are below 2^-126 each, so together under 2^-26 of such a sum);
//  2. every other query goes on a list and is recomputed here by direct FP32
//     differences with a running-minimum shift: per data part the sum
//     S = sum_j 2^(-c2 (dist_j - dmin)) (x the Laplace factor) with dmin the
//     smallest squared distance seen so far (the sum is rescaled when it
//     drops), so the nearest term is 1 and nothing underflows;
//  3. parts are combined in FP64 and out = log(S) - dmin / (2 h^2) + log(scale).
// The result is deterministic: the list order varies from run to run, but
// each query's value comes from a fixed partition of the data.
#include "fsk_common.cuh"
#include "fsk_kernels.cuh"

namespace fsk {

namespace {
constexpr int LS_THREADS = 256;   // 8 warps: the data parts of one item split 8 ways
constexpr int LS_WARPS = LS_THREADS / 32;
constexpr int LS_QG = 64;         // queries per work item (2 per lane)
constexpr int LS_TN = 32;         // data points per warp tile

// queries flagged by the reduction: out = log(scale * sum) for the others
__global__ void reduce_rows_logexact_kernel(const double* __restrict__ partials, int splits, int64_t m,
                                            double scale, double tiny, float* __restrict__ out,
                                            uint32_t* __restrict__ count, uint32_t* __restrict__ list) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m) return;
  double s = 0.0;
  for (int k = 0; k < splits; ++k) s += partials[(int64_t)k * m + i];
  if (s >= tiny) {
    out[i] = (float)log(s * scale);
  } else {
    const uint32_t slot = atomicAdd(count, 1u);
    if (in_bounds(slot, m, 56)) list[slot] = (uint32_t)i;
  }
}

// data parts per query group: enough work items to fill the grid
__device__ __forceinline__ int ls_parts(int64_t groups, int grid) {
  const int64_t want = (grid + groups - 1) / groups;
  return (int)(want < 1 ? 1 : (want > FSK_LS_PARTS ? FSK_LS_PARTS : want));
}

// Running state of a lane's two queries (x and y halves), packed so that
// one f32x2 instruction serves both: the smallest squared distance (kept
// negated) and the compensated sum s + c of 2^(-c2 (dist - dmin)) (x the
// Laplace factor).
struct Shifted2 {
  float2 ndmin;
  float2 s, c;
};

__device__ __forceinline__ void rescale(float& ndmin, float& s, float& c, float dist, float c2) {
  const float f = ex2_approx(-c2 * (-ndmin - dist));   // 0 for the first point (dmin = inf)
  s *= f;
  c *= f;
  ndmin = -dist;
}

template <bool LAPLACE>
__device__ __forceinline__ void shifted_add2(Shifted2& a, float2 dist, float c2, float c1) {
  if (dist.x < -a.ndmin.x) rescale(a.ndmin.x, a.s.x, a.c.x, dist.x, c2);
  if (dist.y < -a.ndmin.y) rescale(a.ndmin.y, a.s.y, a.c.y, dist.y, c2);
  const float2 t = __fmul2_rn(__fadd2_rn(dist, a.ndmin), make_float2(-c2, -c2));
  float2 e = make_float2(ex2_approx(t.x), ex2_approx(t.y));
  if (LAPLACE)
    e = __fmul2_rn(e, __ffma2_rn(make_float2(-c1, -c1), dist, make_float2(1.0f + 0.5f * FSK_D, 1.0f + 0.5f * FSK_D)));
  // compensated add (TwoSum) of both lanes
  const float2 u = __fadd2_rn(a.s, e);
  const float2 z = __fadd2_rn(u, make_float2(-a.s.x, -a.s.y));
  const float2 r1 = __fadd2_rn(a.s, make_float2(z.x - u.x, z.y - u.y));
  const float2 r2 = __fadd2_rn(e, make_float2(-z.x, -z.y));
  a.c = __fadd2_rn(a.c, __fadd2_rn(r1, r2));
  a.s = u;
}

// Work item = (group of LS_QG listed queries, data part).  Warp w of the block
// takes the part's data tiles w, w + 8, ...; the block then merges its warps
// in FP64 and writes one (dmin, sum) per query and part.
template <bool LAPLACE>
__global__ void __launch_bounds__(LS_THREADS) logspace_kde16_kernel(
    const float* __restrict__ q, const float* __restrict__ x, int64_t n, const uint32_t* __restrict__ count_ptr,
    const uint32_t* __restrict__ list, float c2, float c1, double c2d, float* __restrict__ pd,
    double* __restrict__ ps, int64_t m) {
  __shared__ __align__(16) float4 xs[LS_WARPS][LS_TN][FSK_D / 4];
  __shared__ float wd[LS_WARPS][LS_QG];
  __shared__ double wsum[LS_WARPS][LS_QG];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t count = *count_ptr;
  if (count == 0) return;
  const int64_t groups = (count + LS_QG - 1) / LS_QG;
  const int parts = ls_parts(groups, (int)gridDim.x);
  const int64_t items = groups * parts;
  const int64_t n_tiles = (n + LS_TN - 1) / LS_TN;
  const int64_t tpp = (n_tiles + parts - 1) / parts;
  for (int64_t it = blockIdx.x; it < items; it += gridDim.x) {
    const int64_t grp = it / parts;
    const int part = (int)(it % parts);
    // the lane's two queries, feature by feature as (first, second) pairs
    float2 qq[FSK_D];
    {
      const int64_t s0 = grp * LS_QG + lane, s1 = s0 + 32;
      const int64_t q0 = s0 < count ? (int64_t)list[s0] : -1;
      const int64_t q1 = s1 < count ? (int64_t)list[s1] : -1;
      // scalar loads: the caller's rows need only 4-byte alignment
#pragma unroll
      for (int k = 0; k < FSK_D; ++k)
        qq[k] = make_float2(q0 >= 0 ? q[q0 * FSK_D + k] : 0.f, q1 >= 0 ? q[q1 * FSK_D + k] : 0.f);
    }
    Shifted2 acc;
    acc.ndmin = make_float2(-__int_as_float(0x7f800000), -__int_as_float(0x7f800000));
    acc.s = make_float2(0.f, 0.f);
    acc.c = make_float2(0.f, 0.f);
    const int64_t t0 = (int64_t)part * tpp;
    const int64_t t1 = t0 + tpp < n_tiles ? t0 + tpp : n_tiles;
    float* tile = reinterpret_cast<float*>(&xs[warp][0][0]);
    for (int64_t t = t0 + warp; t < t1; t += LS_WARPS) {
      const int valid = (int)(n - t * LS_TN < LS_TN ? n - t * LS_TN : LS_TN);
      // the tile's valid rows, negated, contiguous in x: coalesced scalar loads
      const float* src = x + t * LS_TN * FSK_D;
      for (int e = lane; e < valid * FSK_D; e += 32) tile[e] = -src[e];
      __syncwarp();
      for (int r = 0; r < valid; ++r) {
        // squared distances of both queries: four f32x2 FMA chains joined
        // pairwise (the summation order of sqdist16)
        float2 a0 = make_float2(0.f, 0.f), a1 = a0, a2 = a0, a3 = a0;
#pragma unroll
        for (int k = 0; k < FSK_D / 4; ++k) {
          const float4 v = xs[warp][r][k];
          const float2 d0 = __fadd2_rn(qq[4 * k], make_float2(v.x, v.x));
          const float2 d1 = __fadd2_rn(qq[4 * k + 1], make_float2(v.y, v.y));
          const float2 d2 = __fadd2_rn(qq[4 * k + 2], make_float2(v.z, v.z));
          const float2 d3 = __fadd2_rn(qq[4 * k + 3], make_float2(v.w, v.w));
          a0 = __ffma2_rn(d0, d0, a0);
          a1 = __ffma2_rn(d1, d1, a1);
          a2 = __ffma2_rn(d2, d2, a2);
          a3 = __ffma2_rn(d3, d3, a3);
        }
        shifted_add2<LAPLACE>(acc, __fadd2_rn(__fadd2_rn(a0, a1), __fadd2_rn(a2, a3)), c2, c1);
      }
      __syncwarp();
    }
    wd[warp][lane] = -acc.ndmin.x;
    wd[warp][32 + lane] = -acc.ndmin.y;
    wsum[warp][lane] = (double)acc.s.x + (double)acc.c.x;
    wsum[warp][32 + lane] = (double)acc.s.y + (double)acc.c.y;
    __syncthreads();
    if (threadIdx.x < LS_QG) {
      const int qs = threadIdx.x;
      float dm = wd[0][qs];
#pragma unroll
      for (int w = 1; w < LS_WARPS; ++w) dm = fminf(dm, wd[w][qs]);
      double sum = 0.0;
      if (dm < __int_as_float(0x7f800000)) {
#pragma unroll
        for (int w = 0; w < LS_WARPS; ++w)
          if (wd[w][qs] < __int_as_float(0x7f800000)) sum += wsum[w][qs] * exp2(-c2d * ((double)wd[w][qs] - (double)dm));
      }
      const int64_t slot = grp * LS_QG + qs;
      if (slot < count) {
        pd[(int64_t)part * m + slot] = dm;
        ps[(int64_t)part * m + slot] = sum;
      }
    }
    __syncthreads();
  }
}

// out[list[slot]] = log(S) - dmin / (2 h^2) + log(scale) over the parts
__global__ void logspace_combine_kernel(const uint32_t* __restrict__ count_ptr, const uint32_t* __restrict__ list,
                                        const float* __restrict__ pd, const double* __restrict__ ps, int64_t m,
                                        int ls_grid, double c2d, double c1d, double log_scale,
                                        float* __restrict__ out) {
  const int64_t count = *count_ptr;
  if (count == 0) return;
  const int parts = ls_parts((count + LS_QG - 1) / LS_QG, ls_grid);
  for (int64_t slot = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; slot < count;
       slot += (int64_t)gridDim.x * blockDim.x) {
    float dm = pd[slot];
    for (int p = 1; p < parts; ++p) dm = fminf(dm, pd[(int64_t)p * m + slot]);
    double sum = 0.0;
    for (int p = 0; p < parts; ++p) {
      const float d = pd[(int64_t)p * m + slot];
      if (d < __int_as_float(0x7f800000)) sum += ps[(int64_t)p * m + slot] * exp2(-c2d * ((double)d - (double)dm));
    }
    const int64_t q = list[slot];
    if (in_bounds(q, m, 55)) out[q] = (float)(log(sum) - c1d * (double)dm + log_scale);
  }
}
}  // namespace

void take_logexact(WsCarver& c, int64_t m, LogExactBufs* b) {
  LogExactBufs t;
  t.count = c.take<uint32_t>(1);
  t.list = c.take<uint32_t>((size_t)m);
  t.pd = c.take<float>((size_t)FSK_LS_PARTS * m);
  t.ps = c.take<double>((size_t)FSK_LS_PARTS * m);
  if (b) *b = t;
}

void launch_reduce_logexact(const float* q, int64_t m, const float* x, int64_t n, double h, bool laplace,
                            const double* partials, int splits, double scale, const LogExactBufs& b, float* out,
                            cudaStream_t s) {
  cudaMemsetAsync(b.count, 0, sizeof(uint32_t), s);
  const int T = 256;
  const double tiny = ldexp((double)n, -100);
  reduce_rows_logexact_kernel<<<(unsigned)((m + T - 1) / T), T, 0, s>>>(partials, splits, m, scale, tiny, out,
                                                                      b.count, b.list);
  count_launch();
  const double c2d = FSK_LOG2E / (2.0 * h * h);
  const double c1d = 1.0 / (2.0 * h * h);
  const int grid = 4 * sm_count();
  {
    TimerScope ts(K_KDE16_LOGSPACE, 0.0, s);
    if (laplace)
      logspace_kde16_kernel<true><<<grid, LS_THREADS, 0, s>>>(q, x, n, b.count, b.list, (float)c2d, (float)c1d, c2d,
                                                              b.pd, b.ps, m);
    else
      logspace_kde16_kernel<false><<<grid, LS_THREADS, 0, s>>>(q, x, n, b.count, b.list, (float)c2d, (float)c1d, c2d,
                                                               b.pd, b.ps, m);
    count_launch();
  }
  logspace_combine_kernel<<<2 * sm_count(), 256, 0, s>>>(b.count, b.list, b.pd, b.ps, m, grid, c2d, c1d, log(scale),
                                                          out);
  count_launch();
}

unsigned int logspace_take_device_error() { return take_unit_device_error(); }

}  // namespace fsk
