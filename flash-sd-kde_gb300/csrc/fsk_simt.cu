// fsk_simt.cu - CUDA-core kernels of the Flash-SD-KDE hot path.
//
// * 16-D KDE and empirical score in the "fp32_ieee" precision mode: every
//   pair distance is formed from direct FP32 differences sum_k (q_k - x_k)^2
//   (no cancellation), exp on the SFU (ex2.approx), and per-split compensated
//   FP32 sums written as FP64 partials [split][row].  Follows the math of
//   flash_sd_kde/reference.py:216-235 (KDE) and :263-284 (score); the split-K
//   decomposition follows kernels/kde_eval_16d_stream_splitk.py:14-81 and
//   kernels/emp_score_16d_ordered_splitk.py:14-92.
// * Symmetric score (phi_ij = phi_ji): upper-triangle tile pairs, row and
//   column contributions scattered with FP64 atomics, after
//   kernels/emp_score_16d_symmetric_atomic.py:10-103.
// * 1-D KDE and 1-D KDE score (pdf + derivative sums), after
//   kernels/kde_eval_1d_splitk.py:13-52 and kernels/flash_sd_kde/kde.py:59-100.
//
// Distances come from direct FP32 differences of the original coordinates
// (four FMA chains joined pairwise) and the exponent product dist * log2(e)/(2h^2)
// is carried in double-float (exp2_neg_scaled), so no step needs centring.
#include "fsk_common.cuh"

#include "fsk_kernels.cuh"

namespace fsk {

// ---------------------------------------------------------------------------
// 16-D KDE, direct differences.  Block: 128 threads x QPT queries each.
// grid.x = query blocks, grid.y = splits; each split covers `tiles_per_split`
// data tiles of TN points.  A thread's two queries share every f32x2
// instruction (difference, square-accumulate, exponent, sum): the roundings
// of the scalar code, half the issue slots (8.5e11 vs 7.9e11 pairs/s at
// 2^20 x 2^20, bitwise the same results).
// ---------------------------------------------------------------------------
namespace {
constexpr int SIMT_TN = 64;
constexpr int SIMT_THREADS = 128;
constexpr int SIMT_QPT = 2;
}  // namespace

template <bool LAPLACE>
__global__ void __launch_bounds__(SIMT_THREADS) kde16_simt_kernel(
    const float* __restrict__ q, int64_t m, const float* __restrict__ x, int64_t n,
    float c2, float c2_lo, float c1, int64_t tiles_per_split,
    double* __restrict__ partials, double* __restrict__ atomic_acc) {
  __shared__ __align__(16) float xs[SIMT_TN][FSK_D];

  const int64_t q0 = (int64_t)blockIdx.x * (SIMT_THREADS * SIMT_QPT);
  float qr[SIMT_QPT][FSK_D];
  bool qvalid[SIMT_QPT];
#pragma unroll
  for (int u = 0; u < SIMT_QPT; ++u) {
    int64_t qi = q0 + threadIdx.x + u * SIMT_THREADS;
    qvalid[u] = qi < m;
#pragma unroll
    for (int k = 0; k < FSK_D; ++k) qr[u][k] = qvalid[u] ? q[qi * FSK_D + k] : 0.f;
  }
  Comp acc[SIMT_QPT];
#pragma unroll
  for (int u = 0; u < SIMT_QPT; ++u) acc[u] = Comp{0.f, 0.f};
  float2 q2[FSK_D];
#pragma unroll
  for (int k = 0; k < FSK_D; ++k) q2[k] = make_float2(qr[0][k], qr[1][k]);

  const int64_t n_tiles = (n + SIMT_TN - 1) / SIMT_TN;
  const int64_t t_begin = (int64_t)blockIdx.y * tiles_per_split;
  const int64_t t_end = min(n_tiles, t_begin + tiles_per_split);
  for (int64_t t = t_begin; t < t_end; ++t) {
    const int64_t j0 = t * SIMT_TN;
    const int valid = (int)imin<int64_t>(SIMT_TN, n - j0);
    __syncthreads();
    for (int e = threadIdx.x; e < SIMT_TN * FSK_D; e += SIMT_THREADS) {
      int r = e / FSK_D, k = e % FSK_D;
      xs[r][k] = r < valid ? x[(j0 + r) * FSK_D + k] : 0.f;
    }
    __syncthreads();
    static_assert(SIMT_QPT == 2, "two queries per f32x2 lane pair");
    float2 part = make_float2(0.f, 0.f);
    for (int r = 0; r < valid; ++r) {
      float2 s0 = make_float2(0.f, 0.f), s1 = s0, s2 = s0, s3 = s0;
#pragma unroll
      for (int k = 0; k < FSK_D; k += 4) {
        const float4 v = *reinterpret_cast<const float4*>(&xs[r][k]);
        // q - x for both queries, four features in four chains (the order of sqdist16)
        const float2 d0 = __fadd2_rn(q2[k], make_float2(-v.x, -v.x));
        const float2 d1 = __fadd2_rn(q2[k + 1], make_float2(-v.y, -v.y));
        const float2 d2 = __fadd2_rn(q2[k + 2], make_float2(-v.z, -v.z));
        const float2 d3 = __fadd2_rn(q2[k + 3], make_float2(-v.w, -v.w));
        s0 = __ffma2_rn(d0, d0, s0);
        s1 = __ffma2_rn(d1, d1, s1);
        s2 = __ffma2_rn(d2, d2, s2);
        s3 = __ffma2_rn(d3, d3, s3);
      }
      const float2 dist = __fadd2_rn(__fadd2_rn(s0, s1), __fadd2_rn(s2, s3));
      float2 e = exp2_neg_scaled2(dist, c2, c2_lo);
      if (LAPLACE) e = __fmul2_rn(e, __ffma2_rn(make_float2(-c1, -c1), dist, make_float2(1.0f + 0.5f * FSK_D, 1.0f + 0.5f * FSK_D)));
      part = __fadd2_rn(part, e);
    }
    acc[0].add(part.x);
    acc[1].add(part.y);
  }
#pragma unroll
  for (int u = 0; u < SIMT_QPT; ++u) {
    int64_t qi = q0 + threadIdx.x + u * SIMT_THREADS;
    if (!qvalid[u]) continue;
    double v = (double)acc[u].s + (double)acc[u].c;
    if (atomic_acc) {
      if (in_bounds(qi, m, 44)) atomicAdd(&atomic_acc[qi], v);
    } else {
      const int64_t idx = (int64_t)blockIdx.y * m + qi;
      if (in_bounds(idx, (int64_t)gridDim.y * m, 45)) partials[idx] = v;
    }
  }
}

void launch_kde16_simt(const float* q, int64_t m, const float* x, int64_t n, double h, bool laplace,
                       int splits, double* partials, double* atomic_acc, cudaStream_t s) {
  const int64_t n_tiles = (n + SIMT_TN - 1) / SIMT_TN;
  const int64_t tps = (n_tiles + splits - 1) / splits;
  const int qblocks = (int)((m + SIMT_THREADS * SIMT_QPT - 1) / (SIMT_THREADS * SIMT_QPT));
  dim3 grid(qblocks, (unsigned)((n_tiles + tps - 1) / tps));
  const double c2d = FSK_LOG2E / (2.0 * h * h);
  const float c2 = (float)c2d, c2_lo = (float)(c2d - (double)c2);
  const float c1 = (float)(1.0 / (2.0 * h * h));
  TimerScope ts(K_KDE16_SIMT, (double)m * (double)n, s);
  if (laplace)
    kde16_simt_kernel<true><<<grid, SIMT_THREADS, 0, s>>>(q, m, x, n, c2, c2_lo, c1, tps, partials, atomic_acc);
  else
    kde16_simt_kernel<false><<<grid, SIMT_THREADS, 0, s>>>(q, m, x, n, c2, c2_lo, c1, tps, partials, atomic_acc);
  count_launch();
}

// Effective split count: the launchers give each split ceil(n_tiles/splits)
// tiles, so the number of non-empty splits is ceil(n_tiles / tps); the
// partial buffers and reductions use exactly this count.
static int effective_splits(int64_t n_tiles, int64_t splits) {
  splits = imax<int64_t>(1, imin<int64_t>(splits, n_tiles));
  const int64_t tps = (n_tiles + splits - 1) / splits;
  return (int)((n_tiles + tps - 1) / tps);
}

int simt_kde16_splits(int64_t m, int64_t n) {
  const int64_t n_tiles = (n + SIMT_TN - 1) / SIMT_TN;
  const int64_t qblocks = (m + SIMT_THREADS * SIMT_QPT - 1) / (SIMT_THREADS * SIMT_QPT);
  const int64_t target = 4LL * sm_count() * 4;  // ~4 waves of 4 resident blocks/SM
  int64_t splits = (target + qblocks - 1) / qblocks;
  splits = imax<int64_t>(1, imin<int64_t>(splits, n_tiles / 4 > 0 ? n_tiles / 4 : 1));
  return effective_splits(n_tiles, imin<int64_t>(splits, 65535));
}

// ---------------------------------------------------------------------------
// 16-D empirical score, ordered split-K.  One row i per thread.  Writes
// partial pdf [split][n] and partial weighted [split][n][16].  Distances use
// the original coordinates; the weighted sums accumulate x_j - mu (centred,
// so the compensated FP32 sums carry the spread, not the offset) and the
// mean is added back in FP64 by the reduction.  Two data points share every
// f32x2 instruction (the tile kept as point pairs in shared memory; even and
// odd points in separate chains, added per tile): 2616 -> 2155 ms at 2^20.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(SIMT_THREADS) score16_simt_kernel(
    const float* __restrict__ x, int64_t n, const float* __restrict__ mu, float c2, float c2_lo,
    int64_t tiles_per_split, double* __restrict__ ppdf, double* __restrict__ pw) {
  // the data tile as point pairs: xs2[rp][k] = -(x_{2rp}, x_{2rp+1})[k], xcs2 the centred values
  __shared__ __align__(16) float2 xs2[SIMT_TN / 2][FSK_D];
  __shared__ __align__(16) float2 xcs2[SIMT_TN / 2][FSK_D];
  __shared__ float mus[FSK_D];
  if (threadIdx.x < FSK_D) mus[threadIdx.x] = mu[threadIdx.x];
  __syncthreads();
  const int64_t i = (int64_t)blockIdx.x * SIMT_THREADS + threadIdx.x;
  const bool valid_i = i < n;
  float2 xi2[FSK_D];
#pragma unroll
  for (int k = 0; k < FSK_D; ++k) {
    const float v = valid_i ? x[i * FSK_D + k] : 0.f;
    xi2[k] = make_float2(v, v);
  }
  Comp pdf{0.f, 0.f};
  Comp w[FSK_D];
#pragma unroll
  for (int k = 0; k < FSK_D; ++k) w[k] = Comp{0.f, 0.f};

  const int64_t n_tiles = (n + SIMT_TN - 1) / SIMT_TN;
  const int64_t t_begin = (int64_t)blockIdx.y * tiles_per_split;
  const int64_t t_end = min(n_tiles, t_begin + tiles_per_split);
  for (int64_t t = t_begin; t < t_end; ++t) {
    const int64_t j0 = t * SIMT_TN;
    const int valid = (int)imin<int64_t>(SIMT_TN, n - j0);
    __syncthreads();
    for (int e = threadIdx.x; e < SIMT_TN * FSK_D; e += SIMT_THREADS) {
      int r = e / FSK_D, k = e % FSK_D;
      const float v = r < valid ? x[(j0 + r) * FSK_D + k] : 0.f;
      reinterpret_cast<float*>(&xs2[r >> 1][k])[r & 1] = -v;
      reinterpret_cast<float*>(&xcs2[r >> 1][k])[r & 1] = r < valid ? v - mus[k] : 0.f;
    }
    __syncthreads();
    // two data points per f32x2 instruction; even and odd points in separate chains
    float2 ps2 = make_float2(0.f, 0.f), wp2[FSK_D];
#pragma unroll
    for (int k = 0; k < FSK_D; ++k) wp2[k] = make_float2(0.f, 0.f);
    for (int rp = 0; 2 * rp < valid; ++rp) {
      const float4* xr = reinterpret_cast<const float4*>(&xs2[rp][0]);
      float2 d0 = make_float2(0.f, 0.f), d1 = d0, d2 = d0, d3 = d0;
#pragma unroll
      for (int kk = 0; kk < 4; ++kk) {
        const float4 va = xr[2 * kk], vb = xr[2 * kk + 1];   // features 4kk, 4kk+1 | 4kk+2, 4kk+3
        const float2 a0 = __fadd2_rn(xi2[4 * kk], make_float2(va.x, va.y));
        const float2 a1 = __fadd2_rn(xi2[4 * kk + 1], make_float2(va.z, va.w));
        const float2 a2 = __fadd2_rn(xi2[4 * kk + 2], make_float2(vb.x, vb.y));
        const float2 a3 = __fadd2_rn(xi2[4 * kk + 3], make_float2(vb.z, vb.w));
        d0 = __ffma2_rn(a0, a0, d0);
        d1 = __ffma2_rn(a1, a1, d1);
        d2 = __ffma2_rn(a2, a2, d2);
        d3 = __ffma2_rn(a3, a3, d3);
      }
      float2 e = exp2_neg_scaled2(__fadd2_rn(__fadd2_rn(d0, d1), __fadd2_rn(d2, d3)), c2, c2_lo);
      if (2 * rp + 1 >= valid) e.y = 0.f;   // the padding point of an odd tile
      ps2 = __fadd2_rn(ps2, e);
      const float4* xcr = reinterpret_cast<const float4*>(&xcs2[rp][0]);
#pragma unroll
      for (int kk = 0; kk < 8; ++kk) {
        const float4 c = xcr[kk];   // features 2kk, 2kk+1 of both points
        wp2[2 * kk] = __ffma2_rn(e, make_float2(c.x, c.y), wp2[2 * kk]);
        wp2[2 * kk + 1] = __ffma2_rn(e, make_float2(c.z, c.w), wp2[2 * kk + 1]);
      }
    }
    pdf.add(ps2.x + ps2.y);
#pragma unroll
    for (int k = 0; k < FSK_D; ++k) w[k].add(wp2[k].x + wp2[k].y);
  }
  if (!valid_i) return;
  const int64_t row = (int64_t)blockIdx.y * n + i;
  if (in_bounds(row, (int64_t)gridDim.y * n, 46)) ppdf[row] = (double)pdf.s + (double)pdf.c;
  if (!in_bounds(row, (int64_t)gridDim.y * n, 47)) return;   // the row's 16 features
  double* wo = pw + row * FSK_D;
#pragma unroll
  for (int k = 0; k < FSK_D; ++k) wo[k] = (double)w[k].s + (double)w[k].c;
}

void launch_score16_simt(const float* x, int64_t n, const float* mu, double h, int splits,
                         double* ppdf, double* pw, cudaStream_t s) {
  const int64_t n_tiles = (n + SIMT_TN - 1) / SIMT_TN;
  const int64_t tps = (n_tiles + splits - 1) / splits;
  dim3 grid((unsigned)((n + SIMT_THREADS - 1) / SIMT_THREADS), (unsigned)((n_tiles + tps - 1) / tps));
  const double c2d = FSK_LOG2E / (2.0 * h * h);
  const float c2 = (float)c2d, c2_lo = (float)(c2d - (double)c2);
  TimerScope ts(K_SCORE16_SIMT, (double)n * (double)n, s);
  score16_simt_kernel<<<grid, SIMT_THREADS, 0, s>>>(x, n, mu, c2, c2_lo, tps, ppdf, pw);
  count_launch();
}

int simt_score16_splits(int64_t n) {
  const int64_t n_tiles = (n + SIMT_TN - 1) / SIMT_TN;
  const int64_t rblocks = (n + SIMT_THREADS - 1) / SIMT_THREADS;
  const int64_t target = 4LL * sm_count() * 4;
  int64_t splits = (target + rblocks - 1) / rblocks;
  splits = imax<int64_t>(1, imin<int64_t>(splits, n_tiles / 4 > 0 ? n_tiles / 4 : 1));
  return effective_splits(n_tiles, imin<int64_t>(splits, 65535));
}

// ---------------------------------------------------------------------------
// 16-D empirical score, symmetric (phi_ij = phi_ji: each pair's exp once).
// Block = one row tile I (SYM_R points, thread t owns row i = I*SYM_R + t)
// against a run of up to SYM_L column tiles J of SYM_C points, J*SYM_C >=
// I*SYM_R (upper triangle, the diagonal tiles masked).  Per column tile:
//   phase 1 (thread = row i): phi_ij for the tile's points from direct FP32
//     differences of the original coordinates; the row sums pdf_i and
//     W_i += phi_ij (x_j - mu) accumulate in registers over the run; phi_ij
//     goes to shared memory;
//   phase 2 (thread = column j = J*SYM_C + t % SYM_C, rows t / SYM_C of the
//     tile's two row halves): the column sums sum_i phi_ij and
//     sum_i phi_ij (x_i - mu) from shared memory, added to the FP64
//     accumulators with atomics once per tile.
// The row sums go to the FP64 accumulators once per run.  Pairs with j > i
// count on both sides; the self pair counts once (row side).  Both phases
// use f32x2 instructions: phase 1 evaluates two column points per
// instruction (the tile kept as point pairs in shared memory), phase 2 sums
// two rows per instruction (the row tile kept as row pairs); each sum is
// carried as an even and an odd chain and the two are added at the end of
// the tile (2383 -> 2077 ms at n = 2^20).
// ---------------------------------------------------------------------------
namespace {
constexpr int SYM_R = 128;  // rows per block (threads)
constexpr int SYM_C = 64;   // points per column tile
constexpr int SYM_L = 16;   // column tiles per block
}

__global__ void __launch_bounds__(SYM_R) score16_sym_simt_kernel(
    const float* __restrict__ x, int64_t n, const float* __restrict__ mu, float c2, float c2_lo,
    int64_t n_col_tiles, double* __restrict__ acc_pdf, double* __restrict__ acc_w) {
  const int64_t I = blockIdx.x;
  const int64_t i0 = I * SYM_R;
  // first column tile touching the upper triangle of this row tile
  const int64_t Jfirst = i0 / SYM_C;
  const int64_t J0 = Jfirst + (int64_t)blockIdx.y * SYM_L;
  if (J0 >= n_col_tiles) return;   // beyond the end of this row tile's run (uniform per block)
  const int64_t J1 = imin<int64_t>(n_col_tiles, J0 + SYM_L);

  // column tile as point pairs: xs2[rp][k] = -(x_{2rp}, x_{2rp+1})[k], xcs2 the centred values
  __shared__ __align__(16) float2 xs2[SYM_C / 2][FSK_D];
  __shared__ __align__(16) float2 xcs2[SYM_C / 2][FSK_D];
  __shared__ __align__(16) float2 xic2[SYM_R / 2][FSK_D];   // row tile as row pairs, x - mu (phase 2)
  __shared__ __align__(16) float phi[SYM_C][SYM_R + 2];      // [column][row]; even stride: 8-byte row pairs
  __shared__ float mus[FSK_D];
  const int t = threadIdx.x;
  if (t < FSK_D) mus[t] = mu[t];
  __syncthreads();
  const int64_t i = i0 + t;
  const bool vi = i < n;
  float2 xi2[FSK_D];
#pragma unroll
  for (int k = 0; k < FSK_D; ++k) {
    const float v = vi ? x[i * FSK_D + k] : 0.f;
    xi2[k] = make_float2(v, v);
    reinterpret_cast<float*>(&xic2[t >> 1][k])[t & 1] = vi ? v - mus[k] : 0.f;
  }
  float prow = 0.f, wrow[FSK_D];
#pragma unroll
  for (int k = 0; k < FSK_D; ++k) wrow[k] = 0.f;
  const int cj = t % SYM_C, rh = t / SYM_C;   // phase 2: column and row half

  for (int64_t J = J0; J < J1; ++J) {
    const int64_t j0 = J * SYM_C;
    const int validj = (int)imin<int64_t>(SYM_C, n - j0);
    __syncthreads();   // previous tile's phase 2 is done with phi / xs
    for (int e = t; e < SYM_C * FSK_D; e += SYM_R) {
      const int r = e / FSK_D, k = e % FSK_D;
      const float v = r < validj ? x[(j0 + r) * FSK_D + k] : 0.f;
      reinterpret_cast<float*>(&xs2[r >> 1][k])[r & 1] = -v;
      reinterpret_cast<float*>(&xcs2[r >> 1][k])[r & 1] = r < validj ? v - mus[k] : 0.f;
    }
    __syncthreads();
    // phase 1: row i against the tile's points, two points per instruction
    // (j <= i drops from the column side, j < i from both)
    float2 ps2 = make_float2(0.f, 0.f), wp2[FSK_D];
#pragma unroll
    for (int k = 0; k < FSK_D; ++k) wp2[k] = make_float2(0.f, 0.f);
    const int64_t dj = i - j0;   // column index of the diagonal in this tile (may be outside)
    for (int rp = 0; rp < SYM_C / 2; ++rp) {
      const float4* xr = reinterpret_cast<const float4*>(&xs2[rp][0]);
      float2 d0 = make_float2(0.f, 0.f), d1 = d0, d2 = d0, d3 = d0;
#pragma unroll
      for (int kk = 0; kk < 4; ++kk) {
        const float4 va = xr[2 * kk], vb = xr[2 * kk + 1];   // features 4kk, 4kk+1 | 4kk+2, 4kk+3
        const float2 a0 = __fadd2_rn(xi2[4 * kk], make_float2(va.x, va.y));
        const float2 a1 = __fadd2_rn(xi2[4 * kk + 1], make_float2(va.z, va.w));
        const float2 a2 = __fadd2_rn(xi2[4 * kk + 2], make_float2(vb.x, vb.y));
        const float2 a3 = __fadd2_rn(xi2[4 * kk + 3], make_float2(vb.z, vb.w));
        d0 = __ffma2_rn(a0, a0, d0);
        d1 = __ffma2_rn(a1, a1, d1);
        d2 = __ffma2_rn(a2, a2, d2);
        d3 = __ffma2_rn(a3, a3, d3);
      }
      const int r = 2 * rp;
      float2 e = exp2_neg_scaled2(__fadd2_rn(__fadd2_rn(d0, d1), __fadd2_rn(d2, d3)), c2, c2_lo);
      if (!(vi && r < validj && r >= dj)) e.x = 0.f;            // j >= i
      if (!(vi && r + 1 < validj && r + 1 >= dj)) e.y = 0.f;
      ps2 = __fadd2_rn(ps2, e);
      const float4* xcr = reinterpret_cast<const float4*>(&xcs2[rp][0]);
#pragma unroll
      for (int kk = 0; kk < 8; ++kk) {
        const float4 c = xcr[kk];   // features 2kk, 2kk+1 of both points
        wp2[2 * kk] = __ffma2_rn(e, make_float2(c.x, c.y), wp2[2 * kk]);
        wp2[2 * kk + 1] = __ffma2_rn(e, make_float2(c.z, c.w), wp2[2 * kk + 1]);
      }
      phi[r][t] = r > dj ? e.x : 0.f;   // column side: j > i only
      phi[r + 1][t] = r + 1 > dj ? e.y : 0.f;
    }
    prow += ps2.x + ps2.y;
#pragma unroll
    for (int k = 0; k < FSK_D; ++k) wrow[k] += wp2[k].x + wp2[k].y;
    __syncthreads();
    // phase 2: column j = j0 + cj against rows rh * SYM_C .. +SYM_C of the tile, two rows
    // per instruction
    if (cj < validj) {
      float2 pc2 = make_float2(0.f, 0.f), wc2[FSK_D];
#pragma unroll
      for (int k = 0; k < FSK_D; ++k) wc2[k] = make_float2(0.f, 0.f);
      const int rbeg = rh * SYM_C;
      for (int r = rbeg; r < rbeg + SYM_C; r += 2) {
        const float2 e = *reinterpret_cast<const float2*>(&phi[cj][r]);
        const float4* c4 = reinterpret_cast<const float4*>(&xic2[r >> 1][0]);
#pragma unroll
        for (int kk = 0; kk < 8; ++kk) {
          const float4 c = c4[kk];
          wc2[2 * kk] = __ffma2_rn(e, make_float2(c.x, c.y), wc2[2 * kk]);
          wc2[2 * kk + 1] = __ffma2_rn(e, make_float2(c.z, c.w), wc2[2 * kk + 1]);
        }
        pc2 = __fadd2_rn(pc2, e);
      }
      const float pc = pc2.x + pc2.y;
      if (pc != 0.f && in_bounds(j0 + cj, n, 48)) {
        const int64_t j = j0 + cj;
        atomicAdd(&acc_pdf[j], (double)pc);
#pragma unroll
        for (int k = 0; k < FSK_D; ++k) atomicAdd(&acc_w[j * FSK_D + k], (double)(wc2[k].x + wc2[k].y));
      }
    }
  }
  if (vi && in_bounds(i, n, 49)) {
    atomicAdd(&acc_pdf[i], (double)prow);
#pragma unroll
    for (int k = 0; k < FSK_D; ++k) atomicAdd(&acc_w[i * FSK_D + k], (double)wrow[k]);
  }
}

void launch_score16_sym_simt(const float* x, int64_t n, const float* mu, double h, double* acc_pdf,
                             double* acc_w, cudaStream_t s) {
  const int64_t row_tiles = (n + SYM_R - 1) / SYM_R;
  const int64_t col_tiles = (n + SYM_C - 1) / SYM_C;
  const double c2d = FSK_LOG2E / (2.0 * h * h);
  const float c2 = (float)c2d, c2_lo = (float)(c2d - (double)c2);
  // grid.x: row tile; grid.y: run index (runs past the last column tile exit at once)
  const dim3 grid((unsigned)row_tiles, (unsigned)((col_tiles + SYM_L - 1) / SYM_L));
  TimerScope ts(K_SCORE16_SYM_SIMT, 0.5 * (double)n * (double)(n + 1), s);
  score16_sym_simt_kernel<<<grid, SYM_R, 0, s>>>(x, n, mu, c2, c2_lo, col_tiles, acc_pdf, acc_w);
  count_launch();
}

int64_t sym_simt_pairs(int64_t n) {
  const int64_t col_tiles = (n + SYM_C - 1) / SYM_C;
  return col_tiles * (col_tiles + 1) / 2;
}

// ---------------------------------------------------------------------------
// 1-D KDE.  Block 128 threads x K1_Q queries; data tiles of K1_T points in SMEM.
// phi = exp(-(q - x)^2 / (2 h^2)) (times 1.5 - (q-x)^2/(2h^2) with Laplace).
// A thread's queries are held negated in f32x2 pairs, so one packed
// instruction forms x - q, its square and the exponent for two queries: the
// FP32 work per pair drops below the ex2 rate and the exp pipe is the bound.
// Per query the arithmetic (x - q = -(q - x) exactly, squared, times
// -log2(e)/(2h^2), ex2, summed in data order) is that of a scalar loop.
// ---------------------------------------------------------------------------
namespace {
constexpr int K1_THREADS = 128;
constexpr int K1_Q = 8;
constexpr int K1_P = K1_Q / 2;   // query pairs per thread
constexpr int K1_T = 1024;

// Visits the valid points r0 .. rend-1 of a staged tile in order: four at a
// time (one 16-byte shared load) for a full 32-point group, else one by one.
// (The exp stays on the exp pipe here: per pair the kernel also issues four
// FP32 lane operations, so the FP32 pipe is as busy as the exp pipe and the
// FMA-pipe exp2 would only move the bound: measured 6.6e12 vs 8.3e12 pair
// evaluations per second with an eighth of the exps moved.)
template <typename F>
__device__ __forceinline__ void for_points(const float* xs, int r0, int rend, F&& f) {
  if (rend - r0 == 32) {
    const float4* xs4 = reinterpret_cast<const float4*>(xs + r0);
#pragma unroll 2
    for (int k = 0; k < 8; ++k) {
      const float4 v = xs4[k];
      f(v.x);
      f(v.y);
      f(v.z);
      f(v.w);
    }
  } else {
    for (int r = r0; r < rend; ++r) f(xs[r]);
  }
}
}  // namespace

template <bool LAPLACE>
__global__ void __launch_bounds__(K1_THREADS) kde1d_kernel(
    const float* __restrict__ q, int64_t m, const float* __restrict__ x, int64_t n, float nc2,
    float c1, int64_t tiles_per_split, double* __restrict__ partials, double* __restrict__ atomic_acc) {
  __shared__ __align__(16) float xs[K1_T];
  const int64_t q0 = (int64_t)blockIdx.x * (K1_THREADS * K1_Q);
  float2 nq[K1_P];   // -q of queries (2p, 2p + 1)
#pragma unroll
  for (int p = 0; p < K1_P; ++p) {
    const int64_t qa = q0 + threadIdx.x + (2 * p) * K1_THREADS, qb = qa + K1_THREADS;
    nq[p] = make_float2(qa < m ? -q[qa] : 0.f, qb < m ? -q[qb] : 0.f);
  }
  Comp acc[K1_Q];
#pragma unroll
  for (int u = 0; u < K1_Q; ++u) acc[u] = Comp{0.f, 0.f};
  const float2 nc2_2 = make_float2(nc2, nc2);
  const float2 mc1_2 = make_float2(-c1, -c1);
  const float2 c15_2 = make_float2(1.5f, 1.5f);
  const int64_t n_tiles = (n + K1_T - 1) / K1_T;
  const int64_t t_begin = (int64_t)blockIdx.y * tiles_per_split;
  const int64_t t_end = min(n_tiles, t_begin + tiles_per_split);
  for (int64_t t = t_begin; t < t_end; ++t) {
    const int64_t j0 = t * K1_T;
    const int valid = (int)imin<int64_t>(K1_T, n - j0);
    __syncthreads();
    for (int e = threadIdx.x; e < K1_T; e += K1_THREADS) xs[e] = e < valid ? x[j0 + e] : 0.f;
    __syncthreads();
    for (int r0 = 0; r0 < valid; r0 += 32) {
      float2 part[K1_P];
#pragma unroll
      for (int p = 0; p < K1_P; ++p) part[p] = make_float2(0.f, 0.f);
      for_points(xs, r0, min(valid, r0 + 32), [&](float xv) {
        const float2 x2 = make_float2(xv, xv);
#pragma unroll
        for (int p = 0; p < K1_P; ++p) {
          const float2 d = __fadd2_rn(x2, nq[p]);
          const float2 t2 = __fmul2_rn(d, d);
          const float2 a = __fmul2_rn(t2, nc2_2);
          float2 e = make_float2(ex2_approx(a.x), ex2_approx(a.y));
          if (LAPLACE) e = __fmul2_rn(e, __ffma2_rn(mc1_2, t2, c15_2));
          part[p] = __fadd2_rn(part[p], e);
        }
      });
#pragma unroll
      for (int p = 0; p < K1_P; ++p) {
        acc[2 * p].add(part[p].x);
        acc[2 * p + 1].add(part[p].y);
      }
    }
  }
#pragma unroll
  for (int u = 0; u < K1_Q; ++u) {
    int64_t qi = q0 + threadIdx.x + u * K1_THREADS;
    if (qi >= m) continue;
    double v = (double)acc[u].s + (double)acc[u].c;
    if (atomic_acc) {
      if (in_bounds(qi, m, 50)) atomicAdd(&atomic_acc[qi], v);
    } else {
      const int64_t idx = (int64_t)blockIdx.y * m + qi;
      if (in_bounds(idx, (int64_t)gridDim.y * m, 51)) partials[idx] = v;
    }
  }
}

int kde1d_splits(int64_t m, int64_t n) {
  const int64_t n_tiles = (n + K1_T - 1) / K1_T;
  const int64_t qblocks = (m + K1_THREADS * K1_Q - 1) / (K1_THREADS * K1_Q);
  const int64_t target = 8LL * sm_count() * 4;
  int64_t splits = (target + qblocks - 1) / qblocks;
  return effective_splits(n_tiles, imin<int64_t>(splits, 65535));
}

void launch_kde1d(const float* q, int64_t m, const float* x, int64_t n, double h, bool laplace,
                  int splits, double* partials, double* atomic_acc, cudaStream_t s) {
  const int64_t n_tiles = (n + K1_T - 1) / K1_T;
  const int64_t tps = (n_tiles + splits - 1) / splits;
  dim3 grid((unsigned)((m + K1_THREADS * K1_Q - 1) / (K1_THREADS * K1_Q)), (unsigned)((n_tiles + tps - 1) / tps));
  const float nc2 = (float)(-FSK_LOG2E / (2.0 * h * h));
  const float c1 = (float)(1.0 / (2.0 * h * h));
  TimerScope ts(K_KDE1D, (double)m * (double)n, s);
  if (laplace)
    kde1d_kernel<true><<<grid, K1_THREADS, 0, s>>>(q, m, x, n, nc2, c1, tps, partials, atomic_acc);
  else
    kde1d_kernel<false><<<grid, K1_THREADS, 0, s>>>(q, m, x, n, nc2, c1, tps, partials, atomic_acc);
  count_launch();
}

// 1-D pdf + derivative sums: S0 = sum phi, S1 = sum (x - q) phi  (= -h * sum z phi).
__global__ void __launch_bounds__(K1_THREADS) kde1d_score_kernel(
    const float* __restrict__ q, int64_t m, const float* __restrict__ x, int64_t n, float nc2,
    int64_t tiles_per_split, double* __restrict__ p0, double* __restrict__ p1) {
  __shared__ __align__(16) float xs[K1_T];
  const int64_t q0 = (int64_t)blockIdx.x * (K1_THREADS * K1_Q);
  float2 nq[K1_P];   // -q of queries (2p, 2p + 1)
#pragma unroll
  for (int p = 0; p < K1_P; ++p) {
    const int64_t qa = q0 + threadIdx.x + (2 * p) * K1_THREADS, qb = qa + K1_THREADS;
    nq[p] = make_float2(qa < m ? -q[qa] : 0.f, qb < m ? -q[qb] : 0.f);
  }
  const float2 nc2_2 = make_float2(nc2, nc2);
  Comp a0[K1_Q], a1[K1_Q];
#pragma unroll
  for (int u = 0; u < K1_Q; ++u) { a0[u] = Comp{0.f, 0.f}; a1[u] = Comp{0.f, 0.f}; }
  const int64_t n_tiles = (n + K1_T - 1) / K1_T;
  const int64_t t_begin = (int64_t)blockIdx.y * tiles_per_split;
  const int64_t t_end = min(n_tiles, t_begin + tiles_per_split);
  for (int64_t t = t_begin; t < t_end; ++t) {
    const int64_t j0 = t * K1_T;
    const int valid = (int)imin<int64_t>(K1_T, n - j0);
    __syncthreads();
    for (int e = threadIdx.x; e < K1_T; e += K1_THREADS) xs[e] = e < valid ? x[j0 + e] : 0.f;
    __syncthreads();
    for (int r0 = 0; r0 < valid; r0 += 32) {
      float2 s0[K1_P], s1[K1_P];
#pragma unroll
      for (int p = 0; p < K1_P; ++p) { s0[p] = make_float2(0.f, 0.f); s1[p] = make_float2(0.f, 0.f); }
      for_points(xs, r0, min(valid, r0 + 32), [&](float xv) {
        const float2 x2 = make_float2(xv, xv);
#pragma unroll
        for (int p = 0; p < K1_P; ++p) {
          const float2 d = __fadd2_rn(x2, nq[p]);    // x - q
          const float2 a = __fmul2_rn(__fmul2_rn(d, d), nc2_2);
          const float2 e = make_float2(ex2_approx(a.x), ex2_approx(a.y));
          s0[p] = __fadd2_rn(s0[p], e);
          s1[p] = __ffma2_rn(d, e, s1[p]);
        }
      });
#pragma unroll
      for (int p = 0; p < K1_P; ++p) {
        a0[2 * p].add(s0[p].x);
        a0[2 * p + 1].add(s0[p].y);
        a1[2 * p].add(s1[p].x);
        a1[2 * p + 1].add(s1[p].y);
      }
    }
  }
#pragma unroll
  for (int u = 0; u < K1_Q; ++u) {
    int64_t qi = q0 + threadIdx.x + u * K1_THREADS;
    if (qi >= m) continue;
    const int64_t idx = (int64_t)blockIdx.y * m + qi;
    if (!in_bounds(idx, (int64_t)gridDim.y * m, 52)) continue;
    p0[idx] = (double)a0[u].s + (double)a0[u].c;
    p1[idx] = (double)a1[u].s + (double)a1[u].c;
  }
}

void launch_kde1d_score(const float* q, int64_t m, const float* x, int64_t n, double h, int splits,
                        double* p0, double* p1, cudaStream_t s) {
  const int64_t n_tiles = (n + K1_T - 1) / K1_T;
  const int64_t tps = (n_tiles + splits - 1) / splits;
  dim3 grid((unsigned)((m + K1_THREADS * K1_Q - 1) / (K1_THREADS * K1_Q)), (unsigned)((n_tiles + tps - 1) / tps));
  const float nc2 = (float)(-FSK_LOG2E / (2.0 * h * h));
  TimerScope ts(K_KDE1D_SCORE, (double)m * (double)n, s);
  kde1d_score_kernel<<<grid, K1_THREADS, 0, s>>>(q, m, x, n, nc2, tps, p0, p1);
  count_launch();
}

unsigned int simt_take_device_error() { return take_unit_device_error(); }

}  // namespace fsk
