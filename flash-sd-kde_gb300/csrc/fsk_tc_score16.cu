// fsk_tc_score16.cu - tensor-core (tcgen05 / TMEM) empirical-score
// accumulators of the 16-D SD-KDE, GB300-native.
//
// What it computes, for every data point x_i (queries = data):
//   pdf_sum_i      = sum_j phi_ij,          phi_ij = exp(-||x_i - x_j||^2 / (2 h^2))
//   weighted_sum_i = sum_j phi_ij x_j
// the accumulators of kernels/flash_sd_kde/empirical.py:72-131 and
// kernels/emp_score_16d_ordered_splitk.py:20-95 (both tl.dot products with
// allow_tf32), as FP64 partials per data split; the weighted sum is kept
// centred (sum_j phi_ij (x_j - mu)) and mu * pdf_sum is added back in FP64.
//
// How (per 128-query x 64-point tile):
//  * S = the log2-domain exponent a2 + 15, from the same fp16 hi/lo + bias
//    operand images and four tcgen05.mma as the KDE kernel (fsk_tc_kde16.cu);
//    the +15 rides in the query's bias term, so 2^S = phi * 2^15 and the
//    weights keep fp16 normal range down to phi ~ 2^-29.
//  * Epilogue: tcgen05.ld, ex2.approx, pdf chunk sums, the exact near-pair
//    recompute of the KDE kernel (the recomputed value also replaces the
//    approximate one in the weights), then the weights are split into fp16
//    hi + lo and stored to tensor memory with tcgen05.st.
//  * W += Phi_hi X_hi + Phi_hi X_lo + Phi_lo X_hi: tcgen05.mma with the A
//    operand (weights, M=128 x K=64) read from tensor memory and the B operand
//    ((x_j - mu) 2^ew, fp16 hi/lo, K-major over the data points) from the
//    data stage in shared memory, N = 16 features, FP32 accumulation over a
//    group of S_GROUP tiles, then added into compensated FP32 sums.
//
// Pipeline (one persistent CTA per SM, 18 warps):
//   warp 16 : producer (bulk copies of query images per unit, data stages).
//   warp 17 : owns TMEM, issues S(t) then W(t-1) (one lane).
//   warps 0-15: epilogue; warp w: query tile w/8, data-column half (w/4)&1,
//             TMEM lane quarter w&3.  The two column halves of a row keep
//             separate pdf partials (written as two virtual splits) and
//             read disjoint halves of the weighted-sum features.
// TMEM: S [2 buffers][2 query tiles][64] | Phi [2 tiles][hi 32 | lo 32]
//       | W [2 group parities][2 tiles][16].
#include <cuda_fp16.h>

#include "fsk_kernels.cuh"
#include "fsk_tc.cuh"
#include "fsk_tc_ops.cuh"

namespace fsk {
namespace tc {

namespace {

constexpr int SNQT = 2;                                    // query tiles per unit (256 queries)
constexpr int SNS = 8;                                     // data stages
constexpr int XT_ROW_BYTES = NT * 2;                       // one feature row over 64 points, fp16
constexpr int XT_BYTES = FSK_D * XT_ROW_BYTES;             // 2 KB
constexpr int S_XTH_OFFSET = B_H_BYTES + B_L_BYTES;        // 6 KB
constexpr int S_XTL_OFFSET = S_XTH_OFFSET + XT_BYTES;      // 8 KB
constexpr int S_X_OFFSET = S_XTL_OFFSET + XT_BYTES;        // 10 KB: original FP32 rows
constexpr int S_STAGE_BYTES = S_X_OFFSET + NT * FSK_D * 4; // 14 KB
constexpr int S_A_BYTES = SNQT * A_TILE_BYTES;             // 24 KB
constexpr int S_EPI_WARPS = 8 * SNQT;
constexpr int S_PRODUCER_WARP = S_EPI_WARPS;
constexpr int S_MMA_WARP = S_EPI_WARPS + 1;
constexpr int S_THREADS = (S_EPI_WARPS + 2) * 32;
constexpr int S_GROUP = 4;                                 // data tiles per W accumulation
constexpr int T_S = 0;
constexpr int T_PHI = 2 * SNQT * NT;                       // 256
constexpr int T_W = T_PHI + SNQT * NT;                     // 384
constexpr int S_TMEM_COLS = 512;
// exact-recompute corrections of the weighted sums: [unit parity][column half][256 rows][16] FP32
constexpr int S_WCORR_OFFSET = S_A_BYTES + SNS * S_STAGE_BYTES + 512;
constexpr int S_WCORR_BYTES = 2 * 2 * SNQT * QT * FSK_D * 4;          // 64 KB
constexpr int S_SMEM_BYTES = S_WCORR_OFFSET + S_WCORR_BYTES;
constexpr float PHI_LOG2_SCALE = 15.0f;                    // weights are phi * 2^15
static_assert(T_W + 2 * SNQT * FSK_D <= S_TMEM_COLS, "TMEM budget");
static_assert(S_STAGE_BYTES % 16 == 0 && S_A_BYTES % 16 == 0, "bulk copy granularity");
static_assert(S_SMEM_BYTES <= 227 * 1024, "shared memory");

struct ScParams {
  const uint8_t* qimg;
  const uint8_t* ximg;
  const float* qexact;
  const TcScales* scales;
  const float* mu;
  int64_t n;
  int64_t n_tiles, q_blocks, splits, tiles_per_split;
  float c2, c2_lo;
  double* ppdf;   // [2 * splits][n]  (split sp, column half h at 2 sp + h), self pair excluded
  double* pw;     // [splits][n][16]  centred weighted sums, self pair excluded
};

// f32 pair -> packed fp16 hi and lo parts (hi + lo = v to ~22 bits)
__device__ __forceinline__ void split_pack(float v0, float v1, uint32_t& hi, uint32_t& lo) {
  const __half2 h = __floats2half2_rn(v0, v1);
  const float2 hf = __half22float2(h);
  const float2 r = __fadd2_rn(make_float2(v0, v1), make_float2(-hf.x, -hf.y));
  const __half2 l = __floats2half2_rn(r.x, r.y);
  hi = *reinterpret_cast<const uint32_t*>(&h);
  lo = *reinterpret_cast<const uint32_t*>(&l);
}

__global__ void __launch_bounds__(S_THREADS, 1) score16_tc_kernel(ScParams p) {
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t* sA = smem_raw;
  uint8_t* sB = smem_raw + S_A_BYTES;
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem_raw + S_A_BYTES + SNS * S_STAGE_BYTES);
  uint64_t* full = bars;                      // [SNS] stage loaded
  uint64_t* empty = bars + SNS;               // [SNS] stage consumed (W MMA + epilogue)
  uint64_t* tfull = bars + 2 * SNS;           // [2] S buffer written
  uint64_t* tempty = bars + 2 * SNS + 2;      // [2] S buffer read
  uint64_t* pready = bars + 2 * SNS + 4;      // [SNQT] weights of a tile stored
  uint64_t* pfree = bars + 2 * SNS + 6;       // [SNQT] weights consumed by the W MMA
  uint64_t* wfull = bars + 2 * SNS + 8;       // [2] W group accumulated
  uint64_t* wempty = bars + 2 * SNS + 10;     // [2] W group read
  uint64_t* qready = bars + 2 * SNS + 12;
  uint64_t* qempty = bars + 2 * SNS + 13;
  uint64_t* drain = bars + 2 * SNS + 14;      // all MMAs of this CTA finished (exit path)
  uint64_t* cready = bars + 2 * SNS + 15;     // unit's W corrections written (epilogue warps)
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 2 * SNS + 16);
  float* wcorr = reinterpret_cast<float*>(smem_raw + S_WCORR_OFFSET);
  int64_t n_stage_copies = 0, n_query_copies = 0;   // producer: bulk copies issued

  const int warp = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;

  if (threadIdx.x == 0) {
    for (int s = 0; s < SNS; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1 + S_EPI_WARPS);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&tfull[b], 1);
      mbar_init(&tempty[b], S_EPI_WARPS);
      mbar_init(&wfull[b], 1);
      mbar_init(&wempty[b], S_EPI_WARPS);
    }
    for (int a = 0; a < SNQT; ++a) {
      mbar_init(&pready[a], 8);
      mbar_init(&pfree[a], 1);
    }
    mbar_init(qready, 1);
    mbar_init(qempty, 1);
    mbar_init(drain, 1);
    mbar_init(cready, S_EPI_WARPS);
    fence_barrier_init();
  }
  if (warp == S_MMA_WARP) {
    tmem_alloc(tmem_slot, S_TMEM_COLS);
    tmem_relinquish();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem_base = *tmem_slot;
  const int64_t units = p.q_blocks * p.splits;
  const int64_t u_begin = (int64_t)blockIdx.x * units / gridDim.x;
  const int64_t u_end = (int64_t)(blockIdx.x + 1) * units / gridDim.x;

  if (warp == S_PRODUCER_WARP) {
    if (lane == 0) {
      int64_t& g = n_stage_copies;
      int64_t& k = n_query_copies;
      for (int64_t u = u_begin; u < u_end; ++u) {
        const int64_t qb = u / p.splits, sp = u % p.splits;
        if (!mbar_wait(qempty, (uint32_t)((k & 1) ^ 1), 21)) goto done;
        mbar_arrive_expect_tx(qready, S_A_BYTES);
        bulk_g2s(sA, p.qimg + qb * (int64_t)S_A_BYTES, S_A_BYTES, qready);
        ++k;
        const int64_t t0 = sp * p.tiles_per_split;
        const int64_t t1 = imin<int64_t>(p.n_tiles, t0 + p.tiles_per_split);
        for (int64_t t = t0; t < t1; ++t) {
          const int s = (int)(g % SNS);
          if (!mbar_wait(&empty[s], (uint32_t)(((g / SNS) & 1) ^ 1), 22)) goto done;
          mbar_arrive_expect_tx(&full[s], S_STAGE_BYTES);
          bulk_g2s(sB + s * S_STAGE_BYTES, p.ximg + t * (int64_t)S_STAGE_BYTES, S_STAGE_BYTES, &full[s]);
          ++g;
        }
      }
    }
  } else if (warp == S_MMA_WARP) {
    if (lane == 0) {
      const uint32_t idesc_s = idesc_f16_f32(QT, NT);
      const uint32_t idesc_w = idesc_f16_f32(QT, FSK_D);
      int64_t g = 0, k = 0, grp = 0;
      for (int64_t u = u_begin; u < u_end; ++u, ++k) {
        const int64_t sp = u % p.splits;
        if (!mbar_wait(qready, (uint32_t)(k & 1), 23)) goto done;
        const int64_t t0 = sp * p.tiles_per_split;
        const int64_t t1 = imin<int64_t>(p.n_tiles, t0 + p.tiles_per_split);
        // iteration t issues S(t) (t < t1) and then W(t-1) (t > t0)
        for (int64_t t = t0; t <= t1; ++t) {
          if (t < t1) {
            const int s = (int)(g % SNS);
            const int b = (int)(g & 1);
            if (!mbar_wait(&full[s], (uint32_t)((g / SNS) & 1), 24)) goto done;
            if (!mbar_wait(&tempty[b], (uint32_t)(((g >> 1) & 1) ^ 1), 25)) goto done;
            tc_fence_after();
            const uint32_t bs = smem_u32(sB + s * S_STAGE_BYTES);
            const uint64_t b_hf = smem_desc_kmajor(bs, 128, 8 * H_ROW_BYTES);
            const uint64_t b_hb = smem_desc_kmajor(bs + 256, 128, 8 * H_ROW_BYTES);
            const uint64_t b_l = smem_desc_kmajor(bs + B_H_BYTES, 128, 8 * L_ROW_BYTES);
#pragma unroll
            for (int a = 0; a < SNQT; ++a) {
              const uint32_t as = smem_u32(sA + a * A_TILE_BYTES);
              const uint64_t a_hf = smem_desc_kmajor(as, 128, 8 * H_ROW_BYTES);
              const uint64_t a_hb = smem_desc_kmajor(as + 256, 128, 8 * H_ROW_BYTES);
              const uint64_t a_l = smem_desc_kmajor(as + A_H_BYTES, 128, 8 * L_ROW_BYTES);
              const uint32_t d = tmem_base + (uint32_t)(T_S + b * (SNQT * NT) + a * NT);
              mma_f16_ss(d, a_l, b_hf, idesc_s, 0u);
              mma_f16_ss(d, a_hf, b_l, idesc_s, 1u);
              mma_f16_ss(d, a_hf, b_hf, idesc_s, 1u);
              mma_f16_ss(d, a_hb, b_hb, idesc_s, 1u);
            }
            mma_commit(&tfull[b]);
            if (t == t1 - 1) mma_commit(qempty);   // last read of the query images
          }
          if (t > t0) {
            // weighted sums of the previous tile
            const int64_t gw = g - 1;
            const int64_t pos = (t - 1 - t0) % S_GROUP;
            const bool first = pos == 0;
            const bool last = pos == S_GROUP - 1 || t == t1;
            const int par = (int)(grp & 1);
            const int sw = (int)(gw % SNS);
            if (first && !mbar_wait(&wempty[par], (uint32_t)(((grp >> 1) & 1) ^ 1), 26)) goto done;
            const uint32_t bs = smem_u32(sB + sw * S_STAGE_BYTES);
#pragma unroll
            for (int a = 0; a < SNQT; ++a) {
              if (!mbar_wait(&pready[a], (uint32_t)(gw & 1), 27)) goto done;
              tc_fence_after();
              const uint32_t d = tmem_base + (uint32_t)(T_W + par * (SNQT * FSK_D) + a * FSK_D);
              const uint32_t ph = tmem_base + (uint32_t)(T_PHI + a * NT);
#pragma unroll
              for (int ks = 0; ks < NT / 16; ++ks) {
                const uint64_t xh = smem_desc_kmajor(bs + S_XTH_OFFSET + 256 * ks, 128, 8 * XT_ROW_BYTES);
                const uint64_t xl = smem_desc_kmajor(bs + S_XTL_OFFSET + 256 * ks, 128, 8 * XT_ROW_BYTES);
                mma_f16_ts(d, ph + 8 * ks, xh, idesc_w, (first && ks == 0) ? 0u : 1u);
                mma_f16_ts(d, ph + 8 * ks, xl, idesc_w, 1u);
                mma_f16_ts(d, ph + NT / 2 + 8 * ks, xh, idesc_w, 1u);
              }
              mma_commit(&pfree[a]);
            }
            mma_commit(&empty[sw]);
            if (last) {
              mma_commit(&wfull[par]);
              ++grp;
            }
          }
          if (t < t1) ++g;
        }
      }
    }
  } else {
    // ---------------- epilogue warps ----------------
    // The self pair (data index == query index) is left out of every sum
    // here; the reduce pass adds it exactly (phi = 1, weight x_i).  Its
    // weight still counts in the near-pair threshold: pdf_sum >= 1.
    const int qt = warp >> 3;             // query tile
    const int half = (warp >> 2) & 1;     // data-column half
    const int quarter = warp & 3;         // TMEM lane quarter
    const int row = quarter * 32 + lane;
    const uint32_t lane_off = (uint32_t)(quarter * 32) << 16;
    const float out_mul = p.scales->out_mul;
    const bool scaled = out_mul != 1.0f;
    const float phi_scale = 32768.0f;     // 2^PHI_LOG2_SCALE
    const double w_unscale = ldexp(1.0, -(int)PHI_LOG2_SCALE - p.scales->pad[2]);
    const double p_unscale = ldexp(1.0, -(int)PHI_LOG2_SCALE);
    const double c_unscale = ldexp(1.0, -(int)PHI_LOG2_SCALE);
    // correction rows: wcorr[parity][half][qt*128 + row][16]
    const int wc_row = (qt * QT + row) * FSK_D;
    constexpr int WC_HALF = SNQT * QT * FSK_D, WC_PAR = 2 * WC_HALF;
#pragma unroll
    for (int par = 0; par < 2; ++par)
#pragma unroll
      for (int k = 0; k < FSK_D; k += 4)
        *reinterpret_cast<float4*>(wcorr + par * WC_PAR + half * WC_HALF + wc_row + k) =
            make_float4(0.f, 0.f, 0.f, 0.f);
    int g = 0, grp = 0, k_unit = 0;
    int prev_qb = -1;
    float s_carry = 0.f;
    const int splits = (int)p.splits, tps = (int)p.tiles_per_split, n_tiles = (int)p.n_tiles;
    for (int u = (int)u_begin; u < (int)u_end; ++u, ++k_unit) {
      const int qb = u / splits, sp = u % splits;
      if (qb != prev_qb) {
        s_carry = phi_scale;   // the self pair
        prev_qb = qb;
      }
      const int gi = qb * (SNQT * QT) + qt * QT + row;
      const int diag_col = qb * (SNQT * QT) + qt * QT + quarter * 32;   // this warp's rows
      float* wc = wcorr + (k_unit & 1) * WC_PAR + half * WC_HALF + wc_row;
      Comp acc{0.f, 0.f};
      float corr = 0.f;
      Comp wacc[FSK_D / 2];
#pragma unroll
      for (int k = 0; k < FSK_D / 2; ++k) wacc[k] = Comp{0.f, 0.f};
      const int t0 = sp * tps;
      const int t1 = imin(n_tiles, t0 + tps);
      bool pend = false;     // a W group ended at the previous tile and is not read yet
      for (int t = t0; t < t1; ++t, ++g) {
        const int s = g % SNS;
        const int b = g & 1;
        const int valid = (int)imin<int64_t>(NT, p.n - (int64_t)t * NT);
        if (!mbar_wait(&tfull[b], (uint32_t)((g >> 1) & 1), 28)) goto done;
        tc_fence_after();
        const uint8_t* stage = sB + s * S_STAGE_BYTES;
        uint32_t r[32];
        tmem_ld32(tmem_base + lane_off + (uint32_t)(T_S + b * (SNQT * NT) + qt * NT + half * 32), r);
        tmem_ld_wait();
        tc_fence_before();
        __syncwarp();
        if (lane == 0) mbar_arrive(&tempty[b]);
        float e[32];
        if (scaled) {
#pragma unroll
          for (int j = 0; j < 32; ++j) e[j] = __uint_as_float(r[j]) * out_mul;
        } else {
#pragma unroll
          for (int j = 0; j < 32; ++j) e[j] = __uint_as_float(r[j]);
        }
#pragma unroll
        for (int j = 0; j < 32; ++j) e[j] = ex2_approx(e[j]);
        if (valid < NT) {
#pragma unroll
          for (int j = 0; j < 32; ++j)
            if (half * 32 + j >= valid) e[j] = 0.f;
        }
        if (t * NT + half * 32 == diag_col) {
          // this chunk's 32 columns are this warp's 32 rows: drop the self pair
#pragma unroll
          for (int j = 0; j < 32; ++j)
            if (j == lane) e[j] = 0.f;
        }
        float2 pa = make_float2(e[0], e[1]), pb = make_float2(e[2], e[3]);
#pragma unroll
        for (int j = 4; j < 32; j += 4) {
          pa = __fadd2_rn(pa, make_float2(e[j], e[j + 1]));
          pb = __fadd2_rn(pb, make_float2(e[j + 2], e[j + 3]));
        }
        pa = __fadd2_rn(pa, pb);
        const float cs = pa.x + pa.y;
        const bool trig = cs > (s_carry + acc.s + cs) * NEAR_FRACTION;
        if (__any_sync(0xffffffffu, trig)) {
          // The chunk's largest weight is recomputed exactly (argmax on keys
          // = value bits with the column in the low 5 bits, as in the KDE
          // kernel).  With A the keyed approximation, the pdf gets ex - A
          // (corr) and the weighted sum (ex - A)(x_j - mu) (shared-memory
          // corrections), so both see the same weight e_j - A + ex.
          if (trig) {
            uint32_t key[16];
#pragma unroll
            for (int j = 0; j < 16; ++j)
              key[j] = max((__float_as_uint(e[j]) & ~31u) | (uint32_t)j,
                           (__float_as_uint(e[j + 16]) & ~31u) | (uint32_t)(j + 16));
#pragma unroll
            for (int w = 8; w >= 1; w >>= 1)
#pragma unroll
              for (int j = 0; j < w; ++j) key[j] = max(key[j], key[j + w]);
            const uint32_t kmax = key[0];
            const int j = (int)(kmax & 31u);
            float qx[FSK_D];   // the query's original coordinates (L1-resident after first use)
#pragma unroll
            for (int kk = 0; kk < FSK_D; kk += 4) {
              const float4 v = __ldg(reinterpret_cast<const float4*>(p.qexact + (int64_t)gi * FSK_D + kk));
              qx[kk] = v.x; qx[kk + 1] = v.y; qx[kk + 2] = v.z; qx[kk + 3] = v.w;
            }
            const int col = half * 32 + j;
            const float dist = exact_dist(stage, col, qx, S_X_OFFSET);
            float ex = exp2_neg_scaled(dist, p.c2, p.c2_lo) * phi_scale;
            if (col >= valid || t * NT + col == gi) ex = 0.f;
            const float delta = ex - __uint_as_float(kmax);
            corr += delta;
            const float4* xr = reinterpret_cast<const float4*>(stage + S_X_OFFSET + col * (FSK_D * 4));
#pragma unroll
            for (int kk = 0; kk < 4; ++kk) {
              const float4 xv = xr[kk];
              const float4 mv = __ldg(reinterpret_cast<const float4*>(p.mu) + kk);
              float4 cv = *reinterpret_cast<float4*>(wc + 4 * kk);
              cv.x = fmaf(delta, xv.x - mv.x, cv.x);
              cv.y = fmaf(delta, xv.y - mv.y, cv.y);
              cv.z = fmaf(delta, xv.z - mv.z, cv.z);
              cv.w = fmaf(delta, xv.w - mv.w, cv.w);
              *reinterpret_cast<float4*>(wc + 4 * kk) = cv;
            }
          }
          __syncwarp();
        }
        acc.add(cs);
        // fp16 hi / lo weights for the W product; the previous tile's W MMA
        // must have finished reading this query tile's weight columns.
        uint32_t hi[16], lo[16];
#pragma unroll
        for (int j = 0; j < 16; ++j) split_pack(e[2 * j], e[2 * j + 1], hi[j], lo[j]);
        if (g > 0 && !mbar_wait(&pfree[qt], (uint32_t)((g - 1) & 1), 29)) goto done;
        tc_fence_after();
        tmem_st16(tmem_base + lane_off + (uint32_t)(T_PHI + qt * NT + half * 16), hi);
        tmem_st16(tmem_base + lane_off + (uint32_t)(T_PHI + qt * NT + NT / 2 + half * 16), lo);
        tmem_st_wait();
        tc_fence_before();
        __syncwarp();
        if (lane == 0) {
          mbar_arrive(&pready[qt]);
          mbar_arrive(&empty[s]);
        }
        // read a W group that ended at the previous tile (its MMAs were
        // issued after that tile's weights, so by now they are usually done)
        const int pos = (t - t0) % S_GROUP;
        const bool last = pos == S_GROUP - 1 || t == t1 - 1;
        for (int pass = 0; pass < 2; ++pass) {
          const bool do_read = pass == 0 ? pend : (last && t == t1 - 1);
          if (!do_read) continue;
          const int par = grp & 1;
          if (!mbar_wait(&wfull[par], (uint32_t)((grp >> 1) & 1), 30)) goto done;
          tc_fence_after();
          uint32_t wv[8];
          tmem_ld8(tmem_base + lane_off + (uint32_t)(T_W + par * (SNQT * FSK_D) + qt * FSK_D + half * 8), wv);
          tmem_ld_wait();
          tc_fence_before();
          __syncwarp();
          if (lane == 0) mbar_arrive(&wempty[par]);
#pragma unroll
          for (int k = 0; k < 8; ++k) wacc[k].add(__uint_as_float(wv[k]));
          ++grp;
          if (pass == 0) pend = false;
        }
        if (last && t != t1 - 1) pend = true;
      }
      s_carry += acc.s + corr;
      // Combine the two column halves' corrections of this row for the 8
      // features this warp outputs.  Buffers alternate by unit parity; the
      // previous parity is cleared once every warp has passed this unit's
      // barrier (so has finished reading it).
      __syncwarp();
      if (lane == 0) mbar_arrive(cready);
      if (!mbar_wait(cready, (uint32_t)(k_unit & 1), 35)) goto done;
      {
        float* wc_next = wcorr + ((k_unit + 1) & 1) * WC_PAR + half * WC_HALF + wc_row;
#pragma unroll
        for (int k = 0; k < FSK_D; k += 4)
          *reinterpret_cast<float4*>(wc_next + k) = make_float4(0.f, 0.f, 0.f, 0.f);
      }
      if (gi < p.n) {
        p.ppdf[(int64_t)(2 * sp + half) * p.n + gi] = ((double)acc.s + (double)acc.c + (double)corr) * p_unscale;
        double* wrow = p.pw + ((int64_t)sp * p.n + gi) * FSK_D + half * 8;
        const float* c0 = wcorr + (k_unit & 1) * WC_PAR + wc_row + half * 8;
        const float* c1 = c0 + WC_HALF;
#pragma unroll
        for (int k = 0; k < 8; ++k)
          wrow[k] = ((double)wacc[k].s + (double)wacc[k].c) * w_unscale +
                    ((double)c0[k] + (double)c1[k]) * c_unscale;
      }
    }
  }
done:
  // Exit path (also after a timed-out wait): let this CTA's bulk copies and
  // MMAs finish before shared and tensor memory are released.
  if (warp == S_PRODUCER_WARP && lane == 0) {
    for (int64_t i = imax<int64_t>(0, n_stage_copies - SNS); i < n_stage_copies; ++i)
      mbar_wait(&full[i % SNS], (uint32_t)((i / SNS) & 1), 32);
    if (n_query_copies > 0) mbar_wait(qready, (uint32_t)((n_query_copies - 1) & 1), 33);
  }
  if (warp == S_MMA_WARP && lane == 0) {
    mma_commit(drain);
    mbar_wait(drain, 0, 34);
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == S_MMA_WARP) tmem_dealloc(tmem_base, S_TMEM_COLS);
}

// Data stage image: [H (64 x 32 fp16) | L (64 x 16 fp16) | XT hi (16 x 64 fp16)
// | XT lo | x (64 x 16 FP32)].  XT rows are features, K-major over the points.
__global__ void prep_score_data_kernel(const float* __restrict__ x, int64_t n, int64_t n_pad,
                                       const float* __restrict__ mu, float c2,
                                       const TcScales* __restrict__ sc, uint8_t* __restrict__ img) {
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n_pad) return;
  const bool ok = j < n;
  float xo[FSK_D], v[FSK_D];
  float nrm = 0.f;
  const float ws = ldexpf(1.f, sc->pad[2]);
  uint8_t* tile = img + (j / NT) * (int64_t)S_STAGE_BYTES;
  const int r = (int)(j % NT);
#pragma unroll
  for (int k = 0; k < FSK_D; ++k) {
    xo[k] = ok ? x[j * FSK_D + k] : 0.f;
    const float cv = xo[k] - mu[k];
    nrm = fmaf(cv, cv, nrm);
    v[k] = ok ? cv * sc->x_scale : 0.f;
    const float w = ok ? cv * ws : 0.f;
    const __half wh = __float2half_rn(w);
    const __half wl = __float2half_rn(w - __half2float(wh));
    put_h(tile + S_XTH_OFFSET, k, r, XT_ROW_BYTES, wh);
    put_h(tile + S_XTL_OFFSET, k, r, XT_ROW_BYTES, wl);
  }
  const float beta = ok ? -c2 * nrm * sc->b_scale : 0.f;
  write_operand_row(tile, tile + B_H_BYTES, r, v, beta, ok ? ldexpf(1.f, sc->pad[0]) : 0.f, true);
  float4* xr = reinterpret_cast<float4*>(tile + S_X_OFFSET + r * (FSK_D * 4));
#pragma unroll
  for (int k = 0; k < 4; ++k) xr[k] = make_float4(xo[4 * k], xo[4 * k + 1], xo[4 * k + 2], xo[4 * k + 3]);
}

}  // namespace

TcPlan plan_score16(int64_t n) {
  TcPlan pl;
  pl.m_pad = (n + SNQT * QT - 1) / (SNQT * QT) * (SNQT * QT);
  pl.n_tiles = (n + NT - 1) / NT;
  pl.n_pad = pl.n_tiles * NT;
  pl.q_blocks = pl.m_pad / (SNQT * QT);
  plan_splits(pl);
  return pl;
}

size_t tc_score16_ws_bytes(const TcPlan& pl, int64_t n) {
  size_t b = 0;
  b += align_up(sizeof(TcScales), 256);
  b += align_up((size_t)pl.q_blocks * S_A_BYTES, 256);
  b += align_up((size_t)pl.m_pad * FSK_D * sizeof(float), 256);
  b += align_up((size_t)pl.n_tiles * S_STAGE_BYTES, 256);
  b += align_up((size_t)2 * pl.splits * n * sizeof(double), 256);
  b += align_up((size_t)pl.splits * n * FSK_D * sizeof(double), 256);
  return b;
}

int launch_score16_tc(const float* x, int64_t n, const float* mu, double h, const TcPlan& pl, WsCarver& c,
                      double** ppdf_out, double** pw_out, cudaStream_t s) {
  TcScales* sc = c.take<TcScales>(1);
  uint8_t* qimg = c.take<uint8_t>((size_t)pl.q_blocks * S_A_BYTES);
  float* qexact = c.take<float>((size_t)pl.m_pad * FSK_D);
  uint8_t* ximg = c.take<uint8_t>((size_t)pl.n_tiles * S_STAGE_BYTES);
  double* ppdf = c.take<double>((size_t)2 * pl.splits * n);
  double* pw = c.take<double>((size_t)pl.splits * n * FSK_D);
  if (!c.fits()) return FSK_ERR_WORKSPACE_TOO_SMALL;
  *ppdf_out = ppdf;
  *pw_out = pw;

  const double c2d = FSK_LOG2E / (2.0 * h * h);
  const float c2 = (float)c2d;
  const float c2_lo = (float)(c2d - (double)c2);
  scale_init_kernel<<<1, 32, 0, s>>>(sc);
  count_launch();
  const int sblocks = (int)imin<int64_t>(1024, (n + 255) / 256);
  scale_stats_kernel<<<sblocks, 256, 0, s>>>(x, n, mu, c2, 1, PHI_LOG2_SCALE, sc);
  count_launch();
  scale_stats_kernel<<<sblocks, 256, 0, s>>>(x, n, mu, c2, 0, 0.f, sc);
  count_launch();
  scale_select_kernel<<<1, 32, 0, s>>>(sc);
  count_launch();
  prep_score_data_kernel<<<(unsigned)((pl.n_pad + 255) / 256), 256, 0, s>>>(x, n, pl.n_pad, mu, c2, sc, ximg);
  count_launch();
  prep_query_kernel<<<(unsigned)((pl.m_pad + 255) / 256), 256, 0, s>>>(x, n, pl.m_pad, mu, c2, PHI_LOG2_SCALE,
                                                                        sc, qimg, qexact);
  count_launch();

  ScParams p;
  p.qimg = qimg;
  p.ximg = ximg;
  p.qexact = qexact;
  p.scales = sc;
  p.mu = mu;
  p.n = n;
  p.n_tiles = pl.n_tiles;
  p.q_blocks = pl.q_blocks;
  p.splits = pl.splits;
  p.tiles_per_split = pl.tiles_per_split;
  p.c2 = c2;
  p.c2_lo = c2_lo;
  p.ppdf = ppdf;
  p.pw = pw;
  cudaError_t e = cudaFuncSetAttribute(score16_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       S_SMEM_BYTES);
  if (e != cudaSuccess) return cuda_status(e);
  TimerScope ts(K_SCORE16_TC, (double)n * (double)n, s);
  score16_tc_kernel<<<pl.grid, S_THREADS, S_SMEM_BYTES, s>>>(p);
  count_launch();
  return cuda_status(cudaGetLastError());
}

// ---- layout probe: D (128 x 16) = A (128 x 64) . B (16 x 64)^T, fp16 ------------
// A is stored to tensor memory with tcgen05.st (two fp16 per 32-bit column,
// row = TMEM lane) and read by tcgen05.mma as its A operand; B uses the
// transposed-feature image layout of the score kernel's data stages (rows of
// 64 points, 128 B).  Four K=16 steps.  Inputs FP32, rounded to fp16 here.
namespace {
__global__ void __launch_bounds__(128, 1) mma_ts_probe_kernel(const float* __restrict__ a,
                                                              const float* __restrict__ b,
                                                              float* __restrict__ d) {
  __shared__ __align__(1024) uint8_t sb[XT_BYTES];
  __shared__ uint64_t bar;
  __shared__ uint32_t slot;
  const int t = threadIdx.x;
  const int warp = t >> 5;
  for (int i = t; i < FSK_D * NT; i += 128)
    put_h(sb, i / NT, i % NT, XT_ROW_BYTES, __float2half_rn(b[i]));
  if (t == 0) {
    mbar_init(&bar, 1);
    fence_barrier_init();
  }
  if (warp == 0) {
    tmem_alloc(&slot, 128);
    tmem_relinquish();
  }
  fence_proxy_async_smem();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tbase = slot;
  const uint32_t lane_off = (uint32_t)(warp * 32) << 16;
#pragma unroll
  for (int c = 0; c < 2; ++c) {
    uint32_t v[16];
#pragma unroll
    for (int j = 0; j < 16; ++j) {
      const __half2 h2 = __floats2half2_rn(a[t * NT + c * 32 + 2 * j], a[t * NT + c * 32 + 2 * j + 1]);
      v[j] = *reinterpret_cast<const uint32_t*>(&h2);
    }
    tmem_st16(tbase + lane_off + (uint32_t)(c * 16), v);
  }
  tmem_st_wait();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (t == 0) {
    const uint32_t idesc = idesc_f16_f32(QT, FSK_D);
    for (int ks = 0; ks < NT / 16; ++ks)
      mma_f16_ts(tbase + 64, tbase + (uint32_t)(8 * ks),
                 smem_desc_kmajor(smem_u32(sb) + 256 * ks, 128, 8 * XT_ROW_BYTES), idesc, ks ? 1u : 0u);
    mma_commit(&bar);
  }
  __syncwarp();
  const bool ok = mbar_wait(&bar, 0, 31);
  tc_fence_after();
  if (ok) {
    uint32_t r[16];
    tmem_ld16(tbase + lane_off + 64u, r);
    tmem_ld_wait();
#pragma unroll
    for (int j = 0; j < 16; ++j) d[t * FSK_D + j] = __uint_as_float(r[j]);
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 0) tmem_dealloc(tbase, 128);
}
}  // namespace

int launch_mma_ts_probe(const float* a, const float* b, float* d, cudaStream_t s) {
  mma_ts_probe_kernel<<<1, 128, 0, s>>>(a, b, d);
  count_launch();
  return cuda_status(cudaGetLastError());
}

}  // namespace tc
}  // namespace fsk
