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
// How (per 256-query x 64-point tile):
//  * S = the log2-domain exponent a2 + 15, three-part fp16 product of the
//    operand images of the KDE kernel (fsk_tc_kde16.cu): seven tcgen05.mma
//    per query tile, the query operand (hi | mid | lo rows) read from tensor
//    memory, where the epilogue warps copy it at the start of each unit (an
//    M=128, K=16 MMA with both operands in shared memory costs ~48 cycles,
//    bound by the operand reads; with A in tensor memory it runs at the
//    math rate when enough threads issue).  The +15 rides in the query's
//    bias term, so 2^S = phi * 2^15 and the weights keep fp16 normal range
//    down to phi ~ 2^-29.
//  * Epilogue: tcgen05.ld, ex2.approx, pdf chunk sums, the exact near-pair
//    recompute of the KDE kernel (the recomputed value also replaces the
//    approximate one in the weights), then the weights are split into fp16
//    hi + lo and stored with tcgen05.st over the tensor-memory columns their
//    S came from.
//  * W += Phi_hi [X_hi | X_lo] + Phi_lo X_hi: tcgen05.mma with the A operand
//    (weights, M=128 x K=16 per step) read from tensor memory and the B
//    operand ((x_j - mu) 2^ew as fp16 hi and lo rows, K-major over the data
//    points) from the data stage, FP32 accumulation over a group of S_GROUP
//    tiles, then added into compensated FP32 sums.  Four issuing threads,
//    one per (query tile, weight part), each with its own accumulator: a
//    single thread issues an M=128, K=16, N=32 MMA every ~46 cycles, four
//    reach the tensor core's math rate.
//
// Pipeline (one persistent CTA per SM, 23 warps):
//   warp 16 : producer (bulk copies of query images per unit, data stages).
//   warps 17, 18 : issue S for query tiles 0 and 1 (one lane each), up to
//             NBUF tiles ahead of W; warp 17 owns TMEM.
//   warps 19-22 : issue the weighted-sum MMAs of (query tile, weight part)
//             (0, hi), (0, lo), (1, hi), (1, lo).
//   warps 0-15: epilogue; warp w: query tile w/8, data-column half (w/4)&1,
//             TMEM lane quarter w&3.  The two column halves of a row keep
//             separate pdf partials (written as two virtual splits) and
//             read disjoint halves of the weighted-sum features.
// TMEM: A operands [2 query tiles][hi 16 | mid 8 | lo 8]  (columns 0-63)
//       | S / weights [NBUF buffers][2 query tiles][64]  (64-319)
//       | W [2 group parities][2 query tiles][hi part 32 | lo part 16]  (320-511).
#include <cuda_fp16.h>

#include "fsk_kernels.cuh"
#include "fsk_tc.cuh"
#include "fsk_tc_ops.cuh"

namespace fsk {
namespace tc {

namespace {

constexpr int SNQT = 2;                                    // query tiles per unit (256 queries)
constexpr int SNS = 4;                                     // data stages
constexpr int XT_ROW_BYTES = NT * 2;                       // one feature row over 64 points, fp16
constexpr int XT_BYTES = FSK_D * XT_ROW_BYTES;             // 2 KB
constexpr int S_XTH_OFFSET = B_L_OFFSET + B_L_BYTES;       // 8 KB
constexpr int S_XTL_OFFSET = S_XTH_OFFSET + XT_BYTES;      // 10 KB
constexpr int S_X_OFFSET = S_XTL_OFFSET + XT_BYTES;        // 12 KB: original FP32 rows
constexpr int S_STAGE_BYTES = S_X_OFFSET + NT * FSK_D * 4; // 16 KB
constexpr int S_A_BYTES = SNQT * A_TILE_BYTES;             // 32 KB
constexpr int S_EPI_WARPS = 8 * SNQT;
constexpr int S_PRODUCER_WARP = S_EPI_WARPS;
constexpr int S_MMA_WARP = S_EPI_WARPS + 1;     // issues the S MMAs of query tile 0, owns TMEM
constexpr int S_MMA_WARP2 = S_EPI_WARPS + 2;    // issues the S MMAs of query tile 1
constexpr int W_MMA_WARP = S_EPI_WARPS + 3;     // first of the W_ISSUERS weighted-sum issuers
constexpr int W_ISSUERS = 2 * SNQT;             // (query tile, weight part hi / lo)
constexpr int S_THREADS = (S_EPI_WARPS + 3 + W_ISSUERS) * 32;
constexpr int S_GROUP = 16;                                // data tiles per W accumulation
constexpr int NBUF = 2;                                    // S / weight buffers in TMEM
constexpr int WN = 2 * FSK_D;                              // W MMA N, hi weights: X_hi and X_lo rows
constexpr int WN_LO = FSK_D;                               // W MMA N, lo weights: X_hi rows
constexpr int T_A = 0;                                     // [SNQT][32]: hi 16 | mid 8 | lo 8
constexpr int T_S = 64;
constexpr int T_W = T_S + NBUF * SNQT * NT;                // 320
constexpr int W_TILE_COLS = WN + WN_LO;                    // 48 per (parity, query tile)
constexpr int S_TMEM_COLS = 512;
// exact-recompute corrections of the weighted sums: [unit parity][column half][256 rows][16] FP32
// original coordinates of the unit's 256 queries (exact near-pair recompute)
constexpr int S_QX_OFFSET = S_A_BYTES;
constexpr int S_QX_BYTES = SNQT * QT * FSK_D * 4;                    // 16 KB
constexpr int S_B_OFFSET = S_QX_OFFSET + S_QX_BYTES;
constexpr int S_BAR_OFFSET = S_B_OFFSET + SNS * S_STAGE_BYTES;
constexpr int S_WCORR_OFFSET = S_BAR_OFFSET + 512;
constexpr int S_WCORR_BYTES = 2 * 2 * SNQT * QT * FSK_D * 4;          // 64 KB
// compensated per-thread weighted-sum accumulators (8 features, value + error),
// float4 planes [s0-3, s4-7, c0-3, c4-7][epilogue thread]
constexpr int S_WACC_OFFSET = S_WCORR_OFFSET + S_WCORR_BYTES;
constexpr int S_WACC_BYTES = 4 * S_EPI_WARPS * 32 * 16;                // 32 KB
constexpr int S_MU_OFFSET = S_WACC_OFFSET + S_WACC_BYTES;             // data mean, 16 FP32
constexpr int S_SMEM_BYTES = S_MU_OFFSET + FSK_D * 4;
constexpr float PHI_LOG2_SCALE = 15.0f;                    // weights are phi * 2^15
// Three-part S product as in the KDE kernel, so the same near-pair threshold
// (1/8 of the running sum, the excluded self pair's weight included).
constexpr float SCORE_NEAR_FRACTION = NEAR_FRACTION;
static_assert(T_W + 2 * SNQT * W_TILE_COLS <= S_TMEM_COLS, "TMEM budget");
static_assert(S_XTL_OFFSET == S_XTH_OFFSET + 16 * XT_ROW_BYTES, "X_lo rows follow X_hi rows (one N=32 operand)");
static_assert(S_STAGE_BYTES % 16 == 0 && S_A_BYTES % 16 == 0 && S_QX_BYTES % 16 == 0, "bulk copy granularity");
static_assert(S_SMEM_BYTES <= 227 * 1024, "shared memory");
static_assert((2 * SNS + 3 * NBUF * SNQT + 4 * SNQT + SNQT + 4) * 8 + 4 <= 512, "barrier area");

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

// f32 pair -> packed fp16 hi and lo parts (hi + lo = v to ~22 bits).  The
// residual v - hi is exact in FP32 (hi holds v's leading 11 bits) and comes
// from one mixed-precision FMA per value, fp16 hi times -1 plus the FP32 v.
__device__ __forceinline__ void split_pack(float v0, float v1, uint32_t& hi, uint32_t& lo) {
  asm("cvt.rn.f16x2.f32 %0, %1, %2;" : "=r"(hi) : "f"(v1), "f"(v0));
  float r0, r1;
  const unsigned short minus_one = 0xBC00;   // fp16 -1
  asm("{\n\t.reg .b16 h0, h1;\n\tmov.b32 {h0, h1}, %2;\n\t"
      "fma.rn.f32.f16 %0, h0, %5, %3;\n\tfma.rn.f32.f16 %1, h1, %5, %4;\n\t}"
      : "=f"(r0), "=f"(r1)
      : "r"(hi), "f"(v0), "f"(v1), "h"(minus_one));
  asm("cvt.rn.f16x2.f32 %0, %1, %2;" : "=r"(lo) : "f"(r1), "f"(r0));
}

// Walks the (unit, data tile) sequence of one CTA: units are (query block,
// data split), each split covers tiles [t0, t1).
struct TileCursor {
  int u, u_end, splits, tps, n_tiles, t0, t1, t;
  __device__ void start(int ub, int ue, int sp_count, int tiles_per_split, int tiles) {
    u = ub; u_end = ue; splits = sp_count; tps = tiles_per_split; n_tiles = tiles;
    enter();
  }
  __device__ void enter() {
    if (u < u_end) {
      t0 = (u % splits) * tps;
      t1 = min(n_tiles, t0 + tps);
      t = t0;
    }
  }
  __device__ bool done() const { return u >= u_end; }
  __device__ void next() {
    if (++t >= t1) {
      ++u;
      enter();
    }
  }
};

__global__ void __launch_bounds__(S_THREADS, 1) score16_tc_kernel(ScParams p) {
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t* sA = smem_raw;
  const float* sQ = reinterpret_cast<const float*>(smem_raw + S_QX_OFFSET);
  uint8_t* sB = smem_raw + S_B_OFFSET;
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem_raw + S_BAR_OFFSET);
  float* sMu = reinterpret_cast<float*>(smem_raw + S_MU_OFFSET);
  uint64_t* full = bars;                          // [SNS] stage loaded
  uint64_t* empty = bars + SNS;                   // [SNS] stage consumed (W MMAs + epilogue)
  uint64_t* tfull = bars + 2 * SNS;               // [NBUF][SNQT] S written
  // [NBUF][SNQT] weights stored.  One barrier per buffer and query tile: a
  // buffer's barrier cannot complete again before its weights are consumed.
  uint64_t* pready = tfull + NBUF * SNQT;
  uint64_t* sfree = pready + NBUF * SNQT;         // [NBUF][SNQT] weights read by both W parts
  uint64_t* wfull = sfree + NBUF * SNQT;          // [2 parities][SNQT] W group accumulated
  uint64_t* wempty = wfull + 2 * SNQT;            // [2 parities][SNQT] W group read
  uint64_t* aready = wempty + 2 * SNQT;           // [SNQT] unit's A operand in TMEM
  uint64_t* qready = aready + SNQT;
  uint64_t* qempty = qready + 1;
  uint64_t* drain = qready + 2;                   // all MMAs of this CTA finished (exit path)
  uint64_t* cready = qready + 3;                  // unit's W corrections written (epilogue warps)
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(qready + 4);
  float* wcorr = reinterpret_cast<float*>(smem_raw + S_WCORR_OFFSET);
  float4* wacc = reinterpret_cast<float4*>(smem_raw + S_WACC_OFFSET);
  int64_t n_stage_copies = 0, n_query_copies = 0;   // producer: bulk copies issued

  const int warp = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;

  if (threadIdx.x == 0) {
    for (int s = 0; s < SNS; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], W_ISSUERS + S_EPI_WARPS);   // the W threads' commits + every epilogue warp
    }
    for (int i = 0; i < NBUF * SNQT; ++i) {
      mbar_init(&tfull[i], 1);
      mbar_init(&pready[i], 8);
      mbar_init(&sfree[i], 2);
    }
    for (int i = 0; i < 2 * SNQT; ++i) {
      mbar_init(&wfull[i], 2);
      mbar_init(&wempty[i], 8);
    }
    for (int a = 0; a < SNQT; ++a) mbar_init(&aready[a], 8);
    mbar_init(qready, 1);
    mbar_init(qempty, S_EPI_WARPS);
    mbar_init(drain, 2 + W_ISSUERS);
    mbar_init(cready, S_EPI_WARPS);
    fence_barrier_init();
  }
  if (warp == S_MMA_WARP) {
    tmem_alloc(tmem_slot, S_TMEM_COLS);
    tmem_relinquish();
  }
  if (threadIdx.x < FSK_D) sMu[threadIdx.x] = p.mu[threadIdx.x];
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem_base = *tmem_slot;
  const int64_t units = p.q_blocks * p.splits;
  const int64_t u_begin = (int64_t)blockIdx.x * units / gridDim.x;
  const int64_t u_end = (int64_t)(blockIdx.x + 1) * units / gridDim.x;

  if (warp == S_PRODUCER_WARP) {
    // whole warp runs the loop (32-bit stage / phase counters), lane 0 copies
    {
      int64_t& g = n_stage_copies;
      int64_t& k = n_query_copies;
      int st = 0;
      uint32_t ph = 0;
      for (int64_t u = u_begin; u < u_end; ++u) {
        const int64_t qb = u / p.splits, sp = u % p.splits;
        if (!__all_sync(0xffffffffu, mbar_wait(qempty, (uint32_t)((k & 1) ^ 1), 21))) goto done;
        if (lane == 0) {
          mbar_arrive_expect_tx(qready, S_A_BYTES + S_QX_BYTES);
          bulk_g2s(sA, p.qimg + qb * (int64_t)S_A_BYTES, S_A_BYTES, qready);
          bulk_g2s(smem_raw + S_QX_OFFSET, p.qexact + qb * (int64_t)(SNQT * QT * FSK_D), S_QX_BYTES, qready);
        }
        ++k;
        const int64_t t0 = sp * p.tiles_per_split;
        const int64_t t1 = imin<int64_t>(p.n_tiles, t0 + p.tiles_per_split);
        const uint8_t* src = p.ximg + t0 * (int64_t)S_STAGE_BYTES;
        for (int64_t t = t0; t < t1; ++t, src += S_STAGE_BYTES) {
          if (!__all_sync(0xffffffffu, mbar_wait(&empty[st], ph ^ 1u, 22))) goto done;
          if (lane == 0) {
            mbar_arrive_expect_tx(&full[st], S_STAGE_BYTES);
            bulk_g2s(sB + st * S_STAGE_BYTES, src, S_STAGE_BYTES, &full[st]);
          }
          ++g;
          if (++st == SNS) {
            st = 0;
            ph ^= 1u;
          }
        }
      }
    }
  } else if (warp == S_MMA_WARP || warp == S_MMA_WARP2) {
    // S(g) of one query tile for every tile, up to NBUF tiles ahead of W:
    // buffer g % NBUF is reused once both W parts of tile g - NBUF have read
    // its weights (sfree).  S and W are issued by different threads because
    // tcgen05.commit tracks every earlier MMA of its thread.  The whole warp
    // runs the loop (warp-uniform values stay in uniform registers); lane 0
    // issues the MMAs and commits.
    {
      const int a = warp == S_MMA_WARP ? 0 : 1;
      const uint32_t idesc_s = idesc_f16_f32(QT, NT);
      const uint32_t a_h = tmem_base + (uint32_t)(T_A + a * 32);   // hi: features | bias; mid at +16, lo at +24
      // descriptors are advanced by adding (bytes >> 4) to the start-address
      // field (shared addresses stay below 2^18 B, so the field cannot carry)
      const uint32_t b0 = smem_u32(sB);
      const uint64_t dh0 = smem_desc_kmajor(b0, 128, 8 * H_ROW_BYTES);
      const uint64_t dm0 = smem_desc_kmajor(b0 + B_M_OFFSET, 128, 8 * L_ROW_BYTES);
      const uint64_t dl0 = smem_desc_kmajor(b0 + B_L_OFFSET, 128, 8 * L_ROW_BYTES);
      TileCursor cs;
      cs.start((int)u_begin, (int)u_end, (int)p.splits, (int)p.tiles_per_split, (int)p.n_tiles);
      int gs = 0, ku = 0;
      while (!cs.done()) {
        const int s = gs % SNS;
        const int b = gs % NBUF;
        if (cs.t == cs.t0) {   // first tile of a unit: its A operand in TMEM
          if (!__all_sync(0xffffffffu, mbar_wait(&aready[a], (uint32_t)(ku & 1), 23))) goto done;
          ++ku;
        }
        if (gs >= NBUF &&
            !__all_sync(0xffffffffu, mbar_wait(&sfree[b * SNQT + a], (uint32_t)(((gs / NBUF) - 1) & 1), 25)))
          goto done;
        if (!__all_sync(0xffffffffu, mbar_wait(&full[s], (uint32_t)((gs / SNS) & 1), 24))) goto done;
        tc_fence_after();
        const uint64_t so = (uint64_t)((s * S_STAGE_BYTES) >> 4);
        const uint32_t d = tmem_base + (uint32_t)(T_S + b * (SNQT * NT) + a * NT);
        const uint64_t b_h = dh0 + so;
        // three-part product, small terms first (the order of mma_s_tile)
        const uint64_t b_m = dm0 + so, b_l = dl0 + so;
        if (lane == 0) {
          mma_f16_ts(d, a_h + 16u, b_m, idesc_s, 0u);                    // mid . mid
          mma_f16_ts(d, a_h, b_l, idesc_s, 1u);                          // hi . lo
          mma_f16_ts(d, a_h + 24u, b_h, idesc_s, 1u);                    // lo . hi
          mma_f16_ts(d, a_h, b_m, idesc_s, 1u);                          // hi . mid
          mma_f16_ts(d, a_h + 16u, b_h, idesc_s, 1u);                    // mid . hi
          mma_f16_ts(d, a_h, b_h, idesc_s, 1u);                          // hi . hi
          mma_f16_ts(d, a_h + 8u, b_h + (uint64_t)(256 >> 4), idesc_s, 1u);   // bias . bias
          mma_commit(&tfull[b * SNQT + a]);
        }
        __syncwarp();
        ++gs;
        cs.next();
      }
    }
  } else if (warp >= W_MMA_WARP) {
    // W(g) of one (query tile, weight part) once the epilogue warps of that
    // query tile have stored tile g's weights (whole warp runs the loop, lane
    // 0 issues).
    {
      const int wi = warp - W_MMA_WARP;
      const int a = wi >> 1, part = wi & 1;   // part 0: hi weights x [X_hi | X_lo]; 1: lo weights x X_hi
      const uint32_t idesc_w = idesc_f16_f32(QT, part ? WN_LO : WN);
      const uint64_t dx0 = smem_desc_kmajor(smem_u32(sB) + S_XTH_OFFSET, 128, 8 * XT_ROW_BYTES);
      TileCursor cw;
      cw.start((int)u_begin, (int)u_end, (int)p.splits, (int)p.tiles_per_split, (int)p.n_tiles);
      int gw = 0, grp = 0;
      while (!cw.done()) {
        const int b = gw % NBUF;
        const int s = gw % SNS;
        const int pos = (cw.t - cw.t0) % S_GROUP;
        const bool first = pos == 0;
        const bool last = pos == S_GROUP - 1 || cw.t == cw.t1 - 1;
        const int par = grp & 1;
        if (first &&
            !__all_sync(0xffffffffu, mbar_wait(&wempty[par * SNQT + a], (uint32_t)(((grp >> 1) & 1) ^ 1), 26)))
          goto done;
        if (!__all_sync(0xffffffffu, mbar_wait(&pready[b * SNQT + a], (uint32_t)((gw / NBUF) & 1), 27))) goto done;
        tc_fence_after();
        const uint64_t xd0 = dx0 + (uint64_t)((s * S_STAGE_BYTES) >> 4);
        const uint32_t ph = tmem_base + (uint32_t)(T_S + b * (SNQT * NT) + a * NT + part * 16);
        const uint32_t d = tmem_base + (uint32_t)(T_W + par * (SNQT * W_TILE_COLS) + a * W_TILE_COLS + part * WN);
        if (lane == 0) {
#pragma unroll
          for (int ks = 0; ks < NT / 16; ++ks) {
            // data columns 16 ks .. +15: column half ks/2; weights hi at +0, lo at +16
            const uint32_t wa = ph + (uint32_t)(32 * (ks >> 1) + 8 * (ks & 1));
            mma_f16_ts(d, wa, xd0 + (uint64_t)(ks * (256 >> 4)), idesc_w, (first && ks == 0) ? 0u : 1u);
          }
          mma_commit(&sfree[b * SNQT + a]);
          mma_commit(&empty[s]);
          if (last) mma_commit(&wfull[par * SNQT + a]);
        }
        __syncwarp();
        if (last) ++grp;
        ++gw;
        cw.next();
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
    int s = 0;   // data stage of tile g (g % SNS, advanced per tile)
    // valid columns of the last (possibly ragged) data tile; every other tile has NT
    const int last_t = (int)p.n_tiles - 1;
    const int last_valid = (int)(p.n - (int64_t)last_t * NT);
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
      // The unit's query images: this row's A operand to TMEM (column half 0
      // copies the hi row, half 1 the mid and lo rows).  The S MMAs of the previous
      // unit have all completed: this warp consumed their accumulators.
      if (!__all_sync(0xffffffffu, mbar_wait(qready, (uint32_t)(k_unit & 1), 36))) goto done;
      {
        const uint8_t* tile = sA + qt * A_TILE_BYTES;
        const uint32_t ta = tmem_base + lane_off + (uint32_t)(T_A + qt * 32);
        if (half == 0) {
          uint32_t w[16];
#pragma unroll
          for (int c = 0; c < 4; ++c) {
            const uint4 v = *reinterpret_cast<const uint4*>(tile + cm_offset(row, 8 * c, H_ROW_BYTES));
            w[4 * c] = v.x; w[4 * c + 1] = v.y; w[4 * c + 2] = v.z; w[4 * c + 3] = v.w;
          }
          tmem_st16(ta, w);
        } else {
          uint32_t w[16];   // mid row, then lo row
#pragma unroll
          for (int c = 0; c < 4; ++c) {
            const uint4 v = *reinterpret_cast<const uint4*>(tile + (c < 2 ? A_M_OFFSET : A_L_OFFSET) +
                                                            cm_offset(row, 8 * (c & 1), L_ROW_BYTES));
            w[4 * c] = v.x; w[4 * c + 1] = v.y; w[4 * c + 2] = v.z; w[4 * c + 3] = v.w;
          }
          tmem_st16(ta + 16u, w);
        }
        tmem_st_wait();
        tc_fence_before();
        __syncwarp();
        if (lane == 0) mbar_arrive(&aready[qt]);
      }
      Comp acc{0.f, 0.f};
      float corr = 0.f;
      constexpr int EPI_T = S_EPI_WARPS * 32;
#pragma unroll
      for (int k = 0; k < 4; ++k) wacc[k * EPI_T + threadIdx.x] = make_float4(0.f, 0.f, 0.f, 0.f);
      const int t0 = sp * tps;
      const int t1 = imin(n_tiles, t0 + tps);
      bool pend = false;     // a W group ended at the previous tile and is not read yet
      for (int t = t0; t < t1; ++t, ++g, s = (s + 1 == SNS) ? 0 : s + 1) {
        const int b = g % NBUF;
        const int valid = t == last_t ? last_valid : NT;
        if (!__all_sync(0xffffffffu, mbar_wait(&tfull[b * SNQT + qt], (uint32_t)((g / NBUF) & 1), 28))) goto done;
        tc_fence_after();
        const uint8_t* stage = sB + s * S_STAGE_BYTES;
        // this warp's 32 S columns; its weights go back into the same columns
        const uint32_t my_cols = tmem_base + lane_off + (uint32_t)(T_S + b * (SNQT * NT) + qt * NT + half * 32);
        uint32_t r[32];
        tmem_ld32(my_cols, r);
        tmem_ld_wait();
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
        const bool trig = cs > (s_carry + acc.s + cs) * SCORE_NEAR_FRACTION;
        if (__any_sync(0xffffffffu, trig)) {
          // The chunk's largest weight is recomputed exactly (argmax on keys
          // = value bits with the column in the low 5 bits, as in the KDE
          // kernel).  With A the keyed approximation, the pdf gets ex - A
          // (corr) and the weighted sum (ex - A)(x_j - mu) (shared-memory
          // corrections), so both see the same weight e_j - A + ex.
          if (trig) {
            // four interleaved max chains keep the register peak low
            uint32_t k0 = 0u, k1 = 0u, k2 = 0u, k3 = 0u;
#pragma unroll
            for (int j = 0; j < 32; j += 4) {
              k0 = max(k0, (__float_as_uint(e[j]) & ~31u) | (uint32_t)j);
              k1 = max(k1, (__float_as_uint(e[j + 1]) & ~31u) | (uint32_t)(j + 1));
              k2 = max(k2, (__float_as_uint(e[j + 2]) & ~31u) | (uint32_t)(j + 2));
              k3 = max(k3, (__float_as_uint(e[j + 3]) & ~31u) | (uint32_t)(j + 3));
            }
            const uint32_t kmax = max(max(k0, k1), max(k2, k3));
            const int j = (int)(kmax & 31u);
            const int col = half * 32 + j;
            const float4* xr = reinterpret_cast<const float4*>(stage + S_X_OFFSET + col * (FSK_D * 4));
            // exact squared distance, four features at a time
            const float4* qr = reinterpret_cast<const float4*>(sQ + (qt * QT + row) * FSK_D);
            float d0 = 0.f, d1 = 0.f, d2 = 0.f, d3 = 0.f;
#pragma unroll
            for (int kk = 0; kk < 4; ++kk) {
              const float4 qv = qr[kk], xv = xr[kk];
              const float a0 = qv.x - xv.x, a1 = qv.y - xv.y, a2 = qv.z - xv.z, a3 = qv.w - xv.w;
              d0 = fmaf(a0, a0, d0);
              d1 = fmaf(a1, a1, d1);
              d2 = fmaf(a2, a2, d2);
              d3 = fmaf(a3, a3, d3);
            }
            const float dist = (d0 + d1) + (d2 + d3);
            float ex = exp2_neg_scaled(dist, p.c2, p.c2_lo) * phi_scale;
            if (col >= valid || t * NT + col == gi) ex = 0.f;
            const float delta = ex - __uint_as_float(kmax);
            corr += delta;
#pragma unroll
            for (int kk = 0; kk < 4; ++kk) {
              const float4 xv = xr[kk];
              const float4 mv = reinterpret_cast<const float4*>(sMu)[kk];
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
        // fp16 hi / lo weights for the W product, written over this warp's
        // S columns (hi: 16 columns of packed pairs, then lo), eight pairs at
        // a time to keep the register peak low
#pragma unroll
        for (int h8 = 0; h8 < 2; ++h8) {
          uint32_t hi[8], lo[8];
#pragma unroll
          for (int j = 0; j < 8; ++j) split_pack(e[16 * h8 + 2 * j], e[16 * h8 + 2 * j + 1], hi[j], lo[j]);
          tmem_st8(my_cols + (uint32_t)(8 * h8), hi);
          tmem_st8(my_cols + (uint32_t)(16 + 8 * h8), lo);
        }
        tmem_st_wait();
        tc_fence_before();
        __syncwarp();
        if (lane == 0) {
          mbar_arrive(&pready[b * SNQT + qt]);
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
          if (!__all_sync(0xffffffffu, mbar_wait(&wfull[par * SNQT + qt], (uint32_t)((grp >> 1) & 1), 30))) goto done;
          tc_fence_after();
          // this warp's 8 features: hi weights x X_hi, hi weights x X_lo, lo weights x X_hi
          uint32_t wv[8], wl[8], wm[8];
          const uint32_t wcol = tmem_base + lane_off + (uint32_t)(T_W + par * (SNQT * W_TILE_COLS) + qt * W_TILE_COLS + half * 8);
          tmem_ld8(wcol, wv);
          tmem_ld8(wcol + FSK_D, wl);
          tmem_ld8(wcol + WN, wm);
          tmem_ld_wait();
#pragma unroll
          for (int k = 0; k < 8; ++k)
            wv[k] = __float_as_uint(__uint_as_float(wv[k]) + (__uint_as_float(wl[k]) + __uint_as_float(wm[k])));
          tc_fence_before();
          __syncwarp();
          if (lane == 0) mbar_arrive(&wempty[par * SNQT + qt]);
          {
            float4 s0 = wacc[threadIdx.x], s1 = wacc[EPI_T + threadIdx.x];
            float4 e0 = wacc[2 * EPI_T + threadIdx.x], e1 = wacc[3 * EPI_T + threadIdx.x];
            Comp c;
#define FSK_WADD(S, E, V) c = Comp{S, E}; c.add(__uint_as_float(V)); S = c.s; E = c.c;
            FSK_WADD(s0.x, e0.x, wv[0]) FSK_WADD(s0.y, e0.y, wv[1])
            FSK_WADD(s0.z, e0.z, wv[2]) FSK_WADD(s0.w, e0.w, wv[3])
            FSK_WADD(s1.x, e1.x, wv[4]) FSK_WADD(s1.y, e1.y, wv[5])
            FSK_WADD(s1.z, e1.z, wv[6]) FSK_WADD(s1.w, e1.w, wv[7])
#undef FSK_WADD
            wacc[threadIdx.x] = s0;
            wacc[EPI_T + threadIdx.x] = s1;
            wacc[2 * EPI_T + threadIdx.x] = e0;
            wacc[3 * EPI_T + threadIdx.x] = e1;
          }
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
      if (lane == 0) {
        mbar_arrive(cready);
        mbar_arrive(qempty);   // done with this unit's query images and rows in shared memory
      }
      if (!__all_sync(0xffffffffu, mbar_wait(cready, (uint32_t)(k_unit & 1), 35))) goto done;
      {
        float* wc_next = wcorr + ((k_unit + 1) & 1) * WC_PAR + half * WC_HALF + wc_row;
#pragma unroll
        for (int k = 0; k < FSK_D; k += 4)
          *reinterpret_cast<float4*>(wc_next + k) = make_float4(0.f, 0.f, 0.f, 0.f);
      }
      if (gi < p.n) {
        const double p_unscale = 1.0 / 32768.0;   // 2^-PHI_LOG2_SCALE
        const double c_unscale = p_unscale;
        const double w_unscale = ldexp(p_unscale, -p.scales->pad[2]);
        const int64_t pidx = (int64_t)(2 * sp + half) * p.n + gi;
        if (in_bounds(pidx, 2 * p.splits * p.n, 42))
          p.ppdf[pidx] = ((double)acc.s + (double)acc.c + (double)corr) * p_unscale;
        const int64_t wbase = ((int64_t)sp * p.n + gi) * FSK_D + half * 8;   // 8 features from here
        const bool w_ok = in_bounds(wbase, p.splits * p.n * FSK_D - 7, 43);
        double* wrow = p.pw + wbase;
        const float* c0 = wcorr + (k_unit & 1) * WC_PAR + wc_row + half * 8;
        const float* c1 = c0 + WC_HALF;
        const float4 s0 = wacc[threadIdx.x], s1 = wacc[EPI_T + threadIdx.x];
        const float4 e0 = wacc[2 * EPI_T + threadIdx.x], e1 = wacc[3 * EPI_T + threadIdx.x];
        const float ws[8] = {s0.x, s0.y, s0.z, s0.w, s1.x, s1.y, s1.z, s1.w};
        const float we[8] = {e0.x, e0.y, e0.z, e0.w, e1.x, e1.y, e1.z, e1.w};
        if (w_ok) {
#pragma unroll
          for (int k = 0; k < 8; ++k)
            wrow[k] = ((double)ws[k] + (double)we[k]) * w_unscale + ((double)c0[k] + (double)c1[k]) * c_unscale;
        }
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
  if ((warp == S_MMA_WARP || warp == S_MMA_WARP2 || warp >= W_MMA_WARP) && lane == 0) {
    mma_commit(drain);   // one arrival per issuing thread, when its MMAs have finished
    mbar_wait(drain, 0, 34);
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == S_MMA_WARP) tmem_dealloc(tmem_base, S_TMEM_COLS);
}

// Data stage image: [H (64 x 32 fp16) | M (64 x 16 fp16) | L (64 x 16 fp16)
// | XT hi (16 x 64 fp16) | XT lo | x (64 x 16 FP32)].  XT rows are features, K-major over the points.
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
  write_operand_row(tile, tile + B_M_OFFSET, tile + B_L_OFFSET, r, v, beta, ok ? ldexpf(1.f, sc->pad[0]) : 0.f,
                    true);
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
  pl.part_rows = 2 * pl.splits;   // pdf rows: one per (split, column half)
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

// ---- layout probe: tcgen05.cp of a query operand image into tensor memory -----
// A (128 x 32, rounded to fp16) is written in the "hi" operand image layout
// (64-byte rows, no-swizzle K-major core matrices), copied to TMEM columns
// 0-15 with two 128x256b copies (K 0-15 at +0 B, K 16-31 at +256 B) and read
// back with tcgen05.ld: out[r][c] is column c of lane r (two fp16 per word).
namespace {
__global__ void __launch_bounds__(128, 1) tmem_cp_probe_kernel(const float* __restrict__ a,
                                                               uint32_t* __restrict__ out) {
  __shared__ __align__(1024) uint8_t sa[QT * H_ROW_BYTES];
  __shared__ uint64_t bar;
  __shared__ uint32_t slot;
  const int t = threadIdx.x;
  const int warp = t >> 5;
#pragma unroll 4
  for (int k = 0; k < KH; ++k) put_h(sa, t, k, H_ROW_BYTES, __float2half_rn(a[t * KH + k]));
  if (t == 0) {
    mbar_init(&bar, 1);
    fence_barrier_init();
  }
  if (warp == 0) {
    tmem_alloc(&slot, 32);
    tmem_relinquish();
  }
  fence_proxy_async_smem();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tbase = slot;
  if (t == 0) {
    tmem_cp_128x256b(tbase, smem_desc_kmajor(smem_u32(sa), 128, 8 * H_ROW_BYTES));
    tmem_cp_128x256b(tbase + 8u, smem_desc_kmajor(smem_u32(sa) + 256, 128, 8 * H_ROW_BYTES));
    mma_commit(&bar);
  }
  __syncwarp();
  const bool ok = mbar_wait(&bar, 0, 37);
  tc_fence_after();
  if (ok) {
    uint32_t r[16];
    tmem_ld16(tbase + ((uint32_t)(warp * 32) << 16), r);
    tmem_ld_wait();
#pragma unroll
    for (int j = 0; j < 16; ++j) out[t * 16 + j] = r[j];
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 0) tmem_dealloc(tbase, 32);
}
}  // namespace

}  // namespace tc

unsigned int score16_take_device_error() { return take_unit_device_error(); }

namespace tc {

int launch_tmem_cp_probe(const float* a, uint32_t* out, cudaStream_t s) {
  tmem_cp_probe_kernel<<<1, 128, 0, s>>>(a, out);
  count_launch();
  return cuda_status(cudaGetLastError());
}

int launch_mma_ts_probe(const float* a, const float* b, float* d, cudaStream_t s) {
  mma_ts_probe_kernel<<<1, 128, 0, s>>>(a, b, d);
  count_launch();
  return cuda_status(cudaGetLastError());
}

}  // namespace tc
}  // namespace fsk
