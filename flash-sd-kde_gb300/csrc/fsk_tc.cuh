// fsk_tc.cuh - tile geometry, parameters and launchers of the tcgen05 kernels.
#pragma once
#include "fsk_common.cuh"

namespace fsk {
namespace tc {

// ---- geometry -----------------------------------------------------------------
constexpr int QT = 128;                 // queries per MMA tile (M, one TMEM lane each)
constexpr int NT = 64;                  // data points per 64-row operand image (score kernel stages)
// KDE kernel: 2 query tiles x 128 data points per tile (an M=128, K=16 MMA
// costs ~46 cycles for any N <= 64 and 64 cycles at N = 128, so N = 128
// halves the instruction count of the S product per pair).
constexpr int NQT = 2;                  // KDE: query tiles per work unit (256 queries)
constexpr int KNT = 128;                // KDE: data points per stage (MMA N)
constexpr int NS = 6;                   // KDE: shared-memory data stages
constexpr int KH = 32;                  // K of the "hi" operand: 16 features + 16 bias columns
// Operand images, fp16, no-swizzle K-major core-matrix layout: 8-row groups,
// each group = (K/8) core matrices of 8 rows x 16 B stored back to back.
constexpr int H_ROW_BYTES = KH * 2;     // 64 B: features (2 K-chunks) + bias (2 K-chunks)
constexpr int L_ROW_BYTES = 16 * 2;     // 32 B: features only (mid and lo parts)
// Operands are split in three fp16 parts v = hi + mid + lo (~33 significant
// bits): H holds hi and the bias columns, M the mid parts, L the lo parts.
constexpr int A_H_BYTES = QT * H_ROW_BYTES;       // 8 KB
constexpr int A_M_BYTES = QT * L_ROW_BYTES;       // 4 KB
constexpr int A_L_BYTES = QT * L_ROW_BYTES;       // 4 KB
constexpr int A_M_OFFSET = A_H_BYTES;
constexpr int A_L_OFFSET = A_H_BYTES + A_M_BYTES;
constexpr int A_TILE_BYTES = A_L_OFFSET + A_L_BYTES;  // 16 KB
constexpr int A_BYTES = NQT * A_TILE_BYTES;       // 32 KB per KDE unit
constexpr int B_H_BYTES = NT * H_ROW_BYTES;       // 4 KB
constexpr int B_M_BYTES = NT * L_ROW_BYTES;       // 2 KB
constexpr int B_L_BYTES = NT * L_ROW_BYTES;       // 2 KB
constexpr int B_M_OFFSET = B_H_BYTES;
constexpr int B_L_OFFSET = B_H_BYTES + B_M_BYTES;
constexpr int B_X_OFFSET = B_L_OFFSET + B_L_BYTES; // original FP32 rows, 64 B each
// KDE data stage: [H (128 x 32 fp16) | M (128 x 16) | L (128 x 16) | x (128 x 16 FP32)]
constexpr int KB_H_BYTES = KNT * H_ROW_BYTES;                 // 8 KB
constexpr int KB_M_OFFSET = KB_H_BYTES;
constexpr int KB_L_OFFSET = KB_M_OFFSET + KNT * L_ROW_BYTES;  // 12 KB
constexpr int KB_X_OFFSET = KB_L_OFFSET + KNT * L_ROW_BYTES;  // 16 KB
constexpr int KB_STAGE_BYTES = KB_X_OFFSET + KNT * FSK_D * 4; // 24 KB
constexpr int EPI_WARPS = 8 * NQT;      // KDE: (lane quarter, column half) per query tile
constexpr int PRODUCER_WARP = EPI_WARPS;
constexpr int MMA_WARP = EPI_WARPS + 1;   // owns TMEM, issues the MMAs of query tile 0
constexpr int MMA_WARP2 = EPI_WARPS + 2;  // issues the MMAs of query tile 1
constexpr int MMA_ISSUERS = 2;
constexpr int THREADS = (EPI_WARPS + 3) * 32;
constexpr int TMEM_COLS = 2 * NQT * KNT; // double-buffered accumulators
constexpr int K_BAR_OFFSET = A_BYTES + NS * KB_STAGE_BYTES;
// KDE: one 64-byte slot per epilogue thread for its query's FP32 row (read by
// the exact recompute; each thread writes its own slot at the start of a unit)
constexpr int K_QX_OFFSET = K_BAR_OFFSET + 256;
constexpr int SMEM_BYTES = K_QX_OFFSET + EPI_WARPS * 32 * FSK_D * 4;
// A term is recomputed exactly when its 32-column chunk holds more than this
// fraction of the running sum of its query (the chunk included).  With the
// three-part operands the exponent of any other term is off by at most
// ~2^-25 * 2 c2 |q - mu| |x - mu| (one FP32 rounding at the magnitude of the
// cross product), so a term below an eighth of the sum moves it by well
// under 1e-6.
constexpr float NEAR_FRACTION = 1.0f / 8.0f;
constexpr float FP16_TARGET = 8192.0f;  // largest operand magnitude aimed for

static_assert(TMEM_COLS == 512, "TMEM budget");
static_assert(KB_STAGE_BYTES % 16 == 0 && A_BYTES % 16 == 0, "bulk copy granularity");
static_assert(SMEM_BYTES <= 227 * 1024, "shared memory");

// Device-side scale state written by the prep kernels (see fsk_tc_kde16.cu).
struct TcScales {
  unsigned int qmax_bits, xmax_bits, amax_bits, bmax_bits;  // maxima (FP32 bits, >= 0)
  float q_scale;   // q' = q_scale * (q - mu)       (= 2 c2 2^eq)
  float x_scale;   // x' = x_scale * (x - mu)       (= 2^ex)
  float a_scale;   // alpha part scale  2^-ea  (A bias col holds alpha*a_scale, B holds 1/a_scale)
  float b_scale;   // beta part scale   2^-eb
  float out_mul;   // a2 = out_mul * D  (1 unless the product had to be scaled down)
  int pad[3];      // ea, eb, ew: x'' = (x - mu) 2^ew is the weighted-sum operand
};

struct TcParams {
  const uint8_t* qimg;
  const uint8_t* ximg;
  const float* qexact;
  const TcScales* scales;
  int64_t m, n;
  int64_t n_tiles;
  int64_t q_blocks;
  int64_t splits;
  int64_t tiles_per_split;
  float c2, c2_lo, c1;
  double* partials;
  double* atomic_acc;
};

struct TcPlan {
  int64_t m_pad, n_pad, n_tiles, q_blocks, splits, tiles_per_split;
  int64_t part_rows;   // FP64 partial rows per query written by the kernel
  int grid;
};

// Fills splits / tiles_per_split / grid from q_blocks and n_tiles.
void plan_splits(TcPlan& pl);
TcPlan plan_kde16(int64_t m, int64_t n);

// Prep kernels shared by the tensor-core kernels (fsk_tc_kde16.cu).
__global__ void scale_init_kernel(TcScales* sc);
__global__ void scale_stats_kernel(const float* __restrict__ pts, int64_t count, const float* __restrict__ mu,
                                   float c2, int is_query, float alpha_off, TcScales* __restrict__ sc);
__global__ void scale_select_kernel(TcScales* sc);
__global__ void prep_query_kernel(const float* __restrict__ q, int64_t m, int64_t m_pad,
                                  const float* __restrict__ mu, float c2, float alpha_off,
                                  const TcScales* __restrict__ sc, uint8_t* __restrict__ img,
                                  float* __restrict__ qexact);
size_t tc_kde16_ws_bytes(const TcPlan& pl, int64_t m, bool atomic);
int launch_kde16_tc(const float* q, int64_t m, const float* x, int64_t n, const float* mu, double h,
                    bool laplace, bool single, bool poly, const TcPlan& pl, WsCarver& c, double** partials_out,
                    bool atomic, cudaStream_t s);
TcPlan plan_score16(int64_t n);
size_t tc_score16_ws_bytes(const TcPlan& pl, int64_t n);
// Empirical-score partials: ppdf [2 * splits][n], pw [splits][n][16] (centred).
int launch_score16_tc(const float* x, int64_t n, const float* mu, double h, const TcPlan& pl, WsCarver& c,
                      double** ppdf_out, double** pw_out, cudaStream_t s);
int launch_mma_probe(const float* a, const float* b, float* d, cudaStream_t s);
int launch_mma_ts_probe(const float* a, const float* b, float* d, cudaStream_t s);
int launch_tmem_cp_probe(const float* a, uint32_t* out, cudaStream_t s);
int launch_wait_timeout_probe(int* out, cudaStream_t s);

// fp16 core-matrix offset of element (row r, k) in an image whose rows are
// `row_bytes` wide (K = row_bytes / 2).
__host__ __device__ __forceinline__ uint32_t cm_offset(int r, int k, int row_bytes) {
  return (uint32_t)(r >> 3) * (uint32_t)(8 * row_bytes) + (uint32_t)(k >> 3) * 128u +
         (uint32_t)(r & 7) * 16u + (uint32_t)(k & 7) * 2u;
}

}  // namespace tc
}  // namespace fsk
