// fsk_tc_ops.cuh - device helpers shared by the tcgen05 kernels: fp16
// instruction descriptors and MMA issue, the fp16 operand-image writers
// (core-matrix layout, hi/mid/lo parts and the bias columns that fold the
// norm terms into the accumulator), the six-product S MMA sequence and the
// exact direct-difference distance.
#pragma once
#include <cuda_fp16.h>

#include "fsk_tc.cuh"

namespace fsk {
namespace tc {

// ---- idesc / descriptors for fp16 operands ---------------------------------------
__host__ __device__ constexpr uint32_t idesc_f16_f32(int M, int N) {
  return (1u << 4)                      // D format F32
         | (0u << 7) | (0u << 10)       // A, B format F16
         | (uint32_t(N >> 3) << 17) | (uint32_t(M >> 4) << 24);
}

__device__ __forceinline__ void mma_f16_ss(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc,
                                           uint32_t idesc, uint32_t accumulate) {
  mma_bf16_ss(d_tmem, a_desc, b_desc, idesc, accumulate);  // same instruction, kind::f16
}

// D = a2 for one 128-query tile x one data tile (smallest products first, so
// the large hi.hi and bias terms meet last, then the bias K step).
// a_h / b_h: H images (hi | bias), a_m / b_m: mid, a_l / b_l: lo images.
// The six products whose error terms exceed ~2^-33, then the bias: seven MMAs.
__device__ __forceinline__ void mma_s_tile(uint32_t d, uint64_t a_h, uint64_t a_m, uint64_t a_l, uint64_t b_h,
                                           uint64_t b_m, uint64_t b_l, uint32_t idesc) {
  const uint64_t bias = 256 >> 4;   // bias K step: +256 B in the start-address field
  mma_f16_ss(d, a_m, b_m, idesc, 0u);       // mid . mid
  mma_f16_ss(d, a_h, b_l, idesc, 1u);       // hi . lo
  mma_f16_ss(d, a_l, b_h, idesc, 1u);       // lo . hi
  mma_f16_ss(d, a_h, b_m, idesc, 1u);       // hi . mid
  mma_f16_ss(d, a_m, b_h, idesc, 1u);       // mid . hi
  mma_f16_ss(d, a_h, b_h, idesc, 1u);       // hi . hi
  mma_f16_ss(d, a_h + bias, b_h + bias, idesc, 1u);   // beta_j + alpha_i
}

// Single-pass rung: hi.hi cross product and the bias K step (two MMAs); the
// norms in the bias columns keep their three-part precision.
__device__ __forceinline__ void mma_s_tile_single(uint32_t d, uint64_t a_h, uint64_t b_h, uint32_t idesc) {
  const uint64_t bias = 256 >> 4;
  mma_f16_ss(d, a_h, b_h, idesc, 0u);
  mma_f16_ss(d, a_h + bias, b_h + bias, idesc, 1u);
}

// sum_k (q_k - x_k)^2 from the original FP32 coordinates of data row r.
__device__ __forceinline__ float exact_dist(const uint8_t* stage, int r, const float (&q)[FSK_D],
                                            int x_offset = B_X_OFFSET) {
  const float4* xr = reinterpret_cast<const float4*>(stage + x_offset + r * (FSK_D * 4));
  float xv[FSK_D];
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const float4 v = xr[k];
    xv[4 * k] = v.x; xv[4 * k + 1] = v.y; xv[4 * k + 2] = v.z; xv[4 * k + 3] = v.w;
  }
  return sqdist16(q, xv);
}

__device__ __forceinline__ void atomic_max_pos(unsigned int* addr, float v) {
  atomicMax(addr, __float_as_uint(fmaxf(v, 0.f)));  // non-negative floats order as integers
}

// Splits v into three fp16 parts (hi, mid, lo) that sum to v to ~33 bits.
__device__ __forceinline__ void split3_f16(float v, __half& a, __half& b, __half& c) {
  a = __float2half_rn(v);
  const float r1 = v - __half2float(a);
  b = __float2half_rn(r1);
  c = __float2half_rn(r1 - __half2float(b));
}

__device__ __forceinline__ void put_h(uint8_t* img, int r, int k, int row_bytes, __half v) {
  *reinterpret_cast<__half*>(img + cm_offset(r, k, row_bytes)) = v;
}

// Writes one operand row: H image (features hi + 16 bias columns), M image
// (features mid) and L image (features lo), v = hi + mid + lo.  own_term:
// this row's norm term, as three parts in its bias columns; pow_other: the
// exact power of two multiplying the other side's parts.  Each 8-element
// K chunk of a row is 16 contiguous bytes in the core-matrix layout, so the
// row goes out as 16-byte stores (4 for H, 2 each for M and L).
__device__ __forceinline__ void write_operand_row(uint8_t* h_img, uint8_t* m_img, uint8_t* l_img, int r,
                                                  const float (&v)[FSK_D], float own_term, float pow_other,
                                                  bool own_first) {
  __align__(16) __half hrow[KH], mrow[FSK_D], lrow[FSK_D];
#pragma unroll
  for (int k = 0; k < FSK_D; ++k) split3_f16(v[k], hrow[k], mrow[k], lrow[k]);
  __half p0, p1, p2;
  split3_f16(own_term, p0, p1, p2);
  const __half one = __float2half_rn(pow_other);
  const __half zero = __float2half_rn(0.f);
  // bias columns 16..21: A = [2^eb x3 | alpha parts x3], B = [beta parts x3 | 2^ea x3]
  const int own = own_first ? 16 : 19, oth = own_first ? 19 : 16;
  hrow[own + 0] = p0;
  hrow[own + 1] = p1;
  hrow[own + 2] = p2;
  hrow[oth + 0] = one;
  hrow[oth + 1] = one;
  hrow[oth + 2] = one;
#pragma unroll
  for (int k = 22; k < KH; ++k) hrow[k] = zero;
#pragma unroll
  for (int c = 0; c < KH / 8; ++c)
    *reinterpret_cast<uint4*>(h_img + cm_offset(r, 8 * c, H_ROW_BYTES)) = *reinterpret_cast<const uint4*>(hrow + 8 * c);
#pragma unroll
  for (int c = 0; c < FSK_D / 8; ++c) {
    *reinterpret_cast<uint4*>(m_img + cm_offset(r, 8 * c, L_ROW_BYTES)) = *reinterpret_cast<const uint4*>(mrow + 8 * c);
    *reinterpret_cast<uint4*>(l_img + cm_offset(r, 8 * c, L_ROW_BYTES)) = *reinterpret_cast<const uint4*>(lrow + 8 * c);
  }
}

}  // namespace tc
}  // namespace fsk
