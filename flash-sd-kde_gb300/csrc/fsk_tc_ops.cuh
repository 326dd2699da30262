// fsk_tc_ops.cuh - device helpers shared by the tcgen05 kernels: fp16
// instruction descriptors and MMA issue, the fp16 operand-image writers
// (core-matrix layout, hi/lo parts and the bias columns that fold the norm
// terms into the accumulator) and the exact direct-difference distance.
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

// Writes one operand row: H image (features hi + 16 bias columns) and L
// image (features lo).  bias_own: three parts of this row's own norm term;
// pow_other: the exact power of two multiplying the other side's parts.
__device__ __forceinline__ void write_operand_row(uint8_t* h_img, uint8_t* l_img, int r, const float (&v)[FSK_D],
                                                  float own_term, float pow_other, bool own_first) {
#pragma unroll
  for (int k = 0; k < FSK_D; ++k) {
    const __half hi = __float2half_rn(v[k]);
    const __half lo = __float2half_rn(v[k] - __half2float(hi));
    put_h(h_img, r, k, H_ROW_BYTES, hi);
    put_h(l_img, r, k, L_ROW_BYTES, lo);
  }
  __half p0, p1, p2;
  split3_f16(own_term, p0, p1, p2);
  const __half one = __float2half_rn(pow_other);
  const __half zero = __float2half_rn(0.f);
  // bias columns 16..21: A = [2^eb x3 | alpha parts x3], B = [beta parts x3 | 2^ea x3]
  const int own = own_first ? 16 : 19, oth = own_first ? 19 : 16;
  put_h(h_img, r, own + 0, H_ROW_BYTES, p0);
  put_h(h_img, r, own + 1, H_ROW_BYTES, p1);
  put_h(h_img, r, own + 2, H_ROW_BYTES, p2);
  put_h(h_img, r, oth + 0, H_ROW_BYTES, one);
  put_h(h_img, r, oth + 1, H_ROW_BYTES, one);
  put_h(h_img, r, oth + 2, H_ROW_BYTES, one);
#pragma unroll
  for (int k = 22; k < KH; ++k) put_h(h_img, r, k, H_ROW_BYTES, zero);
}

}  // namespace tc
}  // namespace fsk
