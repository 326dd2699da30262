// fsk_tc_kde16.cu - tensor-core (tcgen05 / TMEM) 16-D Gaussian KDE, the
// "fast_tf32" precision mode of the reference, GB300-native.
//
// What it computes (per query q_i): sum_j exp(-||q_i - x_j||^2 / (2 h^2)),
// optionally times the Laplace factor (1 + d/2 - ||q_i-x_j||^2/(2h^2)); the
// quantity of kernels/kde_eval_16d_stream_splitk.py:14-81 (pass A) and
// kernels/flash_sd_kde/kde.py:103-144, as FP64 partial sums per data split.
//
// How:
//  * Coordinates are centred on the data mean mu (FP32).  With c2 =
//    log2(e)/(2h^2), the log2-domain exponent of a pair is
//        a2 = 2 c2 (q-mu).(x-mu) + beta_j + alpha_i,
//    beta_j = -c2 |x_j-mu|^2, alpha_i = -c2 |q_i-mu|^2.
//  * Operands are fp16 triples v = hi + mid + lo (~33 significant bits): queries as
//    q' = 2 c2 (q-mu) 2^eq, data as x' = (x-mu) 2^ex with power-of-two
//    scales chosen on the device so every operand stays in fp16 range and
//    eq + ex = 0 (or the product is scaled down and multiplied back).  Each
//    hi operand row carries 16 extra "bias" K-columns holding beta_j and
//    alpha_i as three fp16 parts each against exact powers of two, so one
//    accumulator D = mid.mid + hi.lo + lo.hi + hi.mid + mid.hi + hi.hi +
//    bias.bias (seven tcgen05.mma kind::f16, M=128, N=128, FP32 accumulation
//    in tensor memory) *is* a2, to one FP32 rounding at the magnitude of the
//    cross product.
//  * Epilogue: tcgen05.ld one query row per thread, 2^D on the SFU
//    (ex2.approx), 32-column chunk sums, compensated (TwoSum) per query.
//  * Exact near-pair recompute: when a 32-column chunk holds more than 1/8
//    of its query's running sum (carried across the data splits a CTA runs
//    for that query block), the chunk's largest term is recomputed from
//    direct FP32 differences of the original coordinates (kept in the data
//    stage) with the exponent product in double-float, and replaces its
//    approximation.  The argmax rides in the low 5 mantissa bits, so all
//    triggered lanes of a warp recompute one pair each in lock-step.  Other
//    terms carry the ~2^-25 relative error of the accumulation, which
//    averages out.
//
// Pipeline (one persistent CTA per SM, 19 warps):
//   warp 16 : producer - bulk (TMA) copies of query images per unit and of
//             data-tile images (128 points) per stage into shared memory
//             (mbarrier tx).
//   warps 17, 18 : issue the MMAs of query tiles 0 and 1 (one lane each);
//             warp 17 owns TMEM (512 columns).
//   warps 0-15: epilogue; warp w reads TMEM lanes 32*(w%4).. and columns
//             64*((w/4)%2).. of query tile w/8.
// A work unit is 256 queries (two M=128 tiles) x one data split; TMEM holds
// two accumulator buffers x two query tiles x 128 columns.  Each query's sum
// is kept as two column halves by two threads and written as two FP64
// partial rows per split.
#include <cuda_fp16.h>

#include "fsk_kernels.cuh"
#include "fsk_tc.cuh"
#include "fsk_tc_ops.cuh"

namespace fsk {
namespace tc {

// SINGLE: the single-pass precision rung (FSK_PREC_FP16_SINGLE) - only the
// hi.hi cross product (one fp16 product per feature, FP32 accumulation) and
// the bias step, no exact near-pair recompute.
// POLY: the last POLY_COLS columns of every 32-column chunk take the FMA-pipe
// exp2 (exp2_poly2) instead of ex2.approx, moving a quarter of the exps off
// the exp pipe (the FP32 pipe carries ~one lane operation per pair here).
constexpr int POLY_COLS = 8;
template <bool LAPLACE, bool SINGLE, bool POLY>
__global__ void __launch_bounds__(THREADS, 1) kde16_tc_kernel(TcParams p) {
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t* sA = smem_raw;                               // NQT query tiles: H | M | L
  uint8_t* sB = smem_raw + A_BYTES;                     // NS data stages
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem_raw + K_BAR_OFFSET);
  uint64_t* full = bars;                 // [NS] data stage loaded
  uint64_t* empty = bars + NS;           // [NS] data stage consumed (MMAs + epilogue)
  uint64_t* tfull = bars + 2 * NS;       // [2 buffers][NQT] accumulator written
  uint64_t* tempty = bars + 2 * NS + 4;  // [2 buffers][NQT] accumulator drained
  uint64_t* qready = bars + 2 * NS + 8;  // query images loaded
  uint64_t* qempty = bars + 2 * NS + 9;  // query images no longer read by the MMAs
  uint64_t* drain = bars + 2 * NS + 10;  // all MMAs of this CTA finished (exit path)
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 2 * NS + 11);
  uint32_t n_stage_copies = 0, n_query_copies = 0;   // producer: bulk copies issued

  const int warp = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;

  if (threadIdx.x == 0) {
    for (int s = 0; s < NS; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], MMA_ISSUERS + EPI_WARPS);
    }
    for (int i = 0; i < 2 * NQT; ++i) {
      mbar_init(&tfull[i], 1);
      mbar_init(&tempty[i], EPI_WARPS / NQT);
    }
    mbar_init(qready, 1);
    mbar_init(qempty, MMA_ISSUERS);
    mbar_init(drain, MMA_ISSUERS);
    fence_barrier_init();
  }
  if (warp == MMA_WARP) {
    tmem_alloc(tmem_slot, TMEM_COLS);
    tmem_relinquish();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem_base = *tmem_slot;
  // Work units are (query block, data split), query-block-major; each CTA
  // takes one contiguous range of units so consecutive splits of a query
  // block run back to back and the epilogue can carry its running sums.
  const int64_t units = p.q_blocks * p.splits;
  const int64_t u_begin = (int64_t)blockIdx.x * units / gridDim.x;
  const int64_t u_end = (int64_t)(blockIdx.x + 1) * units / gridDim.x;
  const int64_t qb_begin = u_begin / p.splits;
  const int64_t sp_begin = u_begin - qb_begin * p.splits;

  if (warp == PRODUCER_WARP) {
    // the whole warp runs the loop (warp-uniform values stay in uniform
    // registers); lane 0 issues the copies
    {
      uint32_t& g = n_stage_copies;
      uint32_t& k = n_query_copies;
      int s = 0;
      uint32_t ph = 0;
      int64_t qb = qb_begin, sp = sp_begin;
      for (int64_t u = u_begin; u < u_end; ++u) {
        if (!__all_sync(0xffffffffu, mbar_wait(qempty, (k & 1u) ^ 1u, 1))) goto done;
        if (lane == 0) {
          mbar_arrive_expect_tx(qready, A_BYTES);
          bulk_g2s(sA, p.qimg + qb * (int64_t)A_BYTES, A_BYTES, qready);
        }
        ++k;
        const int64_t t0 = sp * p.tiles_per_split;
        const int64_t t1 = imin<int64_t>(p.n_tiles, t0 + p.tiles_per_split);
        const uint8_t* src = p.ximg + t0 * (int64_t)KB_STAGE_BYTES;
        for (int64_t t = t0; t < t1; ++t, src += KB_STAGE_BYTES) {
          if (!__all_sync(0xffffffffu, mbar_wait(&empty[s], ph ^ 1u, 2))) goto done;
          if (lane == 0) {
            mbar_arrive_expect_tx(&full[s], KB_STAGE_BYTES);
            bulk_g2s(sB + s * KB_STAGE_BYTES, src, KB_STAGE_BYTES, &full[s]);
          }
          ++g;
          if (++s == NS) {
            s = 0;
            ph ^= 1u;
          }
        }
        if (++sp == p.splits) {
          sp = 0;
          ++qb;
        }
      }
    }
  } else if (warp == MMA_WARP || warp == MMA_WARP2) {
    // Two issuing threads, one query tile each, with their own accumulator
    // barriers: a tile's MMAs wait only for the 8 epilogue warps reading that
    // tile.  The per-tile path is kept to the waits, the MMAs and the commits
    // (descriptors of stage s = stage 0 + s * 1 KiB in the 16-byte address
    // field).  The whole warp runs the loop; lane 0 issues and commits.
    {
      const uint32_t idesc = idesc_f16_f32(QT, KNT);
      const int a = (warp == MMA_WARP) ? 0 : 1;
      const uint32_t as = smem_u32(sA + a * A_TILE_BYTES);
      const uint64_t a_h = smem_desc_kmajor(as, 128, 8 * H_ROW_BYTES);
      const uint64_t a_m = smem_desc_kmajor(as + A_M_OFFSET, 128, 8 * L_ROW_BYTES);
      const uint64_t a_l = smem_desc_kmajor(as + A_L_OFFSET, 128, 8 * L_ROW_BYTES);
      const uint32_t bs0 = smem_u32(sB);
      const uint64_t b_h0 = smem_desc_kmajor(bs0, 128, 8 * H_ROW_BYTES);
      const uint64_t b_m0 = smem_desc_kmajor(bs0 + KB_M_OFFSET, 128, 8 * L_ROW_BYTES);
      const uint64_t b_l0 = smem_desc_kmajor(bs0 + KB_L_OFFSET, 128, 8 * L_ROW_BYTES);
      const uint32_t d0 = tmem_base + (uint32_t)(a * KNT);
      uint32_t g = 0, k = 0, ph = 0;
      int s = 0;
      int64_t sp = sp_begin;
      for (int64_t u = u_begin; u < u_end; ++u, ++k) {
        if (!__all_sync(0xffffffffu, mbar_wait(qready, k & 1u, 3))) goto done;
        const int64_t t0 = sp * p.tiles_per_split;
        const int nt = (int)(imin<int64_t>(p.n_tiles, t0 + p.tiles_per_split) - t0);
        for (int i = 0; i < nt; ++i, ++g) {
          const uint32_t b = g & 1u;
          if (!__all_sync(0xffffffffu, mbar_wait(&full[s], ph, 4))) goto done;
          if (!__all_sync(0xffffffffu, mbar_wait(&tempty[b * NQT + a], ((g >> 1) & 1u) ^ 1u, 5))) goto done;
          tc_fence_after();
          const uint64_t so = (uint64_t)(s * (KB_STAGE_BYTES >> 4));
          if (lane == 0) {
            if (SINGLE)
              mma_s_tile_single(d0 + b * (uint32_t)(NQT * KNT), a_h, b_h0 + so, idesc);
            else
              mma_s_tile(d0 + b * (uint32_t)(NQT * KNT), a_h, a_m, a_l, b_h0 + so, b_m0 + so, b_l0 + so, idesc);
            mma_commit(&tfull[b * NQT + a]);
            mma_commit(&empty[s]);
          }
          __syncwarp();
          if (++s == NS) {
            s = 0;
            ph ^= 1u;
          }
        }
        if (lane == 0) mma_commit(qempty);
        __syncwarp();
        if (++sp == p.splits) sp = 0;
      }
    }
  } else {
    // ---------------- epilogue warps ----------------
    const int qt = warp >> 3;          // query tile within the unit
    const int half = (warp >> 2) & 1;  // column half of the 128-point data tile
    const int quarter = warp & 3;      // TMEM lane quarter
    const uint32_t lane_off = (uint32_t)(quarter * 32) << 16;
    const float out_mul = p.scales->out_mul;
    const bool scaled = out_mul != 1.0f;
    // slot float4 kk of thread t at [kk][t]: a warp's 16-byte accesses are contiguous
    float4* qslot = reinterpret_cast<float4*>(smem_raw + K_QX_OFFSET) + (warp * 32 + lane);
    constexpr int QS_STRIDE = EPI_WARPS * 32;
    uint32_t g = 0;
    int s = 0;
    int64_t prev_qb = -1;
    int64_t qb = qb_begin, sp = sp_begin;
    float s_carry = 0.f;   // approximate sum of this query's half over the splits already done here
    for (int64_t u = u_begin; u < u_end; ++u) {
      if (qb != prev_qb) {
        s_carry = 0.f;
        prev_qb = qb;
      }
      const int64_t gi = qb * (NQT * QT) + qt * QT + quarter * 32 + lane;   // padded query index
      // this query's FP32 row into the thread's own shared-memory slot (read
      // only by the exact recompute; the slot is rewritten only by this thread)
      {
        const float4* src = reinterpret_cast<const float4*>(p.qexact + gi * FSK_D);
#pragma unroll
        for (int kk = 0; kk < FSK_D / 4; ++kk) qslot[kk * QS_STRIDE] = src[kk];
      }
      Comp acc{0.f, 0.f};
      float corr = 0.f;
      const int64_t t0 = sp * p.tiles_per_split;
      const int nt = (int)(imin<int64_t>(p.n_tiles, t0 + p.tiles_per_split) - t0);
      // columns of this thread's half of tile t0 + i: first data index and valid count
      // valid columns of this thread's half of the last (possibly ragged) data
      // tile; every other tile has KNT / 2
      const int last_i = (int)(p.n_tiles - 1 - t0);
      const int last_valid = (int)imin<int64_t>(KNT / 2, p.n - ((p.n_tiles - 1) * KNT + half * (KNT / 2)));
      for (int i = 0; i < nt; ++i, ++g) {
        const uint32_t b = g & 1u;
        const int valid = i == last_i ? last_valid : KNT / 2;   // may be <= 0 on the last tile
        // (a timed-out wait ends the whole warp: it must stay converged)
        if (!__all_sync(0xffffffffu, mbar_wait(&tfull[b * NQT + qt], (g >> 1) & 1u, 6))) goto done;
        tc_fence_after();
        const uint8_t* xrows = sB + s * KB_STAGE_BYTES + KB_X_OFFSET + half * (KNT / 2) * (FSK_D * 4);
        float tsum = 0.f;
        // Both 32-column chunks are loaded before either is processed, so the
        // accumulator buffer goes back to the MMA issuer as early as possible.
        uint32_t ra[32], rb[32];
        {
          const uint32_t col = tmem_base + lane_off + b * (uint32_t)(NQT * KNT) + (uint32_t)(qt * KNT + half * (KNT / 2));
          tmem_ld32(col, ra);
          tmem_ld32(col + 32u, rb);
          tmem_ld_wait();
          tc_fence_before();
          __syncwarp();
          if (lane == 0) mbar_arrive(&tempty[b * NQT + qt]);
        }
        auto chunk = [&](const uint32_t (&r)[32], const int c) {
            float e[32];
            if (scaled) {
#pragma unroll
              for (int j = 0; j < 32; j += 2) {
                const float2 v = __fmul2_rn(make_float2(__uint_as_float(r[j]), __uint_as_float(r[j + 1])),
                                            make_float2(out_mul, out_mul));
                e[j] = v.x;
                e[j + 1] = v.y;
              }
            } else {
#pragma unroll
              for (int j = 0; j < 32; ++j) e[j] = __uint_as_float(r[j]);
            }
#pragma unroll
            for (int j = 0; j < 32; ++j) {
              if (POLY && j >= 32 - POLY_COLS) continue;
              float v = ex2_approx(e[j]);
              // Laplace factor 1 + d/2 - dist/(2h^2) = 9 + a2 ln 2   (a2 = -c2 dist)
              if (LAPLACE) v *= fmaf(e[j], 0.69314718055994531f, 1.0f + 0.5f * FSK_D);
              e[j] = v;
            }
            if (POLY) {
#pragma unroll
              for (int j = 32 - POLY_COLS; j < 32; j += 2) {
                const float2 v = exp2_poly2(make_float2(e[j], e[j + 1]));
                e[j] = v.x;
                e[j + 1] = v.y;
              }
            }
            const int cvalid = valid - c * 32;   // valid columns of this chunk (may be <= 0 or > 32)
            if (cvalid < 32) {  // ragged last data tile: drop padding columns
#pragma unroll
              for (int j = 0; j < 32; ++j)
                if (j >= cvalid) e[j] = 0.f;
            }
            // packed pairwise sum (f32x2 adds on register pairs)
            float2 pa = make_float2(e[0], e[1]), pb = make_float2(e[2], e[3]);
#pragma unroll
            for (int j = 4; j < 32; j += 4) {
              pa = __fadd2_rn(pa, make_float2(e[j], e[j + 1]));
              pb = __fadd2_rn(pb, make_float2(e[j + 2], e[j + 3]));
            }
            pa = __fadd2_rn(pa, pb);
            float cs = pa.x + pa.y;
            // Near-pair test: a chunk holding more than NEAR_FRACTION of the
            // running sum (this chunk included) may contain a dominant term.
            const float run = s_carry + fabsf(acc.s) + fabsf(tsum);
            const bool trig = !SINGLE && fabsf(cs) > (run + fabsf(cs)) * NEAR_FRACTION;
            if (!SINGLE && __any_sync(0xffffffffu, trig)) {
              // Triggered lanes replace their chunk's largest term by its exact
              // value.  The argmax rides in the low 5 mantissa bits of each term
              // (key = |e| with bits[4:0] := column); the chunk is re-summed
              // from those keyed values, so subtracting the keyed maximum
              // removes exactly what was added.  All triggered lanes recompute
              // one pair each, in lock-step.
              if (trig) {
                uint32_t key[32];
                float2 qa = make_float2(0.f, 0.f), qc = make_float2(0.f, 0.f);
#pragma unroll
                for (int j = 0; j < 32; j += 2) {
                  // terms are >= 0 except with the Laplace factor
                  const float a0 = LAPLACE ? fabsf(e[j]) : e[j], a1 = LAPLACE ? fabsf(e[j + 1]) : e[j + 1];
                  key[j] = (__float_as_uint(a0) & ~31u) | (uint32_t)j;
                  key[j + 1] = (__float_as_uint(a1) & ~31u) | (uint32_t)(j + 1);
                  const float v0 = LAPLACE ? copysignf(__uint_as_float(key[j]), e[j]) : __uint_as_float(key[j]);
                  const float v1 = LAPLACE ? copysignf(__uint_as_float(key[j + 1]), e[j + 1]) : __uint_as_float(key[j + 1]);
                  if (j & 2) qc = __fadd2_rn(qc, make_float2(v0, v1));
                  else qa = __fadd2_rn(qa, make_float2(v0, v1));
                }
                // max tree over the keys
#pragma unroll
                for (int w = 16; w >= 1; w >>= 1)
#pragma unroll
                  for (int j = 0; j < w; ++j) key[j] = max(key[j], key[j + w]);
                const uint32_t kmax = key[0];
                qa = __fadd2_rn(qa, qc);
                cs = qa.x + qa.y;
                const int j = (int)(kmax & 31u);
                float approx = __uint_as_float(kmax);
                if (LAPLACE) {
#pragma unroll
                  for (int jj = 0; jj < 32; ++jj)
                    if (jj == j) approx = copysignf(approx, e[jj]);
                }
                float qx[FSK_D];
#pragma unroll
                for (int kk = 0; kk < FSK_D; kk += 4) {
                  const float4 v = qslot[(kk / 4) * QS_STRIDE];
                  qx[kk] = v.x; qx[kk + 1] = v.y; qx[kk + 2] = v.z; qx[kk + 3] = v.w;
                }
                const float dist = exact_dist(xrows, c * 32 + j, qx, 0);
                float ex = exp2_neg_scaled(dist, p.c2, p.c2_lo);
                if (LAPLACE) ex *= fmaf(-p.c1, dist, 1.0f + 0.5f * FSK_D);
                if (j >= cvalid) ex = 0.f;
                corr += ex - approx;
              }
              __syncwarp();
            }
            tsum += cs;
        };
        chunk(ra, 0);
        chunk(rb, 1);
        acc.add(tsum);
        // the stage's x rows are no longer read by this warp
        __syncwarp();
        if (lane == 0) mbar_arrive(&empty[s]);
        if (++s == NS) s = 0;
      }
      s_carry += fabsf(acc.s + corr);
      if (gi < p.m) {
        const double v = (double)acc.s + (double)acc.c + (double)corr;
        if (p.atomic_acc) {
          if (in_bounds(gi, p.m, 40)) atomicAdd(&p.atomic_acc[gi], v);
        } else {
          const int64_t idx = (2 * sp + half) * p.m + gi;
          if (in_bounds(idx, 2 * p.splits * p.m, 41)) p.partials[idx] = v;
        }
      }
      if (++sp == p.splits) {
        sp = 0;
        ++qb;
      }
    }
  }
done:
  // Exit path (also after a timed-out wait): let this CTA's bulk copies and
  // MMAs finish before shared and tensor memory are released.
  if (warp == PRODUCER_WARP && lane == 0) {
    for (uint32_t i = n_stage_copies > (uint32_t)NS ? n_stage_copies - NS : 0u; i < n_stage_copies; ++i)
      mbar_wait(&full[i % NS], (i / NS) & 1u, 7);
    if (n_query_copies > 0) mbar_wait(qready, (n_query_copies - 1) & 1u, 8);
  }
  if ((warp == MMA_WARP || warp == MMA_WARP2) && lane == 0) {
    mma_commit(drain);   // one arrival per issuing thread, when its MMAs have finished
    mbar_wait(drain, 0, 9);
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == MMA_WARP) tmem_dealloc(tmem_base, TMEM_COLS);
}

// ---- prep ----------------------------------------------------------------------------
// Maxima for the scale selection: |2 c2 (q-mu)|, c2 |q-mu|^2 over queries and
// |x-mu|, c2 |x-mu|^2 over data.  One thread per row; block-reduced.
__global__ void scale_stats_kernel(const float* __restrict__ pts, int64_t count, const float* __restrict__ mu,
                                   float c2, int is_query, float alpha_off, TcScales* __restrict__ sc) {
  float vmax = 0.f, nmax = 0.f;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count;
       i += (int64_t)gridDim.x * blockDim.x) {
    float nrm = 0.f, mx = 0.f;
#pragma unroll
    for (int k = 0; k < FSK_D; ++k) {
      const float v = pts[i * FSK_D + k] - mu[k];
      nrm = fmaf(v, v, nrm);
      mx = fmaxf(mx, fabsf(v));
    }
    vmax = fmaxf(vmax, is_query ? 2.0f * c2 * mx : mx);
    nmax = fmaxf(nmax, fabsf(c2 * nrm - (is_query ? alpha_off : 0.f)));
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    vmax = fmaxf(vmax, __shfl_xor_sync(0xffffffffu, vmax, off));
    nmax = fmaxf(nmax, __shfl_xor_sync(0xffffffffu, nmax, off));
  }
  if ((threadIdx.x & 31) == 0) {
    atomic_max_pos(is_query ? &sc->qmax_bits : &sc->xmax_bits, vmax);
    atomic_max_pos(is_query ? &sc->amax_bits : &sc->bmax_bits, nmax);
  }
}

__global__ void scale_init_kernel(TcScales* sc) {
  if (threadIdx.x == 0) {
    sc->qmax_bits = sc->xmax_bits = sc->amax_bits = sc->bmax_bits = 0u;
  }
}

// Chooses the power-of-two scales (one thread).  q' max and x' max are
// balanced around sqrt(Lq Lx 2^-es) <= FP16_TARGET; alpha and beta parts are
// scaled into range against exact powers of two (<= 2^15) in the other
// operand's bias columns.
__global__ void scale_select_kernel(TcScales* sc) {
  if (threadIdx.x != 0) return;
  const float T = FP16_TARGET;
  float lq = fmaxf(__uint_as_float(sc->qmax_bits), 1e-30f);
  float lx = fmaxf(__uint_as_float(sc->xmax_bits), 1e-30f);
  const float am = __uint_as_float(sc->amax_bits), bm = __uint_as_float(sc->bmax_bits);
  int es = 0;
  for (int it = 0; it < 64; ++it) {
    const double prod = (double)lq * (double)lx * ldexp(1.0, -es);
    const int eaa = am * ldexpf(1.f, -es) > T ? (int)ceil(log2((double)am * ldexp(1.0, -es) / T)) : 0;
    const int ebb = bm * ldexpf(1.f, -es) > T ? (int)ceil(log2((double)bm * ldexp(1.0, -es) / T)) : 0;
    if (prod <= (double)T * T && eaa <= 15 && ebb <= 15) break;
    ++es;
  }
  // x' = (x-mu) 2^ex, q' = 2c2 (q-mu) 2^eq, eq + ex = -es, balanced
  const int ex = (int)floor(0.5 * (log2((double)lq) - log2((double)lx) - es));
  const int eq = -es - ex;
  const int ea = am * ldexpf(1.f, -es) > T ? (int)ceil(log2((double)am * ldexp(1.0, -es) / T)) : 0;
  const int eb = bm * ldexpf(1.f, -es) > T ? (int)ceil(log2((double)bm * ldexp(1.0, -es) / T)) : 0;
  sc->x_scale = ldexpf(1.f, ex);
  sc->q_scale = ldexpf(1.f, eq);          // times 2 c2, applied in the prep kernel
  sc->a_scale = ldexpf(1.f, -es - ea);    // alpha * a_scale in A, 2^ea in B
  sc->b_scale = ldexpf(1.f, -es - eb);    // beta * b_scale in B, 2^eb in A
  sc->pad[0] = ea;
  sc->pad[1] = eb;
  // scale of the (x - mu) operand of the weighted-sum product: max |x'| <= T
  sc->pad[2] = (int)floor(log2((double)T / (double)lx));
  sc->out_mul = ldexpf(1.f, es);
}

// data tile image: [H (128 x 32 fp16) | M (128 x 16 fp16) | L (128 x 16 fp16) | x (128 x 16 FP32)]
__global__ void prep_data_kernel(const float* __restrict__ x, int64_t n, int64_t n_pad,
                                 const float* __restrict__ mu, float c2, const TcScales* __restrict__ sc,
                                 uint8_t* __restrict__ img) {
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n_pad) return;
  const bool ok = j < n;
  float xo[FSK_D], v[FSK_D];
  float nrm = 0.f;
#pragma unroll
  for (int k = 0; k < FSK_D; ++k) {
    xo[k] = ok ? x[j * FSK_D + k] : 0.f;
    const float cv = xo[k] - mu[k];
    nrm = fmaf(cv, cv, nrm);
    v[k] = ok ? cv * sc->x_scale : 0.f;
  }
  uint8_t* tile = img + (j / KNT) * (int64_t)KB_STAGE_BYTES;
  const int r = (int)(j % KNT);
  const float beta = ok ? -c2 * nrm * sc->b_scale : 0.f;
  write_operand_row(tile, tile + KB_M_OFFSET, tile + KB_L_OFFSET, r, v, beta, ok ? ldexpf(1.f, sc->pad[0]) : 0.f,
                    true);
  float4* xr = reinterpret_cast<float4*>(tile + KB_X_OFFSET + r * (FSK_D * 4));
#pragma unroll
  for (int k = 0; k < 4; ++k) xr[k] = make_float4(xo[4 * k], xo[4 * k + 1], xo[4 * k + 2], xo[4 * k + 3]);
}

// query tile image: [H (QT x 32 fp16) | L (QT x 16 fp16)], plus the original
// coordinates for the exact recompute.
__global__ void prep_query_kernel(const float* __restrict__ q, int64_t m, int64_t m_pad,
                                  const float* __restrict__ mu, float c2, float alpha_off,
                                  const TcScales* __restrict__ sc, uint8_t* __restrict__ img,
                                  float* __restrict__ qexact) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m_pad) return;
  const bool ok = i < m;
  float qo[FSK_D], v[FSK_D];
  float nrm = 0.f;
  const float qs = 2.0f * c2 * sc->q_scale;
#pragma unroll
  for (int k = 0; k < FSK_D; ++k) {
    qo[k] = ok ? q[i * FSK_D + k] : 0.f;
    const float cv = qo[k] - mu[k];
    nrm = fmaf(cv, cv, nrm);
    v[k] = ok ? cv * qs : 0.f;
  }
  uint8_t* tile = img + (i / QT) * (int64_t)A_TILE_BYTES;
  const float alpha = ok ? (alpha_off - c2 * nrm) * sc->a_scale : 0.f;
  write_operand_row(tile, tile + A_M_OFFSET, tile + A_L_OFFSET, (int)(i % QT), v, alpha,
                    ok ? ldexpf(1.f, sc->pad[1]) : 0.f, false);
#pragma unroll
  for (int k = 0; k < FSK_D; ++k) qexact[i * FSK_D + k] = qo[k];
}

void plan_splits(TcPlan& pl) {
  const int64_t sms = sm_count();
  // Data splits only add parallelism: pick the smallest split count giving
  // every CTA >= 4 units with a near-integral number of units per CTA.
  const int64_t s_min = imax<int64_t>(1, imin<int64_t>(pl.n_tiles, (4 * sms + pl.q_blocks - 1) / pl.q_blocks));
  const int64_t s_max = imin<int64_t>(pl.n_tiles, 4 * s_min + 16);
  int64_t best = s_min;
  double best_eff = -1.0;
  for (int64_t sp = s_min; sp <= s_max; ++sp) {
    const int64_t tps = (pl.n_tiles + sp - 1) / sp;
    const int64_t eff_splits = (pl.n_tiles + tps - 1) / tps;
    const int64_t u = pl.q_blocks * eff_splits;
    const int64_t g = imin<int64_t>(u, sms);
    const double eff = (double)u / (double)(g * ((u + g - 1) / g));
    if (eff > best_eff + 1e-9) {
      best_eff = eff;
      best = sp;
    }
    if (eff >= 0.97) break;
  }
  pl.tiles_per_split = (pl.n_tiles + best - 1) / best;
  pl.splits = (pl.n_tiles + pl.tiles_per_split - 1) / pl.tiles_per_split;  // all splits non-empty
  pl.grid = (int)imin<int64_t>(pl.q_blocks * pl.splits, sms);
}

TcPlan plan_kde16(int64_t m, int64_t n) {
  TcPlan pl;
  pl.m_pad = (m + NQT * QT - 1) / (NQT * QT) * (NQT * QT);
  pl.n_tiles = (n + KNT - 1) / KNT;
  pl.n_pad = pl.n_tiles * KNT;
  pl.q_blocks = pl.m_pad / (NQT * QT);
  plan_splits(pl);
  pl.part_rows = 2 * pl.splits;   // one row per (split, column half)
  return pl;
}

size_t tc_kde16_ws_bytes(const TcPlan& pl, int64_t m, bool atomic) {
  size_t b = 0;
  b += align_up(sizeof(TcScales), 256);
  b += align_up((size_t)pl.q_blocks * A_BYTES, 256);
  b += align_up((size_t)pl.m_pad * FSK_D * sizeof(float), 256);
  b += align_up((size_t)pl.n_tiles * KB_STAGE_BYTES, 256);
  b += align_up((size_t)(atomic ? 1 : pl.part_rows) * m * sizeof(double), 256);
  return b;
}

template <bool LAPLACE, bool SINGLE, bool POLY = false>
static cudaError_t launch_kde16_tc_kernel(const TcPlan& pl, const TcParams& p, cudaStream_t s) {
  const cudaError_t e = cudaFuncSetAttribute(kde16_tc_kernel<LAPLACE, SINGLE, POLY>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES);
  if (e != cudaSuccess) return e;
  kde16_tc_kernel<LAPLACE, SINGLE, POLY><<<pl.grid, THREADS, SMEM_BYTES, s>>>(p);
  return cudaGetLastError();
}

int launch_kde16_tc(const float* q, int64_t m, const float* x, int64_t n, const float* mu, double h,
                    bool laplace, bool single, bool poly, const TcPlan& pl, WsCarver& c, double** partials_out,
                    bool atomic, cudaStream_t s) {
  TcScales* sc = c.take<TcScales>(1);
  uint8_t* qimg = c.take<uint8_t>((size_t)pl.q_blocks * A_BYTES);
  float* qexact = c.take<float>((size_t)pl.m_pad * FSK_D);
  uint8_t* ximg = c.take<uint8_t>((size_t)pl.n_tiles * KB_STAGE_BYTES);
  double* part = c.take<double>((size_t)(atomic ? 1 : pl.part_rows) * m);
  if (!c.fits()) return FSK_ERR_WORKSPACE_TOO_SMALL;
  *partials_out = part;

  const double c2d = FSK_LOG2E / (2.0 * h * h);
  const float c2 = (float)c2d;
  const float c2_lo = (float)(c2d - (double)c2);
  scale_init_kernel<<<1, 32, 0, s>>>(sc);
  count_launch();
  const int sblocks_q = (int)imin<int64_t>(1024, (m + 255) / 256);
  const int sblocks_x = (int)imin<int64_t>(1024, (n + 255) / 256);
  scale_stats_kernel<<<sblocks_q, 256, 0, s>>>(q, m, mu, c2, 1, 0.f, sc);
  count_launch();
  scale_stats_kernel<<<sblocks_x, 256, 0, s>>>(x, n, mu, c2, 0, 0.f, sc);
  count_launch();
  scale_select_kernel<<<1, 32, 0, s>>>(sc);
  count_launch();
  prep_data_kernel<<<(unsigned)((pl.n_pad + 255) / 256), 256, 0, s>>>(x, n, pl.n_pad, mu, c2, sc, ximg);
  count_launch();
  prep_query_kernel<<<(unsigned)((pl.m_pad + 255) / 256), 256, 0, s>>>(q, m, pl.m_pad, mu, c2, 0.f, sc, qimg,
                                                                        qexact);
  count_launch();
  if (atomic) launch_zero(part, m, s);

  TcParams p;
  p.qimg = qimg;
  p.ximg = ximg;
  p.qexact = qexact;
  p.scales = sc;
  p.m = m;
  p.n = n;
  p.n_tiles = pl.n_tiles;
  p.q_blocks = pl.q_blocks;
  p.splits = pl.splits;
  p.tiles_per_split = pl.tiles_per_split;
  p.c2 = c2;
  p.c2_lo = c2_lo;
  p.c1 = (float)(1.0 / (2.0 * h * h));
  p.partials = atomic ? nullptr : part;
  p.atomic_acc = atomic ? part : nullptr;
  cudaError_t e;
  TimerScope ts(K_KDE16_TC, (double)m * (double)n, s);
  if (laplace)
    e = single ? launch_kde16_tc_kernel<true, true>(pl, p, s) : launch_kde16_tc_kernel<true, false>(pl, p, s);
  else if (single)
    e = launch_kde16_tc_kernel<false, true>(pl, p, s);
  else
    e = poly ? launch_kde16_tc_kernel<false, false, true>(pl, p, s) : launch_kde16_tc_kernel<false, false>(pl, p, s);
  count_launch();
  return cuda_status(e);
}

// ---- layout probe: D (128 x 64) = A (128 x 32) . B (64 x 32)^T, fp16 ----------------
// Two K=16 tcgen05.mma steps over the 64-byte-row core-matrix images used by
// the KDE kernel (the second step at +256 B, like its bias columns).  Inputs
// are FP32, rounded to fp16 here; D is written row-major FP32.
__global__ void __launch_bounds__(128, 1) mma_probe_kernel(const float* __restrict__ a,
                                                           const float* __restrict__ b,
                                                           float* __restrict__ d) {
  __shared__ __align__(1024) uint8_t sa[QT * H_ROW_BYTES];
  __shared__ __align__(1024) uint8_t sb[NT * H_ROW_BYTES];
  __shared__ uint64_t bar;
  __shared__ uint32_t slot;
  const int t = threadIdx.x;
#pragma unroll 4
  for (int k = 0; k < KH; ++k) {
    put_h(sa, t, k, H_ROW_BYTES, __float2half_rn(a[t * KH + k]));
    if (t < NT) put_h(sb, t, k, H_ROW_BYTES, __float2half_rn(b[t * KH + k]));
  }
  if (t == 0) {
    mbar_init(&bar, 1);
    fence_barrier_init();
  }
  const int warp = t >> 5;
  if (warp == 0) {
    tmem_alloc(&slot, 64);
    tmem_relinquish();
  }
  fence_proxy_async_smem();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tbase = slot;
  if (t == 0) {
    const uint32_t idesc = idesc_f16_f32(QT, NT);
    mma_f16_ss(tbase, smem_desc_kmajor(smem_u32(sa), 128, 8 * H_ROW_BYTES),
               smem_desc_kmajor(smem_u32(sb), 128, 8 * H_ROW_BYTES), idesc, 0u);
    mma_f16_ss(tbase, smem_desc_kmajor(smem_u32(sa) + 256, 128, 8 * H_ROW_BYTES),
               smem_desc_kmajor(smem_u32(sb) + 256, 128, 8 * H_ROW_BYTES), idesc, 1u);
    mma_commit(&bar);
  }
  __syncwarp();
  const bool ok = mbar_wait(&bar, 0, 20);
  tc_fence_after();
  if (ok) {
    for (int c = 0; c < NT / 32; ++c) {
      uint32_t r[32];
      tmem_ld32(tbase + ((uint32_t)(warp * 32) << 16) + (uint32_t)(c * 32), r);
      tmem_ld_wait();
#pragma unroll
      for (int j = 0; j < 32; ++j) d[(int64_t)t * NT + c * 32 + j] = __uint_as_float(r[j]);
    }
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 0) tmem_dealloc(tbase, 64);
}

int launch_mma_probe(const float* a, const float* b, float* d, cudaStream_t s) {
  mma_probe_kernel<<<1, 128, 0, s>>>(a, b, d);
  count_launch();
  return cuda_status(cudaGetLastError());
}

// Waits on an mbarrier that nothing arrives on: the bounded wait gives up
// (about 2 s), records FSK_ERR_DEVICE_TIMEOUT in the device error word and
// the kernel returns normally.  Tests the failure path without a GPU fault.
__global__ void wait_timeout_probe_kernel(int* out) {
  __shared__ uint64_t bar;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    fence_barrier_init();
  }
  __syncthreads();
  if (threadIdx.x == 0) *out = mbar_wait(&bar, 0, 30) ? 1 : 0;
}

}  // namespace tc

unsigned int kde16_take_device_error() { return take_unit_device_error(); }

namespace tc {

int launch_wait_timeout_probe(int* out, cudaStream_t s) {
  wait_timeout_probe_kernel<<<1, 32, 0, s>>>(out);
  count_launch();
  return cuda_status(cudaGetLastError());
}

}  // namespace tc
}  // namespace fsk
