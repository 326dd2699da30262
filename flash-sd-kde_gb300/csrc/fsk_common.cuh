// fsk_common.cuh - shared definitions for the sm_103a Flash-SD-KDE kernels:
// status plumbing, launch accounting, and thin inline-PTX wrappers for
// mbarrier, bulk (TMA) copies and the tcgen05 tensor-core / tensor-memory
// instructions.  Every spin-wait here is bounded: when it gives up it records
// FSK_ERR_DEVICE_TIMEOUT in the device error word and returns false, so the
// caller can drain and exit without hanging the GPU.
#pragma once

#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>
#include <stdint.h>
#include <string.h>

#include "../../include/fsk.h"

#define FSK_D 16            // feature count of the 16-D path
#define FSK_LOG2E 1.4426950408889634

namespace fsk {

// ---- device error word ----------------------------------------------------
// 0 = ok; otherwise an fsk_status code plus a site id in the upper bits.  Most
// units are built without relocatable device code (no device symbol is
// shared between units), so every translation unit has its own word; the
// units whose kernels record errors export a take function (fsk_kernels.cuh)
// and fsk_device_status reads and clears all of them.
static __device__ unsigned int g_device_error = 0u;

__device__ __forceinline__ void record_error(unsigned int code, unsigned int site) {
  atomicCAS(&g_device_error, 0u, code | (site << 8));
}

// Bounds-check build (-DFSK_BOUNDS_CHECK; fsk._build.build(checked=True)
// makes libfsk_checked.so): the global writes of the hot kernels first check
// their index against the extent of the buffer they write; an index outside
// it records FSK_ERR_DEVICE_BOUNDS with the call site and the write is
// skipped (nothing traps).  In the normal build the check compiles away.
__device__ __forceinline__ bool in_bounds(int64_t i, int64_t limit, unsigned int site) {
#ifdef FSK_BOUNDS_CHECK
  if (i >= 0 && i < limit) return true;
  record_error(FSK_ERR_DEVICE_BOUNDS, site);
  return false;
#else
  (void)i;
  (void)limit;
  (void)site;
  return true;
#endif
}

// This translation unit's error word, read and cleared from the host
// (synchronous; the caller has synchronised the stream).
static inline unsigned int take_unit_device_error() {
  unsigned int v = 0u, zero = 0u;
  if (cudaMemcpyFromSymbol(&v, g_device_error, sizeof(v)) != cudaSuccess) return (unsigned int)FSK_ERR_CUDA;
  if (v != 0u && cudaMemcpyToSymbol(g_device_error, &zero, sizeof(zero)) != cudaSuccess)
    return (unsigned int)FSK_ERR_CUDA;
  return v;
}

// ---- host helpers -----------------------------------------------------------
void count_launch();                     // bump the launch counter
int sm_count();                          // SMs of the current device
int check_device();                      // FSK_OK if current device is sm_103
int cuda_status(cudaError_t e);          // map a CUDA error to fsk_status

// Hot-path kernel ids reported by fsk_timer_collect.
enum KernelId {
  K_KDE16_TC = 1,
  K_KDE16_SIMT = 2,
  K_SCORE16_SIMT = 3,
  K_SCORE16_SYM_SIMT = 4,
  K_KDE1D = 5,
  K_KDE1D_SCORE = 6,
  K_SCORE16_TC = 7,
  K_MLP_INFER = 9,   // work unit: one (query, ensemble member) evaluation
  K_KDE16_LOGSPACE = 10,   // shifted recompute of underflowing queries (work not known on the host)
  K_KDE_ND = 11,
  K_SCORE_ND = 12,
};

// Host-side NVTX range around one C-ABI entry point, so profilers (ncu
// --nvtx, Nsight Systems) show each phase (score, debias, KDE, ...) by name;
// NVTX v3 is header-only and its calls do nothing unless a tool is attached.
class NvtxRange {
 public:
  explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
  NvtxRange(const NvtxRange&) = delete;
  NvtxRange& operator=(const NvtxRange&) = delete;
};

// RAII bracket of one kernel launch with CUDA events on its stream when the
// library timer is enabled (fsk_timer.cu); `work` = pair evaluations.
class TimerScope {
 public:
  TimerScope(int id, double work, cudaStream_t s);
  ~TimerScope();

 private:
  bool active_;
  size_t idx_;
  cudaStream_t s_;
};

inline size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

template <typename T> __host__ __device__ __forceinline__ T imin(T a, T b) { return a < b ? a : b; }
template <typename T> __host__ __device__ __forceinline__ T imax(T a, T b) { return a < b ? b : a; }

// Carves aligned sub-buffers out of a caller workspace.
struct WsCarver {
  char* base;
  size_t cap, used;
  WsCarver(void* b, size_t c) : base(static_cast<char*>(b)), cap(c), used(0) {}
  template <typename T> T* take(size_t count) {
    used = align_up(used, 256);
    T* p = reinterpret_cast<T*>(base ? base + used : nullptr);
    used += count * sizeof(T);
    return p;
  }
  bool fits() const { return used <= cap; }
};

// ---- compensated FP32 accumulation (TwoSum) --------------------------------
struct Comp {
  float s, c;  // value = s + c
  __device__ __forceinline__ void add(float x) {
    float t = s + x;
    float z = t - s;
    c += (s - (t - z)) + (x - z);
    s = t;
  }
};

__device__ __forceinline__ float ex2_approx(float x) {
  float y;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

// 2^a for a <= 0 on the FP32 FMA pipe, two lanes per instruction: the
// exp pipe's work moved to the FMA pipe where that pipe has spare issue
// slots.  a = j + r with j = round(a) (adding 1.5 * 2^23 leaves j in the low
// mantissa bits) and r in [-1/2, 1/2]; 2^r from a degree-5 polynomial whose
// coefficients minimise the maximum relative error on [-1/2, 1/2] (Remez
// exchange, csrc/exp2_poly_remez.py; 7.5e-8 in exact arithmetic, 2.1e-7 with
// the FP32 Horner evaluation, about the error of ex2.approx.f32); j is added
// to the exponent field by one integer multiply-add.  Inputs below -125 are
// clamped (result ~2^-125 * 2^r, where ex2.approx.ftz returns 0 for
// a < -126: negligible against any sum with a term above 2^-100).
__device__ __forceinline__ float2 exp2_poly2(float2 a) {
  const float2 magic = make_float2(12582912.0f, 12582912.0f);   // 1.5 * 2^23
  a.x = fmaxf(a.x, -125.0f);
  a.y = fmaxf(a.y, -125.0f);
  const float2 t = __fadd2_rn(a, magic);
  const float2 j = __fadd2_rn(t, make_float2(-12582912.0f, -12582912.0f));      // round(a), exact
  const float2 r = __ffma2_rn(j, make_float2(-1.0f, -1.0f), a);                 // a - j, exact
  float2 p = __ffma2_rn(make_float2(1.327647245e-03f, 1.327647245e-03f), r,
                        make_float2(9.675540961e-03f, 9.675540961e-03f));
  p = __ffma2_rn(p, r, make_float2(5.550713092e-02f, 5.550713092e-02f));
  p = __ffma2_rn(p, r, make_float2(2.402212024e-01f, 2.402212024e-01f));
  p = __ffma2_rn(p, r, make_float2(6.931469440e-01f, 6.931469440e-01f));
  p = __ffma2_rn(p, r, make_float2(1.000000119e+00f, 1.000000119e+00f));
  // (bits(t) << 23) == (j << 23) mod 2^32: the magic's low nine bits are zero
  return make_float2(__uint_as_float((__float_as_uint(t.x) << 23) + __float_as_uint(p.x)),
                     __uint_as_float((__float_as_uint(t.y) << 23) + __float_as_uint(p.y)));
}

// Packed two-lane FP32 add / fma (one issue slot for two lane operations).
__device__ __forceinline__ void fadd2(float& d0, float& d1, float a0, float a1, float b0, float b1) {
  uint64_t ra, rb, rd;
  asm("mov.b64 %0, {%1, %2};" : "=l"(ra) : "f"(a0), "f"(a1));
  asm("mov.b64 %0, {%1, %2};" : "=l"(rb) : "f"(b0), "f"(b1));
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(rd) : "l"(ra), "l"(rb));
  asm("mov.b64 {%0, %1}, %2;" : "=f"(d0), "=f"(d1) : "l"(rd));
}

__device__ __forceinline__ void ffma2(float& d0, float& d1, float a0, float a1, float b0, float b1,
                                      float c0, float c1) {
  uint64_t ra, rb, rc, rd;
  asm("mov.b64 %0, {%1, %2};" : "=l"(ra) : "f"(a0), "f"(a1));
  asm("mov.b64 %0, {%1, %2};" : "=l"(rb) : "f"(b0), "f"(b1));
  asm("mov.b64 %0, {%1, %2};" : "=l"(rc) : "f"(c0), "f"(c1));
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(rd) : "l"(ra), "l"(rb), "l"(rc));
  asm("mov.b64 {%0, %1}, %2;" : "=f"(d0), "=f"(d1) : "l"(rd));
}

// sum_k (a_k - b_k)^2 over 16 features from direct FP32 differences, four
// FMA chains joined pairwise (shorter rounding chains than one sequence).
__device__ __forceinline__ float sqdist16(const float* a, const float* b) {
  float s0 = 0.f, s1 = 0.f, s2 = 0.f, s3 = 0.f;
#pragma unroll
  for (int k = 0; k < 16; k += 4) {
    const float d0 = a[k] - b[k], d1 = a[k + 1] - b[k + 1];
    const float d2 = a[k + 2] - b[k + 2], d3 = a[k + 3] - b[k + 3];
    s0 = fmaf(d0, d0, s0);
    s1 = fmaf(d1, d1, s1);
    s2 = fmaf(d2, d2, s2);
    s3 = fmaf(d3, d3, s3);
  }
  return (s0 + s1) + (s2 + s3);
}

// 2^(-dist * c) with c = c2 + c2_lo carried in double-float: the rounding
// residual e of dist*c2 is applied as the first-order factor (1 - e ln 2),
// so the exponent is not limited by the FP32 rounding of dist*c2.
__device__ __forceinline__ float exp2_neg_scaled(float dist, float c2, float c2_lo) {
  const float p = dist * c2;
  const float e = fmaf(dist, c2, -p) + dist * c2_lo;
  const float y = ex2_approx(-p);
  return fmaf(y, -e * 0.69314718055994531f, y);
}

// exp2_neg_scaled for two lanes with f32x2 instructions (the same roundings).
__device__ __forceinline__ float2 exp2_neg_scaled2(float2 dist, float c2, float c2_lo) {
  const float2 np = __fmul2_rn(dist, make_float2(-c2, -c2));                       // -p
  const float2 e = __fadd2_rn(__ffma2_rn(dist, make_float2(c2, c2), np), __fmul2_rn(dist, make_float2(c2_lo, c2_lo)));
  const float2 y = make_float2(ex2_approx(np.x), ex2_approx(np.y));
  return __ffma2_rn(y, __fmul2_rn(e, make_float2(-0.69314718055994531f, -0.69314718055994531f)), y);
}

// ---- shared-memory address / mbarrier ---------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}

__device__ __forceinline__ void fence_barrier_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Non-blocking probe of an mbarrier phase (try_wait may suspend the thread
// for a hardware time slice when the phase is incomplete; test_wait returns
// at once).  For issuers that poll several barriers.
__device__ __forceinline__ bool mbar_test_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

__device__ __forceinline__ uint64_t globaltimer_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Bounded wait on an mbarrier phase.  Gives up after ~2 s of wall time,
// records FSK_ERR_DEVICE_TIMEOUT (with the call-site id) and returns false.
// (The error word is not consulted here: a stale error from an earlier,
// unacknowledged launch must not cut short the waits of a later one.)
// After the first probe the thread waits with a suspend-time hint of 50 us:
// it sleeps until the phase completes (or the hint runs out) instead of
// spinning, so a waiting warp takes no issue slots from the busy warps of
// its scheduler.
__device__ __forceinline__ bool mbar_try_wait_sleep(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity), "r"(50000u)
      : "memory");
  return ok != 0;
}

__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, unsigned int site) {
  if (mbar_try_wait(bar, parity)) return true;
  const uint64_t t0 = globaltimer_ns();
  for (;;) {
    if (mbar_try_wait_sleep(bar, parity)) return true;
    if (globaltimer_ns() - t0 > 2000000000ull) {
      record_error(FSK_ERR_DEVICE_TIMEOUT, site);
      return false;
    }
  }
}

// ---- bulk (non-tensor TMA) copy global -> shared -----------------------------
// dst, src 16-byte aligned, bytes a multiple of 16; completes tx on bar.
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

// ---- tcgen05 ------------------------------------------------------------------
__device__ __forceinline__ void tmem_alloc(uint32_t* dst_smem, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                   smem_u32(dst_smem)),
               "r"(ncols)
               : "memory");
}
__device__ __forceinline__ void tmem_relinquish() {
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols)
               : "memory");
}
__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

// D[tmem] (+)= A[smem] * B[smem]^T, kind::f16 (bf16 inputs, FP32 accumulate).
__device__ __forceinline__ void mma_bf16_ss(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc,
                                            uint32_t idesc, uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accumulate)
      : "memory");
}

// Arrive on bar once all previously issued tcgen05.mma of this thread completed.
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          smem_u32(bar))
      : "memory");
}

// Instruction descriptor: kind::f16, A=B=BF16, D=F32, both K-major, M x N.
__host__ __device__ constexpr uint32_t idesc_bf16_f32(int M, int N) {
  return (1u << 4)                          // D format F32
         | (1u << 7)                        // A format BF16
         | (1u << 10)                       // B format BF16
         | (uint32_t(N >> 3) << 17)         // N / 8
         | (uint32_t(M >> 4) << 24);        // M / 16
}

// Shared-memory matrix descriptor, no swizzle, K-major "core matrix" layout:
// a core matrix is 8 rows x 16 bytes stored as 128 contiguous bytes; lbo is
// the byte distance between core matrices adjacent along K, sbo between
// core matrices adjacent along M/N (8-row groups).
__device__ __forceinline__ uint64_t smem_desc_kmajor(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= uint64_t((saddr >> 4) & 0x3FFFu);
  d |= uint64_t((lbo >> 4) & 0x3FFFu) << 16;
  d |= uint64_t((sbo >> 4) & 0x3FFFu) << 32;
  d |= uint64_t(1) << 46;  // descriptor version for tcgen05
  // base offset 0, lbo mode 0, layout type 0 (no swizzle)
  return d;
}

// 32 lanes x 32 consecutive 32-bit columns: thread t of the warp gets lane
// (quarter*32 + t), columns [col, col+32).
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&r)[32]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
      "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]),
        "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]),
        "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
}
__device__ __forceinline__ void tmem_ld_wait() {
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// 32 lanes x 16 consecutive 32-bit columns.
__device__ __forceinline__ void tmem_ld8(uint32_t taddr, uint32_t (&r)[8]) {
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
                 "=r"(r[7])
               : "r"(taddr));
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&r)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
      "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
}

// Store 16 consecutive 32-bit columns of this thread's TMEM lane.
__device__ __forceinline__ void tmem_st2(uint32_t taddr, const uint32_t (&r)[2]) {
  asm volatile("tcgen05.st.sync.aligned.32x32b.x2.b32 [%0], {%1,%2};" ::"r"(taddr), "r"(r[0]), "r"(r[1]));
}

__device__ __forceinline__ void tmem_st4(uint32_t taddr, const uint32_t (&r)[4]) {
  asm volatile("tcgen05.st.sync.aligned.32x32b.x4.b32 [%0], {%1,%2,%3,%4};" ::"r"(taddr), "r"(r[0]), "r"(r[1]),
               "r"(r[2]), "r"(r[3]));
}

__device__ __forceinline__ void tmem_st8(uint32_t taddr, const uint32_t (&r)[8]) {
  asm volatile("tcgen05.st.sync.aligned.32x32b.x8.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8};" ::"r"(taddr), "r"(r[0]),
               "r"(r[1]), "r"(r[2]), "r"(r[3]), "r"(r[4]), "r"(r[5]), "r"(r[6]), "r"(r[7])
               : "memory");
}

__device__ __forceinline__ void tmem_st16(uint32_t taddr, const uint32_t (&r)[16]) {
  asm volatile(
      "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], "
      "{%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16};" ::"r"(taddr),
      "r"(r[0]), "r"(r[1]), "r"(r[2]), "r"(r[3]), "r"(r[4]), "r"(r[5]), "r"(r[6]), "r"(r[7]),
      "r"(r[8]), "r"(r[9]), "r"(r[10]), "r"(r[11]), "r"(r[12]), "r"(r[13]), "r"(r[14]), "r"(r[15])
      : "memory");
}
__device__ __forceinline__ void tmem_st_wait() {
  asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
}

// Asynchronous copy of a 128-row x 256-bit shared-memory tile (described by a
// matrix descriptor, as for tcgen05.mma) to tensor memory: row r -> lane r,
// eight consecutive 32-bit columns.  Ordered with the issuing thread's other
// tcgen05 operations; its completion is tracked by tcgen05.commit.
__device__ __forceinline__ void tmem_cp_128x256b(uint32_t taddr, uint64_t sdesc) {
  asm volatile("tcgen05.cp.cta_group::1.128x256b [%0], %1;" ::"r"(taddr), "l"(sdesc) : "memory");
}

// D[tmem] (+)= A[tmem] * B[smem]^T, kind::f16 (fp16 inputs, FP32 accumulate);
// A is M x K with row m in TMEM lane m, two fp16 per 32-bit column.
__device__ __forceinline__ void mma_f16_ts(uint32_t d_tmem, uint32_t a_tmem, uint64_t b_desc,
                                           uint32_t idesc, uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], [%1], %2, %3, p;\n\t}" ::"r"(d_tmem),
      "r"(a_tmem), "l"(b_desc), "r"(idesc), "r"(accumulate)
      : "memory");
}

// ---- bf16 splitting -----------------------------------------------------------
// Round-to-nearest-even FP32 -> BF16 bits.
__host__ __device__ __forceinline__ uint16_t f32_to_bf16_rn(float f) {
  uint32_t u;
#ifdef __CUDA_ARCH__
  u = __float_as_uint(f);
#else
  memcpy(&u, &f, 4);
#endif
  uint32_t r = u + 0x7FFFu + ((u >> 16) & 1u);
  return uint16_t(r >> 16);
}
__host__ __device__ __forceinline__ float bf16_to_f32(uint16_t b) {
  uint32_t u = uint32_t(b) << 16;
#ifdef __CUDA_ARCH__
  return __uint_as_float(u);
#else
  float f;
  memcpy(&f, &u, 4);
  return f;
#endif
}

}  // namespace fsk
