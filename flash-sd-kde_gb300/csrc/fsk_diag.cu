// fsk_diag.cu - pipe-throughput microbenchmarks for the exp-bound roofline.
//
// Measures, on the current device, the sustained rate of
//   ex2.approx.ftz.f32 (SFU / MUFU), fma.rn.f32 and fma.rn.f32x2 (FMA pipe)
// with independent dependency chains in every thread, timed with CUDA events.
// Rates are returned in operations per second (an f32x2 FMA counts as two).
#include "fsk_kernels.cuh"

namespace fsk {

namespace {
constexpr int DIAG_THREADS = 256;
constexpr int DIAG_CHAINS = 8;
}  // namespace

__global__ void __launch_bounds__(DIAG_THREADS) diag_ex2_kernel(int iters, float* sink) {
  float a[DIAG_CHAINS];
#pragma unroll
  for (int c = 0; c < DIAG_CHAINS; ++c) a[c] = 0.1f * (c + 1) + 1e-6f * threadIdx.x;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int c = 0; c < DIAG_CHAINS; ++c) {
      float y;
      asm volatile("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(-a[c]));
      a[c] = y;
    }
  }
  float s = 0.f;
#pragma unroll
  for (int c = 0; c < DIAG_CHAINS; ++c) s += a[c];
  if (s == 12345.f) sink[blockIdx.x] = s;
}

__global__ void __launch_bounds__(DIAG_THREADS) diag_ffma_kernel(int iters, float* sink) {
  float a[DIAG_CHAINS];
#pragma unroll
  for (int c = 0; c < DIAG_CHAINS; ++c) a[c] = 0.1f * (c + 1) + 1e-6f * threadIdx.x;
  const float m = 0.999f, b = 1e-3f;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int c = 0; c < DIAG_CHAINS; ++c) asm volatile("fma.rn.f32 %0, %0, %1, %2;" : "+f"(a[c]) : "f"(m), "f"(b));
  }
  float s = 0.f;
#pragma unroll
  for (int c = 0; c < DIAG_CHAINS; ++c) s += a[c];
  if (s == 12345.f) sink[blockIdx.x] = s;
}

__global__ void __launch_bounds__(DIAG_THREADS) diag_ffma2_kernel(int iters, float* sink) {
  uint64_t a[DIAG_CHAINS];
#pragma unroll
  for (int c = 0; c < DIAG_CHAINS; ++c) {
    const float lo = 0.1f * (c + 1), hi = 0.2f * (c + 1) + 1e-6f * threadIdx.x;
    asm("mov.b64 %0, {%1, %2};" : "=l"(a[c]) : "f"(lo), "f"(hi));
  }
  uint64_t m, b;
  asm("mov.b64 %0, {%1, %2};" : "=l"(m) : "f"(0.999f), "f"(0.998f));
  asm("mov.b64 %0, {%1, %2};" : "=l"(b) : "f"(1e-3f), "f"(2e-3f));
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int c = 0; c < DIAG_CHAINS; ++c) asm volatile("fma.rn.f32x2 %0, %0, %1, %2;" : "+l"(a[c]) : "l"(m), "l"(b));
  }
  float s = 0.f;
#pragma unroll
  for (int c = 0; c < DIAG_CHAINS; ++c) {
    float lo, hi;
    asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(a[c]));
    s += lo + hi;
  }
  if (s == 12345.f) sink[blockIdx.x] = s;
}

int diag_pipe_rates(double* out3, cudaStream_t s) {
  const int sms = sm_count();
  const int blocks = sms * 8;
  float* sink = nullptr;
  cudaError_t e = cudaMalloc(&sink, blocks * sizeof(float));  // diagnostics only
  if (e != cudaSuccess) return cuda_status(e);
  cudaEvent_t t0, t1;
  cudaEventCreate(&t0);
  cudaEventCreate(&t1);
  const int iters = 4096;
  const double ops = (double)blocks * DIAG_THREADS * iters * DIAG_CHAINS;
  for (int which = 0; which < 3; ++which) {
    float best = 1e30f;
    for (int rep = 0; rep < 3; ++rep) {
      cudaEventRecord(t0, s);
      if (which == 0) diag_ex2_kernel<<<blocks, DIAG_THREADS, 0, s>>>(iters, sink);
      else if (which == 1) diag_ffma_kernel<<<blocks, DIAG_THREADS, 0, s>>>(iters, sink);
      else diag_ffma2_kernel<<<blocks, DIAG_THREADS, 0, s>>>(iters, sink);
      count_launch();
      cudaEventRecord(t1, s);
      cudaEventSynchronize(t1);
      float ms = 0.f;
      cudaEventElapsedTime(&ms, t0, t1);
      if (rep > 0 && ms < best) best = ms;
    }
    out3[which] = ops * (which == 2 ? 2.0 : 1.0) / (best * 1e-3);
  }
  cudaEventDestroy(t0);
  cudaEventDestroy(t1);
  cudaFree(sink);
  return cuda_status(cudaGetLastError());
}

}  // namespace fsk

extern "C" int fsk_diag_pipe_rates(double* rates_out, void* stream) {
  if (!rates_out) return FSK_ERR_INVALID_ARGUMENT;
  int st = fsk::check_device();
  if (st) return st;
  return fsk::diag_pipe_rates(rates_out, static_cast<cudaStream_t>(stream));
}
