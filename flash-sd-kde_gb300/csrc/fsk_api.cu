// fsk_api.cu - the extern "C" boundary (include/fsk.h).  Validates arguments,
// sizes and carves the caller's workspace, and enqueues the kernels on the
// caller's stream.  No allocation, no synchronisation (except
// fsk_device_status), no host fallback.
#include <math.h>

#include <atomic>

#include "fsk_kernels.cuh"
#include "fsk_tc.cuh"

namespace fsk {


static std::atomic<int64_t> g_launches{0};
void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }

int sm_count() {
  int dev = 0, v = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 148;
  if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || v <= 0) return 148;
  return v;
}

int check_device() {
  int dev = 0, major = 0, minor = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return FSK_ERR_CUDA;
  if (cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev) != cudaSuccess) return FSK_ERR_CUDA;
  if (cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev) != cudaSuccess) return FSK_ERR_CUDA;
  if (major != 10 || minor != 3) return FSK_ERR_UNSUPPORTED_DEVICE;
  return FSK_OK;
}

int cuda_status(cudaError_t e) { return e == cudaSuccess ? FSK_OK : FSK_ERR_CUDA; }

namespace {

bool bad_bw(double h) { return !(h > 0.0) || !isfinite(h); }

// ---- 16-D KDE workspace plan ---------------------------------------------------
struct Kde16Plan {
  bool ieee, atomic, log_exact;
  int simt_splits;
  tc::TcPlan tcp;
};

Kde16Plan plan16(int64_t m, int64_t n, int flags) {
  Kde16Plan p{};
  p.ieee = (flags & FSK_PREC_IEEE) != 0;
  p.atomic = (flags & FSK_ATOMIC) != 0;
  p.log_exact = (flags & FSK_OUT_LOG_EXACT) != 0;
  if (p.ieee) p.simt_splits = simt_kde16_splits(m, n);
  else p.tcp = tc::plan_kde16(m, n);
  return p;
}

// common prefix: mean scratch, mu, mu64
struct CenterBufs {
  double* scratch;
  float* mu;
  double* mu64;
};
CenterBufs take_center(WsCarver& c, int64_t n) {
  CenterBufs b;
  b.scratch = c.take<double>(mean_scratch_doubles(n));
  b.mu = c.take<float>(FSK_D);
  b.mu64 = c.take<double>(FSK_D);
  return b;
}

size_t kde16_bytes(int64_t m, int64_t n, const Kde16Plan& p) {
  WsCarver c(nullptr, 0);
  take_center(c, n);
  if (p.ieee) {
    c.take<double>((size_t)(p.atomic ? 1 : p.simt_splits) * m);
  } else {
    c.used = align_up(c.used, 256) + tc::tc_kde16_ws_bytes(p.tcp, m, p.atomic);
  }
  if (p.log_exact) take_logexact(c, m, nullptr);
  return align_up(c.used, 256);
}

constexpr int KNOWN_FLAGS = FSK_PREC_IEEE | FSK_LAPLACE | FSK_OUT_LOG | FSK_ATOMIC | FSK_WEIGHTED_FEATURE_MAJOR |
                            FSK_OUT_LOG_EXACT | FSK_PREC_FP16_SINGLE | FSK_EXP_OFFLOAD;

// FSK_OUT_LOG_EXACT: only with FSK_OUT_LOG, out_eps = 0 and m < 2^32 (list indices)
bool bad_log_exact(int flags, double out_eps, int64_t m) {
  if (!(flags & FSK_OUT_LOG_EXACT)) return false;
  return !(flags & FSK_OUT_LOG) || out_eps != 0.0 || m >= (int64_t(1) << 32);
}

}  // namespace

int validate_kde16_args(const float* q, int64_t m, const float* x, int64_t n, double h, int flags,
                        double out_eps, const float* out) {
  if (!q || !x || !out || m < 1 || n < 1 || bad_bw(h)) return FSK_ERR_INVALID_ARGUMENT;
  if (flags & ~KNOWN_FLAGS) return FSK_ERR_INVALID_ARGUMENT;
  if ((flags & FSK_PREC_FP16_SINGLE) && (flags & FSK_PREC_IEEE)) return FSK_ERR_INVALID_ARGUMENT;
  if (bad_log_exact(flags, out_eps, m)) return FSK_ERR_INVALID_ARGUMENT;
  return FSK_OK;
}

}  // namespace fsk

using namespace fsk;

extern "C" {

int fsk_version(void) { return 10000; }

int64_t fsk_launch_count(void) { return g_launches.load(); }

const char* fsk_strerror(int status) {
  switch (status) {
    case FSK_OK: return "ok";
    case FSK_ERR_INVALID_ARGUMENT: return "invalid argument";
    case FSK_ERR_WORKSPACE_TOO_SMALL: return "workspace too small";
    case FSK_ERR_CUDA: return "CUDA runtime error";
    case FSK_ERR_DEVICE_TIMEOUT: return "bounded device wait timed out";
    case FSK_ERR_UNSUPPORTED_DEVICE: return "device is not sm_103 (GB300)";
    case FSK_ERR_SCRATCH_LIMIT: return "request exceeds the fixed scratch limit";
    case FSK_ERR_DEVICE_BOUNDS: return "device index out of bounds (bounds-check build)";
    default: return "unknown status";
  }
}

int fsk_device_status(void* stream) {
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  cudaError_t e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return FSK_ERR_CUDA;
  // every unit's word is read (and cleared), the first error found is returned
  const unsigned int words[3] = {kde16_take_device_error(), score16_take_device_error(), mlp_tc_take_device_error()};
  for (unsigned int v : words)
    if (v != 0u) return (int)(v & 0xFFu);
#ifdef FSK_BOUNDS_CHECK
  // units whose only device errors are the bounds checks
  const unsigned int checked[3] = {simt_take_device_error(), reduce_take_device_error(), logspace_take_device_error()};
  for (unsigned int v : checked)
    if (v != 0u) return (int)(v & 0xFFu);
#endif
  return FSK_OK;
}

size_t fsk_kde16_workspace_bytes(int64_t m, int64_t n, int flags) {
  if (m < 1 || n < 1) return 0;
  return kde16_bytes(m, n, plan16(m, n, flags));
}

int fsk_kde16(const float* queries, int64_t m, const float* data, int64_t n, double bandwidth, int flags,
              double out_scale, double out_eps, float* out, void* workspace, size_t workspace_bytes,
              void* stream) {
  NvtxRange nvtx_range("fsk_kde16");
  int st = validate_kde16_args(queries, m, data, n, bandwidth, flags, out_eps, out);
  if (st) return st;
  st = check_device();
  if (st) return st;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const Kde16Plan p = plan16(m, n, flags);
  if (!workspace || workspace_bytes < kde16_bytes(m, n, p)) return FSK_ERR_WORKSPACE_TOO_SMALL;
  WsCarver c(workspace, workspace_bytes);
  CenterBufs cb = take_center(c, n);
  const bool laplace = (flags & FSK_LAPLACE) != 0;
  double* part = nullptr;
  int splits = 1;
  if (p.ieee) {
    splits = p.atomic ? 1 : p.simt_splits;
    part = c.take<double>((size_t)splits * m);
    if (!c.fits()) return FSK_ERR_WORKSPACE_TOO_SMALL;
    if (p.atomic) launch_zero(part, m, s);
    launch_kde16_simt(queries, m, data, n, bandwidth, laplace, p.simt_splits,
                      p.atomic ? nullptr : part, p.atomic ? part : nullptr, s);
  } else {
    launch_mean16(data, n, cb.scratch, cb.mu, cb.mu64, s);
    st = tc::launch_kde16_tc(queries, m, data, n, cb.mu, bandwidth, laplace, (flags & FSK_PREC_FP16_SINGLE) != 0,
                             (flags & FSK_EXP_OFFLOAD) != 0, p.tcp, c, &part, p.atomic, s);
    if (st) return st;
    splits = p.atomic ? 1 : (int)p.tcp.part_rows;
  }
  if (p.log_exact) {
    LogExactBufs lb;
    take_logexact(c, m, &lb);
    if (!c.fits()) return FSK_ERR_WORKSPACE_TOO_SMALL;
    launch_reduce_logexact(queries, m, data, n, bandwidth, laplace, part, splits, out_scale, lb, out, s);
  } else {
    launch_reduce_rows(part, splits, m, out_scale, out_eps, (flags & FSK_OUT_LOG) != 0, out, s);
  }
  return cuda_status(cudaGetLastError());
}

// ---- empirical score ------------------------------------------------------------
// Ordered variant: the tcgen05 split-K kernel (tensor precision) or the
// CUDA-core split-K kernel (FSK_PREC_IEEE).  Symmetric variant: the
// upper-triangle kernel, each pair's exp evaluated once, row and column sums
// scattered with FP64 atomics.
static size_t empscore_bytes(int64_t n, int variant, int flags) {
  WsCarver c(nullptr, 0);
  take_center(c, n);
  c.take<double>(reduce_score_scratch_doubles(n));
  size_t b = c.used;
  if (variant == FSK_SCORE_SYMMETRIC) {
    c.take<double>((size_t)n);
    c.take<double>((size_t)n * FSK_D);
    b = c.used;
  } else if (!(flags & FSK_PREC_IEEE)) {
    b = align_up(b, 256) + tc::tc_score16_ws_bytes(tc::plan_score16(n), n);
  } else {
    const int splits = simt_score16_splits(n);
    c.take<double>((size_t)splits * n);
    c.take<double>((size_t)splits * n * FSK_D);
    b = c.used;
  }
  return align_up(b, 256);
}

size_t fsk_empscore16_workspace_bytes(int64_t n, int variant, int flags) {
  if (n < 1) return 0;
  return empscore_bytes(n, variant, flags);
}

int fsk_empscore16(const float* data, int64_t n, double bandwidth, int variant, int flags, float* pdf_sum,
                   float* weighted_sum, void* workspace, size_t workspace_bytes, void* stream) {
  NvtxRange nvtx_range("fsk_empscore16");
  if (!data || !pdf_sum || !weighted_sum || n < 1 || bad_bw(bandwidth)) return FSK_ERR_INVALID_ARGUMENT;
  if (variant != FSK_SCORE_ORDERED && variant != FSK_SCORE_SYMMETRIC) return FSK_ERR_INVALID_ARGUMENT;
  if (flags & ~(KNOWN_FLAGS & ~(FSK_PREC_FP16_SINGLE | FSK_EXP_OFFLOAD))) return FSK_ERR_INVALID_ARGUMENT;
  int st = check_device();
  if (st) return st;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (!workspace || workspace_bytes < empscore_bytes(n, variant, flags)) return FSK_ERR_WORKSPACE_TOO_SMALL;
  WsCarver c(workspace, workspace_bytes);
  CenterBufs cb = take_center(c, n);
  double* rscratch = c.take<double>(reduce_score_scratch_doubles(n));
  launch_mean16(data, n, cb.scratch, cb.mu, cb.mu64, s);
  const bool fm = (flags & FSK_WEIGHTED_FEATURE_MAJOR) != 0;
  const int64_t ws_row = fm ? 1 : FSK_D, ws_col = fm ? n : 1;
  if (variant == FSK_SCORE_SYMMETRIC) {
    double* apdf = c.take<double>((size_t)n);
    double* aw = c.take<double>((size_t)n * FSK_D);
    launch_zero(apdf, n, s);
    launch_zero(aw, n * FSK_D, s);
    launch_score16_sym_simt(data, n, cb.mu, bandwidth, apdf, aw, s);
    launch_reduce_score(apdf, aw, 1, 1, n, cb.mu64, nullptr, pdf_sum, weighted_sum, ws_row, ws_col, rscratch, s);
  } else if (!(flags & FSK_PREC_IEEE)) {
    const tc::TcPlan pl = tc::plan_score16(n);
    double *ppdf = nullptr, *pw = nullptr;
    st = tc::launch_score16_tc(data, n, cb.mu, bandwidth, pl, c, &ppdf, &pw, s);
    if (st) return st;
    launch_reduce_score(ppdf, pw, (int)(2 * pl.splits), (int)pl.splits, n, cb.mu64, data, pdf_sum,
                        weighted_sum, ws_row, ws_col, rscratch, s);
  } else {
    const int splits = simt_score16_splits(n);
    double* ppdf = c.take<double>((size_t)splits * n);
    double* pw = c.take<double>((size_t)splits * n * FSK_D);
    launch_score16_simt(data, n, cb.mu, bandwidth, splits, ppdf, pw, s);
    launch_reduce_score(ppdf, pw, splits, splits, n, cb.mu64, nullptr, pdf_sum, weighted_sum, ws_row, ws_col,
                        rscratch, s);
  }
  return cuda_status(cudaGetLastError());
}

int fsk_debias16(const float* data, int64_t n, const float* pdf_sum, const float* weighted_sum,
                 int64_t w_row_stride, int64_t w_col_stride, double bandwidth, double eps, float* debiased,
                 float* score, void* stream) {
  NvtxRange nvtx_range("fsk_debias16");
  if (!data || !pdf_sum || !weighted_sum || !debiased || n < 1 || bad_bw(bandwidth) || !(eps >= 0.0))
    return FSK_ERR_INVALID_ARGUMENT;
  int st = check_device();
  if (st) return st;
  launch_debias16(data, n, pdf_sum, weighted_sum, w_row_stride, w_col_stride, bandwidth, eps, debiased,
                  score, static_cast<cudaStream_t>(stream));
  return cuda_status(cudaGetLastError());
}

// ---- one-call SD-KDE: score -> debias -> KDE --------------------------------------
// Workspace: pdf_sum (n) | weighted_sum (n, 16) | debiased (n, 16) unless the
// caller takes it | the larger of the score and KDE workspaces (they run one
// after the other on the stream and share it).
static const int kSdkdeScoreFlags = FSK_PREC_IEEE;
static const int kSdkdeKdeFlags = FSK_PREC_IEEE | FSK_OUT_LOG | FSK_OUT_LOG_EXACT | FSK_ATOMIC;

static size_t sdkde_bytes(int64_t n, int64_t m, int flags) {
  WsCarver c(nullptr, 0);
  c.take<float>((size_t)n);
  c.take<float>((size_t)n * FSK_D);
  c.take<float>((size_t)n * FSK_D);
  const size_t a = fsk_empscore16_workspace_bytes(n, FSK_SCORE_ORDERED, flags & kSdkdeScoreFlags);
  const size_t b = fsk_kde16_workspace_bytes(m, n, flags & kSdkdeKdeFlags);
  c.used = align_up(c.used, 256) + (a > b ? a : b);
  return align_up(c.used, 256);
}

size_t fsk_sdkde16_workspace_bytes(int64_t n, int64_t m, int flags) {
  if (n < 1 || m < 1) return 0;
  return sdkde_bytes(n, m, flags);
}

int fsk_sdkde16(const float* data, int64_t n, const float* queries, int64_t m, double bandwidth, int flags,
                double eps, double out_scale, double out_eps, float* debiased, float* out, void* workspace,
                size_t workspace_bytes, void* stream) {
  NvtxRange nvtx_range("fsk_sdkde16");
  if (!data || !queries || !out || n < 1 || m < 1 || bad_bw(bandwidth) || !(eps >= 0.0))
    return FSK_ERR_INVALID_ARGUMENT;
  if (flags & ~kSdkdeKdeFlags) return FSK_ERR_INVALID_ARGUMENT;
  int st = validate_kde16_args(queries, m, data, n, bandwidth, flags & kSdkdeKdeFlags, out_eps, out);
  if (st) return st;
  st = check_device();
  if (st) return st;
  if (!workspace || workspace_bytes < sdkde_bytes(n, m, flags)) return FSK_ERR_WORKSPACE_TOO_SMALL;
  WsCarver c(workspace, workspace_bytes);
  float* pdf = c.take<float>((size_t)n);
  float* w = c.take<float>((size_t)n * FSK_D);
  float* deb_ws = c.take<float>((size_t)n * FSK_D);
  float* deb = debiased ? debiased : deb_ws;
  c.used = align_up(c.used, 256);
  void* rest = static_cast<char*>(workspace) + c.used;
  const size_t rest_bytes = workspace_bytes - c.used;
  st = fsk_empscore16(data, n, bandwidth, FSK_SCORE_ORDERED, flags & kSdkdeScoreFlags, pdf, w, rest, rest_bytes,
                      stream);
  if (st) return st;
  st = fsk_debias16(data, n, pdf, w, FSK_D, 1, bandwidth, eps, deb, nullptr, stream);
  if (st) return st;
  return fsk_kde16(queries, m, deb, n, bandwidth, flags & kSdkdeKdeFlags, out_scale, out_eps, out, rest, rest_bytes,
                   stream);
}

// ---- any d <= FSK_ND_MAX (CUDA cores) ------------------------------------------------
size_t fsk_kde_nd_workspace_bytes(int64_t m, int64_t n, int d, int flags) {
  (void)flags;
  if (m < 1 || n < 1 || d < 1 || d > FSK_ND_MAX) return 0;
  return align_up((size_t)kde_nd_splits(m, n, d) * m * sizeof(double), 256);
}

int fsk_kde_nd(const float* queries, int64_t m, const float* data, int64_t n, int d, double bandwidth, int flags,
               double out_scale, double out_eps, float* out, void* workspace, size_t workspace_bytes, void* stream) {
  NvtxRange nvtx_range("fsk_kde_nd");
  if (!queries || !data || !out || m < 1 || n < 1 || d < 1 || d > FSK_ND_MAX || bad_bw(bandwidth))
    return FSK_ERR_INVALID_ARGUMENT;
  if (flags & ~(FSK_PREC_IEEE | FSK_LAPLACE | FSK_OUT_LOG | FSK_ATOMIC)) return FSK_ERR_INVALID_ARGUMENT;
  int st = check_device();
  if (st) return st;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (!workspace || workspace_bytes < fsk_kde_nd_workspace_bytes(m, n, d, flags)) return FSK_ERR_WORKSPACE_TOO_SMALL;
  const int splits = kde_nd_splits(m, n, d);
  double* part = static_cast<double*>(workspace);
  launch_kde_nd(queries, m, data, n, d, bandwidth, (flags & FSK_LAPLACE) != 0, splits, part, s);
  launch_reduce_rows(part, splits, m, out_scale, out_eps, (flags & FSK_OUT_LOG) != 0, out, s);
  return cuda_status(cudaGetLastError());
}

static size_t empscore_nd_bytes(int64_t n, int d) {
  WsCarver c(nullptr, 0);
  const int splits = score_nd_splits(n);
  c.take<double>((size_t)FSK_ND_MAX);
  c.take<float>((size_t)FSK_ND_MAX);
  c.take<double>((size_t)splits * n);
  c.take<double>((size_t)splits * n * d);
  return align_up(c.used, 256);
}

size_t fsk_empscore_nd_workspace_bytes(int64_t n, int d) {
  if (n < 1 || d < 1 || d > FSK_ND_MAX) return 0;
  return empscore_nd_bytes(n, d);
}

int fsk_empscore_nd(const float* data, int64_t n, int d, double bandwidth, float* pdf_sum, float* weighted_sum,
                    void* workspace, size_t workspace_bytes, void* stream) {
  NvtxRange nvtx_range("fsk_empscore_nd");
  if (!data || !pdf_sum || !weighted_sum || n < 1 || d < 1 || d > FSK_ND_MAX || bad_bw(bandwidth))
    return FSK_ERR_INVALID_ARGUMENT;
  int st = check_device();
  if (st) return st;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (!workspace || workspace_bytes < empscore_nd_bytes(n, d)) return FSK_ERR_WORKSPACE_TOO_SMALL;
  WsCarver c(workspace, workspace_bytes);
  const int splits = score_nd_splits(n);
  double* mu64 = c.take<double>((size_t)FSK_ND_MAX);
  float* mu = c.take<float>((size_t)FSK_ND_MAX);
  double* ppdf = c.take<double>((size_t)splits * n);
  double* pw = c.take<double>((size_t)splits * n * d);
  launch_score_nd(data, n, d, bandwidth, splits, mu64, mu, ppdf, pw, pdf_sum, weighted_sum, s);
  return cuda_status(cudaGetLastError());
}

int fsk_debias_nd(const float* data, int64_t n, int d, const float* pdf_sum, const float* weighted_sum,
                  double bandwidth, double eps, float* debiased, float* score, void* stream) {
  NvtxRange nvtx_range("fsk_debias_nd");
  if (!data || !pdf_sum || !weighted_sum || !debiased || n < 1 || d < 1 || d > FSK_ND_MAX || bad_bw(bandwidth) ||
      !(eps >= 0.0))
    return FSK_ERR_INVALID_ARGUMENT;
  int st = check_device();
  if (st) return st;
  launch_debias_nd(data, n, d, pdf_sum, weighted_sum, bandwidth, eps, debiased, score,
                   static_cast<cudaStream_t>(stream));
  return cuda_status(cudaGetLastError());
}

// ---- 1-D ------------------------------------------------------------------------
size_t fsk_kde1d_workspace_bytes(int64_t m, int64_t n, int flags) {
  if (m < 1 || n < 1) return 0;
  const int splits = (flags & FSK_ATOMIC) ? 1 : kde1d_splits(m, n);
  // the score variant needs two partial arrays
  return align_up((size_t)2 * splits * m * sizeof(double), 256);
}

int fsk_kde1d(const float* queries, int64_t m, const float* data, int64_t n, double bandwidth, int flags,
              double out_scale, double out_eps, float* out, void* workspace, size_t workspace_bytes,
              void* stream) {
  NvtxRange nvtx_range("fsk_kde1d");
  if (!queries || !data || !out || m < 1 || n < 1 || bad_bw(bandwidth)) return FSK_ERR_INVALID_ARGUMENT;
  if (flags & ~KNOWN_FLAGS) return FSK_ERR_INVALID_ARGUMENT;
  int st = check_device();
  if (st) return st;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (!workspace || workspace_bytes < fsk_kde1d_workspace_bytes(m, n, flags)) return FSK_ERR_WORKSPACE_TOO_SMALL;
  const bool atomic = (flags & FSK_ATOMIC) != 0;
  const int splits = kde1d_splits(m, n);
  double* part = static_cast<double*>(workspace);
  if (atomic) launch_zero(part, m, s);
  launch_kde1d(queries, m, data, n, bandwidth, (flags & FSK_LAPLACE) != 0, splits, atomic ? nullptr : part,
               atomic ? part : nullptr, s);
  launch_reduce_rows(part, atomic ? 1 : splits, m, out_scale, out_eps, (flags & FSK_OUT_LOG) != 0, out, s);
  return cuda_status(cudaGetLastError());
}

int fsk_kde1d_score(const float* queries, int64_t m, const float* data, int64_t n, double bandwidth,
                    float* score, float* pdf, float* deriv, void* workspace, size_t workspace_bytes,
                    void* stream) {
  NvtxRange nvtx_range("fsk_kde1d_score");
  if (!queries || !data || m < 1 || n < 1 || bad_bw(bandwidth)) return FSK_ERR_INVALID_ARGUMENT;
  int st = check_device();
  if (st) return st;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (!workspace || workspace_bytes < fsk_kde1d_workspace_bytes(m, n, 0)) return FSK_ERR_WORKSPACE_TOO_SMALL;
  const int splits = kde1d_splits(m, n);
  double* p0 = static_cast<double*>(workspace);
  double* p1 = p0 + (size_t)splits * m;
  launch_kde1d_score(queries, m, data, n, bandwidth, splits, p0, p1, s);
  launch_reduce_kde1d_score(p0, p1, splits, m, n, bandwidth, score, pdf, deriv, s);
  return cuda_status(cudaGetLastError());
}

// ---- bandwidth --------------------------------------------------------------------
size_t fsk_silverman_workspace_bytes(int64_t n, int d) {
  if (n < 1 || d < 1) return 0;
  return silverman_ws_bytes(n, d);
}

int fsk_silverman(const float* data, int64_t n, int d, int rule, double* h_out, void* workspace,
                  size_t workspace_bytes, void* stream) {
  NvtxRange nvtx_range("fsk_silverman");
  if (!data || !h_out || n < 1 || d < 1 || d > 64) return FSK_ERR_INVALID_ARGUMENT;
  if (rule != FSK_RULE_SILVERMAN && rule != FSK_RULE_SDKDE_1D) return FSK_ERR_INVALID_ARGUMENT;
  if (rule == FSK_RULE_SDKDE_1D && d != 1) return FSK_ERR_INVALID_ARGUMENT;
  int st = check_device();
  if (st) return st;
  if (!workspace || workspace_bytes < silverman_ws_bytes(n, d)) return FSK_ERR_WORKSPACE_TOO_SMALL;
  return run_silverman(data, n, d, rule, h_out, workspace, workspace_bytes, static_cast<cudaStream_t>(stream));
}

int fsk_reduce_partials(const float* partials, int64_t splits, int64_t count, float* out, void* stream) {
  NvtxRange nvtx_range("fsk_reduce_partials");
  if (!partials || !out || splits < 1 || count < 0) return FSK_ERR_INVALID_ARGUMENT;
  if (count == 0) return FSK_OK;
  int st = check_device();
  if (st) return st;
  launch_reduce_f32_partials(partials, splits, count, out, static_cast<cudaStream_t>(stream));
  return cuda_status(cudaGetLastError());
}

// ---- diagnostics: single-MMA probe (not part of fsk.h's hot path) ----------------
int fsk_diag_wait_timeout_probe(int* out, void* stream) {
  if (!out) return FSK_ERR_INVALID_ARGUMENT;
  int st = check_device();
  if (st) return st;
  return tc::launch_wait_timeout_probe(out, static_cast<cudaStream_t>(stream));
}

int fsk_diag_mma_probe(const float* a, const float* b, float* d, void* stream) {
  if (!a || !b || !d) return FSK_ERR_INVALID_ARGUMENT;
  int st = check_device();
  if (st) return st;
  return tc::launch_mma_probe(a, b, d, static_cast<cudaStream_t>(stream));
}

int fsk_diag_mma_ts_probe(const float* a, const float* b, float* d, void* stream) {
  if (!a || !b || !d) return FSK_ERR_INVALID_ARGUMENT;
  int st = check_device();
  if (st) return st;
  return tc::launch_mma_ts_probe(a, b, d, static_cast<cudaStream_t>(stream));
}

int fsk_diag_tmem_cp_probe(const float* a, uint32_t* out, void* stream) {
  if (!a || !out) return FSK_ERR_INVALID_ARGUMENT;
  int st = check_device();
  if (st) return st;
  return tc::launch_tmem_cp_probe(a, out, static_cast<cudaStream_t>(stream));
}

}  // extern "C"
