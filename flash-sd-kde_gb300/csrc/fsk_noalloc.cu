// fsk_noalloc.cu - the 16-D KDE for callers that cannot allocate device memory.
//
// Who needs it: hosts that reach this library only through its C ABI (an FFI
// binding from another language runtime, a database or server plug-in) and
// have no device allocator they may call, processes whose GPU memory is
// owned and budgeted by some other allocator, and latency-sensitive loops in
// which a cudaMalloc/cudaFree pair would synchronise the whole device.  For
// them fsk_kde16_noalloc computes exactly what fsk_kde16 computes, but keeps
// its scratch (data/query operand images, split partial sums, centring and
// scale state) in one fixed file-scope device array instead of a workspace
// passed in by the caller.  It calls no cudaMalloc, cudaFree or allocating
// library routine.
//
// What the caller must know:
//  * The array is FSK_NOALLOC_SCRATCH_BYTES (32 MiB) on every GPU that loads
//    this library, held until the process exits.  A request whose
//    fsk_kde16_workspace_bytes(m, n, flags) exceeds it is rejected with
//    FSK_ERR_SCRATCH_LIMIT before any work is enqueued.
//  * All calls on a device share the array and it keeps the previous call's
//    contents; each call writes or clears (the atomic accumulator, the scale
//    maxima) everything it reads, so no state leaks between calls.  Calls
//    whose GPU work overlaps - on two streams, or from two host threads
//    without ordering - race on the array and must be serialised by the
//    caller.
//  * The first call on each device, with that device current, looks up the
//    array's device address (cudaGetSymbolAddress) and caches it; make that
//    first call before any stream capture on that device.
#include <mutex>

#include "fsk_kernels.cuh"

static __device__ __align__(256) unsigned char g_noalloc_scratch[FSK_NOALLOC_SCRATCH_BYTES];

namespace {
constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mu;
void* g_noalloc_ptr[kMaxDevices];  // device address of the array, per device ordinal

// Device address of the scratch array on the current device (set up once).
int noalloc_scratch(void** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return FSK_ERR_CUDA;
  if (dev < 0 || dev >= kMaxDevices) return FSK_ERR_UNSUPPORTED_DEVICE;
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  if (g_noalloc_ptr[dev] == nullptr) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || p == nullptr) return FSK_ERR_CUDA;
    g_noalloc_ptr[dev] = p;
  }
  *out = g_noalloc_ptr[dev];
  return FSK_OK;
}
}  // namespace

extern "C" int fsk_kde16_noalloc(const float* queries, int64_t m, const float* data, int64_t n,
                                 double bandwidth, int flags, double out_scale, double out_eps,
                                 float* out, void* stream) {
  if (!queries || !data || !out || m < 1 || n < 1) return FSK_ERR_INVALID_ARGUMENT;
  const size_t need = fsk_kde16_workspace_bytes(m, n, flags);
  if (need == 0) return FSK_ERR_INVALID_ARGUMENT;
  if (need > (size_t)FSK_NOALLOC_SCRATCH_BYTES) return FSK_ERR_SCRATCH_LIMIT;
  int st = fsk::check_device();
  if (st) return st;
  void* ws = nullptr;
  st = noalloc_scratch(&ws);
  if (st) return st;
  return fsk_kde16(queries, m, data, n, bandwidth, flags, out_scale, out_eps, out, ws,
                   (size_t)FSK_NOALLOC_SCRATCH_BYTES, stream);
}
