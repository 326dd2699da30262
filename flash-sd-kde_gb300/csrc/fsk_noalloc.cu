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
//    FSK_ERR_SCRATCH_LIMIT before any work is enqueued (after the argument
//    checks of fsk_kde16, so a bad argument gives FSK_ERR_INVALID_ARGUMENT
//    whatever the size).
//  * All calls on a device share the array and it keeps the previous call's
//    contents; each call writes or clears (the atomic accumulator, the scale
//    maxima, the exact-log query counter) everything it reads, so no state
//    leaks between calls.  Calls whose GPU work overlaps - on two streams, or
//    from two host threads without ordering - race on the array and must be
//    serialised by the caller.
//  * Every call looks up the array's address in the calling thread's current
//    CUDA context (cudaGetSymbolAddress: a host-side query that allocates
//    nothing and does not synchronise), so the address stays right when the
//    caller switches contexts (cuCtxPushCurrent) or after cudaDeviceReset.
//    The first call in a context loads this library's device code into it;
//    make that first call before any stream capture in that context.
#include "fsk_kernels.cuh"

static __device__ __align__(256) unsigned char g_noalloc_scratch[FSK_NOALLOC_SCRATCH_BYTES];

extern "C" int fsk_kde16_noalloc(const float* queries, int64_t m, const float* data, int64_t n,
                                 double bandwidth, int flags, double out_scale, double out_eps,
                                 float* out, void* stream) {
  int st = fsk::validate_kde16_args(queries, m, data, n, bandwidth, flags, out_eps, out);
  if (st) return st;
  if (fsk_kde16_workspace_bytes(m, n, flags) > (size_t)FSK_NOALLOC_SCRATCH_BYTES) return FSK_ERR_SCRATCH_LIMIT;
  st = fsk::check_device();
  if (st) return st;
  // Device address of the array in the current context.  In host code the
  // name g_noalloc_scratch is only a host-side stand-in for it.
  void* ws = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&ws, g_noalloc_scratch);
  if (e != cudaSuccess || ws == nullptr) return FSK_ERR_CUDA;
  return fsk_kde16(queries, m, data, n, bandwidth, flags, out_scale, out_eps, out, ws,
                   (size_t)FSK_NOALLOC_SCRATCH_BYTES, stream);
}
