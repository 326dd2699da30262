// fsk_mlp_api.cu - the extern "C" entry points of the learned surrogate
// (include/fsk.h, "learned surrogate").  Argument checks, workspace
// carving, kernel launches on the caller's stream; no allocation, no
// synchronisation, no host fallback.
#include "fsk_kernels.cuh"
#include "fsk_mlp.cuh"

using namespace fsk;

namespace {
constexpr int MAX_MEMBERS = 8;
bool bad_members(int m) { return m < 1 || m > MAX_MEMBERS; }
size_t train_bytes(int members, int64_t batch) {
  WsCarver c(nullptr, 0);
  mlp::carve_train(c, members, batch);
  return align_up(c.used, 256);
}
}  // namespace

extern "C" {

size_t fsk_mlp_train_workspace_bytes(int members, int64_t batch) {
  if (bad_members(members) || batch < 1) return 0;
  return train_bytes(members, batch);
}

int fsk_mlp_fwd(const float* params, int members, const float* x, int64_t batch, const float* in_mean,
                const float* in_inv_std, float* y, void* workspace, size_t workspace_bytes, void* stream) {
  if (!params || !x || !in_mean || !in_inv_std || !y || bad_members(members) || batch < 1 || batch > (1LL << 31))
    return FSK_ERR_INVALID_ARGUMENT;
  int st = check_device();
  if (st) return st;
  if (!workspace || workspace_bytes < train_bytes(members, batch)) return FSK_ERR_WORKSPACE_TOO_SMALL;
  WsCarver c(workspace, workspace_bytes);
  const mlp::TrainBufs t = mlp::carve_train(c, members, batch);
  mlp::launch_forward(params, members, x, batch, in_mean, in_inv_std, t, y, static_cast<cudaStream_t>(stream));
  return cuda_status(cudaGetLastError());
}

int fsk_mlp_bwd(const float* params, int members, int64_t batch, const float* dy, float* grads, void* workspace,
                size_t workspace_bytes, void* stream) {
  if (!params || !dy || !grads || bad_members(members) || batch < 1 || batch > (1LL << 31))
    return FSK_ERR_INVALID_ARGUMENT;
  int st = check_device();
  if (st) return st;
  if (!workspace || workspace_bytes < train_bytes(members, batch)) return FSK_ERR_WORKSPACE_TOO_SMALL;
  WsCarver c(workspace, workspace_bytes);
  const mlp::TrainBufs t = mlp::carve_train(c, members, batch);
  mlp::launch_backward(params, members, batch, t, dy, grads, static_cast<cudaStream_t>(stream));
  return cuda_status(cudaGetLastError());
}

int fsk_mlp_mse(const float* y, const float* target, int64_t batch, int members, float* dy, double* loss,
                void* stream) {
  if (!y || !target || !dy || bad_members(members) || batch < 1) return FSK_ERR_INVALID_ARGUMENT;
  int st = check_device();
  if (st) return st;
  mlp::launch_mse(y, target, batch, members, dy, loss, static_cast<cudaStream_t>(stream));
  return cuda_status(cudaGetLastError());
}

int fsk_mlp_adam(float* params, const float* grads, float* m, float* v, int64_t count, float lr, float beta1,
                 float beta2, float eps, float weight_decay, int step, void* stream) {
  if (!params || !grads || !m || !v || count < 1 || step < 1 || !(lr >= 0.f) || !(beta1 >= 0.f && beta1 < 1.f) ||
      !(beta2 >= 0.f && beta2 < 1.f) || !(eps > 0.f) || !(weight_decay >= 0.f))
    return FSK_ERR_INVALID_ARGUMENT;
  int st = check_device();
  if (st) return st;
  mlp::launch_adam(params, grads, m, v, count, lr, beta1, beta2, eps, weight_decay, step,
                   static_cast<cudaStream_t>(stream));
  return cuda_status(cudaGetLastError());
}

size_t fsk_mlp_packed_bytes(int members) { return bad_members(members) ? 0 : mlp::packed_bytes(members); }

int fsk_mlp_pack(const float* params, int members, const float* in_mean, const float* in_inv_std, float out_scale,
                 float out_shift, void* packed, void* stream) {
  if (!params || !in_mean || !in_inv_std || !packed || bad_members(members) || (reinterpret_cast<uintptr_t>(packed) & 15))
    return FSK_ERR_INVALID_ARGUMENT;
  int st = check_device();
  if (st) return st;
  return mlp::launch_pack(params, members, in_mean, in_inv_std, out_scale, out_shift, packed,
                          static_cast<cudaStream_t>(stream));
}

int fsk_mlp_infer(const void* packed, int members, const float* x, int64_t batch, float* y, void* stream) {
  NvtxRange nvtx_range("fsk_mlp_infer");
  if (!packed || !x || !y || bad_members(members) || batch < 1 || (reinterpret_cast<uintptr_t>(x) & 15) ||
      (reinterpret_cast<uintptr_t>(packed) & 15))
    return FSK_ERR_INVALID_ARGUMENT;
  int st = check_device();
  if (st) return st;
  return mlp::launch_infer(packed, members, x, batch, y, static_cast<cudaStream_t>(stream));
}

int fsk_mlp_combine(const float* y, int members, int64_t batch, const float* x, const float* in_mean,
                    const float* in_inv_std, float base_a, float base_b, float spread_tol, float r2_max, float* mean,
                    float* spread, uint8_t* served, void* stream) {
  NvtxRange nvtx_range("fsk_mlp_combine");
  if (!y || bad_members(members) || batch < 1 || (x && (!in_mean || !in_inv_std))) return FSK_ERR_INVALID_ARGUMENT;
  int st = check_device();
  if (st) return st;
  mlp::launch_combine(y, members, batch, x, in_mean, in_inv_std, base_a, base_b, spread_tol, r2_max, mean, spread,
                      served, static_cast<cudaStream_t>(stream));
  return cuda_status(cudaGetLastError());
}

}  // extern "C"
