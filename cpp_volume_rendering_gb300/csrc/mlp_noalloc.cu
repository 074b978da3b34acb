// mlp_noalloc.cu — the network gradient without any allocation: the same
// training-tile and reduction kernels as cvr_mlp_gradients, with their scratch
// (per-tile gradient partials, the point index list and the reduced gradient)
// in one fixed device array of this file instead of cudaMalloc'd buffers.
//
// Who needs it: a caller that must not allocate device memory while it runs
// its own loop — for example a process whose device memory is held by another
// framework's caching allocator (a cudaMalloc there can fail or fragment that
// pool), or a latency-bound loop in which cudaMalloc / cudaFree would stall
// the device (cudaFree synchronises).  Inputs and outputs are the caller's
// device buffers.
#include <mutex>

#include "ctx.cuh"
#include "mlp.cuh"

using namespace cvr::ctxutil;

namespace {

constexpr int kMaxPoints = CVR_MLP_NOALLOC_MAX_POINTS;
constexpr int kMaxTiles = kMaxPoints / 128;
constexpr size_t kPartFloats = (size_t)kMaxTiles * (kMlpParams + 1);  // per-tile partials
constexpr size_t kRedFloats = ((kMlpParams + 1 + 63) / 64) * 64;      // reduced gradient + loss
constexpr size_t kScratchBytes = (kPartFloats + kRedFloats) * sizeof(float) + (size_t)kMaxPoints * sizeof(int);

// Layout: [partials: kPartFloats floats][reduced: kRedFloats floats][index: kMaxPoints ints].
// The partials and the reduced gradient are fully written by every call
// before they are read; the index list must hold 0, 1, ..., kMaxPoints-1,
// which the set-up writes once per device.
static __device__ __align__(256) unsigned char g_scratch[kScratchBytes];

__global__ void k_fill_identity(int* idx, int n) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) idx[i] = i;
}

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
unsigned char* g_scratch_ptr[kMaxDevices] = {};

// Once per device, with that device current: the scratch address and the
// identity index list.  Synchronises the context stream.
cvr_status setup(cvr_ctx* c, unsigned char** out) {
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (c->device < 0 || c->device >= kMaxDevices)
    return fail(c, CVR_ERR_UNSUPPORTED, "cvr_mlp_gradients_noalloc: device index above 63");
  if (!g_scratch_ptr[c->device]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_scratch);
    if (e != cudaSuccess) return cuda_fail(c, e, "cvr_mlp_gradients_noalloc: cudaGetSymbolAddress");
    int* idx = reinterpret_cast<int*>(static_cast<unsigned char*>(p) + (kPartFloats + kRedFloats) * sizeof(float));
    k_fill_identity<<<(kMaxPoints + 255) / 256, 256, 0, c->stream>>>(idx, kMaxPoints);
    if ((e = cudaGetLastError()) != cudaSuccess) return cuda_fail(c, e, "cvr_mlp_gradients_noalloc: set-up launch");
    if ((e = cudaStreamSynchronize(c->stream)) != cudaSuccess)
      return cuda_fail(c, e, "cvr_mlp_gradients_noalloc: set-up");
    g_scratch_ptr[c->device] = static_cast<unsigned char*>(p);
  }
  *out = g_scratch_ptr[c->device];
  return CVR_OK;
}

}  // namespace

extern "C" {

cvr_status cvr_mlp_gradients_noalloc(cvr_ctx* c, const float* x_dev, const float* t_dev, int n, float* grad_dev,
                                     float* loss_dev) {
  if (!c) return CVR_ERR_INVALID_ARG;
  if (!c->mlp || !c->mlp->ready) return fail(c, CVR_ERR_NOT_READY, "cvr_mlp_gradients_noalloc: no network");
  if (!x_dev || !t_dev || !grad_dev || n <= 0)
    return fail(c, CVR_ERR_INVALID_ARG, "cvr_mlp_gradients_noalloc: bad arguments");
  if (n > kMaxPoints)
    return fail(c, CVR_ERR_INVALID_ARG,
                "cvr_mlp_gradients_noalloc: n exceeds CVR_MLP_NOALLOC_MAX_POINTS (8192); split the batch or use "
                "cvr_mlp_gradients");
  CK(c, cudaSetDevice(c->device));
  unsigned char* base = nullptr;
  cvr_status st = setup(c, &base);
  if (st != CVR_OK) return st;
  float* partials = reinterpret_cast<float*>(base);
  float* reduced = partials + kPartFloats;
  const int* idx = reinterpret_cast<const int*>(reduced + kRedFloats);
  MlpState& s = *c->mlp;
  const int tiles = (n + 127) / 128;
  CK(c, launch_mlp_train_tiles(s.packed, x_dev, t_dev, idx, n, 1.0f / (float)n, partials, nullptr, s.err, c->stream));
  CK(c, launch_mlp_adam(s.params, s.m, s.v, partials, tiles, 0.0f, 0.9f, 0.999f, 1e-8f, nullptr, reduced, c->stream));
  CK(c, cudaMemcpyAsync(grad_dev, reduced, sizeof(float) * kMlpParams, cudaMemcpyDeviceToDevice, c->stream));
  if (loss_dev)
    CK(c, cudaMemcpyAsync(loss_dev, reduced + kMlpParams, sizeof(float), cudaMemcpyDeviceToDevice, c->stream));
  return CVR_OK;
}

}  // extern "C"
