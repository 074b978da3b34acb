// mlp_host.cu — C ABI of the surrogate network: parameters, batch inference,
// gradients, training data and the Adam training loop (one CUDA graph per
// epoch, replayed with a fresh permutation each epoch).
#include <algorithm>
#include <cmath>
#include <numeric>
#include <random>
#include <vector>

#include "ctx.cuh"
#include "mlp.cuh"

using namespace cvr::ctxutil;

namespace {

cvr_status need_mlp(cvr_ctx* c) {
  if (!c) return CVR_ERR_INVALID_ARG;
  if (!c->mlp || !c->mlp->ready) return fail(c, CVR_ERR_NOT_READY, "surrogate network not initialised (cvr_mlp_init)");
  return CVR_OK;
}

cvr_status alloc_mlp(cvr_ctx* c) {
  if (c->mlp && c->mlp->params) return CVR_OK;
  c->mlp.reset(new MlpState());
  MlpState& s = *c->mlp;
  CK(c, cudaSetDevice(c->device));
  CK(c, cudaMalloc((void**)&s.params, sizeof(float) * kMlpParams));
  CK(c, cudaMalloc((void**)&s.m, sizeof(float) * kMlpParams));
  CK(c, cudaMalloc((void**)&s.v, sizeof(float) * kMlpParams));
  CK(c, cudaMalloc((void**)&s.packed, kPkBytes));
  CK(c, cudaMalloc((void**)&s.grad, sizeof(float) * (kMlpParams + 1)));
  CK(c, cudaMalloc((void**)&s.loss_acc, sizeof(float)));
  CK(c, cudaMalloc((void**)&s.err, sizeof(int)));
  CK(c, cudaMalloc((void**)&s.step, sizeof(int)));
  CK(c, cudaMemsetAsync(s.packed, 0, kPkBytes, c->stream));  // padding of the BF16 tiles stays zero
  CK(c, cudaMemsetAsync(s.err, 0, sizeof(int), c->stream));
  return CVR_OK;
}

cvr_status reset_optimizer(cvr_ctx* c) {
  MlpState& s = *c->mlp;
  CK(c, cudaMemsetAsync(s.m, 0, sizeof(float) * kMlpParams, c->stream));
  CK(c, cudaMemsetAsync(s.v, 0, sizeof(float) * kMlpParams, c->stream));
  CK(c, cudaMemsetAsync(s.step, 0, sizeof(int), c->stream));
  return CVR_OK;
}

cvr_status check_err(cvr_ctx* c) {
  int e = 0;
  CK(c, cudaMemcpyAsync(&e, c->mlp->err, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  CK(c, cudaStreamSynchronize(c->stream));
  if (e) {
    cudaMemsetAsync(c->mlp->err, 0, sizeof(int), c->stream);
    return fail(c, CVR_ERR_TIMEOUT, "a tensor-core wait gave up (bounded mbarrier wait)");
  }
  return CVR_OK;
}

template <class T>
cudaError_t grow(T*& p, size_t& cap, size_t n) {
  if (cap >= n && p) return cudaSuccess;
  if (p) cudaFree(p);
  p = nullptr;
  cap = 0;
  cudaError_t e = cudaMalloc((void**)&p, sizeof(T) * n);
  if (e == cudaSuccess) cap = n;
  return e;
}

// Bumps the Adam step counter after an update (single thread).
__global__ void k_step_inc(int* step) { *step += 1; }
__global__ void k_add_loss(float* acc, const float* grad) { *acc += grad[kMlpParams]; }

// One Adam step on the batch of 'count' points starting at idx[offset].
cvr_status enqueue_step(cvr_ctx* c, int offset, int count, float lr) {
  MlpState& s = *c->mlp;
  int tiles = (count + 127) / 128;
  CK(c, launch_mlp_train_tiles(s.packed, s.x, s.t, s.idx + offset, count, 1.0f / (float)count, s.partials, nullptr,
                               s.err, c->stream));
  // step counter: read as step + 1 inside the update
  CK(c, launch_mlp_adam(s.params, s.m, s.v, s.partials, tiles, lr, 0.9f, 0.999f, 1e-8f, s.step, s.grad, c->stream));
  k_add_loss<<<1, 1, 0, c->stream>>>(s.loss_acc, s.grad);
  CK(c, cudaGetLastError());
  k_step_inc<<<1, 1, 0, c->stream>>>(s.step);
  CK(c, cudaGetLastError());
  CK(c, launch_mlp_pack(s.params, s.packed, c->stream));
  return CVR_OK;
}

}  // namespace

extern "C" {

cvr_status cvr_mlp_init(cvr_ctx* c, uint64_t seed) {
  if (!c) return CVR_ERR_INVALID_ARG;
  cvr_status st = alloc_mlp(c);
  if (st != CVR_OK) return st;
  // He-uniform: U(-sqrt(6/fan_in), sqrt(6/fan_in)), zero biases.
  std::vector<float> p(kMlpParams, 0.0f);
  std::mt19937_64 rng(seed);
  auto fill = [&](int off, int n, int fan_in) {
    double a = std::sqrt(6.0 / fan_in);
    std::uniform_real_distribution<double> d(-a, a);
    for (int i = 0; i < n; ++i) p[off + i] = (float)d(rng);
  };
  fill(kOffW1, 64 * 48, 48);
  fill(kOffW2, 64 * 64, 64);
  fill(kOffW3, 2 * 64, 64);
  return cvr_mlp_set_params(c, p.data(), kMlpParams);
}

cvr_status cvr_mlp_set_params(cvr_ctx* c, const float* params, int n) {
  if (!c || !params || n != kMlpParams) return fail(c, CVR_ERR_INVALID_ARG, "cvr_mlp_set_params: need CVR_MLP_PARAMS floats");
  for (int i = 0; i < n; ++i)
    if (!std::isfinite(params[i])) return fail(c, CVR_ERR_INVALID_ARG, "cvr_mlp_set_params: non-finite parameter");
  cvr_status st = alloc_mlp(c);
  if (st != CVR_OK) return st;
  MlpState& s = *c->mlp;
  CK(c, cudaMemcpyAsync(s.params, params, sizeof(float) * kMlpParams, cudaMemcpyHostToDevice, c->stream));
  st = reset_optimizer(c);
  if (st != CVR_OK) return st;
  CK(c, launch_mlp_pack(s.params, s.packed, c->stream));
  CK(c, cudaStreamSynchronize(c->stream));
  s.ready = true;
  return CVR_OK;
}

cvr_status cvr_mlp_get_params(cvr_ctx* c, float* params, int n) {
  cvr_status st = need_mlp(c);
  if (st != CVR_OK) return st;
  if (!params || n != kMlpParams) return fail(c, CVR_ERR_INVALID_ARG, "cvr_mlp_get_params: need CVR_MLP_PARAMS floats");
  CK(c, cudaMemcpyAsync(params, c->mlp->params, sizeof(float) * kMlpParams, cudaMemcpyDeviceToHost, c->stream));
  CK(c, cudaStreamSynchronize(c->stream));
  return CVR_OK;
}

cvr_status cvr_mlp_forward(cvr_ctx* c, const float* x, int n, float* y) {
  cvr_status st = need_mlp(c);
  if (st != CVR_OK) return st;
  if (!x || !y || n <= 0) return fail(c, CVR_ERR_INVALID_ARG, "cvr_mlp_forward: bad arguments");
  MlpState& s = *c->mlp;
  if ((size_t)n > s.io_cap) {
    if (s.io_x) cudaFree(s.io_x);
    if (s.io_y) cudaFree(s.io_y);
    s.io_x = s.io_y = nullptr;
    s.io_cap = 0;
    CK(c, cudaMalloc((void**)&s.io_x, sizeof(float) * 48 * (size_t)n));
    CK(c, cudaMalloc((void**)&s.io_y, sizeof(float) * 2 * (size_t)n));
    s.io_cap = (size_t)n;
  }
  CK(c, cudaMemcpyAsync(s.io_x, x, sizeof(float) * 48 * (size_t)n, cudaMemcpyHostToDevice, c->stream));
  CK(c, launch_mlp_infer(s.packed, s.io_x, n, s.io_y, s.err, c->stream));
  CK(c, cudaMemcpyAsync(y, s.io_y, sizeof(float) * 2 * (size_t)n, cudaMemcpyDeviceToHost, c->stream));
  return check_err(c);
}

cvr_status cvr_mlp_check(cvr_ctx* c) {
  if (!c) return CVR_ERR_INVALID_ARG;
  if (!c->mlp) return CVR_OK;
  CK(c, cudaSetDevice(c->device));
  return check_err(c);
}

cvr_status cvr_mlp_gradients(cvr_ctx* c, const float* x, const float* t, int n, float* grad, float* loss) {
  cvr_status st = need_mlp(c);
  if (st != CVR_OK) return st;
  if (!x || !t || !grad || n <= 0) return fail(c, CVR_ERR_INVALID_ARG, "cvr_mlp_gradients: bad arguments");
  MlpState& s = *c->mlp;
  float* dx = nullptr;
  float* dt = nullptr;
  int* di = nullptr;
  float* parts = nullptr;
  int tiles = (n + 127) / 128;
  cudaError_t e = cudaMalloc((void**)&dx, sizeof(float) * 48 * (size_t)n);
  if (e == cudaSuccess) e = cudaMalloc((void**)&dt, sizeof(float) * 2 * (size_t)n);
  if (e == cudaSuccess) e = cudaMalloc((void**)&di, sizeof(int) * (size_t)n);
  if (e == cudaSuccess) e = cudaMalloc((void**)&parts, sizeof(float) * (kMlpParams + 1) * (size_t)tiles);
  std::vector<int> id(n);
  std::iota(id.begin(), id.end(), 0);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dx, x, sizeof(float) * 48 * (size_t)n, cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dt, t, sizeof(float) * 2 * (size_t)n, cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(di, id.data(), sizeof(int) * (size_t)n, cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess) e = launch_mlp_train_tiles(s.packed, dx, dt, di, n, 1.0f / (float)n, parts, nullptr, s.err, c->stream);
  if (e == cudaSuccess) e = launch_mlp_adam(s.params, s.m, s.v, parts, tiles, 0.0f, 0.9f, 0.999f, 1e-8f, nullptr, s.grad, c->stream);
  std::vector<float> g(kMlpParams + 1);
  if (e == cudaSuccess) e = cudaMemcpyAsync(g.data(), s.grad, sizeof(float) * (kMlpParams + 1), cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  cudaFree(dx);
  cudaFree(dt);
  cudaFree(di);
  cudaFree(parts);
  if (e != cudaSuccess) return cuda_fail(c, e, "cvr_mlp_gradients");
  std::copy(g.begin(), g.begin() + kMlpParams, grad);
  if (loss) *loss = g[kMlpParams];
  return check_err(c);
}

cvr_status cvr_mlp_set_training_data(cvr_ctx* c, const float* x, const float* t, int n) {
  cvr_status st = need_mlp(c);
  if (st != CVR_OK) return st;
  if (n < 0 || (n > 0 && (!x || !t))) return fail(c, CVR_ERR_INVALID_ARG, "cvr_mlp_set_training_data: bad arguments");
  MlpState& s = *c->mlp;
  if (n == 0) {  // clears the training set
    s.n = 0;
    if (s.epoch_graph) {
      cudaGraphExecDestroy(s.epoch_graph);
      s.epoch_graph = nullptr;
    }
    return CVR_OK;
  }
  if ((size_t)n > s.data_cap) {
    if (s.x) cudaFree(s.x);
    if (s.t) cudaFree(s.t);
    s.x = s.t = nullptr;
    s.data_cap = 0;
    CK(c, cudaMalloc((void**)&s.x, sizeof(float) * 48 * (size_t)n));
    CK(c, cudaMalloc((void**)&s.t, sizeof(float) * 2 * (size_t)n));
    s.data_cap = (size_t)n;
  }
  CK(c, cudaMemcpyAsync(s.x, x, sizeof(float) * 48 * (size_t)n, cudaMemcpyHostToDevice, c->stream));
  CK(c, cudaMemcpyAsync(s.t, t, sizeof(float) * 2 * (size_t)n, cudaMemcpyHostToDevice, c->stream));
  CK(c, cudaStreamSynchronize(c->stream));
  s.n = n;
  if (s.epoch_graph) {
    cudaGraphExecDestroy(s.epoch_graph);
    s.epoch_graph = nullptr;
  }
  return CVR_OK;
}

cvr_status cvr_mlp_get_training_data(cvr_ctx* c, float* x, float* t, int n) {
  cvr_status st = need_mlp(c);
  if (st != CVR_OK) return st;
  MlpState& s = *c->mlp;
  if (!x || !t || n != s.n) return fail(c, CVR_ERR_INVALID_ARG, "cvr_mlp_get_training_data: size mismatch");
  CK(c, cudaMemcpyAsync(x, s.x, sizeof(float) * 48 * (size_t)n, cudaMemcpyDeviceToHost, c->stream));
  CK(c, cudaMemcpyAsync(t, s.t, sizeof(float) * 2 * (size_t)n, cudaMemcpyDeviceToHost, c->stream));
  CK(c, cudaStreamSynchronize(c->stream));
  return CVR_OK;
}

int cvr_mlp_training_size(cvr_ctx* c) { return (c && c->mlp) ? c->mlp->n : 0; }

cvr_status cvr_mlp_train(cvr_ctx* c, int epochs, int batch, float lr, uint64_t seed, float* loss_per_epoch) {
  cvr_status st = need_mlp(c);
  if (st != CVR_OK) return st;
  MlpState& s = *c->mlp;
  if (epochs <= 0 || batch <= 0 || batch % 128 || !(lr > 0.0f) || s.n <= 0)
    return fail(c, CVR_ERR_INVALID_ARG, "cvr_mlp_train: need training data, epochs > 0, batch a multiple of 128, lr > 0");
  CK(c, cudaSetDevice(c->device));
  const int n = s.n;
  const int n_batches = (n + batch - 1) / batch;
  CK(c, grow(s.idx, s.idx_cap, (size_t)n));
  CK(c, grow(s.partials, s.partials_cap, (size_t)(batch / 128) * (kMlpParams + 1)));
  // (Re)capture the epoch when the batch structure or the rate changed.
  if (!s.epoch_graph || s.graph_batch != batch || s.graph_n != n || s.graph_lr != lr) {
    if (s.epoch_graph) {
      cudaGraphExecDestroy(s.epoch_graph);
      s.epoch_graph = nullptr;
    }
    cudaGraph_t g = nullptr;
    CK(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
    cudaError_t e = cudaMemsetAsync(s.loss_acc, 0, sizeof(float), c->stream);
    for (int b = 0; b < n_batches && e == cudaSuccess; ++b) {
      int off = b * batch;
      int cnt = std::min(batch, n - off);
      if (enqueue_step(c, off, cnt, lr) != CVR_OK) e = cudaErrorUnknown;
    }
    cudaError_t e2 = cudaStreamEndCapture(c->stream, &g);
    if (e != cudaSuccess || e2 != cudaSuccess) {
      if (g) cudaGraphDestroy(g);
      return cuda_fail(c, e != cudaSuccess ? e : e2, "cvr_mlp_train: epoch capture");
    }
    e = cudaGraphInstantiate(&s.epoch_graph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return cuda_fail(c, e, "cvr_mlp_train: graph instantiate");
    s.graph_batch = batch;
    s.graph_n = n;
    s.graph_lr = lr;
  }
  std::mt19937_64 rng(seed);
  std::vector<int> perm(n);
  std::iota(perm.begin(), perm.end(), 0);
  for (int ep = 0; ep < epochs; ++ep) {
    std::shuffle(perm.begin(), perm.end(), rng);
    CK(c, cudaMemcpyAsync(s.idx, perm.data(), sizeof(int) * (size_t)n, cudaMemcpyHostToDevice, c->stream));
    CK(c, cudaGraphLaunch(s.epoch_graph, c->stream));
    float acc = 0.0f;
    CK(c, cudaMemcpyAsync(&acc, s.loss_acc, sizeof(float), cudaMemcpyDeviceToHost, c->stream));
    CK(c, cudaStreamSynchronize(c->stream));  // perm is reused next epoch
    if (loss_per_epoch) loss_per_epoch[ep] = acc / (float)n_batches;
  }
  return check_err(c);
}

static const char kCkptMagic[8] = {'C', 'V', 'R', 'M', 'L', 'P', '0', '1'};

cvr_status cvr_mlp_save(cvr_ctx* c, const char* path) {
  cvr_status st = need_mlp(c);
  if (st != CVR_OK) return st;
  if (!path) return fail(c, CVR_ERR_INVALID_ARG, "cvr_mlp_save: null path");
  MlpState& s = *c->mlp;
  std::vector<float> buf(3 * (size_t)kMlpParams);
  int step = 0;
  CK(c, cudaMemcpyAsync(buf.data(), s.params, sizeof(float) * kMlpParams, cudaMemcpyDeviceToHost, c->stream));
  CK(c, cudaMemcpyAsync(buf.data() + kMlpParams, s.m, sizeof(float) * kMlpParams, cudaMemcpyDeviceToHost, c->stream));
  CK(c, cudaMemcpyAsync(buf.data() + 2 * kMlpParams, s.v, sizeof(float) * kMlpParams, cudaMemcpyDeviceToHost,
                        c->stream));
  CK(c, cudaMemcpyAsync(&step, s.step, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  CK(c, cudaStreamSynchronize(c->stream));
  FILE* fp = std::fopen(path, "wb");
  if (!fp) return fail(c, CVR_ERR_IO, std::string("cvr_mlp_save: cannot open ") + path);
  const uint32_t hdr[2] = {1u, (uint32_t)kMlpParams};
  bool ok = std::fwrite(kCkptMagic, 1, 8, fp) == 8 && std::fwrite(hdr, sizeof hdr, 1, fp) == 1 &&
            std::fwrite(buf.data(), sizeof(float), buf.size(), fp) == buf.size() &&
            std::fwrite(&step, sizeof step, 1, fp) == 1;
  ok = (std::fclose(fp) == 0) && ok;
  return ok ? CVR_OK : fail(c, CVR_ERR_IO, std::string("cvr_mlp_save: write failed: ") + path);
}

cvr_status cvr_mlp_load(cvr_ctx* c, const char* path) {
  if (!c || !path) return fail(c, CVR_ERR_INVALID_ARG, "cvr_mlp_load: bad arguments");
  FILE* fp = std::fopen(path, "rb");
  if (!fp) return fail(c, CVR_ERR_IO, std::string("cvr_mlp_load: cannot open ") + path);
  char magic[8];
  uint32_t hdr[2] = {0, 0};
  std::vector<float> buf(3 * (size_t)kMlpParams);
  int step = 0;
  bool ok = std::fread(magic, 1, 8, fp) == 8 && std::fread(hdr, sizeof hdr, 1, fp) == 1;
  if (ok && (std::memcmp(magic, kCkptMagic, 8) != 0 || hdr[0] != 1u || hdr[1] != (uint32_t)kMlpParams)) {
    std::fclose(fp);
    return fail(c, CVR_ERR_FORMAT, std::string("cvr_mlp_load: not a version-1 checkpoint of this network: ") + path);
  }
  ok = ok && std::fread(buf.data(), sizeof(float), buf.size(), fp) == buf.size() &&
       std::fread(&step, sizeof step, 1, fp) == 1;
  std::fclose(fp);
  if (!ok) return fail(c, CVR_ERR_FORMAT, std::string("cvr_mlp_load: truncated checkpoint: ") + path);
  cvr_status st = cvr_mlp_set_params(c, buf.data(), kMlpParams);  // also resets the optimiser
  if (st != CVR_OK) return st;
  MlpState& s = *c->mlp;
  CK(c, cudaMemcpyAsync(s.m, buf.data() + kMlpParams, sizeof(float) * kMlpParams, cudaMemcpyHostToDevice, c->stream));
  CK(c, cudaMemcpyAsync(s.v, buf.data() + 2 * kMlpParams, sizeof(float) * kMlpParams, cudaMemcpyHostToDevice,
                        c->stream));
  CK(c, cudaMemcpyAsync(s.step, &step, sizeof(int), cudaMemcpyHostToDevice, c->stream));
  CK(c, cudaStreamSynchronize(c->stream));
  return CVR_OK;
}

}  // extern "C"

namespace cvr {
namespace ctxutil {

cvr_status mlp_check_err(cvr_ctx* c) { return (c && c->mlp && c->mlp->err) ? check_err(c) : CVR_OK; }

cvr_status mlp_reserve_training(cvr_ctx* c, size_t extra, float** x, float** t) {
  cvr_status st = need_mlp(c);
  if (st != CVR_OK) return st;
  MlpState& s = *c->mlp;
  size_t need = (size_t)s.n + extra;
  if (need > (size_t)0x7fffffff) return fail(c, CVR_ERR_INVALID_ARG, "training set larger than 2^31 points");
  if (need > s.data_cap) {
    size_t cap = std::max(need, s.data_cap + s.data_cap / 2);
    float* nx = nullptr;
    float* nt = nullptr;
    cudaError_t e = cudaMalloc((void**)&nx, sizeof(float) * 48 * cap);
    if (e == cudaSuccess) e = cudaMalloc((void**)&nt, sizeof(float) * 2 * cap);
    if (e == cudaSuccess && s.n > 0) {
      e = cudaMemcpyAsync(nx, s.x, sizeof(float) * 48 * (size_t)s.n, cudaMemcpyDeviceToDevice, c->stream);
      if (e == cudaSuccess)
        e = cudaMemcpyAsync(nt, s.t, sizeof(float) * 2 * (size_t)s.n, cudaMemcpyDeviceToDevice, c->stream);
      if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    }
    if (e != cudaSuccess) {
      if (nx) cudaFree(nx);
      if (nt) cudaFree(nt);
      return cuda_fail(c, e, "training set allocation");
    }
    if (s.x) cudaFree(s.x);
    if (s.t) cudaFree(s.t);
    s.x = nx;
    s.t = nt;
    s.data_cap = cap;
  }
  if (s.epoch_graph) {  // the graph captured the old buffers
    cudaGraphExecDestroy(s.epoch_graph);
    s.epoch_graph = nullptr;
  }
  *x = s.x + 48 * (size_t)s.n;
  *t = s.t + 2 * (size_t)s.n;
  return CVR_OK;
}

}  // namespace ctxutil
}  // namespace cvr
