// mlp.cu — tensor-core (tcgen05) kernels of the surrogate network: weight
// packing, batch inference, fused forward + backward of training tiles, and
// the Adam update.  All GEMMs are M = 128 (one row per point of a tile),
// BF16 operands from shared memory, FP32 accumulators in tensor memory.
#include "mlp_tile.cuh"

namespace cvr {


// ---------------------------------------------------------------- pack
__global__ void k_mlp_pack(const float* __restrict__ p, uint8_t* __restrict__ pk) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < 64 * 64) {
    int o = i / 64, k = i % 64;
    uint16_t w1 = k < 48 ? to_bf16(p[kOffW1 + o * 48 + k]) : (uint16_t)0;
    *reinterpret_cast<uint16_t*>(pk + kPkW1 + tile_off(o, k, 128, kRowSbo)) = w1;
    uint16_t w2 = to_bf16(p[kOffW2 + o * 64 + k]);
    *reinterpret_cast<uint16_t*>(pk + kPkW2 + tile_off(o, k, 128, kRowSbo)) = w2;
    *reinterpret_cast<uint16_t*>(pk + kPkW2T + tile_off(k, o, 128, kRowSbo)) = w2;  // W2^T[in][out]
  }
  if (i < 16 * 64) {
    int o = i / 64, k = i % 64;
    uint16_t w3 = o < 2 ? to_bf16(p[kOffW3 + o * 64 + k]) : (uint16_t)0;
    *reinterpret_cast<uint16_t*>(pk + kPkW3 + tile_off(o, k, 128, kRowSbo)) = w3;
    *reinterpret_cast<uint16_t*>(pk + kPkW3T + tile_off(k, o, 128, kRow16Sbo)) = w3;  // W3^T[hidden][out]
  }
  if (i < 130) {
    float* b = reinterpret_cast<float*>(pk + kPkBias);
    b[i] = i < 64 ? p[kOffB1 + i] : (i < 128 ? p[kOffB2 + i - 64] : p[kOffB3 + i - 128]);
  }
}

cudaError_t launch_mlp_pack(const float* params, uint8_t* packed, cudaStream_t st) {
  k_mlp_pack<<<16, 256, 0, st>>>(params, packed);
  return cudaGetLastError();
}

// ---------------------------------------------------------------- inference
__global__ void __launch_bounds__(128, 1) k_mlp_infer(const uint8_t* __restrict__ packed, const float* __restrict__ x,
                                                      int n, float* __restrict__ y, int* err) {
  extern __shared__ __align__(1024) uint8_t sm[];
  uint8_t* w = sm;
  uint8_t* xt = sm + kPkBytes;
  uint8_t* ht = xt + kRowTile;
  uint64_t* bar = reinterpret_cast<uint64_t*>(ht + kRowTile);
  uint32_t* tslot = reinterpret_cast<uint32_t*>(bar + 1);
  mlp_cta_begin(w, packed, bar, tslot);
  const int m = blockIdx.x * 128 + threadIdx.x;
  float v[48];
#pragma unroll
  for (int k = 0; k < 48; ++k) v[k] = m < n ? __ldg(x + (size_t)m * 48 + k) : 0.0f;
  store_row64(xt, threadIdx.x, v, 48);
  fence_async_smem();
  __syncthreads();
  MlpSmem s{w, xt, ht, bar, *tslot, 0u};
  float out[2];
  if (!mlp_forward_tile(s, out)) atomicExch(err, 1);
  if (m < n) {
    y[2 * (size_t)m] = out[0];
    y[2 * (size_t)m + 1] = out[1];
  }
  mlp_cta_end(s.tmem);
}

cudaError_t launch_mlp_infer(const uint8_t* packed, const float* x, int n, float* y, int* err, cudaStream_t st) {
  const size_t smem = kPkBytes + 2 * kRowTile + 16;
  cudaError_t e = cudaFuncSetAttribute(k_mlp_infer, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  if (n <= 0) return cudaSuccess;
  k_mlp_infer<<<(n + 127) / 128, 128, smem, st>>>(packed, x, n, y, err);
  return cudaGetLastError();
}

// ---------------------------------------------------------------- training
// One tile of 128 points: forward, MSE loss gradient, backward; writes this
// CTA's gradient of every parameter (and its loss) to partials[blockIdx.x].
//   L = 1/(2 count) * sum_points sum_o (y_o - t_o)^2
// Weight gradients of layers 1 and 2 come from one M=128 N=128 K=128 MMA of
//   A = [dZ2^T ; dZ1^T]  (128 x points)  and  B = [H1^T ; X^T ; 0]  (128 x points),
// whose diagonal 64x64 blocks are dW2 and dW1 (the off-diagonal blocks are
// discarded).  dW3 and the biases are reduced on the CUDA cores.
__global__ void __launch_bounds__(128, 1) k_mlp_train(const uint8_t* __restrict__ packed, const float* __restrict__ x,
                                                      const float* __restrict__ t, const int* __restrict__ idx, int n,
                                                      float inv_count, float* __restrict__ partials, int* err) {
  extern __shared__ __align__(1024) uint8_t sm[];
  uint8_t* w = sm;
  uint8_t* xt = w + kPkBytes;
  uint8_t* h1 = xt + kRowTile;
  uint8_t* h2 = h1 + kRowTile;
  uint8_t* dz2 = h2 + kRowTile;
  uint8_t* dyt = dz2 + kRowTile;
  uint8_t* at = dyt + kRow16Tile;
  uint8_t* bt = at + kTTile;
  float* dyf = reinterpret_cast<float*>(bt + kTTile);  // dY in FP32, 128 x 2
  uint64_t* bar = reinterpret_cast<uint64_t*>(dyf + 256);
  uint32_t* tslot = reinterpret_cast<uint32_t*>(bar + 1);
  mlp_cta_begin(w, packed, bar, tslot);
  // rows 112..127 of B (past the 48 input features) stay zero
  for (int i = threadIdx.x; i < (int)(2 * kTSbo / 16); i += 128)
    reinterpret_cast<uint4*>(bt + 14 * kTSbo)[i] = make_uint4(0, 0, 0, 0);
  __syncthreads();

  const int tid = threadIdx.x;
  const int slot = blockIdx.x * 128 + tid;
  const bool valid = slot < n;
  const int p = valid ? idx[slot] : 0;
  float v[64];
#pragma unroll
  for (int k = 0; k < 48; ++k) v[k] = valid ? __ldg(x + (size_t)p * 48 + k) : 0.0f;
  float tgt0 = valid ? __ldg(t + 2 * (size_t)p) : 0.0f, tgt1 = valid ? __ldg(t + 2 * (size_t)p + 1) : 0.0f;
  store_row64(xt, tid, v, 48);
  store_col(bt, tid, 64, v, 48);
  sync_tiles();

  const float* bias = reinterpret_cast<const float*>(w + kPkBias);
  MlpSmem s{w, xt, h1, bar, *tslot, 0u};
  bool ok = true;
  uint64_t mask1 = 0, mask2 = 0;
  // ---- layer 1
  if (tid == 0) {
    fence_after_sync();
    issue_k64(s.tmem, xt, w + kPkW1, idesc_bf16(128, 64));
  }
  ok &= complete(bar, s.phase);
  ld_row64(s.tmem, 0, v);
#pragma unroll
  for (int j = 0; j < 64; ++j) {
    float z = v[j] + bias[j];
    if (z > 0.0f) mask1 |= 1ull << j;
    v[j] = fmaxf(z, 0.0f);
  }
  store_row64(h1, tid, v, 64);
  store_col(bt, tid, 0, v, 64);
  sync_tiles();
  // ---- layer 2
  if (tid == 0) {
    fence_after_sync();
    issue_k64(s.tmem + 64, h1, w + kPkW2, idesc_bf16(128, 64));
  }
  ok &= complete(bar, s.phase);
  ld_row64(s.tmem, 64, v);
#pragma unroll
  for (int j = 0; j < 64; ++j) {
    float z = v[j] + bias[64 + j];
    if (z > 0.0f) mask2 |= 1ull << j;
    v[j] = fmaxf(z, 0.0f);
  }
  store_row64(h2, tid, v, 64);
  sync_tiles();
  // ---- layer 3 + loss
  if (tid == 0) {
    fence_after_sync();
    issue_k64(s.tmem, h2, w + kPkW3, idesc_bf16(128, 16));
  }
  ok &= complete(bar, s.phase);
  float o[16];
  tmem_ld16(taddr(s.tmem, (uint32_t)(tid & ~31), 0), o);
  float y0 = o[0] + bias[128], y1 = o[1] + bias[129];
  float e0 = valid ? (y0 - tgt0) : 0.0f, e1 = valid ? (y1 - tgt1) : 0.0f;
  float loss = 0.5f * (e0 * e0 + e1 * e1) * inv_count;
  float dy0 = e0 * inv_count, dy1 = e1 * inv_count;
  dyf[2 * tid] = dy0;
  dyf[2 * tid + 1] = dy1;
  {
    // dY row (K = 16: two values and zero padding)
    uint32_t w0 = (uint32_t)to_bf16(dy0) | ((uint32_t)to_bf16(dy1) << 16);
    uint8_t* rowp = dyt + (uint32_t)(tid >> 3) * kRow16Sbo + (uint32_t)(tid & 7) * 16u;
    *reinterpret_cast<uint4*>(rowp) = make_uint4(w0, 0, 0, 0);
    *reinterpret_cast<uint4*>(rowp + 128) = make_uint4(0, 0, 0, 0);
  }
  sync_tiles();
  // ---- dH2 = dY W3  (K = 16)
  if (tid == 0) {
    fence_after_sync();
    mma_bf16(s.tmem, sdesc(smem_u32(dyt), 128u, kRow16Sbo), sdesc(smem_u32(w + kPkW3T), 128u, kRow16Sbo),
             idesc_bf16(128, 64), 0u);
  }
  ok &= complete(bar, s.phase);
  ld_row64(s.tmem, 0, v);
#pragma unroll
  for (int j = 0; j < 64; ++j) v[j] = (mask2 >> j) & 1ull ? v[j] : 0.0f;
  store_row64(dz2, tid, v, 64);
  store_col(at, tid, 0, v, 64);
  sync_tiles();
  // ---- dH1 = dZ2 W2
  if (tid == 0) {
    fence_after_sync();
    issue_k64(s.tmem + 64, dz2, w + kPkW2T, idesc_bf16(128, 64));
  }
  ok &= complete(bar, s.phase);
  ld_row64(s.tmem, 64, v);
#pragma unroll
  for (int j = 0; j < 64; ++j) v[j] = (mask1 >> j) & 1ull ? v[j] : 0.0f;
  store_col(at, tid, 64, v, 64);
  sync_tiles();
  // ---- [dW2 | dW1] = A B^T over the 128 points (K = 128)
  if (tid == 0) {
    fence_after_sync();
#pragma unroll
    for (int kb = 0; kb < 8; ++kb)
      mma_bf16(s.tmem, sdesc(smem_u32(at) + kb * 2u * kTLbo, kTLbo, kTSbo),
               sdesc(smem_u32(bt) + kb * 2u * kTLbo, kTLbo, kTSbo), idesc_bf16(128, 128), kb > 0);
  }
  ok &= complete(bar, s.phase);
  float* part = partials + (size_t)blockIdx.x * (kMlpParams + 1);
  if (tid < 64) {
    ld_row64(s.tmem, 0, v);  // row j = tid: dW2[j][0..63]
#pragma unroll
    for (int i = 0; i < 64; ++i) part[kOffW2 + tid * 64 + i] = v[i];
  } else {
    ld_row64(s.tmem, 64, v);  // row 64 + j: dW1[j][0..47]
#pragma unroll
    for (int k = 0; k < 48; ++k) part[kOffW1 + (tid - 64) * 48 + k] = v[k];
  }
  // ---- CUDA-core reductions over the 128 points: dW3, db3, db2, db1
  {
    const int oo = tid >> 6, j = tid & 63;
    float acc = 0.0f;
    for (int m = 0; m < 128; ++m) {
      uint16_t hb = *reinterpret_cast<const uint16_t*>(h2 + tile_off(m, j, 128, kRowSbo));
      acc = fmaf(dyf[2 * m + oo], from_bf16(hb), acc);
    }
    part[kOffW3 + oo * 64 + j] = acc;
    // db2 (tid < 64, from dZ2^T rows 0..63) and db1 (tid >= 64, from dZ1^T rows 64..127)
    float sb = 0.0f;
    for (int m = 0; m < 128; ++m)
      sb += from_bf16(*reinterpret_cast<const uint16_t*>(at + tile_off(tid, m, kTLbo, kTSbo)));
    if (tid < 64) part[kOffB2 + tid] = sb;
    else part[kOffB1 + (tid - 64)] = sb;
    if (tid < 2) {
      float sy = 0.0f;
      for (int m = 0; m < 128; ++m) sy += dyf[2 * m + tid];
      part[kOffB3 + tid] = sy;
    }
  }
  // loss of the tile
  for (int off = 16; off > 0; off >>= 1) loss += __shfl_down_sync(0xffffffffu, loss, off);
  __syncthreads();
  if ((tid & 31) == 0) dyf[tid >> 5] = loss;  // dY values are no longer needed
  __syncthreads();
  if (tid == 0) part[kMlpParams] = dyf[0] + dyf[1] + dyf[2] + dyf[3];
  if (!ok) atomicExch(err, 1);
  mlp_cta_end(s.tmem);
}

cudaError_t launch_mlp_train_tiles(const uint8_t* packed, const float* x, const float* t, const int* idx, int n,
                                   float inv_count, float* partials, float* loss_sum, int* err, cudaStream_t st) {
  (void)loss_sum;
  const size_t smem = kPkBytes + 4 * kRowTile + kRow16Tile + 2 * kTTile + 256 * sizeof(float) + 16;
  cudaError_t e = cudaFuncSetAttribute(k_mlp_train, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  if (n <= 0) return cudaSuccess;
  k_mlp_train<<<(n + 127) / 128, 128, smem, st>>>(packed, x, t, idx, n, inv_count, partials, err);
  return cudaGetLastError();
}

// ---------------------------------------------------------------- Adam
// Thread p sums the per-CTA partials of parameter p (slot kMlpParams is the
// loss) and applies one Adam step; lr <= 0 only reduces (gradient check).
__global__ void k_mlp_adam(float* __restrict__ params, float* __restrict__ m, float* __restrict__ v,
                           const float* __restrict__ partials, int n_parts, float lr, float b1, float b2, float eps,
                           const int* __restrict__ step_dev, float* __restrict__ grad_out) {
  int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p > kMlpParams) return;
  const int step = step_dev ? *step_dev + 1 : 1;  // 1-based step of this update
  float g = 0.0f;
  for (int c = 0; c < n_parts; ++c) g += partials[(size_t)c * (kMlpParams + 1) + p];
  if (grad_out) grad_out[p] = g;
  if (p == kMlpParams || lr <= 0.0f) return;
  float mm = b1 * m[p] + (1.0f - b1) * g;
  float vv = b2 * v[p] + (1.0f - b2) * g * g;
  m[p] = mm;
  v[p] = vv;
  float mh = mm / (1.0f - powf(b1, (float)step));
  float vh = vv / (1.0f - powf(b2, (float)step));
  params[p] -= lr * mh / (sqrtf(vh) + eps);
}

cudaError_t launch_mlp_adam(float* params, float* m, float* v, const float* partials, int n_parts, float lr,
                            float beta1, float beta2, float eps, const int* step_dev, float* grad_out, cudaStream_t st) {
  k_mlp_adam<<<(kMlpParams + 1 + 255) / 256, 256, 0, st>>>(params, m, v, partials, n_parts, lr, beta1, beta2, eps,
                                                           step_dev, grad_out);
  return cudaGetLastError();
}

}  // namespace cvr
