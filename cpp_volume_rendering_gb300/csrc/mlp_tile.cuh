// mlp_tile.cuh — device routines of one 128-point tile of the surrogate
// network on the tensor cores, shared by the MLP kernels (mlp.cu) and the
// surrogate-shaded marcher (surrogate.cu).
#pragma once

#include "mlp.cuh"
#include "tc.cuh"

namespace cvr {

using namespace tc;

constexpr uint32_t kPolls = 1u << 22;  // bound of every mbarrier wait

// Tile geometry (bytes): row tiles of K = 64 (lbo 128, sbo 1024), K = 16 row
// tiles (lbo 128, sbo 256), and the transposed K = 128 tiles of the weight
// gradients (lbo 144 so that column-wise 16-bit stores are bank-conflict free).
constexpr uint32_t kRowSbo = 1024, kRow16Sbo = 256;
constexpr uint32_t kTLbo = 144, kTSbo = 16 * 144;
constexpr uint32_t kRowTile = 128 * 128;      // 128 x 64 bf16
constexpr uint32_t kRow16Tile = 16 * 256;     // 128 x 16 bf16
constexpr uint32_t kTTile = 16 * kTSbo;       // 128 x 128 bf16 (transposed layout)

// ---------------------------------------------------------------- helpers
// Row r of a K = 64 row tile from n <= 64 floats (zero padded), 16 B stores.
__device__ __forceinline__ void store_row64(uint8_t* tile, int r, const float* v, int n) {
#pragma unroll
  for (int c = 0; c < 8; ++c) {
    uint32_t w[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      int k0 = c * 8 + 2 * j;
      w[j] = k0 + 1 < n ? pack_bf16(v[k0], v[k0 + 1]) : (k0 < n ? pack_bf16(v[k0], 0.0f) : 0u);
    }
    *reinterpret_cast<uint4*>(tile + (uint32_t)(r >> 3) * kRowSbo + (uint32_t)c * 128u + (uint32_t)(r & 7) * 16u) =
        make_uint4(w[0], w[1], w[2], w[3]);
  }
}

// One 16-byte chunk (k = 8c .. 8c+7) of row r of a K = 64 row tile.
__device__ __forceinline__ void store_chunk(uint8_t* tile, int r, int c, uint32_t w0, uint32_t w1, uint32_t w2,
                                            uint32_t w3) {
  *reinterpret_cast<uint4*>(tile + (uint32_t)(r >> 3) * kRowSbo + (uint32_t)c * 128u + (uint32_t)(r & 7) * 16u) =
      make_uint4(w0, w1, w2, w3);
}

// Hidden layer epilogue: TMEM columns col..col+63 of this thread's row, plus
// bias, ReLU, to BF16 row r of tile; 16 columns at a time.
__device__ __forceinline__ void epilogue_relu64(uint32_t tmem, int col, const float* bias, uint8_t* tile, int r) {
  const uint32_t lane = (uint32_t)(threadIdx.x & ~31);
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    float v[16];
    tmem_ld16(taddr(tmem, lane, (uint32_t)(col + 16 * q)), v);
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int k = 16 * q + 8 * h;
      store_chunk(tile, r, 2 * q + h, pack_bf16_relu(v[8 * h + 0] + bias[k + 0], v[8 * h + 1] + bias[k + 1]),
                  pack_bf16_relu(v[8 * h + 2] + bias[k + 2], v[8 * h + 3] + bias[k + 3]),
                  pack_bf16_relu(v[8 * h + 4] + bias[k + 4], v[8 * h + 5] + bias[k + 5]),
                  pack_bf16_relu(v[8 * h + 6] + bias[k + 6], v[8 * h + 7] + bias[k + 7]));
    }
  }
}

// Column m (rows r0 .. r0+n-1) of a transposed K = 128 tile.
__device__ __forceinline__ void store_col(uint8_t* tile, int m, int r0, const float* v, int n) {
  for (int r = 0; r < n; ++r)
    *reinterpret_cast<uint16_t*>(tile + tile_off(r0 + r, m, kTLbo, kTSbo)) = to_bf16(v[r]);
}

__device__ __forceinline__ void issue_k64(uint32_t d, const uint8_t* a, const uint8_t* b, uint32_t idesc) {
#pragma unroll
  for (int kb = 0; kb < 4; ++kb)
    mma_bf16(d, sdesc(smem_u32(a) + kb * 256u, 128u, kRowSbo), sdesc(smem_u32(b) + kb * 256u, 128u, kRowSbo), idesc,
             kb > 0);
}

// Runs one commit/wait round trip: the issuing thread has queued MMAs.
__device__ __forceinline__ bool complete(uint64_t* bar, uint32_t& phase) {
  if (threadIdx.x == 0) commit(bar);
  bool ok = mbar_wait(bar, phase, kPolls);
  phase ^= 1u;
  fence_after_sync();
  return ok;
}

__device__ __forceinline__ void ld_row64(uint32_t tmem, int col, float* v) {
  const uint32_t lane = (uint32_t)(threadIdx.x & ~31);
#pragma unroll
  for (int c = 0; c < 4; ++c) tmem_ld16(taddr(tmem, lane, (uint32_t)(col + 16 * c)), v + 16 * c);
}

__device__ __forceinline__ void sync_tiles() {
  fence_before_sync();
  fence_async_smem();
  __syncthreads();
}

// Forward of the 128-point tile whose input rows are in s.x; returns this
// thread's two outputs.  Must be called by all 128 threads.  Every layer
// accumulates into TMEM columns 0..63 (a layer's result is read out before
// the next is issued), and the hidden activations go to s.h, which may be
// the same buffer as s.x (the input is dead once layer 1 has completed).
__device__ __forceinline__ bool mlp_forward_tile(MlpSmem& s, float y[2]) {
  const float* bias = reinterpret_cast<const float*>(s.w + kPkBias);
  bool ok = true;
  if (threadIdx.x == 0) {
    fence_after_sync();
    issue_k64(s.tmem, s.x, s.w + kPkW1, idesc_bf16(128, 64));
  }
  ok &= complete(s.bar, s.phase);
  epilogue_relu64(s.tmem, 0, bias, s.h, threadIdx.x);
  sync_tiles();
  if (threadIdx.x == 0) {
    fence_after_sync();
    issue_k64(s.tmem, s.h, s.w + kPkW2, idesc_bf16(128, 64));
  }
  ok &= complete(s.bar, s.phase);
  epilogue_relu64(s.tmem, 0, bias + 64, s.h, threadIdx.x);
  sync_tiles();
  if (threadIdx.x == 0) {
    fence_after_sync();
    issue_k64(s.tmem, s.h, s.w + kPkW3, idesc_bf16(128, 16));
  }
  ok &= complete(s.bar, s.phase);
  float o[16];
  tmem_ld16(taddr(s.tmem, (uint32_t)(threadIdx.x & ~31), 0), o);
  y[0] = o[0] + bias[128];
  y[1] = o[1] + bias[129];
  fence_before_sync();
  return ok;
}

// Shared set-up of an MLP CTA: TMEM allocation, mbarrier, the first 'bytes'
// of the weight image (kPkBytes, or kPkFwdBytes for the forward pass only).
__device__ __forceinline__ void mlp_cta_begin(uint8_t* w, const uint8_t* packed, uint64_t* bar, uint32_t* tslot,
                                              uint32_t tmem_cols = 128, uint32_t bytes = kPkBytes) {
  if (threadIdx.x < 32) tmem_alloc(tslot, tmem_cols);
  if (threadIdx.x == 0) {
    mbar_init(bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  const uint4* src = reinterpret_cast<const uint4*>(packed);
  uint4* dst = reinterpret_cast<uint4*>(w);
  for (int i = threadIdx.x; i < (int)(bytes / 16); i += blockDim.x) dst[i] = src[i];
}

__device__ __forceinline__ void mlp_cta_end(uint32_t tmem, uint32_t tmem_cols = 128) {
  fence_before_sync();
  __syncthreads();
  if (threadIdx.x < 32) {
    fence_after_sync();
    tmem_dealloc(tmem, tmem_cols);
  }
}

}  // namespace cvr
