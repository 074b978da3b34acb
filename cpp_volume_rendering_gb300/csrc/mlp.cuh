// mlp.cuh — the occlusion/shadow surrogate network: 48 -> 64 -> 64 -> 2,
// ReLU hidden layers, BF16 operands with FP32 accumulation on tcgen05.
//
// Parameter vector (FP32 master copy, CVR_MLP_PARAMS floats):
//   W1[64][48], b1[64], W2[64][64], b2[64], W3[2][64], b3[2]   (W[out][in])
// Packed image (what a CTA copies into shared memory): the BF16 operand tiles
// in the K-major core-matrix layout of tc.cuh plus the FP32 biases.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace cvr {

constexpr int kMlpIn = 48;
constexpr int kMlpHidden = 64;
constexpr int kMlpOut = 2;
constexpr int kMlpK = 64;  // input width padded to a multiple of 16
constexpr int kMlpParams = 64 * 48 + 64 + 64 * 64 + 64 + 2 * 64 + 2;  // 7426
constexpr int kOffW1 = 0, kOffB1 = 64 * 48, kOffW2 = kOffB1 + 64, kOffB2 = kOffW2 + 64 * 64, kOffW3 = kOffB2 + 64,
              kOffB3 = kOffW3 + 2 * 64;

// Packed image byte offsets (all multiples of 128).  The forward operands
// and the biases come first, so a forward-only CTA copies kPkFwdBytes.
constexpr uint32_t kPkW1 = 0;        // 64 rows x K 64, lbo 128, sbo 1024
constexpr uint32_t kPkW2 = 8192;     // 64 x 64
constexpr uint32_t kPkW3 = 16384;    // 16 rows (2 used) x 64
constexpr uint32_t kPkBias = 18432;  // b1[64], b2[64], b3[2] as FP32
constexpr uint32_t kPkFwdBytes = 18432 + 1024;
constexpr uint32_t kPkW2T = 19456;   // W2^T: 64 (in) x 64 (out)
constexpr uint32_t kPkW3T = 27648;   // W3^T: 64 (hidden) x K 16 (2 used), lbo 128, sbo 256
constexpr uint32_t kPkBytes = 27648 + 2048;

// One 128-point tile of the forward pass on the tensor cores.  Used by the
// batch inference kernel and fused into the surrogate marcher.
struct MlpSmem {
  uint8_t* w;        // packed image (kPkBytes)
  uint8_t* x;        // 128 x 64 input tile (row layout: lbo 128, sbo 1024)
  uint8_t* h;        // 128 x 64 hidden tile
  uint64_t* bar;     // mbarrier
  uint32_t tmem;     // 128-column TMEM allocation
  uint32_t phase;    // parity of the next mbarrier phase
};

cudaError_t launch_mlp_pack(const float* params, uint8_t* packed, cudaStream_t st);
cudaError_t launch_mlp_infer(const uint8_t* packed, const float* x, int n, float* y, int* err, cudaStream_t st);
// Forward + backward of a batch; per-CTA gradient partials (ceil(n/128) x kMlpParams).
cudaError_t launch_mlp_train_tiles(const uint8_t* packed, const float* x, const float* t, const int* idx, int n,
                                   float inv_count, float* partials, float* loss_sum, int* err, cudaStream_t st);
// Sums the partials and applies one Adam step to params (m, v moments); the
// step number is *step_dev + 1 (step_dev may be null: step 1).  lr <= 0 only
// reduces the gradient into grad_out.
cudaError_t launch_mlp_adam(float* params, float* m, float* v, const float* partials, int n_parts, float lr,
                            float beta1, float beta2, float eps, const int* step_dev, float* grad_out,
                            cudaStream_t st);

}  // namespace cvr
