// textures.cu — texture-unit copies of the volume and of the extinction
// pyramid levels: 3D CUDA arrays sampled with hardware trilinear filtering,
// normalised coordinates and clamp-to-edge addressing (the OpenGL
// GL_LINEAR / GL_CLAMP_TO_EDGE sampling of the reference's textures).
#include <algorithm>

#include <cuda_fp16.h>

#include "ctx.cuh"

using namespace cvr::ctxutil;

namespace {

__global__ void k_to_half(const float* __restrict__ src, __half* __restrict__ dst, long long n) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) dst[i] = __float2half_rn(src[i]);
}

cudaError_t launch_to_half(const float* src, __half* dst, long long n, cudaStream_t st) {
  k_to_half<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(src, dst, n);
  return cudaGetLastError();
}

cudaError_t make_texture(cvr_ctx* c, TexImage& t, const void* src, size_t elem, cudaChannelFormatDesc desc, int w,
                         int h, int d, cudaTextureReadMode mode) {
  t.release();
  cudaExtent ext = make_cudaExtent((size_t)w, (size_t)h, (size_t)d);
  cudaError_t e = cudaMalloc3DArray(&t.arr, &desc, ext);
  if (e != cudaSuccess) return e;
  cudaMemcpy3DParms cp{};
  cp.srcPtr = make_cudaPitchedPtr(const_cast<void*>(src), (size_t)w * elem, (size_t)w, (size_t)h);
  cp.dstArray = t.arr;
  cp.extent = ext;
  cp.kind = cudaMemcpyDeviceToDevice;
  if ((e = cudaMemcpy3DAsync(&cp, c->stream)) != cudaSuccess) return e;
  cudaResourceDesc rd{};
  rd.resType = cudaResourceTypeArray;
  rd.res.array.array = t.arr;
  cudaTextureDesc td{};
  td.addressMode[0] = td.addressMode[1] = td.addressMode[2] = cudaAddressModeClamp;
  td.filterMode = cudaFilterModeLinear;
  td.readMode = mode;
  td.normalizedCoords = 1;
  return cudaCreateTextureObject(&t.tex, &rd, &td, nullptr);
}

}  // namespace

namespace cvr {
namespace ctxutil {

cvr_status ensure_volume_texture(cvr_ctx* c) {
  if (c->tex.vol_valid) return CVR_OK;
  if (!c->has_volume) return fail(c, CVR_ERR_NO_VOLUME, "volume texture: no volume");
  cudaChannelFormatDesc desc = c->dtype == CVR_U8 ? cudaCreateChannelDesc<unsigned char>()
                                                  : cudaCreateChannelDesc<unsigned short>();
  cudaError_t e = make_texture(c, c->tex.vol, c->d_vol, c->dtype == CVR_U8 ? 1 : 2, desc, c->nx, c->ny, c->nz,
                               cudaReadModeNormalizedFloat);
  if (e != cudaSuccess) {
    c->tex.vol.release();
    return cuda_fail(c, e, "volume texture");
  }
  c->tex.vol_valid = true;
  return CVR_OK;
}

// Pyramid levels as FP16 textures (the reference keeps the pyramid in R16F,
// extcoefvolumegenerator.cpp:246-252): half the bytes of the texture reads.
cvr_status ensure_pyramid_textures(cvr_ctx* c) {
  if (c->tex.pyr_valid) return CVR_OK;
  if (!c->pyr_ready) return fail(c, CVR_ERR_NOT_READY, "pyramid textures: no pyramid");
  for (auto& t : c->tex.pyr) t.release();
  c->tex.n_pyr = 0;
  long long total = 0;
  for (int l = 0; l < c->pyr.n_levels; ++l)
    total = std::max(total, (long long)c->pyr.dims[l][0] * c->pyr.dims[l][1] * c->pyr.dims[l][2]);
  __half* tmp = nullptr;
  CK(c, cudaMalloc((void**)&tmp, sizeof(__half) * (size_t)total));
  cudaError_t e = cudaSuccess;
  for (int l = 0; l < c->pyr.n_levels && e == cudaSuccess; ++l) {
    const int* d = c->pyr.dims[l];
    const long long n = (long long)d[0] * d[1] * d[2];
    e = launch_to_half(c->d_pyr + c->pyr.offset[l], tmp, n, c->stream);
    if (e == cudaSuccess)
      e = make_texture(c, c->tex.pyr[l], tmp, sizeof(__half), cudaCreateChannelDescHalf(), d[0], d[1], d[2],
                       cudaReadModeElementType);
    // the array copy reads tmp on the stream: finish before the next level reuses it
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e == cudaSuccess) c->tex.n_pyr = l + 1;
  }
  cudaFree(tmp);
  if (e != cudaSuccess) {
    for (auto& t : c->tex.pyr) t.release();
    return cuda_fail(c, e, "pyramid texture");
  }
  c->tex.pyr_valid = true;
  return CVR_OK;
}

// The gradient as an RGBA16F texture (the reference's RGB16F gradient
// texture, utils.cpp:274-278, with a fourth channel for 8-byte texels).
cvr_status ensure_gradient_texture(cvr_ctx* c) {
  if (c->tex.grad_valid) return CVR_OK;
  if (!c->grad_ready) return fail(c, CVR_ERR_NOT_READY, "gradient texture: no gradient");
  cudaError_t e = make_texture(c, c->tex.grad, c->d_grad, sizeof(uint2), cudaCreateChannelDescHalf4(), c->nx, c->ny,
                               c->nz, cudaReadModeElementType);
  if (e != cudaSuccess) {
    c->tex.grad.release();
    return cuda_fail(c, e, "gradient texture");
  }
  c->tex.grad_valid = true;
  return CVR_OK;
}

}  // namespace ctxutil
}  // namespace cvr

extern "C" {

cvr_status cvr_set_sampling(cvr_ctx* c, int flags) {
  if (!c) return CVR_ERR_INVALID_ARG;
  if (flags & ~(CVR_SAMPLING_TEX_FEATURES | CVR_SAMPLING_TEX_VOLUME | CVR_SAMPLING_TEX_PYRAMID))
    return fail(c, CVR_ERR_INVALID_ARG, "cvr_set_sampling: unknown flags");
  c->sampling = flags;
  return CVR_OK;
}

int cvr_get_sampling(cvr_ctx* c) { return c ? c->sampling : 0; }

}  // extern "C"
