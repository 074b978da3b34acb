// postpass.cu — pixel multiscaling of the renderer output
// (BaseVolumeRenderer::MULTISCALING, cppvolrend/volrenderbase.h:28-33, and
// vis::RenderFrameToScreen, libs/vis_utils/renderoutputframe.cpp:265-539):
// a frame rendered at a multiple (or fraction) of the output size is brought
// to the output size on the device by
//   multisample  bilinear texture() lookup at the output pixel centres
//                (renderoutputframe/multisample_filter.comp),
//   downscale    the reconstruction kernel summed over the generated texels
//                under its support, scaled by the area ratio
//                (downscaling_filter.comp),
//   upscale      the kernel evaluated at the generated texels around the
//                output pixel (upscaling_filter.comp),
// with the cardinal B-spline and OMOMS kernels' recursive digital filter
// (cbs_digital_filter.comp, comoms_digital_filter.comp) run on the output
// (downscale) or on the generated frame (upscale), rows then columns.
// texelFetch outside the frame reads 0.
#include "ctx.cuh"

using namespace cvr::ctxutil;

namespace {

// IMAGE_FILTER_KERNEL (libs/vis_utils/filters/utils.hpp:8-15); support and
// weight of each (renderoutputframe/*_filter.comp).
__device__ __forceinline__ float kernel_support(int k) { return k == 0 ? 1.0f : (k == 1 ? 2.0f : 4.0f); }

__device__ __forceinline__ float kernel_weight(int k, float x) {
  if (k == 0) return (x <= -0.5f || x > 0.5f) ? 0.0f : 1.0f;  // box
  x = fabsf(x);
  if (k == 1) return x > 1.0f ? 0.0f : 1.0f - x;  // hat
  if (x > 2.0f) return 0.0f;
  const bool outer = x > 1.0f;
  const float u = outer ? 2.0f - x : 1.0f - x;  // k0(2 - x) on (1, 2], k1(1 - x) on [0, 1]
  switch (k) {
    case 2:  // Catmull-Rom
      return outer ? ((0.5f * u - 0.5f) * u) * u : ((-1.5f * u + 2.0f) * u + 0.5f) * u;
    case 3:  // Mitchell-Netravali
      return outer ? (((7.0f / 18.0f) * u - 1.0f / 3.0f) * u) * u
                   : (((-7.0f / 6.0f) * u + 1.5f) * u + 0.5f) * u + 1.0f / 18.0f;
    case 4:  // cardinal cubic B-spline (pieces times 6)
      return outer ? (u * u) * u : ((-3.0f * u + 3.0f) * u + 3.0f) * u + 1.0f;
    default:  // 5: cardinal OMOMS-3
      return outer ? ((0.875f * u) * u + 0.125f) * u : ((-2.625f * u + 2.625f) * u + 2.25f) * u + 1.0f;
  }
}

__device__ __forceinline__ float4 fetch(const float4* __restrict__ img, int w, int h, int x, int y) {
  if (x < 0 || y < 0 || x >= w || y >= h) return make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  return img[(size_t)y * w + x];
}

__device__ __forceinline__ void axpy(float4& acc, float a, float4 v) {
  acc.x = fmaf(a, v.x, acc.x); acc.y = fmaf(a, v.y, acc.y); acc.z = fmaf(a, v.z, acc.z); acc.w = fmaf(a, v.w, acc.w);
}

// multisample_filter.comp: texture(TexGeneratedFrame, (pixel + 0.5) / size),
// GL_LINEAR with clamp-to-edge.
__global__ void k_multisample(const float4* __restrict__ src, int sw, int sh, float4* __restrict__ dst, int dw,
                              int dh) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= dw || y >= dh) return;
  const Tap a = axis_tap(((float(x) + 0.5f) / float(dw)) * float(sw) - 0.5f, sw);
  const Tap b = axis_tap(((float(y) + 0.5f) / float(dh)) * float(sh) - 0.5f, sh);
  const float4 c00 = src[(size_t)b.i0 * sw + a.i0], c10 = src[(size_t)b.i0 * sw + a.i1];
  const float4 c01 = src[(size_t)b.i1 * sw + a.i0], c11 = src[(size_t)b.i1 * sw + a.i1];
  auto lerp = [](float t, float4 p, float4 q) {
    return make_float4(fmaf(t, q.x - p.x, p.x), fmaf(t, q.y - p.y, p.y), fmaf(t, q.z - p.z, p.z),
                       fmaf(t, q.w - p.w, p.w));
  };
  dst[(size_t)y * dw + x] = lerp(b.t, lerp(a.t, c00, c10), lerp(a.t, c01, c11));
}

// downscaling_filter.comp main().
__global__ void k_downscale(const float4* __restrict__ src, int sw, int sh, float4* __restrict__ dst, int dw, int dh,
                            int kern) {
  const int jc = blockIdx.x * blockDim.x + threadIdx.x, jr = blockIdx.y * blockDim.y + threadIdx.y;
  if (jc >= dw || jr >= dh) return;
  const float s_r = float(dh) / float(sh), s_c = float(dw) / float(sw);
  const float kr = 0.5f * kernel_support(kern);
  const float x_r = (float(jr) + 0.5f) / float(dh);
  const int il_r = (int)ceilf((x_r - kr / float(dh)) * float(sh) - 0.5f);
  const int ir_r = (int)floorf((x_r + kr / float(dh)) * float(sh) - 0.5f);
  const float x_c = (float(jc) + 0.5f) / float(dw);
  const int il_c = (int)ceilf((x_c - kr / float(dw)) * float(sw) - 0.5f);
  const int ir_c = (int)floorf((x_c + kr / float(dw)) * float(sw) - 0.5f);
  float4 acc = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  for (int ir = il_r; ir <= ir_r; ++ir) {
    const float wr = kernel_weight(kern, (x_r - (float(ir) + 0.5f) / float(sh)) * float(dh));
    for (int ic = il_c; ic <= ir_c; ++ic)
      axpy(acc, wr * kernel_weight(kern, (x_c - (float(ic) + 0.5f) / float(sw)) * float(dw)),
           fetch(src, sw, sh, ic, ir));
  }
  const float s = s_r * s_c;
  dst[(size_t)jr * dw + jc] = make_float4(acc.x * s, acc.y * s, acc.z * s, acc.w * s);
}

// upscaling_filter.comp main().
__global__ void k_upscale(const float4* __restrict__ src, int sw, int sh, float4* __restrict__ dst, int dw, int dh,
                          int kern) {
  const int jc = blockIdx.x * blockDim.x + threadIdx.x, jr = blockIdx.y * blockDim.y + threadIdx.y;
  if (jc >= dw || jr >= dh) return;
  const float kr = 0.5f * kernel_support(kern);
  const float xi_r = ((float(jr) + 0.5f) / float(dh)) * float(sh) - 0.5f;
  const int il_r = (int)ceilf(xi_r - kr), ir_r = (int)floorf(xi_r + kr);
  const float xi_c = ((float(jc) + 0.5f) / float(dw)) * float(sw) - 0.5f;
  const int il_c = (int)ceilf(xi_c - kr), ir_c = (int)floorf(xi_c + kr);
  float4 acc = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  for (int ir = il_r; ir <= ir_r; ++ir) {
    const float wr = kernel_weight(kern, xi_r - float(ir));
    for (int ic = il_c; ic <= ir_c; ++ic) axpy(acc, wr * kernel_weight(kern, xi_c - float(ic)), fetch(src, sw, sh, ic, ir));
  }
  dst[(size_t)jr * dw + jc] = acc;
}

// The pre-factored LU solve of the B-spline / OMOMS digital filters
// (cbs_digital_filter.comp, comoms_digital_filter.comp): one thread per row
// (dir 0) or column (dir 1), in place; lines shorter than the factor table
// (where the shader would read and write past the line) are left as they are.
struct LuTable {
  int m;
  float L[9];
};

// The digital filter (cbs_digital_filter.comp / comoms_digital_filter.comp:
// the LU solve of the interpolation condition along every row, then every
// column) as chunked first-order recursions.  Forward y[i] = f[i] - L y[i-1]
// and reverse o[i] = L (y[i] - o[i+1]) both have |L| < 0.35 from the m-th
// entry on, so a chunk of a line can start kDfWarm entries before its first
// one from a zero state: the start's error is scaled by L^kDfWarm (< 2e-15)
// before the chunk begins.  The chunk holding the line's first m entries (the
// varying L) starts exactly at the line's end, as does the last chunk of the
// reverse.  One thread per chunk of kDfChunk entries: many threads per line
// instead of one long dependent walk.  Forward reads f and writes y to a
// second buffer, reverse reads y and writes the result over f (a chunk's
// warm-up reads its neighbour's entries, so neither pass runs in place).
constexpr int kDfChunk = 64, kDfWarm = 32;

struct DfLine {
  size_t base, step;
  int n, s, e;  // line length, chunk [s, e)
};
__device__ __forceinline__ bool df_line(int w, int h, int dir, DfLine& d) {
  const int lines = dir == 0 ? h : w, n = dir == 0 ? w : h;
  const int chunks = (n + kDfChunk - 1) / kDfChunk;
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long long)lines * chunks) return false;
  int line, chunk;
  if (dir == 0) { chunk = (int)(idx % chunks); line = (int)(idx / chunks); }  // rows: a thread per chunk of a row
  else { line = (int)(idx % lines); chunk = (int)(idx / lines); }             // columns: lanes on adjacent columns
  d.base = dir == 0 ? (size_t)line * w : (size_t)line;
  d.step = dir == 0 ? 1 : (size_t)w;
  d.n = n;
  d.s = chunk * kDfChunk;
  d.e = min(d.s + kDfChunk, n);
  return true;
}

__global__ void k_df_forward(const float4* __restrict__ f, float4* __restrict__ y, int w, int h, int dir, LuTable t) {
  DfLine d;
  if (!df_line(w, h, dir, d)) return;
  const int m = t.m;
  const float L_inf = t.L[m - 1];
  const float4* __restrict__ fp = f + d.base;
  float4* __restrict__ yp = y + d.base;
  int i = d.s - kDfWarm;
  float4 prev = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  if (i <= 0) {  // exact start: y[0] = f[0]
    prev = fp[0];
    if (d.s == 0) yp[0] = prev;
    i = 1;
  }
#pragma unroll 4
  for (; i < d.e; ++i) {
    const float l = i < m ? t.L[i - 1] : L_inf;
    float4 v = fp[(size_t)i * d.step];
    v.x -= l * prev.x; v.y -= l * prev.y; v.z -= l * prev.z; v.w -= l * prev.w;
    if (i >= d.s) yp[(size_t)i * d.step] = v;
    prev = v;
  }
}

__global__ void k_df_reverse(const float4* __restrict__ y, float4* __restrict__ o, int w, int h, int dir, LuTable t) {
  DfLine d;
  if (!df_line(w, h, dir, d)) return;
  const int m = t.m;
  const float L_inf = t.L[m - 1], v_inv = L_inf / (1.0f + L_inf);
  const float4* __restrict__ yp = y + d.base;
  float4* __restrict__ op = o + d.base;
  const int n = d.n;
  int i = d.e - 1 + kDfWarm;
  float4 next = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  if (i >= n - 1) {  // exact start: o[n-1] = y[n-1] * v_inv (p_inv = 1)
    const float4 v = yp[(size_t)(n - 1) * d.step];
    next = make_float4(v.x * v_inv, v.y * v_inv, v.z * v_inv, v.w * v_inv);
    if (d.e == n) op[(size_t)(n - 1) * d.step] = next;
    i = n - 2;
  }
#pragma unroll 4
  for (; i >= d.s; --i) {
    const float l = i >= m - 1 ? L_inf : t.L[i];
    float4 v = yp[(size_t)i * d.step];
    v.x = l * (v.x - next.x); v.y = l * (v.y - next.y); v.z = l * (v.z - next.z); v.w = l * (v.w - next.w);
    if (i < d.e) op[(size_t)i * d.step] = v;
    next = v;
  }
}

LuTable lu_table(int kern) {
  LuTable t{};
  if (kern == CVR_FILTER_CARDINAL_BSPLINE3) {
    const float L[8] = {.2f, .26315789f, .26760563f, .26792453f, .26794742f, .26794907f, .26794918f, .26794919f};
    t.m = 8;
    for (int i = 0; i < 8; ++i) t.L[i] = L[i];
  } else {
    const float L[9] = {.23529412f, .33170732f, .34266611f, .34395774f, .34411062f,
                        .34412872f, .34413087f, .34413112f, .34413115f};
    t.m = 9;
    for (int i = 0; i < 9; ++i) t.L[i] = L[i];
  }
  return t;
}

// Rows then columns (lines shorter than m are left as they are, as the
// shaders skip them); scratch holds w x h float4.
cudaError_t digital_filter(float4* img, float4* scratch, int w, int h, int kern, cudaStream_t st) {
  const LuTable t = lu_table(kern);
  for (int dir = 0; dir < 2; ++dir) {
    const int lines = dir == 0 ? h : w, n = dir == 0 ? w : h;
    if (n < t.m) continue;
    const long long threads = (long long)lines * ((n + kDfChunk - 1) / kDfChunk);
    const unsigned blocks = (unsigned)((threads + 127) / 128);
    k_df_forward<<<blocks, 128, 0, st>>>(img, scratch, w, h, dir, t);
    k_df_reverse<<<blocks, 128, 0, st>>>(scratch, img, w, h, dir, t);
  }
  return cudaGetLastError();
}

bool has_digital_filter(int kern) { return kern == CVR_FILTER_CARDINAL_BSPLINE3 || kern == CVR_FILTER_CARDINAL_OMOMS3; }

}  // namespace

namespace cvr {
namespace ctxutil {

// The generated frame's size for an output of w x h (UpdateScreenResolutionMultiScaling,
// renderoutputframe.cpp:89-115: x factor, or integer division for up-scaling).
void multiscale_size(int mode, int fw, int fh, int w, int h, int* gw, int* gh) {
  if (mode == CVR_MULTISCALE_UPSCALE) { *gw = w / fw; *gh = h / fh; }
  else if (mode == CVR_MULTISCALE_SINGLE) { *gw = w; *gh = h; }
  else { *gw = w * fw; *gh = h * fh; }
}

size_t multiscale_scratch(int mode, int kern, int gw, int gh, int w, int h) {
  if (!has_digital_filter(kern) || mode == CVR_MULTISCALE_MULTISAMPLE) return 0;
  return (mode == CVR_MULTISCALE_UPSCALE ? (size_t)gw * gh : (size_t)w * h) * sizeof(float4);
}

// src (gw x gh) -> dst (w x h); src is modified in place by the up-scaling
// digital filter; scratch has multiscale_scratch bytes.
cudaError_t launch_multiscale(int mode, int kern, float4* src, int gw, int gh, float4* dst, int w, int h,
                              float4* scratch, cudaStream_t st) {
  const dim3 block(16, 8);
  const dim3 grid((w + 15) / 16, (h + 7) / 8);
  cudaError_t e = cudaSuccess;
  if (mode == CVR_MULTISCALE_MULTISAMPLE) {
    k_multisample<<<grid, block, 0, st>>>(src, gw, gh, dst, w, h);
    return cudaGetLastError();
  }
  if (mode == CVR_MULTISCALE_DOWNSCALE) {
    k_downscale<<<grid, block, 0, st>>>(src, gw, gh, dst, w, h, kern);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    return has_digital_filter(kern) ? digital_filter(dst, scratch, w, h, kern, st) : cudaSuccess;
  }
  if (has_digital_filter(kern) && (e = digital_filter(src, scratch, gw, gh, kern, st)) != cudaSuccess) return e;
  k_upscale<<<grid, block, 0, st>>>(src, gw, gh, dst, w, h, kern);
  return cudaGetLastError();
}

}  // namespace ctxutil
}  // namespace cvr

extern "C" {

cvr_status cvr_set_multiscaling(cvr_ctx* c, int mode, int kernel, int factor_w, int factor_h) {
  if (!c) return CVR_ERR_INVALID_ARG;
  if (mode < CVR_MULTISCALE_SINGLE || mode > CVR_MULTISCALE_UPSCALE || kernel < CVR_FILTER_BOX ||
      kernel > CVR_FILTER_CARDINAL_OMOMS3 || factor_w < 1 || factor_h < 1 || factor_w > 8 || factor_h > 8)
    return fail(c, CVR_ERR_INVALID_ARG, "cvr_set_multiscaling: mode 0..3, kernel 0..5, factors 1..8");
  c->ms_mode = mode;
  c->ms_kernel = kernel;
  c->ms_fw = factor_w;
  c->ms_fh = factor_h;
  return CVR_OK;
}

cvr_status cvr_get_multiscaling(cvr_ctx* c, int* mode, int* kernel, int* factor_w, int* factor_h) {
  if (!c) return CVR_ERR_INVALID_ARG;
  if (mode) *mode = c->ms_mode;
  if (kernel) *kernel = c->ms_kernel;
  if (factor_w) *factor_w = c->ms_fw;
  if (factor_h) *factor_h = c->ms_fh;
  return CVR_OK;
}

cvr_status cvr_rescale_frame(cvr_ctx* c, int mode, int kernel, const float* src_dev, int sw, int sh, float* dst_dev,
                             int w, int h) {
  if (!c || !src_dev || !dst_dev || sw <= 0 || sh <= 0 || w <= 0 || h <= 0 || sw > 32768 || sh > 32768 ||
      w > 32768 || h > 32768 || mode < CVR_MULTISCALE_MULTISAMPLE || mode > CVR_MULTISCALE_UPSCALE ||
      kernel < CVR_FILTER_BOX || kernel > CVR_FILTER_CARDINAL_OMOMS3)
    return fail(c, CVR_ERR_INVALID_ARG, "cvr_rescale_frame: bad arguments");
  CK(c, cudaSetDevice(c->device));
  const size_t bytes = (size_t)sw * sh * sizeof(float4);
  CK(c, ensure(c->d_ms, c->ms_cap, bytes));
  if (const size_t sb = multiscale_scratch(mode, kernel, sw, sh, w, h))
    CK(c, ensure(c->d_msf, c->msf_cap, sb));
  CK(c, cudaMemcpyAsync(c->d_ms, src_dev, bytes, cudaMemcpyDeviceToDevice, c->stream));
  CK(c, launch_multiscale(mode, kernel, c->d_ms, sw, sh, reinterpret_cast<float4*>(dst_dev), w, h, c->d_msf,
                          c->stream));
  return CVR_OK;
}

}  // extern "C"
