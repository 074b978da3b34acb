// surrogate_host.cu — C ABI of surrogate shading: shading-point collection,
// labelling with the ground-truth integrator, evaluation against it, and the
// CVR_METHOD_SURROGATE launch of cvr_render.
#include <algorithm>
#include <cmath>

#include "ctx.cuh"
#include "mlp.cuh"
#include "surrogate.cuh"

using namespace cvr::ctxutil;

namespace {

constexpr size_t kChunk = 1u << 20;  // points per labelling / evaluation chunk

cvr_status need_sur(cvr_ctx* c) {
  if (!c) return CVR_ERR_INVALID_ARG;
  CK(c, cudaSetDevice(c->device));
  if (!c->sur) c->sur.reset(new SurState());
  SurState& s = *c->sur;
  if (!s.counter) CK(c, cudaMalloc((void**)&s.counter, sizeof(unsigned int)));
  if (!s.acc) CK(c, cudaMalloc((void**)&s.acc, sizeof(double) * 8));
  return CVR_OK;
}

cvr_status grow_points(cvr_ctx* c, size_t cap) {
  SurState& s = *c->sur;
  if (s.pts_cap >= cap && s.pts) return CVR_OK;
  float4* np = nullptr;
  CK(c, cudaMalloc((void**)&np, sizeof(float4) * 2 * cap));
  if (s.n_pts > 0) {
    cudaError_t e = cudaMemcpyAsync(np, s.pts, sizeof(float4) * 2 * (size_t)s.n_pts, cudaMemcpyDeviceToDevice, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) {
      cudaFree(np);
      return cuda_fail(c, e, "point list copy");
    }
  }
  if (s.pts) cudaFree(s.pts);
  s.pts = np;
  s.pts_cap = cap;
  return CVR_OK;
}

cvr_status grow_chunk(cvr_ctx* c) {
  SurState& s = *c->sur;
  if (s.chunk_cap >= kChunk) return CVR_OK;
  CK(c, cudaMalloc((void**)&s.cx, sizeof(float) * kMlpIn * kChunk));
  CK(c, cudaMalloc((void**)&s.ct, sizeof(float) * 2 * kChunk));
  CK(c, cudaMalloc((void**)&s.cy, sizeof(float) * 2 * kChunk));
  CK(c, cudaMalloc((void**)&s.cd, sizeof(float) * 2 * kChunk));
  s.chunk_cap = kChunk;
  return CVR_OK;
}

// Volume, transfer function and geometry of a frame (no camera / image).
FrameArgs base_frame(cvr_ctx* c) {
  FrameArgs f{};
  f.vol = volume_view(c);
  f.tf = c->d_rgbt;
  f.tf_n = c->tf_n;
  f.tile_w = 16;
  f.tile_h = 8;
  return f;
}

SurArgs sur_args(cvr_ctx* c, const cvr_light* light, const cvr_gt_params* p, int apply_occ, int apply_sdw) {
  const int shadow_type = p->shadow_type;
  const float ka = p->ka, kd = p->kd;
  SurArgs a{};
  a.sdw_dist = p->sdw_distance;
  if (pyramid_view(c, &a.pyr) != CVR_OK) {  // a failed copy leaves the plain levels
    a.pyr = c->pyr;
    a.pyr.data = c->d_pyr;
    a.pyr.quads = nullptr;
  }
  a.packed = c->mlp ? c->mlp->packed : nullptr;
  a.apply_occ = apply_occ;
  a.apply_sdw = apply_sdw;
  a.shadow_type = shadow_type;
  a.light_pos = make3(light->position);
  a.light_fwd = make3(light->forward);
  a.ka = ka;
  a.kd = kd;
  a.unit = (c->sx + c->sy + c->sz) / 3.0f;
  for (int l = 0; l < kSurLevels; ++l) a.ptex[l] = c->tex.pyr_valid ? c->tex.pyr[l].tex : 0;
  return a;
}

// Texture-unit sampling of the network inputs (cvr_set_sampling).
bool use_tex(cvr_ctx* c) { return (c->sampling & CVR_SAMPLING_TEX_FEATURES) != 0; }

cvr_status prepare_textures(cvr_ctx* c) {
  if (!use_tex(c)) return CVR_OK;
  return ensure_pyramid_textures(c);
}

GtArgs gt_args(cvr_ctx* c, const cvr_gt_params* p, const cvr_light* light) {
  GtArgs a{};
  a.occ_vec = c->d_occ_vec; a.sdw_vec = c->d_sdw_vec;
  a.n_occ = c->n_occ; a.n_sdw = c->n_sdw;
  a.gap = p->light_ray_initial_gap; a.lstep = p->light_ray_step_size;
  a.apply_occ = 1; a.apply_sdw = 1; a.shadow_type = p->shadow_type;
  a.occ_dist = p->occ_distance; a.sdw_dist = p->sdw_distance;
  a.light_pos = make3(light->position); a.light_fwd = make3(light->forward);
  a.light_up = make3(light->up); a.light_right = make3(light->right);
  a.ka = p->ka; a.kd = p->kd;
  return a;
}

DosArgs dos_args(cvr_ctx* c, const cvr_dos_params* p, const cvr_light* light) {
  DosArgs a{};
  if (pyramid_view(c, &a.pyr) != CVR_OK) {  // a failed copy leaves the plain levels
    a.pyr = c->pyr;
    a.pyr.data = c->d_pyr;
    a.pyr.quads = nullptr;
  }
  a.occ_sections = c->d_occ_sec; a.sdw_sections = c->d_sdw_sec;
  a.occ = c->occ; a.sdw = c->sdw;
  a.apply_occ = 1; a.apply_sdw = 1; a.shadow_type = p->shadow_type;
  a.light_pos = make3(light->position); a.light_fwd = make3(light->forward);
  a.light_up = make3(light->up); a.light_right = make3(light->right);
  a.spot_cos_max = light->spot_cos_max;
  a.ka = p->ka; a.kd = p->kd;
  return a;
}

cvr_status need_inputs(cvr_ctx* c, const char* who) {
  if (!c->has_volume) return fail(c, CVR_ERR_NO_VOLUME, std::string(who) + ": no volume loaded");
  if (c->tf_n == 0) return fail(c, CVR_ERR_NOT_READY, std::string(who) + ": no transfer function");
  if (c->tf_n * sizeof(float4) > 24 * 1024) return fail(c, CVR_ERR_UNSUPPORTED, std::string(who) + ": TF larger than 1536 entries");
  return CVR_OK;
}

cvr_status need_pyramid(cvr_ctx* c, const char* who) {
  if (!c->pyr_ready || c->pyr.n_levels < kSurLevels)
    return fail(c, CVR_ERR_NOT_READY, std::string(who) + ": needs an extinction pyramid of at least 6 levels");
  return CVR_OK;
}

cvr_status need_gt(cvr_ctx* c, const cvr_gt_params* p, const char* who) {
  if (!c->gt_ready || c->n_occ < 1 || c->n_sdw < 1)
    return fail(c, CVR_ERR_NOT_READY, std::string(who) + ": needs GT kernel vectors (at least one of each)");
  const float min_step = 1.0e-6f * std::sqrt((float)(c->nx * c->sx) * (c->nx * c->sx) +
                                             (float)(c->ny * c->sy) * (c->ny * c->sy) +
                                             (float)(c->nz * c->sz) * (c->nz * c->sz));
  if (!(p->light_ray_step_size >= min_step) || !std::isfinite(p->light_ray_step_size))
    return fail(c, CVR_ERR_INVALID_ARG, std::string(who) + ": light_ray_step_size must be >= 1e-6 * diagonal");
  return CVR_OK;
}

// Error sums of one chunk: acc[0..1] network squared errors, [2..3] cone
// squared errors, [4..5] target sums, [6] largest |occlusion error| (as the
// bits of a non-negative float).
__global__ void k_sur_errors(const float* __restrict__ y, const float* __restrict__ t, const float* __restrict__ d,
                             int n, double* acc) {
  double s[6] = {0, 0, 0, 0, 0, 0};
  float mx = 0.0f;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    float t0 = t[2 * i], t1 = t[2 * i + 1];
    float y0 = fminf(fmaxf(y[2 * i], 0.0f), 1.0f), y1 = fminf(fmaxf(y[2 * i + 1], 0.0f), 1.0f);
    s[0] += (double)(y0 - t0) * (y0 - t0);
    s[1] += (double)(y1 - t1) * (y1 - t1);
    if (d) {
      float d0 = d[2 * i], d1 = d[2 * i + 1];
      s[2] += (double)(d0 - t0) * (d0 - t0);
      s[3] += (double)(d1 - t1) * (d1 - t1);
    }
    s[4] += t0;
    s[5] += t1;
    mx = fmaxf(mx, fabsf(y0 - t0));
  }
#pragma unroll
  for (int k = 0; k < 6; ++k) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s[k] += __shfl_down_sync(0xffffffffu, s[k], o);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_down_sync(0xffffffffu, mx, o));
  if ((threadIdx.x & 31) == 0) {
#pragma unroll
    for (int k = 0; k < 6; ++k) atomicAdd(acc + k, s[k]);
    atomicMax(reinterpret_cast<unsigned long long*>(acc + 6), (unsigned long long)__float_as_uint(mx));
  }
}

}  // namespace

namespace cvr {
namespace ctxutil {

cvr_status sur_job_args(cvr_ctx* c, const cvr_gt_params* p, const cvr_light* light, SurArgs* a, bool* tex) {
  if (!c->mlp || !c->mlp->ready) return fail(c, CVR_ERR_NOT_READY, "cvr_render: surrogate network not initialised");
  cvr_status st = need_pyramid(c, "cvr_render");
  if (st != CVR_OK) return st;
  if (c->tf_n * sizeof(float4) > 24 * 1024) return fail(c, CVR_ERR_UNSUPPORTED, "cvr_render: TF larger than 1536 entries");
  if (p->shadow_type < 0 || p->shadow_type > 2) return fail(c, CVR_ERR_INVALID_ARG, "shadow_type must be 0, 1 or 2");
  st = need_sur(c);
  if (st == CVR_OK) st = prepare_textures(c);
  if (st != CVR_OK) return st;
  *a = sur_args(c, light, p, p->apply_occlusion, p->apply_shadow);
  *tex = use_tex(c);
  return CVR_OK;
}

cvr_status render_surrogate(cvr_ctx* c, const FrameArgs& f, const cvr_gt_params* p, const cvr_light* light) {
  SurArgs a{};
  bool tex = false;
  cvr_status st = sur_job_args(c, p, light, &a, &tex);
  if (st != CVR_OK) return st;
  CK(c, cudaMemsetAsync(c->sur->counter, 0, sizeof(unsigned int), c->stream));
  CK(c, launch_surrogate(f, a, tex, sur_spiral(f), c->sur->counter, c->mlp->err, c->stream));
  return CVR_OK;
}

}  // namespace ctxutil
}  // namespace cvr

extern "C" {

cvr_status cvr_surrogate_collect(cvr_ctx* c, const cvr_camera* cam, int w, int h, float step_size, float rate,
                                 uint64_t seed, int max_points, int* n_added) {
  if (!c || !cam || w <= 0 || h <= 0 || w > 32768 || h > 32768 || !(rate > 0.0f && rate <= 1.0f) || max_points < 0)
    return fail(c, CVR_ERR_INVALID_ARG, "cvr_surrogate_collect: bad arguments");
  cvr_status st = need_inputs(c, "cvr_surrogate_collect");
  if (st != CVR_OK) return st;
  st = need_sur(c);
  if (st != CVR_OK) return st;
  FrameArgs f = base_frame(c);
  const float min_step = 1.0e-6f * std::sqrt(dot3(f.vol.grid, f.vol.grid));
  if (!(step_size >= min_step) || !std::isfinite(step_size))
    return fail(c, CVR_ERR_INVALID_ARG, "cvr_surrogate_collect: step_size must be >= 1e-6 * diagonal");
  SurState& s = *c->sur;
  if (n_added) *n_added = 0;
  if (max_points <= s.n_pts) return CVR_OK;
  st = grow_points(c, (size_t)max_points);
  if (st != CVR_OK) return st;
  f.cam = camera_view(cam, w, h);
  f.step = step_size;
  f.W = w;
  f.H = h;
  CK(c, cudaMemsetAsync(s.counter, 0, sizeof(unsigned int), c->stream));
  CK(c, launch_sur_collect(f, rate, (unsigned long long)seed, s.pts + 2 * (size_t)s.n_pts, max_points - s.n_pts,
                           s.counter, c->stream));
  unsigned int got = 0;
  CK(c, cudaMemcpyAsync(&got, s.counter, sizeof got, cudaMemcpyDeviceToHost, c->stream));
  CK(c, cudaStreamSynchronize(c->stream));
  int added = (int)std::min<unsigned long long>(got, (unsigned long long)(max_points - s.n_pts));
  s.n_pts += added;
  if (n_added) *n_added = added;
  return CVR_OK;
}

cvr_status cvr_surrogate_clear_points(cvr_ctx* c) {
  if (!c) return CVR_ERR_INVALID_ARG;
  if (c->sur) c->sur->n_pts = 0;
  return CVR_OK;
}

int cvr_surrogate_point_count(cvr_ctx* c) { return (c && c->sur) ? c->sur->n_pts : 0; }

cvr_status cvr_surrogate_set_points(cvr_ctx* c, const float* pts, int n) {
  if (!c || n < 0 || (n > 0 && !pts)) return fail(c, CVR_ERR_INVALID_ARG, "cvr_surrogate_set_points: bad arguments");
  cvr_status st = need_sur(c);
  if (st != CVR_OK) return st;
  c->sur->n_pts = 0;
  st = grow_points(c, (size_t)std::max(n, 1));
  if (st != CVR_OK) return st;
  std::vector<float4> hp(2 * (size_t)n);
  for (int i = 0; i < n; ++i) {
    const float* q = pts + 6 * (size_t)i;
    hp[2 * (size_t)i] = make_float4(q[0], q[1], q[2], 0.0f);
    hp[2 * (size_t)i + 1] = make_float4(q[3], q[4], q[5], 0.0f);
  }
  if (n > 0)
    CK(c, cudaMemcpyAsync(c->sur->pts, hp.data(), sizeof(float4) * hp.size(), cudaMemcpyHostToDevice, c->stream));
  CK(c, cudaStreamSynchronize(c->stream));
  c->sur->n_pts = n;
  return CVR_OK;
}

cvr_status cvr_surrogate_get_points(cvr_ctx* c, float* pts, int n) {
  if (!c || !pts || !c->sur || n != c->sur->n_pts)
    return fail(c, CVR_ERR_INVALID_ARG, "cvr_surrogate_get_points: size mismatch");
  std::vector<float4> hp(2 * (size_t)n);
  if (n > 0) {
    CK(c, cudaMemcpyAsync(hp.data(), c->sur->pts, sizeof(float4) * hp.size(), cudaMemcpyDeviceToHost, c->stream));
    CK(c, cudaStreamSynchronize(c->stream));
  }
  for (int i = 0; i < n; ++i) {
    float* q = pts + 6 * (size_t)i;
    float4 a = hp[2 * (size_t)i], b = hp[2 * (size_t)i + 1];
    q[0] = a.x; q[1] = a.y; q[2] = a.z; q[3] = b.x; q[4] = b.y; q[5] = b.z;
  }
  return CVR_OK;
}

cvr_status cvr_surrogate_label(cvr_ctx* c, const cvr_light* light, const cvr_gt_params* p, int append_training,
                               float* x_host, float* t_host, int n) {
  if (!c || !light || !p) return fail(c, CVR_ERR_INVALID_ARG, "cvr_surrogate_label: bad arguments");
  cvr_status st = need_inputs(c, "cvr_surrogate_label");
  if (st == CVR_OK) st = need_pyramid(c, "cvr_surrogate_label");
  if (st == CVR_OK) st = need_gt(c, p, "cvr_surrogate_label");
  if (st == CVR_OK) st = need_sur(c);
  if (st == CVR_OK) st = prepare_textures(c);
  if (st != CVR_OK) return st;
  SurState& s = *c->sur;
  if ((x_host || t_host) && n != s.n_pts)
    return fail(c, CVR_ERR_INVALID_ARG, "cvr_surrogate_label: n must equal the point count");
  if (p->shadow_type < 0 || p->shadow_type > 2) return fail(c, CVR_ERR_INVALID_ARG, "shadow_type must be 0, 1 or 2");
  const int np = s.n_pts;
  if (np == 0) return CVR_OK;
  FrameArgs f = base_frame(c);
  SurArgs a = sur_args(c, light, p, 1, 1);
  GtArgs g = gt_args(c, p, light);
  float* tx = nullptr;
  float* tt = nullptr;
  if (append_training) {
    st = mlp_reserve_training(c, (size_t)np, &tx, &tt);
    if (st != CVR_OK) return st;
  }
  st = grow_chunk(c);
  if (st != CVR_OK) return st;
  for (size_t off = 0; off < (size_t)np; off += kChunk) {
    int cnt = (int)std::min(kChunk, (size_t)np - off);
    float* xo = append_training ? tx + kMlpIn * off : s.cx;
    float* to = append_training ? tt + 2 * off : s.ct;
    CK(c, launch_sur_label(s.pts + 2 * off, cnt, f, a, use_tex(c), &g, nullptr, xo, to, nullptr, c->stream));
    if (x_host)
      CK(c, cudaMemcpyAsync(x_host + kMlpIn * off, xo, sizeof(float) * kMlpIn * cnt, cudaMemcpyDeviceToHost, c->stream));
    if (t_host) CK(c, cudaMemcpyAsync(t_host + 2 * off, to, sizeof(float) * 2 * cnt, cudaMemcpyDeviceToHost, c->stream));
    CK(c, cudaStreamSynchronize(c->stream));
  }
  if (append_training) c->mlp->n += np;
  return CVR_OK;
}

cvr_status cvr_surrogate_evaluate(cvr_ctx* c, const cvr_light* light, const cvr_gt_params* p,
                                  const cvr_dos_params* cone, double out[8]) {
  if (!c || !light || !p || !out) return fail(c, CVR_ERR_INVALID_ARG, "cvr_surrogate_evaluate: bad arguments");
  if (!c->mlp || !c->mlp->ready) return fail(c, CVR_ERR_NOT_READY, "cvr_surrogate_evaluate: no network");
  cvr_status st = need_inputs(c, "cvr_surrogate_evaluate");
  if (st == CVR_OK) st = need_pyramid(c, "cvr_surrogate_evaluate");
  if (st == CVR_OK) st = need_gt(c, p, "cvr_surrogate_evaluate");
  if (st == CVR_OK && cone && !c->cone_ready)
    st = fail(c, CVR_ERR_NOT_READY, "cvr_surrogate_evaluate: cone tables not set");
  if (st == CVR_OK) st = need_sur(c);
  if (st == CVR_OK) st = prepare_textures(c);
  if (st != CVR_OK) return st;
  if (p->shadow_type < 0 || p->shadow_type > 2 || (cone && (cone->shadow_type < 0 || cone->shadow_type > 2)))
    return fail(c, CVR_ERR_INVALID_ARG, "shadow_type must be 0, 1 or 2");
  st = grow_chunk(c);
  if (st != CVR_OK) return st;
  SurState& s = *c->sur;
  const int np = s.n_pts;
  FrameArgs f = base_frame(c);
  SurArgs a = sur_args(c, light, p, 1, 1);
  GtArgs g = gt_args(c, p, light);
  DosArgs d{};
  if (cone) d = dos_args(c, cone, light);
  CK(c, cudaMemsetAsync(s.acc, 0, sizeof(double) * 8, c->stream));
  for (size_t off = 0; off < (size_t)np; off += kChunk) {
    int cnt = (int)std::min(kChunk, (size_t)np - off);
    CK(c, launch_sur_label(s.pts + 2 * off, cnt, f, a, use_tex(c), &g, cone ? &d : nullptr, s.cx, s.ct,
                           cone ? s.cd : nullptr, c->stream));
    CK(c, launch_mlp_infer(c->mlp->packed, s.cx, cnt, s.cy, c->mlp->err, c->stream));
    k_sur_errors<<<std::min(1024, (cnt + 255) / 256), 256, 0, c->stream>>>(s.cy, s.ct, cone ? s.cd : nullptr, cnt,
                                                                            s.acc);
    CK(c, cudaGetLastError());
  }
  double h[8];
  CK(c, cudaMemcpyAsync(h, s.acc, sizeof h, cudaMemcpyDeviceToHost, c->stream));
  CK(c, cudaStreamSynchronize(c->stream));
  st = mlp_check_err(c);
  if (st != CVR_OK) return st;
  const double inv = np > 0 ? 1.0 / np : 0.0;
  unsigned long long mxbits = 0;
  std::memcpy(&mxbits, &h[6], sizeof mxbits);
  uint32_t mx32 = (uint32_t)mxbits;
  float mx = 0.0f;
  std::memcpy(&mx, &mx32, sizeof mx);
  out[0] = std::sqrt(h[0] * inv);
  out[1] = std::sqrt(h[1] * inv);
  out[2] = cone ? std::sqrt(h[2] * inv) : 0.0;
  out[3] = cone ? std::sqrt(h[3] * inv) : 0.0;
  out[4] = (double)np;
  out[5] = h[4] * inv;
  out[6] = h[5] * inv;
  out[7] = mx;
  return CVR_OK;
}

}  // extern "C"
