// ctx.cuh — the cvr_ctx object shared by the translation units of the C ABI
// (context.cu: volume, tables and rendering; mlp_host.cu: the surrogate
// network) and their common error / allocation helpers.
#pragma once

#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <string>
#include <utility>
#include <vector>

#include "../../include/cvr.h"
#include "build_tables.cuh"
#include "march.cuh"
#include "surrogate.cuh"

using namespace cvr;

// Device state of the surrogate network: FP32 master parameters, Adam
// moments, the packed BF16 image, per-CTA gradient partials, the training set.
struct MlpState {
  float* params = nullptr;
  float* m = nullptr;
  float* v = nullptr;
  uint8_t* packed = nullptr;
  float* partials = nullptr;
  size_t partials_cap = 0;
  float* grad = nullptr;     // reduced gradient (+ loss) of the last batch
  float* loss_acc = nullptr; // loss accumulated over an epoch
  int* err = nullptr;        // set by a kernel whose bounded wait gave up
  int* step = nullptr;       // Adam step counter
  float* x = nullptr;        // training features, n x 48
  float* t = nullptr;        // training targets, n x 2
  size_t data_cap = 0;       // points
  int n = 0;
  int* idx = nullptr;        // epoch permutation
  size_t idx_cap = 0;
  float* io_x = nullptr;     // staging of host batches (forward / gradients)
  float* io_y = nullptr;
  size_t io_cap = 0;
  cudaGraphExec_t epoch_graph = nullptr;
  int graph_batch = 0, graph_n = 0;
  float graph_lr = 0.0f;
  bool ready = false;
  ~MlpState() {
    void* bufs[] = {params, m, v, packed, partials, grad, loss_acc, err, step, x, t, idx, io_x, io_y};
    for (void* p : bufs)
      if (p) cudaFree(p);
    if (epoch_graph) cudaGraphExecDestroy(epoch_graph);
  }
};

// Texture-unit copies of the volume and of the pyramid levels (hardware
// trilinear filtering), made on first use after the source changed.
struct TexImage {
  cudaArray_t arr = nullptr;
  cudaTextureObject_t tex = 0;
  void release() {
    if (tex) cudaDestroyTextureObject(tex);
    if (arr) cudaFreeArray(arr);
    tex = 0;
    arr = nullptr;
  }
};
struct TexState {
  TexImage vol;
  bool vol_valid = false;
  TexImage pyr[CVR_MAX_LEVELS];
  int n_pyr = 0;
  bool pyr_valid = false;
  TexImage grad;
  bool grad_valid = false;
  ~TexState() {
    vol.release();
    for (auto& t : pyr) t.release();
    grad.release();
  }
};

inline void swap_tex(TexState& a, TexState& b) {
  std::swap(a.vol, b.vol);
  std::swap(a.vol_valid, b.vol_valid);
  for (int l = 0; l < CVR_MAX_LEVELS; ++l) std::swap(a.pyr[l], b.pyr[l]);
  std::swap(a.n_pyr, b.n_pyr);
  std::swap(a.pyr_valid, b.pyr_valid);
  std::swap(a.grad, b.grad);
  std::swap(a.grad_valid, b.grad_valid);
}

// sat32_F of a context / slot without a valid compact SAT.
constexpr int kNoCompactSat = -1000;
// vbrick_bs of a copy in the x-y quad layout.
constexpr int kQuadCopy = 100;
// Cells of a compact SAT or a quad volume copy: indexed with 32-bit cell
// numbers, so larger grids keep the int64 table / the plain layout.
constexpr size_t kCompactMaxCells = (size_t)1 << 31;

// A resident volume that is not the current one (cvr_select_volume): the
// volume, its SAT, pyramid and texture copies.  The current volume lives in
// the cvr_ctx fields of the same names.
struct VolSlot {
  void* d_vol = nullptr;
  size_t vol_cap = 0;
  int nx = 0, ny = 0, nz = 0, dtype = 0;
  float sx = 1, sy = 1, sz = 1;
  bool has_volume = false;
  long long* d_sat = nullptr;
  size_t sat_cap = 0;
  long long* d_lut = nullptr;
  int sat_frac_bits = 0;
  bool sat_ready = false;
  bool sat_pending = false;
  std::vector<double> sat_ext;
  uint4* d_sat32 = nullptr;
  size_t sat32_cap = 0;
  unsigned* d_lut32 = nullptr;
  size_t lut32_cap = 0;
  int sat32_F = kNoCompactSat;
  double sat32_vmax = 0.0;
  unsigned long long sat32_gen = 0;  // which build of the compact table (walk tables follow it)
  float* d_pyr = nullptr;
  size_t pyr_cap = 0;
  PyramidView pyr{};
  bool pyr_ready = false;
  float4* d_pyrq = nullptr;
  size_t pyrq_cap = 0;
  bool pyrq_ready = false;
  TexState tex;
  void* d_vbrick = nullptr;
  size_t vbrick_cap = 0;
  int vbrick_bs = -1;
  uint2* d_grad = nullptr;
  size_t grad_cap = 0;
  bool grad_ready = false;
  cvr_gradient_params grad_params{CVR_GRADIENT_NONE, 1, 0, 1};
  ~VolSlot() {
    void* bufs[] = {d_vol, d_sat, d_lut, d_pyr, d_vbrick, d_grad, d_sat32, d_lut32, d_pyrq};
    for (void* p : bufs)
      if (p) cudaFree(p);
  }
};

// Shading points of the surrogate (training / evaluation) and its scratch.
struct SurState {
  float4* pts = nullptr;         // 2 float4 per point: position, direction
  size_t pts_cap = 0;            // points
  int n_pts = 0;
  unsigned int* counter = nullptr;  // collection count / marcher ray counter
  float* cx = nullptr;           // per-chunk features, targets, predictions, cone values
  float* ct = nullptr;
  float* cy = nullptr;
  float* cd = nullptr;
  size_t chunk_cap = 0;
  double* acc = nullptr;         // error sums of cvr_surrogate_evaluate
  ~SurState() {
    void* bufs[] = {pts, counter, cx, ct, cy, cd, acc};
    for (void* p : bufs)
      if (p) cudaFree(p);
  }
};

struct cvr_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  std::string err;
  // volume
  void* d_vol = nullptr;
  size_t vol_cap = 0;
  int nx = 0, ny = 0, nz = 0, dtype = 0;
  float sx = 1, sy = 1, sz = 1;
  bool has_volume = false;
  // transfer function
  float4* d_rgbt = nullptr;
  float4* d_rgba = nullptr;
  int tf_n = 0, tf_cap = 0;
  // SAT
  long long* d_sat = nullptr;
  size_t sat_cap = 0;
  long long* d_lut = nullptr;
  int sat_frac_bits = 0;
  bool sat_ready = false;    // cvr_build_sat succeeded for the current volume
  bool sat_pending = false;  // its int64 table is not built yet (ensure_sat)
  // compact SAT (32-bit prefix sums modulo 2^32 at F32 fractional bits) for
  // frames whose boxes are small enough; the extinction table it is built from
  std::vector<double> sat_ext;
  uint4* d_sat32 = nullptr;                  // x-y quad layout
  size_t sat32_cap = 0;
  unsigned* d_lut32 = nullptr;
  size_t lut32_cap = 0;
  int sat32_F = kNoCompactSat;
  double sat32_vmax = 0.0;  // the query extent the current compact table was planned for
  unsigned long long sat32_gen = 0;          // which build of the compact table (walk tables follow it)
  bool compact_sat = true;                   // cvr_set_compact_sat
  bool walk_tables = true;                   // cvr_set_walk_tables
  unsigned* d_satp = nullptr;                // compact builds' plane-prefix scratch (any volume slot)
  size_t satp_cap = 0;
  float* d_pyrs = nullptr;                   // separable pyramid builds' scratch (any volume slot)
  size_t pyrs_cap = 0;
  // the directional shadow's walk table (WalkView) of compact build walk_gen
  uint4* d_walk = nullptr;
  size_t walk_cap = 0;
  unsigned long long walk_gen = 0;
  int walk_axis = -1, walk_w = 0;
  // pyramid, and its x-y quad copy for FP32 taps (built with the first frame that needs it)
  float* d_pyr = nullptr;
  size_t pyr_cap = 0;
  PyramidView pyr{};
  bool pyr_ready = false;
  float4* d_pyrq = nullptr;
  size_t pyrq_cap = 0;
  bool pyrq_ready = false;
  // cone tables
  float4* d_occ_sec = nullptr;
  float4* d_sdw_sec = nullptr;
  ConeTableDev occ{}, sdw{};
  bool cone_ready = false;
  // GT kernel vectors
  float3* d_occ_vec = nullptr;
  float3* d_sdw_vec = nullptr;
  int n_occ = 0, n_sdw = 0;
  bool gt_ready = false;
  // frame
  unsigned long long* d_stats = nullptr;
  float4* d_out = nullptr;
  size_t out_cap = 0;
  void* d_flush = nullptr;
  size_t flush_bytes = 0;
  void* d_probe = nullptr;  // cvr_measure_l1_bandwidth's buffer
  size_t probe_cap = 0;
  cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
  // Pinned staging of the fixed-point tables cvr_build_sat (int64, 65536
  // entries) and the compact rebuild (32-bit) upload, so that the copies are
  // asynchronous; each region is rewritten only after its last copy completed.
  void* h_stage = nullptr;
  cudaEvent_t stage_ev[2] = {nullptr, nullptr};
  int tile_w = 16, tile_h = 8, variant = 0;
  int warp_w = 8;                            // cvr_set_warp_shape (used where the tile holds whole warps)
  bool refill = false;                       // cvr_set_ray_refill: persistent ray-refill marchers
  bool staging = false;                      // cvr_set_brick_staging: the plain marcher's staged variant
  std::unique_ptr<ShadowBoxTable> sdw_table;  // per-frame directional shadow boxes (host staging)
  std::unique_ptr<MlpState> mlp;             // surrogate network (created by cvr_mlp_init)
  std::unique_ptr<SurState> sur;             // surrogate shading points
  TexState tex;                              // texture-unit copies (volume, pyramid)
  int sampling = CVR_SAMPLING_TEX_FEATURES;  // cvr_set_sampling flags
  VolSlot slots[CVR_MAX_VOLUMES];            // the other resident volumes
  int cur_slot = 0;
  // bricked or quad copy of the current volume for the marchers
  // (cvr_set_brick_size, cvr_set_volume_layout)
  int brick_bs = 0;                          // tuning: 0 plain layout, else log2 of the brick edge
  bool quads = false;                        // tuning: the x-y quad layout (takes precedence)
  void* d_vbrick = nullptr;
  size_t vbrick_cap = 0;
  int vbrick_bs = -1;                        // layout of d_vbrick's contents (-1: stale, kQuadCopy: quads)
  // object-space light cache (cvr_set_light_cache): 0 = off
  int lc_dims[3] = {0, 0, 0};
  float2* d_lcache = nullptr;
  size_t lcache_cap = 0;
  // per-voxel gradient of the current volume (cvr_build_gradient) and the
  // Blinn-Phong settings of cvr_set_blinn_phong (context-wide)
  uint2* d_grad = nullptr;
  size_t grad_cap = 0;
  bool grad_ready = false;
  cvr_gradient_params grad_params{CVR_GRADIENT_NONE, 1, 0, 1};
  int grad_kernel = CVR_GRADIENT_KERNEL_AUTO;  // cvr_set_gradient_kernel
  int grad_last = -1;                          // the builder the last build ran
  int* d_kerr = nullptr;                       // set by a table builder whose bounded wait gave up
  cvr_blinn_phong bp{0, 0.5f, 0.5f, 0.8f, 30.0f, {1.0f, 1.0f, 1.0f}};
  // pixel multiscaling (cvr_set_multiscaling) and its generated-frame buffer
  int ms_mode = CVR_MULTISCALE_SINGLE, ms_kernel = CVR_FILTER_HAT, ms_fw = 2, ms_fh = 2;
  float4* d_ms = nullptr;
  size_t ms_cap = 0;
  float4* d_msf = nullptr;  // digital-filter scratch
  size_t msf_cap = 0;
};

// Exchanges the current-volume fields of c with slot s.
inline void swap_volume(cvr_ctx* c, VolSlot& s) {
  std::swap(c->d_vol, s.d_vol);
  std::swap(c->vol_cap, s.vol_cap);
  std::swap(c->nx, s.nx); std::swap(c->ny, s.ny); std::swap(c->nz, s.nz);
  std::swap(c->dtype, s.dtype);
  std::swap(c->sx, s.sx); std::swap(c->sy, s.sy); std::swap(c->sz, s.sz);
  std::swap(c->has_volume, s.has_volume);
  std::swap(c->d_sat, s.d_sat);
  std::swap(c->sat_cap, s.sat_cap);
  std::swap(c->d_lut, s.d_lut);
  std::swap(c->sat_frac_bits, s.sat_frac_bits);
  std::swap(c->sat_ready, s.sat_ready);
  std::swap(c->sat_pending, s.sat_pending);
  std::swap(c->sat_ext, s.sat_ext);
  std::swap(c->d_sat32, s.d_sat32);
  std::swap(c->sat32_cap, s.sat32_cap);
  std::swap(c->d_lut32, s.d_lut32);
  std::swap(c->lut32_cap, s.lut32_cap);
  std::swap(c->sat32_F, s.sat32_F);
  std::swap(c->sat32_vmax, s.sat32_vmax);
  std::swap(c->sat32_gen, s.sat32_gen);
  std::swap(c->d_pyr, s.d_pyr);
  std::swap(c->pyr_cap, s.pyr_cap);
  std::swap(c->pyr, s.pyr);
  std::swap(c->pyr_ready, s.pyr_ready);
  std::swap(c->d_pyrq, s.d_pyrq);
  std::swap(c->pyrq_cap, s.pyrq_cap);
  std::swap(c->pyrq_ready, s.pyrq_ready);
  swap_tex(c->tex, s.tex);
  std::swap(c->d_vbrick, s.d_vbrick);
  std::swap(c->vbrick_cap, s.vbrick_cap);
  std::swap(c->vbrick_bs, s.vbrick_bs);
  std::swap(c->d_grad, s.d_grad);
  std::swap(c->grad_cap, s.grad_cap);
  std::swap(c->grad_ready, s.grad_ready);
  std::swap(c->grad_params, s.grad_params);
}

namespace cvr {
namespace ctxutil {

extern thread_local std::string g_create_err;

// A tile holds whole warps of warp_w x (32 / warp_w) pixels.
inline bool warp_fits(int tile_w, int tile_h, int warp_w) {
  return (warp_w == 4 || warp_w == 8 || warp_w == 16) && tile_w % warp_w == 0 && tile_h % (32 / warp_w) == 0;
}

inline bool finite3(const float* p) { return std::isfinite(p[0]) && std::isfinite(p[1]) && std::isfinite(p[2]); }

inline cvr_status fail(cvr_ctx* c, cvr_status code, const std::string& msg) {
  if (c) c->err = msg;
  return code;
}

// Reads (synchronously) and clears the context's kernel error flag.
cvr_status check_kernel_flag(cvr_ctx* c, const char* what);
// The current pyramid's view for kernels; under the quad layout with its x-y
// quad copy when one can be made (FP32 taps: two loads instead of eight, same
// values).
cvr_status pyramid_view(cvr_ctx* c, PyramidView* out);

inline cvr_status cuda_fail(cvr_ctx* c, cudaError_t e, const char* what) {
  cudaGetLastError();  // clear a sticky launch error where possible
  std::string msg = std::string(what) + ": " + cudaGetErrorString(e);
  return fail(c, e == cudaErrorMemoryAllocation ? CVR_ERR_OUT_OF_MEMORY : CVR_ERR_CUDA, msg);
}

#define CK(ctx, call)                                   \
  do {                                                  \
    cudaError_t e_ = (call);                            \
    if (e_ != cudaSuccess) return cuda_fail(ctx, e_, #call); \
  } while (0)

// Grows a device allocation to at least 'bytes' (contents discarded).
template <class T>
cudaError_t ensure(T*& p, size_t& cap, size_t bytes) {
  if (cap >= bytes && p) return cudaSuccess;
  if (p) cudaFree(p);
  p = nullptr;
  cap = 0;
  cudaError_t e = cudaMalloc((void**)&p, bytes);
  if (e == cudaSuccess) cap = bytes;
  return e;
}

inline VolumeView volume_view(const cvr_ctx* c) {
  VolumeView v;
  v.voxels = c->d_vol;
  v.dtype = c->dtype;
  v.nx = c->nx; v.ny = c->ny; v.nz = c->nz;
  v.spacing = f3(c->sx, c->sy, c->sz);
  v.inv_spacing = f3(1.0f / c->sx, 1.0f / c->sy, 1.0f / c->sz);
  v.grid = f3(c->nx * c->sx, c->ny * c->sy, c->nz * c->sz);
  v.norm = c->dtype == CVR_U8 ? 1.0f / 255.0f : 1.0f / 65535.0f;
  v.tex = 0;
  v.inv_grid = f3(1.0f / v.grid.x, 1.0f / v.grid.y, 1.0f / v.grid.z);
  v.bs = 0;
  v.quad = 0;
  v.stride[0] = 1;
  v.stride[1] = c->nx;
  v.stride[2] = (long long)c->nx * c->ny;
  return v;
}

// glm::lookAt basis in single precision (libs/vis_utils/camera.cpp:281-284).
inline CameraView camera_view(const cvr_camera* cam, int w, int h) {
  float3 eye = make3(cam->eye), ctr = make3(cam->center), up = make3(cam->up);
  float3 fw = ctr - eye;
  float inv = 1.0f / std::sqrt(dot3(fw, fw));
  fw = fw * inv;
  float3 s = cross3(fw, up);
  inv = 1.0f / std::sqrt(dot3(s, s));
  s = s * inv;
  float3 u = cross3(s, fw);
  CameraView cv;
  cv.eye = eye; cv.s = s; cv.u = u; cv.f = fw;
  cv.tan_half_fovy = (float)std::tan((double)cam->fovy_deg * (3.14159265358979323846 / 180.0) / 2.0);
  cv.aspect = cam->aspect > 0.0f ? cam->aspect : (float)w / (float)h;
  return cv;
}

// Surrogate pieces shared between translation units.
// Training-set slots for 'extra' more points (contents kept); *x / *t point
// at the first new slot.  The caller bumps mlp->n once they are written.
cvr_status mlp_reserve_training(cvr_ctx* c, size_t extra, float** x, float** t);
// Reads and clears the network's device error flag (bounded tensor-core waits).
cvr_status mlp_check_err(cvr_ctx* c);
// Texture objects of the volume / pyramid levels, (re)made when stale.
cvr_status ensure_volume_texture(cvr_ctx* c);
cvr_status ensure_pyramid_textures(cvr_ctx* c);
cvr_status ensure_gradient_texture(cvr_ctx* c);
// Gradient shading of a frame of 'method' (f->grad; off unless cvr_set_blinn_phong
// applies it and the volume has a gradient model, built here when stale).
cvr_status grad_args(cvr_ctx* c, int method, const cvr_light* light, FrameArgs* f);
// Pixel multiscaling (postpass.cu): the generated frame's size for an output of
// w x h, and the post-pass from it (modified in place by up-scaling filters).
void multiscale_size(int mode, int fw, int fh, int w, int h, int* gw, int* gh);
cudaError_t launch_multiscale(int mode, int kern, float4* src, int gw, int gh, float4* dst, int w, int h,
                              float4* scratch, cudaStream_t st);
// Bytes of the digital-filter scratch launch_multiscale needs (0: none).
size_t multiscale_scratch(int mode, int kern, int gw, int gh, int w, int h);
// The volume as the marchers read it: the plain layout, or the bricked copy
// of the context's brick size (made on first use after the volume changed).
cvr_status render_volume_view(cvr_ctx* c, VolumeView* v, bool allow_tex = true);
// Frame arguments of a render of the current volume (validated; f.step from
// the params struct's leading step_size, f.counts null, f.stats the context's).
cvr_status frame_args(cvr_ctx* c, const cvr_camera* cam, const void* params, float* out, int w, int h,
                      FrameArgs* f, bool need_tf = true);
// Extinction arguments of the current volume; *table: the directional
// shadow-box table (context-owned staging, valid until the next call) or null.
// With vmax_out the compact SAT is left to the caller: *vmax_out = the largest
// region the frame's queries span (0: the frame cannot use a compact table).
cvr_status ext_args(cvr_ctx* c, const cvr_ext_params* p, const cvr_light* light, const FrameArgs& f, ExtArgs* e,
                    const ShadowBoxTable** table, double* vmax_out = nullptr);
// The compact 32-bit SAT for a frame whose box queries span at most vmax
// cells, (re)built when its fixed point changes; *inv_scale = 2^-F32, or 0
// when the frame keeps the int64 table.
cvr_status ensure_compact_sat(cvr_ctx* c, double vmax, float* inv_scale);
cvr_status ensure_walk_table(cvr_ctx* c, int axis, int w, WalkView* out);
// Enqueues the current volume's pending int64 SAT build (cvr_build_sat defers it).
cvr_status ensure_sat(cvr_ctx* c);
// Staging region r of the pinned table buffer (0: 65536 int64 values, 1:
// 65536 32-bit values), free to write: the region's previous copy has completed.
cvr_status stage_region(cvr_ctx* c, int r, void** out);
// Enqueues the copy of n bytes of staging region r to dev and marks the region busy.
cvr_status stage_upload(cvr_ctx* c, int r, void* dev, size_t n);
// The pieces of it: the fixed point (false: keep the int64 table) and the
// build of the current volume's compact table into dst.
bool compact_plan(const std::vector<double>& ext, double vmax, int* F, std::vector<unsigned>* q);
cvr_status build_compact_sat(cvr_ctx* c, const std::vector<unsigned>& q, uint4* dst);
// Surrogate arguments of the current volume (pyramid, textures, network).
cvr_status sur_job_args(cvr_ctx* c, const cvr_gt_params* p, const cvr_light* light, SurArgs* a, bool* tex);
// The CVR_METHOD_SURROGATE launch of cvr_render.
cvr_status render_surrogate(cvr_ctx* c, const FrameArgs& f, const cvr_gt_params* p, const cvr_light* light);

}  // namespace ctxutil
}  // namespace cvr
