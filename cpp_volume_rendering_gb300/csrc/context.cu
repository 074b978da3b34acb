// context.cu — cvr_ctx and the device entry points of cvr.h.
//
// A context mirrors the GL state a renderer plugin owns between Init() and
// Clean(): the volume texture, transfer-function textures, SAT / pyramid /
// cone-table / kernel-vector textures and the output frame.  Uploads happen
// once (Init); each cvr_render is Update() + Redraw() of one frame.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "ctx.cuh"

using namespace cvr::ctxutil;

thread_local std::string cvr::ctxutil::g_create_err;

namespace {

// The boxes ConeZAxis / ConeYAxis / ConeXAxis (ebs_ray_bbox_marching.comp:190-430)
// walk for a fixed cone direction, evaluated once per frame in double
// precision.  Returns false when the walk has more boxes than the table holds
// (the kernel then evaluates the geometry per sample).
bool build_shadow_table(const cvr_ext_params* p, const float fwd[3], float3 spacing, float3 grid, ShadowBoxTable* t) {
  double c[3] = {fwd[0], fwd[1], fwd[2]};
  double n = std::sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]);
  for (double& v : c) v /= n;
  double a[3] = {std::fabs(c[0]), std::fabs(c[1]), std::fabs(c[2])};
  int ax = (a[2] > a[0] && a[2] > a[1]) ? 2 : (a[1] > a[0] ? 1 : 0);
  const double ang = p->sdw_cone_angle_rad;
  const double p_cs = std::cos(ang), p_sn = std::sin(ang), n_cs = std::cos(-ang), n_sn = std::sin(-ang);
  auto nrm = [](double x, double y, double z, double* o) {
    double l = std::sqrt(x * x + y * y + z * z);
    o[0] = x / l; o[1] = y / l; o[2] = z / l;
  };
  double pa1[3], pa2[3], pb1[3], pb2[3], q1[3], q2[3];
  int sa, sb;
  if (ax == 2) {  // ConeZAxis: secondary axes x (proj_x) and y (proj_y)
    sa = 0; sb = 1;
    nrm(0, c[1], c[2], q1);  // proj_y
    nrm(c[0], 0, c[2], q2);  // proj_x
    nrm(q2[0] * n_cs - q2[2] * n_sn, 0, q2[0] * n_sn + q2[2] * n_cs, pa1);
    nrm(q2[0] * p_cs - q2[2] * p_sn, 0, q2[0] * p_sn + q2[2] * p_cs, pa2);
    nrm(0, q1[1] * n_cs - q1[2] * n_sn, q1[1] * n_sn + q1[2] * n_cs, pb1);
    nrm(0, q1[1] * p_cs - q1[2] * p_sn, q1[1] * p_sn + q1[2] * p_cs, pb2);
  } else if (ax == 1) {  // ConeYAxis: secondary axes x (proj_x) and z (proj_z)
    sa = 0; sb = 2;
    nrm(c[0], c[1], 0, q1);  // proj_x
    nrm(0, c[1], c[2], q2);  // proj_z
    nrm(q1[0] * n_cs - q1[1] * n_sn, q1[0] * n_sn + q1[1] * n_cs, 0, pa1);
    nrm(q1[0] * p_cs - q1[1] * p_sn, q1[0] * p_sn + q1[1] * p_cs, 0, pa2);
    nrm(0, q2[2] * n_sn + q2[1] * n_cs, q2[2] * n_cs - q2[1] * n_sn, pb1);
    nrm(0, q2[2] * p_sn + q2[1] * p_cs, q2[2] * p_cs - q2[1] * p_sn, pb2);
  } else {  // ConeXAxis: secondary axes y (proj_y) and z (proj_z)
    sa = 1; sb = 2;
    nrm(c[0], c[1], 0, q1);  // proj_y
    nrm(c[0], 0, c[2], q2);  // proj_z
    nrm(q1[1] * n_sn + q1[0] * n_cs, q1[1] * n_cs - q1[0] * n_sn, 0, pa1);
    nrm(q1[1] * p_sn + q1[0] * p_cs, q1[1] * p_cs - q1[0] * p_sn, 0, pa2);
    nrm(q2[2] * n_sn + q2[0] * n_cs, 0, q2[2] * n_cs - q2[0] * n_sn, pb1);
    nrm(q2[2] * p_sn + q2[0] * p_cs, 0, q2[2] * p_cs - q2[0] * p_sn, pb2);
  }
  const double sc[3] = {spacing.x, spacing.y, spacing.z};
  const double gr[3] = {grid.x, grid.y, grid.z};
  const double signal = c[ax] < 0.0 ? -1.0 : 1.0;
  const double iw = (double)p->sdw_sample_interval * signal * sc[ax];
  double mp = (double)p->sdw_initial_step * signal * sc[ax];
  int k = 0;
  bool aligned = true;
  while ((mp / c[ax]) < (double)p->sdw_max_distance) {
    if (k == CVR_MAX_SDW_BOXES) return false;
    double mean = std::fabs(mp + iw * 0.5);
    double a1 = pa1[sa] * (mean / std::fabs(pa1[ax])), a2 = pa2[sa] * (mean / std::fabs(pa2[ax]));
    double b1 = pb1[sb] * (mean / std::fabs(pb1[ax])), b2 = pb2[sb] * (mean / std::fabs(pb2[ax]));
    double lo_a = std::min(a1, a2), hi_a = std::max(a1, a2);
    double lo_b = std::min(b1, b2), hi_b = std::max(b1, b2);
    double ad = std::fabs(hi_a - lo_a), bd = std::fabs(hi_b - lo_b);
    double as = (std::ceil(ad / sc[sa]) - (ad / sc[sa])) * 0.5;
    double bs = (std::ceil(bd / sc[sb]) - (bd / sc[sb])) * 0.5;
    lo_a -= as * sc[sa]; hi_a += as * sc[sa];
    lo_b -= bs * sc[sb]; hi_b += bs * sc[sb];
    double lo[3], hi[3];
    lo[ax] = std::min(mp, mp + iw); hi[ax] = std::max(mp, mp + iw);
    lo[sa] = lo_a; hi[sa] = hi_a; lo[sb] = lo_b; hi[sb] = hi_b;
    double volq = (std::fabs(hi[0] - lo[0]) / sc[0]) * (std::fabs(hi[1] - lo[1]) / sc[1]) *
                  (std::fabs(hi[2] - lo[2]) / sc[2]);
    t->lo[k] = make_float4((float)lo[0], (float)lo[1], (float)lo[2], (float)mp);
    t->hi[k] = make_float4((float)hi[0], (float)hi[1], (float)hi[2], (float)((double)p->sdw_ui_weight / volq));
    // integer texel widths (ceil-rounded cross-sections; the walk axis: the
    // interval) for the compact table's equal-fraction query
    int wpk = 0;
    for (int a = 0; a < 3; ++a) {
      const double wd = (hi[a] - lo[a]) / sc[a];
      const double wr = std::nearbyint(wd);
      if (!(std::fabs(wd - wr) <= 1e-6 * std::max(1.0, wr)) || wr < 0.0 || wr > 1023.0) aligned = false;
      else wpk |= (int)wr << (10 * a);
    }
    float pk;
    std::memcpy(&pk, &wpk, sizeof pk);
    t->tx[k] = make_float4((float)(lo[0] / sc[0]), (float)(lo[1] / sc[1]), (float)(lo[2] / sc[2]), pk);
    mp = mp + iw;
    ++k;
  }
  t->aligned = aligned ? 1 : 0;
  t->n = k;
  t->axis = ax;
  t->interval = (float)iw;
  t->vmin = (float)(sc[ax] * 0.5);
  t->vmax = (float)(gr[ax] - sc[ax] * 0.5);
  return true;
}

}  // namespace

namespace cvr {
namespace ctxutil {

cvr_status render_volume_view(cvr_ctx* c, VolumeView* out, bool allow_tex) {
  VolumeView v = volume_view(c);
  // the quad copy is indexed with 32-bit cell numbers
  if (c->quads && (size_t)c->nx * c->ny * c->nz < kCompactMaxCells) {
    if (c->vbrick_bs != kQuadCopy) {
      const size_t n = (size_t)c->nx * c->ny * c->nz;
      CK(c, ensure(c->d_vbrick, c->vbrick_cap, n * 4 * (c->dtype == CVR_U8 ? 1 : 2)));
      CK(c, launch_quad_volume(c->d_vol, c->d_vbrick, c->dtype, c->nx, c->ny, c->nz, c->stream));
      c->vbrick_bs = kQuadCopy;
    }
    v.voxels = c->d_vbrick;
    v.quad = 1;
  } else if (c->brick_bs > 0) {
    if (c->vbrick_bs != c->brick_bs) {
      const long long n = brick_elements(c->nx, c->ny, c->nz, c->brick_bs);
      CK(c, ensure(c->d_vbrick, c->vbrick_cap, (size_t)n * (c->dtype == CVR_U8 ? 1 : 2)));
      CK(c, launch_brick_volume(c->d_vol, c->d_vbrick, c->dtype, c->nx, c->ny, c->nz, c->brick_bs, c->stream));
      c->vbrick_bs = c->brick_bs;
    }
    const int B = 1 << c->brick_bs;
    const long long bx = (c->nx + B - 1) / B, by = (c->ny + B - 1) / B;
    v.voxels = c->d_vbrick;
    v.bs = c->brick_bs;
    v.stride[0] = (long long)B * B * B;
    v.stride[1] = bx * v.stride[0];
    v.stride[2] = by * v.stride[1];
  }
  if (allow_tex && (c->sampling & CVR_SAMPLING_TEX_VOLUME)) {
    cvr_status st = ensure_volume_texture(c);
    if (st != CVR_OK) return st;
    v.tex = c->tex.vol.tex;
  }
  *out = v;
  return CVR_OK;
}

cvr_status frame_args(cvr_ctx* c, const cvr_camera* cam, const void* params, float* out, int w, int h,
                      FrameArgs* fo, bool need_tf) {
  if (!c || !cam || !params || !out || w <= 0 || h <= 0 || w > 32768 || h > 32768)
    return fail(c, CVR_ERR_INVALID_ARG, "cvr_render: bad arguments");
  if (!c->has_volume) return fail(c, CVR_ERR_NO_VOLUME, "cvr_render: no volume loaded");
  if (need_tf && c->tf_n == 0) return fail(c, CVR_ERR_NOT_READY, "cvr_render: no transfer function");
  if (!finite3(cam->eye) || !finite3(cam->center) || !finite3(cam->up))
    return fail(c, CVR_ERR_INVALID_ARG, "cvr_render: non-finite camera");
  FrameArgs f;
  cvr_status vs = render_volume_view(c, &f.vol);
  if (vs != CVR_OK) return vs;
  f.cam = camera_view(cam, w, h);
  f.tf = c->d_rgbt;
  f.tf_n = c->tf_n;
  f.W = w; f.H = h;
  f.tile_w = c->tile_w; f.tile_h = c->tile_h;
  f.warp_w = warp_fits(c->tile_w, c->tile_h, c->warp_w) ? c->warp_w : 8;
  f.variant = c->variant;
  f.out = reinterpret_cast<float4*>(out);
  f.counts = nullptr;
  f.stats = c->d_stats;
  f.work = c->refill ? reinterpret_cast<unsigned*>(c->d_stats + 3) : nullptr;  // zeroed with the stats
  f.grad = GradView{};
  f.step = *static_cast<const float*>(params);  // every params struct starts with step_size
  if (c->tf_n * sizeof(float4) > 48 * 1024) return fail(c, CVR_ERR_UNSUPPORTED, "cvr_render: TF larger than 3072 entries");
  // Steps below 1e-6 of the diagonal would not advance a single-precision
  // ray parameter; they are rejected rather than marched.
  const float min_step = 1.0e-6f * std::sqrt(dot3(f.vol.grid, f.vol.grid));
  if (!(f.step >= min_step) || !std::isfinite(f.step))
    return fail(c, CVR_ERR_INVALID_ARG, "cvr_render: step_size must be finite and >= 1e-6 * diagonal");
  *fo = f;
  return CVR_OK;
}

cvr_status ext_args(cvr_ctx* c, const cvr_ext_params* p, const cvr_light* light, const FrameArgs& f, ExtArgs* eo,
                    const ShadowBoxTable** table, double* vmax_out) {
  if (!c->sat_ready) return fail(c, CVR_ERR_NOT_READY, "cvr_render: extinction SAT not built");
  if (p->apply_occlusion && (p->ao_n_shells < 1 || p->ao_n_shells > CVR_MAX_AO_SHELLS))
    return fail(c, CVR_ERR_INVALID_ARG, "ao_n_shells must be in [1, 32]");
  if (p->apply_shadow && !(p->sdw_sample_interval >= 1.0e-3f))
    return fail(c, CVR_ERR_INVALID_ARG, "sdw_sample_interval must be >= 1e-3 voxels");
  ExtArgs a{};
  a.sat.sx = c->nx + 2; a.sat.sy = c->ny + 2; a.sat.sz = c->nz + 2;
  a.sat.sxy = (unsigned)a.sat.sx * (unsigned)a.sat.sy;
  a.sat.inv_scale = (float)std::ldexp(1.0, -c->sat_frac_bits);
  a.sat.inv_spacing = f.vol.inv_spacing;
  a.sat.min_pos = f.vol.spacing * 0.5f;
  a.sat.max_pos = f.vol.grid + f.vol.spacing * 1.5f;
  a.apply_occ = p->apply_occlusion; a.apply_sdw = p->apply_shadow;
  a.n_shells = p->apply_occlusion ? p->ao_n_shells : 1;
  for (int i = 0; i < CVR_MAX_AO_SHELLS; ++i) a.radii[i] = p->ao_radii[i];
  a.cone_angle = p->sdw_cone_angle_rad; a.interval = p->sdw_sample_interval;
  a.initial = p->sdw_initial_step; a.ui_weight = p->sdw_ui_weight; a.max_dist = p->sdw_max_distance;
  a.shadow_type = p->shadow_type;
  a.light_pos = make3(light->position); a.light_fwd = make3(light->forward);
  a.ka = p->ka; a.kd = p->kd;
  a.ao_aligned = 1;
  for (int i = 0; i < a.n_shells; ++i) {
    const float w2 = 2.0f * p->ao_radii[i];
    if (!(w2 >= 0.0f && w2 <= 1023.0f && w2 == std::nearbyint(w2))) a.ao_aligned = 0;
  }
  *table = nullptr;
  if (p->apply_shadow && p->shadow_type == 1) {
    if (!c->sdw_table) c->sdw_table.reset(new ShadowBoxTable());
    if (build_shadow_table(p, light->forward, f.vol.spacing, f.vol.grid, c->sdw_table.get()))
      *table = c->sdw_table.get();
  }
  // The compact table serves the frame when the largest region any of its
  // box queries spans is known (AO boxes; shadow boxes of a per-frame table)
  if (vmax_out) *vmax_out = 0.0;
  // Without a per-frame table (point lights, or more boxes than it holds) the
  // cone direction varies per sample; its dominant component is at least
  // 1/sqrt(3), so the cone axis leans at most atan(sqrt(2)) off the walk axis
  // and a box's lateral extent at depth zm is at most
  // zm (tan(lean + angle) - tan(lean - angle)) plus one voxel of rounding, with
  // zm below max_dist + interval.  Unbounded when lean + angle reaches 90 deg.
  double cone_extent = -1.0;  // world units, < 0: unknown
  if (p->apply_shadow && !*table) {
    const double lean = std::atan(std::sqrt(2.0)), ang = std::fabs((double)p->sdw_cone_angle_rad);
    const double msc = std::max((double)f.vol.spacing.x, std::max((double)f.vol.spacing.y, (double)f.vol.spacing.z));
    const double iw = (double)p->sdw_sample_interval * msc;
    if (lean + ang < 1.5 && std::isfinite((double)p->sdw_max_distance) && p->sdw_max_distance >= 0.0f) {
      const double zm = (double)p->sdw_max_distance + iw;
      cone_extent = std::max(zm * (std::tan(lean + ang) - std::tan(lean - ang)) + msc, iw);
    }
  }
  if (c->compact_sat && (p->apply_occlusion || p->apply_shadow) && (!p->apply_shadow || *table || cone_extent >= 0.0)) {
    const float3 sc = f.vol.spacing;
    const double sv[3] = {sc.x, sc.y, sc.z};
    const int n[3] = {c->nx, c->ny, c->nz};
    // cells a query on a world extent w may span: its taps reach floor(lo) .. floor(hi) + 1,
    // one more for single-precision positions, at most the SAT's n + 1 cells
    auto cells = [&](double w, int ax) { return std::min(std::ceil(w / sv[ax]) + 3.0, (double)n[ax] + 1.0); };
    double vmax = 0.0;
    if (p->apply_occlusion) {
      float rmax = 0.0f;
      for (int i = 0; i < p->ao_n_shells; ++i) rmax = std::max(rmax, p->ao_radii[i]);
      double v = 1.0;
      for (int ax = 0; ax < 3; ++ax) v *= cells(2.0 * rmax * sv[ax], ax);
      vmax = std::max(vmax, v);
    }
    if (p->apply_shadow && !*table) {
      // lateral extent on two axes, one interval along the walk's (any) axis
      const double iw = (double)p->sdw_sample_interval;
      for (int walk = 0; walk < 3; ++walk) {
        double v = 1.0;
        for (int ax = 0; ax < 3; ++ax) v *= ax == walk ? cells(iw * sv[ax], ax) : cells(cone_extent, ax);
        vmax = std::max(vmax, v);
      }
    } else if (p->apply_shadow) {
      const ShadowBoxTable& t = **table;
      for (int k = 0; k < t.n; ++k) {
        const double v = cells((double)t.hi[k].x - t.lo[k].x, 0) * cells((double)t.hi[k].y - t.lo[k].y, 1) *
                         cells((double)t.hi[k].z - t.lo[k].z, 2);
        vmax = std::max(vmax, v);
      }
    }
    if (vmax_out) {
      *vmax_out = vmax;  // the caller builds the table (batches own theirs)
    } else {
      float inv_scale32 = 0.0f;
      cvr_status cs = ensure_compact_sat(c, vmax, &inv_scale32);
      if (cs != CVR_OK) return cs;
      if (inv_scale32 > 0.0f) {
        a.sat.sat32 = c->d_sat32;
        a.sat.inv_scale32 = inv_scale32;
        // every box of an aligned directional table has the walk depth of the
        // sample interval: its queries read the walk table
        if (*table && (*table)->aligned && c->walk_tables) {
          cs = ensure_walk_table(c, (*table)->axis, (int)std::nearbyint(p->sdw_sample_interval), &a.walk);
          if (cs != CVR_OK) return cs;
        }
      }
    }
  }
  // the int64 table serves frames without a compact table; the caller of
  // vmax_out may fall back to it.  Its pointer is taken after the build,
  // which allocates it the first time.
  if (vmax_out || !a.sat.sat32) {
    cvr_status cs = ensure_sat(c);
    if (cs != CVR_OK) return cs;
  }
  a.sat.sat = c->d_sat;
  *eo = a;
  return CVR_OK;
}

// The walk table of the current compact table for walk axis / depth w
// (rebuilt when the compact table, the axis or the depth changes); without
// room for it the frame's queries read the quads.
cvr_status ensure_walk_table(cvr_ctx* c, int axis, int w, WalkView* out) {
  *out = WalkView{nullptr, axis, w};
  if (w < 1 || w > 1023 || !c->d_sat32) return CVR_OK;
  if (!(c->d_walk && c->walk_gen == c->sat32_gen && c->walk_axis == axis && c->walk_w == w)) {
    const int sx = c->nx + 2, sy = c->ny + 2, sz = c->nz + 2;
    const size_t cells = (size_t)sx * sy * sz;
    c->walk_gen = 0;
    cudaError_t e = ensure(c->d_walk, c->walk_cap, cells * 2 * sizeof(uint4));
    if (e == cudaErrorMemoryAllocation) {
      cudaGetLastError();
      return CVR_OK;
    }
    if (e != cudaSuccess) return cuda_fail(c, e, "walk table");
    CK(c, launch_sat_walk(c->d_sat32, c->d_walk, sx, sy, sz, axis, w, c->stream));
    c->walk_gen = c->sat32_gen;
    c->walk_axis = axis;
    c->walk_w = w;
  }
  out->oct = c->d_walk;
  return CVR_OK;
}

// The fixed point of a compact SAT for queries spanning at most vmax cells:
// round(sigma * 2^F32) with F32 the largest that keeps vmax * max q below
// 2^31, so every sub-box sum, and so every wrapped 32-bit difference of the
// table, is exact.  False when that would resolve the largest extinction in
// fewer than 2^15 steps (the FP32 table of the reference resolves far less).
bool compact_plan(const std::vector<double>& ext, double vmax, int* F_out, std::vector<unsigned>* q) {
  if (ext.empty() || !(vmax >= 1.0)) return false;
  double maxv = 0.0;
  for (double v : ext) maxv = std::max(maxv, v);
  const double limit = 2147483647.0;
  int F = maxv > 0.0 ? (int)std::floor(std::log2(limit / (vmax * maxv))) : 0;
  F = std::min(F, 52);
  q->resize(ext.size());
  for (;; --F) {
    const double scale = std::ldexp(1.0, F);
    double qmax = 0.0;
    for (size_t i = 0; i < q->size(); ++i) {
      const double r = std::rint(ext[i] * scale);  // nearbyint's value without its FP-environment save
      qmax = std::max(qmax, r);
      (*q)[i] = (unsigned)r;
    }
    if (qmax * vmax < limit || F < -64) {
      if (maxv > 0.0 && qmax < 32768.0) return false;
      break;
    }
  }
  *F_out = F;
  return true;
}

// Builds the compact table of the current volume from q into dst, in x-y
// quad layout, asynchronously on the context stream: the plane prefixes go
// to the context's persistent scratch (grown only when a larger volume needs
// it), and q goes through the pinned staging region 1 (q may go when the
// call returns).
cvr_status build_compact_sat(cvr_ctx* c, const std::vector<unsigned>& q, uint4* dst) {
  const size_t cells = (size_t)(c->nx + 2) * (c->ny + 2) * (c->nz + 2);
  CK(c, ensure(c->d_lut32, c->lut32_cap, sizeof(unsigned) * q.size()));
  void* stage = nullptr;
  cvr_status st = stage_region(c, 1, &stage);
  if (st != CVR_OK) return st;
  std::memcpy(stage, q.data(), sizeof(unsigned) * q.size());
  st = stage_upload(c, 1, c->d_lut32, sizeof(unsigned) * q.size());
  if (st != CVR_OK) return st;
  CK(c, ensure(c->d_satp, c->satp_cap, sizeof(unsigned) * cells));
  cudaError_t e = launch_sat_build_quads(c->d_vol, c->dtype, c->nx, c->ny, c->nz, c->d_lut32, c->d_satp, dst,
                                         c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "compact SAT build");
  return CVR_OK;
}

// The context's compact SAT for a frame whose queries span at most vmax
// cells, rebuilt when its fixed point changes; *inv_scale = 2^-F32, or 0 when
// the frame keeps the int64 table.
cvr_status ensure_compact_sat(cvr_ctx* c, double vmax, float* inv_scale) {
  *inv_scale = 0.0f;
  // the table planned for this extent is current (cvr_build_sat and a new
  // volume reset sat32_F): no per-frame pass over the extinction table
  if (c->d_sat32 && c->sat32_F != kNoCompactSat && c->sat32_vmax == vmax) {
    *inv_scale = (float)std::ldexp(1.0, -c->sat32_F);
    return CVR_OK;
  }
  int F;
  std::vector<unsigned> q;
  if (!compact_plan(c->sat_ext, vmax, &F, &q)) return CVR_OK;
  if (c->sat32_F != F || !c->d_sat32) {
    const size_t cells = (size_t)(c->nx + 2) * (c->ny + 2) * (c->nz + 2);
    if (cells >= kCompactMaxCells) return CVR_OK;  // 32-bit cell indices: the int64 table
    c->sat32_F = kNoCompactSat;
    // the quad table is twice the int64 one: without room for it the frame
    // keeps the int64 table
    cudaError_t e = ensure(c->d_sat32, c->sat32_cap, cells * sizeof(uint4));
    if (e == cudaErrorMemoryAllocation) {
      cudaGetLastError();
      return CVR_OK;
    }
    if (e != cudaSuccess) return cuda_fail(c, e, "compact SAT");
    cvr_status st = build_compact_sat(c, q, c->d_sat32);
    if (st == CVR_ERR_OUT_OF_MEMORY) return CVR_OK;
    if (st != CVR_OK) return st;
    c->sat32_F = F;
    static std::atomic<unsigned long long> builds{0};  // distinct id of every compact build
    c->sat32_gen = ++builds;
  }
  c->sat32_vmax = vmax;
  *inv_scale = (float)std::ldexp(1.0, -F);
  return CVR_OK;
}

cvr_status pyramid_view(cvr_ctx* c, PyramidView* out) {
  PyramidView P = c->pyr;
  P.data = c->d_pyr;
  P.quads = nullptr;
  if (!c->quads) {  // the plain layout
    *out = P;
    return CVR_OK;
  }
  if (!c->pyrq_ready) {
    const int L = c->pyr.n_levels - 1;
    const size_t n = (size_t)c->pyr.offset[L] + (size_t)c->pyr.dims[L][0] * c->pyr.dims[L][1] * c->pyr.dims[L][2];
    // without room for the copy the taps read the plain levels
    cudaError_t e = ensure(c->d_pyrq, c->pyrq_cap, n * sizeof(float4));
    if (e == cudaErrorMemoryAllocation) {
      cudaGetLastError();
      *out = P;
      return CVR_OK;
    }
    if (e != cudaSuccess) return cuda_fail(c, e, "pyramid quads");
    CK(c, launch_pyramid_quads(P, c->d_pyr, c->d_pyrq, c->stream));
    c->pyrq_ready = true;
  }
  P.quads = c->d_pyrq;
  *out = P;
  return CVR_OK;
}

cvr_status check_kernel_flag(cvr_ctx* c, const char* what) {
  int e = 0;
  CK(c, cudaMemcpyAsync(&e, c->d_kerr, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  CK(c, cudaStreamSynchronize(c->stream));
  if (e == 0) return CVR_OK;
  CK(c, cudaMemsetAsync(c->d_kerr, 0, sizeof(int), c->stream));
  return fail(c, CVR_ERR_TIMEOUT, what);
}

cvr_status stage_region(cvr_ctx* c, int r, void** out) {
  constexpr size_t kRegion = sizeof(long long) * 65536;
  if (!c->h_stage) {
    CK(c, cudaHostAlloc(&c->h_stage, 2 * kRegion, cudaHostAllocDefault));
    for (cudaEvent_t& e : c->stage_ev) CK(c, cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  }
  CK(c, cudaEventSynchronize(c->stage_ev[r]));  // an event never recorded is complete
  *out = static_cast<char*>(c->h_stage) + (size_t)r * kRegion;
  return CVR_OK;
}

cvr_status stage_upload(cvr_ctx* c, int r, void* dev, size_t n) {
  constexpr size_t kRegion = sizeof(long long) * 65536;
  CK(c, cudaMemcpyAsync(dev, static_cast<char*>(c->h_stage) + (size_t)r * kRegion, n, cudaMemcpyHostToDevice,
                        c->stream));
  CK(c, cudaEventRecord(c->stage_ev[r], c->stream));
  return CVR_OK;
}

cvr_status ensure_sat(cvr_ctx* c) {
  if (!c->sat_ready || !c->sat_pending) return CVR_OK;
  CK(c, cudaSetDevice(c->device));
  size_t cells = (size_t)(c->nx + 2) * (c->ny + 2) * (c->nz + 2);
  CK(c, ensure(c->d_sat, c->sat_cap, cells * sizeof(long long)));
  CK(c, launch_sat_build(c->d_vol, c->dtype, c->nx, c->ny, c->nz, c->d_lut, c->d_sat, c->stream));
  c->sat_pending = false;
  return CVR_OK;
}

}  // namespace ctxutil
}  // namespace cvr

extern "C" {

int cvr_abi_version(void) { return CVR_ABI_VERSION; }

const char* cvr_last_error(const cvr_ctx* ctx) { return ctx ? ctx->err.c_str() : g_create_err.c_str(); }

cvr_status cvr_create(cvr_ctx** out, int device) {
  if (!out) return CVR_ERR_INVALID_ARG;
  *out = nullptr;
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess || n == 0) {
    cudaGetLastError();
    g_create_err = std::string("no CUDA device: ") + cudaGetErrorString(e);
    return CVR_ERR_CUDA;
  }
  if (device < 0 || device >= n) {
    g_create_err = "device index out of range";
    return CVR_ERR_INVALID_ARG;
  }
  cvr_ctx* c = new cvr_ctx();
  c->device = device;
  auto bail = [&](cudaError_t err, const char* what) {
    g_create_err = std::string(what) + ": " + cudaGetErrorString(err);
    cvr_destroy(c);
    return err == cudaErrorMemoryAllocation ? CVR_ERR_OUT_OF_MEMORY : CVR_ERR_CUDA;
  };
  if ((e = cudaSetDevice(device)) != cudaSuccess) return bail(e, "cudaSetDevice");
  if ((e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking)) != cudaSuccess)
    return bail(e, "cudaStreamCreate");
  for (int i = 0; i < 4; ++i)
    if ((e = cudaEventCreate(&c->ev[i])) != cudaSuccess) return bail(e, "cudaEventCreate");
  if ((e = cudaMalloc((void**)&c->d_stats, 4 * sizeof(unsigned long long))) != cudaSuccess)
    return bail(e, "cudaMalloc(stats)");
  if ((e = cudaMalloc((void**)&c->d_kerr, sizeof(int))) != cudaSuccess) return bail(e, "cudaMalloc(kernel flag)");
  if ((e = cudaMemset(c->d_kerr, 0, sizeof(int))) != cudaSuccess) return bail(e, "cudaMemset(kernel flag)");
  *out = c;
  return CVR_OK;
}

void cvr_destroy(cvr_ctx* c) {
  if (!c) return;
  cudaSetDevice(c->device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  void* bufs[] = {c->d_vol, c->d_rgbt, c->d_rgba, c->d_sat, c->d_lut, c->d_pyr, c->d_occ_sec, c->d_sdw_sec,
                  c->d_occ_vec, c->d_sdw_vec, c->d_stats, c->d_out, c->d_flush, c->d_probe, c->d_vbrick, c->d_lcache, c->d_grad, c->d_ms, c->d_msf,
                  c->d_sat32, c->d_lut32, c->d_kerr, c->d_pyrq, c->d_satp, c->d_walk, c->d_pyrs};
  for (void* p : bufs)
    if (p) cudaFree(p);
  for (int i = 0; i < 4; ++i)
    if (c->ev[i]) cudaEventDestroy(c->ev[i]);
  for (cudaEvent_t e : c->stage_ev)
    if (e) cudaEventDestroy(e);
  if (c->h_stage) cudaFreeHost(c->h_stage);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
}

cvr_status cvr_sync(cvr_ctx* c) {
  if (!c) return CVR_ERR_INVALID_ARG;
  CK(c, cudaStreamSynchronize(c->stream));
  return mlp_check_err(c);  // a surrogate frame whose tensor-core wait gave up
}

void* cvr_stream(cvr_ctx* c) { return c ? (void*)c->stream : nullptr; }

static cvr_status set_volume_common(cvr_ctx* c, const void* src, bool src_device, int w, int h, int d, int dtype,
                                    float sx, float sy, float sz) {
  if (!c || !src || w <= 0 || h <= 0 || d <= 0 || (dtype != CVR_U8 && dtype != CVR_U16))
    return fail(c, CVR_ERR_INVALID_ARG, "cvr_set_volume: bad arguments");
  if (!(sx > 0.0f && sy > 0.0f && sz > 0.0f) || !std::isfinite(sx) || !std::isfinite(sy) || !std::isfinite(sz))
    return fail(c, CVR_ERR_INVALID_ARG, "cvr_set_volume: spacing must be positive");
  if ((long long)w * h * d > (1ll << 34)) return fail(c, CVR_ERR_INVALID_ARG, "cvr_set_volume: volume too large");
  CK(c, cudaSetDevice(c->device));
  size_t bytes = (size_t)w * h * d * (dtype == CVR_U8 ? 1 : 2);
  CK(c, ensure(c->d_vol, c->vol_cap, bytes));
  CK(c, cudaMemcpyAsync(c->d_vol, src, bytes, src_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                        c->stream));
  c->nx = w; c->ny = h; c->nz = d; c->dtype = dtype;
  c->sx = sx; c->sy = sy; c->sz = sz;
  c->has_volume = true;
  // Derived tables belong to the previous volume.
  c->sat_ready = false;
  c->sat_pending = false;
  c->sat32_F = kNoCompactSat;
  c->pyr_ready = false;
  c->tex.vol_valid = false;
  c->tex.pyr_valid = false;
  c->vbrick_bs = -1;
  c->grad_ready = false;  // rebuilt with the slot's gradient model on the next shaded frame
  c->tex.grad_valid = false;
  return CVR_OK;
}

cvr_status cvr_set_volume(cvr_ctx* c, const void* host, int w, int h, int d, int dtype, float sx, float sy,
                          float sz) {
  return set_volume_common(c, host, false, w, h, d, dtype, sx, sy, sz);
}

cvr_status cvr_set_volume_device(cvr_ctx* c, const void* dev, int w, int h, int d, int dtype, float sx, float sy,
                                 float sz) {
  return set_volume_common(c, dev, true, w, h, d, dtype, sx, sy, sz);
}

cvr_status cvr_set_transfer_function(cvr_ctx* c, const float* rgbt, const float* rgba, int n) {
  if (!c || !rgbt || n < 2 || n > 65536) return fail(c, CVR_ERR_INVALID_ARG, "cvr_set_transfer_function: bad arguments");
  CK(c, cudaSetDevice(c->device));
  std::vector<float> op;
  if (!rgba) {
    op.assign(rgbt, rgbt + 4 * (size_t)n);
    for (int i = 0; i < n; ++i) op[4 * i + 3] = (float)(1.0 - std::exp(-(double)rgbt[4 * i + 3]));
    rgba = op.data();
  }
  if (n > c->tf_cap) {
    if (c->d_rgbt) cudaFree(c->d_rgbt);
    if (c->d_rgba) cudaFree(c->d_rgba);
    c->d_rgbt = c->d_rgba = nullptr;
    c->tf_cap = 0;
    CK(c, cudaMalloc((void**)&c->d_rgbt, sizeof(float4) * n));
    CK(c, cudaMalloc((void**)&c->d_rgba, sizeof(float4) * n));
    c->tf_cap = n;
  }
  CK(c, cudaMemcpyAsync(c->d_rgbt, rgbt, sizeof(float4) * n, cudaMemcpyHostToDevice, c->stream));
  CK(c, cudaMemcpyAsync(c->d_rgba, rgba, sizeof(float4) * n, cudaMemcpyHostToDevice, c->stream));
  // Host sources may be pageable temporaries: finish before returning.
  CK(c, cudaStreamSynchronize(c->stream));
  c->tf_n = n;
  c->pyr_ready = false;
  c->tex.pyr_valid = false;
  return CVR_OK;
}

cvr_status cvr_build_sat(cvr_ctx* c, const double* ext, int n_values) {
  if (!c || !ext) return fail(c, CVR_ERR_INVALID_ARG, "cvr_build_sat: bad arguments");
  if (!c->has_volume) return fail(c, CVR_ERR_NO_VOLUME, "cvr_build_sat: no volume");
  int need = c->dtype == CVR_U8 ? 256 : 65536;
  if (n_values != need) return fail(c, CVR_ERR_INVALID_ARG, "cvr_build_sat: n_values must be 256 (u8) or 65536 (u16)");
  double maxv = 0.0;
  for (int i = 0; i < n_values; ++i) {
    if (!(ext[i] >= 0.0) || !std::isfinite(ext[i]))
      return fail(c, CVR_ERR_INVALID_ARG, "cvr_build_sat: extinction values must be finite and >= 0");
    maxv = std::max(maxv, ext[i]);
  }
  // Fixed point: the largest possible entry (all voxels at the largest
  // extinction) must stay below 2^62.
  double nvox = (double)c->nx * c->ny * c->nz;
  int F = 52;
  if (maxv > 0.0) F = (int)std::floor(62.0 - std::log2(nvox * maxv));
  F = std::min(52, std::max(0, F));
  CK(c, cudaSetDevice(c->device));
  void* stage = nullptr;
  cvr_status st = stage_region(c, 0, &stage);
  if (st != CVR_OK) return st;
  long long* q = static_cast<long long*>(stage);
  double scale = std::ldexp(1.0, F);
  // llround of a non-negative value: below 2^52, v + 0.5 is exact and its
  // truncation rounds halves up; from 2^52 on, v is an integer already
  for (int i = 0; i < n_values; ++i) {
    const double v = ext[i] * scale;
    q[i] = v < 4503599627370496.0 ? (long long)(v + 0.5) : (long long)v;
  }
  // the table of every possible voxel value (65536 entries covers u8 and u16)
  if (!c->d_lut) CK(c, cudaMalloc((void**)&c->d_lut, sizeof(long long) * 65536));
  st = stage_upload(c, 0, c->d_lut, sizeof(long long) * n_values);
  if (st != CVR_OK) return st;
  c->sat_frac_bits = F;
  c->sat_ready = true;
  c->sat_pending = true;
  c->sat_ext.assign(ext, ext + n_values);
  c->sat32_F = kNoCompactSat;
  return CVR_OK;
}

cvr_status cvr_prepare_sat(cvr_ctx* c) {
  if (!c) return CVR_ERR_INVALID_ARG;
  return ensure_sat(c);
}

cvr_status cvr_get_sat_info(cvr_ctx* c, int dims[3], int* frac_bits) {
  if (!c) return CVR_ERR_INVALID_ARG;
  if (!c->sat_ready) return fail(c, CVR_ERR_NOT_READY, "SAT not built");
  if (dims) { dims[0] = c->nx + 2; dims[1] = c->ny + 2; dims[2] = c->nz + 2; }
  if (frac_bits) *frac_bits = c->sat_frac_bits;
  return CVR_OK;
}

cvr_status cvr_download_sat(cvr_ctx* c, int64_t* host) {
  if (!c || !host) return CVR_ERR_INVALID_ARG;
  if (!c->sat_ready) return fail(c, CVR_ERR_NOT_READY, "SAT not built");
  cvr_status st = ensure_sat(c);
  if (st != CVR_OK) return st;
  size_t cells = (size_t)(c->nx + 2) * (c->ny + 2) * (c->nz + 2);
  CK(c, cudaMemcpyAsync(host, c->d_sat, cells * sizeof(long long), cudaMemcpyDeviceToHost, c->stream));
  CK(c, cudaStreamSynchronize(c->stream));
  return CVR_OK;
}

cvr_status cvr_build_ext_pyramid(cvr_ctx* c, const cvr_pyramid_params* p) {
  if (!c || !p) return fail(c, CVR_ERR_INVALID_ARG, "cvr_build_ext_pyramid: bad arguments");
  if (!c->has_volume) return fail(c, CVR_ERR_NO_VOLUME, "cvr_build_ext_pyramid: no volume");
  if (c->tf_n == 0) return fail(c, CVR_ERR_NOT_READY, "cvr_build_ext_pyramid: no transfer function");
  if (p->base_dims[0] <= 0 || p->base_dims[1] <= 0 || p->base_dims[2] <= 0 || p->base_dims[0] > 4096 ||
      p->base_dims[1] > 4096 || p->base_dims[2] > 4096 || !(p->sigma0 > 0.0f) || p->n_levels < 0)
    return fail(c, CVR_ERR_INVALID_ARG, "cvr_build_ext_pyramid: bad parameters");
  // GL mip chain: level i has max(1, dim >> i) per axis; the chain ends after
  // the level where every axis is 1 (extcoefvolumegenerator.cpp:321-331).
  int maxdim = std::max(p->base_dims[0], std::max(p->base_dims[1], p->base_dims[2]));
  int chain = 1;
  while ((maxdim >> chain) > 0) ++chain;
  int levels = p->n_levels > 0 ? std::min(p->n_levels, chain) : chain;
  levels = std::min(levels, CVR_MAX_LEVELS);
  PyramidView P{};
  long long off = 0;
  for (int l = 0; l < levels; ++l) {
    for (int a = 0; a < 3; ++a) P.dims[l][a] = std::max(1, p->base_dims[a] >> l);
    P.offset[l] = off;
    off += (long long)P.dims[l][0] * P.dims[l][1] * P.dims[l][2];
  }
  if (off >= (1LL << 31))
    return fail(c, CVR_ERR_INVALID_ARG, "cvr_build_ext_pyramid: pyramids hold fewer than 2^31 values");
  P.n_levels = levels;
  CK(c, cudaSetDevice(c->device));
  // the base level's volume taps read the marchers' FP32 layout (bricks or
  // quads; never the texture unit)
  VolumeView v;
  cvr_status vs = render_volume_view(c, &v, false);
  if (vs != CVR_OK) return vs;
  P.grid = v.grid;
  P.inv_grid = f3(1.0f / v.grid.x, 1.0f / v.grid.y, 1.0f / v.grid.z);
  CK(c, ensure(c->d_pyr, c->pyr_cap, (size_t)off * sizeof(float)));
  // scratch of the separable levels (lattice samples and two pass results);
  // without room for it every level takes the direct kernels
  const long long sf = pyramid_scratch_floats(v, P, p->sigma0);
  float* scratch = nullptr;
  if (sf > 0) {
    cudaError_t e = ensure(c->d_pyrs, c->pyrs_cap, (size_t)sf * sizeof(float));
    if (e == cudaErrorMemoryAllocation) cudaGetLastError();
    else if (e != cudaSuccess) return cuda_fail(c, e, "pyramid scratch");
    else scratch = c->d_pyrs;
  }
  CK(c, launch_pyramid_build(v, c->d_rgba, c->tf_n, p->sigma0, P, c->d_pyr, scratch, scratch ? sf : 0, c->stream));
  c->pyr = P;
  c->pyr_ready = true;
  c->pyrq_ready = false;
  c->tex.pyr_valid = false;
  return CVR_OK;
}

cvr_status cvr_get_pyramid_info(cvr_ctx* c, int* n_levels, int (*dims)[3], int max_levels) {
  if (!c) return CVR_ERR_INVALID_ARG;
  if (!c->pyr_ready) return fail(c, CVR_ERR_NOT_READY, "pyramid not built");
  if (n_levels) *n_levels = c->pyr.n_levels;
  if (dims)
    for (int l = 0; l < c->pyr.n_levels && l < max_levels; ++l)
      for (int a = 0; a < 3; ++a) dims[l][a] = c->pyr.dims[l][a];
  return CVR_OK;
}

cvr_status cvr_download_pyramid_level(cvr_ctx* c, int level, float* host) {
  if (!c || !host) return CVR_ERR_INVALID_ARG;
  if (!c->pyr_ready) return fail(c, CVR_ERR_NOT_READY, "pyramid not built");
  if (level < 0 || level >= c->pyr.n_levels) return fail(c, CVR_ERR_INVALID_ARG, "level out of range");
  size_t n = (size_t)c->pyr.dims[level][0] * c->pyr.dims[level][1] * c->pyr.dims[level][2];
  CK(c, cudaMemcpyAsync(host, c->d_pyr + c->pyr.offset[level], n * sizeof(float), cudaMemcpyDeviceToHost, c->stream));
  CK(c, cudaStreamSynchronize(c->stream));
  return CVR_OK;
}

static cvr_status upload_cone(cvr_ctx* c, const cvr_cone_table* t, float4** d, ConeTableDev* out) {
  if (t->n_sections < 0 || t->n_sections > CVR_MAX_CONE_SECTIONS)
    return fail(c, CVR_ERR_INVALID_ARG, "cone table: bad section count");
  int n1 = t->integration_samples[0], n3 = t->integration_samples[1], n7 = t->integration_samples[2];
  if (n1 < 0 || n3 < 0 || n7 < 0 || n1 + n3 + n7 > t->n_sections)
    return fail(c, CVR_ERR_INVALID_ARG, "cone table: integration counts exceed the section count");
  if (*d) { cudaFree(*d); *d = nullptr; }
  size_t bytes = sizeof(float4) * std::max(1, t->n_sections);
  CK(c, cudaMalloc((void**)d, bytes));
  if (t->n_sections) CK(c, cudaMemcpy(*d, t->sections, sizeof(float4) * t->n_sections, cudaMemcpyHostToDevice));
  out->n_sections = t->n_sections;
  out->n1 = n1; out->n3 = n3; out->n7 = n7;
  for (int i = 0; i < 10; ++i) out->axes[i] = make3(t->axes[i]);
  out->initial_step = t->initial_step;
  out->w7 = t->ray7_adj_weight;
  out->ui_weight = t->ui_weight;
  return CVR_OK;
}

cvr_status cvr_set_cone_tables(cvr_ctx* c, const cvr_cone_table* occ, const cvr_cone_table* sdw) {
  if (!c || !occ || !sdw) return fail(c, CVR_ERR_INVALID_ARG, "cvr_set_cone_tables: bad arguments");
  CK(c, cudaSetDevice(c->device));
  cvr_status s = upload_cone(c, occ, &c->d_occ_sec, &c->occ);
  if (s != CVR_OK) return s;
  s = upload_cone(c, sdw, &c->d_sdw_sec, &c->sdw);
  if (s != CVR_OK) return s;
  c->cone_ready = true;
  return CVR_OK;
}

cvr_status cvr_set_gt_kernels(cvr_ctx* c, const float* occ, int n_occ, const float* sdw, int n_sdw) {
  if (!c || n_occ < 0 || n_sdw < 0 || n_occ > CVR_MAX_GT_RAYS || n_sdw > CVR_MAX_GT_RAYS || (n_occ && !occ) ||
      (n_sdw && !sdw))
    return fail(c, CVR_ERR_INVALID_ARG, "cvr_set_gt_kernels: bad arguments (at most 256 rays per cone)");
  CK(c, cudaSetDevice(c->device));
  if (c->d_occ_vec) { cudaFree(c->d_occ_vec); c->d_occ_vec = nullptr; }
  if (c->d_sdw_vec) { cudaFree(c->d_sdw_vec); c->d_sdw_vec = nullptr; }
  CK(c, cudaMalloc((void**)&c->d_occ_vec, sizeof(float3) * std::max(1, n_occ)));
  CK(c, cudaMalloc((void**)&c->d_sdw_vec, sizeof(float3) * std::max(1, n_sdw)));
  if (n_occ) CK(c, cudaMemcpy(c->d_occ_vec, occ, sizeof(float3) * n_occ, cudaMemcpyHostToDevice));
  if (n_sdw) CK(c, cudaMemcpy(c->d_sdw_vec, sdw, sizeof(float3) * n_sdw, cudaMemcpyHostToDevice));
  c->n_occ = n_occ;
  c->n_sdw = n_sdw;
  c->gt_ready = true;
  return CVR_OK;
}


static cvr_status render_frame(cvr_ctx* c, int method, const cvr_camera* cam, const cvr_light* light,
                               const void* params, size_t params_size, float* out, int w, int h, uint32_t* counts,
                               cvr_frame_stats* stats);

// A frame of the context's multiscaling mode: the marcher renders the
// generated frame into the context's buffer, the post-pass writes out.
static cvr_status render_impl(cvr_ctx* c, int method, const cvr_camera* cam, const cvr_light* light,
                              const void* params, size_t params_size, float* out, int w, int h, uint32_t* counts,
                              cvr_frame_stats* stats) {
  if (!c || c->ms_mode == CVR_MULTISCALE_SINGLE)
    return render_frame(c, method, cam, light, params, params_size, out, w, h, counts, stats);
  if (counts) return fail(c, CVR_ERR_UNSUPPORTED, "cvr_render: per-pixel step counts with multiscaling");
  if (!out || w <= 0 || h <= 0) return fail(c, CVR_ERR_INVALID_ARG, "cvr_render: bad arguments");
  int gw, gh;
  multiscale_size(c->ms_mode, c->ms_fw, c->ms_fh, w, h, &gw, &gh);
  if (gw < 1 || gh < 1 || gw > 32768 || gh > 32768)
    return fail(c, CVR_ERR_INVALID_ARG, "cvr_render: multiscaled frame size out of range");
  CK(c, cudaSetDevice(c->device));
  CK(c, ensure(c->d_ms, c->ms_cap, (size_t)gw * gh * sizeof(float4)));
  if (const size_t sb = multiscale_scratch(c->ms_mode, c->ms_kernel, gw, gh, w, h))
    CK(c, ensure(c->d_msf, c->msf_cap, sb));
  // the camera keeps the output's aspect (u_CameraAspectRatio is the screen's)
  cvr_camera cm = cam ? *cam : cvr_camera{};
  if (cam && !(cm.aspect > 0.0f)) cm.aspect = (float)w / (float)h;
  cvr_status s = render_frame(c, method, cam ? &cm : nullptr, light, params, params_size,
                              reinterpret_cast<float*>(c->d_ms), gw, gh, nullptr, stats);
  if (s != CVR_OK) return s;
  CK(c, launch_multiscale(c->ms_mode, c->ms_kernel, c->d_ms, gw, gh, reinterpret_cast<float4*>(out), w, h,
                          c->d_msf, c->stream));
  return CVR_OK;
}

static cvr_status render_frame(cvr_ctx* c, int method, const cvr_camera* cam, const cvr_light* light,
                               const void* params, size_t params_size, float* out, int w, int h, uint32_t* counts,
                               cvr_frame_stats* stats) {
  if (!c) return CVR_ERR_INVALID_ARG;
  CK(c, cudaSetDevice(c->device));
  FrameArgs f;
  cvr_status fs = frame_args(c, cam, params, out, w, h, &f, method != CVR_METHOD_ISO);
  if (fs != CVR_OK) return fs;
  f.counts = counts;
  fs = grad_args(c, method, light, &f);
  if (fs != CVR_OK) return fs;
  // the three counters and the ray counter of the persistent marchers
  CK(c, cudaMemsetAsync(c->d_stats, 0, 4 * sizeof(unsigned long long), c->stream));
  cvr_light dl{};
  if (!light) { light = &dl; }
  cudaError_t e = cudaSuccess;
  if (stats) CK(c, cudaEventRecord(c->ev[2], c->stream));
  switch (method) {
    case CVR_METHOD_PLAIN: {
      if (params_size != sizeof(cvr_plain_params)) return fail(c, CVR_ERR_INVALID_ARG, "plain params size");
      const cvr_plain_params* p = static_cast<const cvr_plain_params*>(params);
      if (!(p->step_size > 0.0f)) return fail(c, CVR_ERR_INVALID_ARG, "step_size must be > 0");
      f.step = p->step_size;
      e = (c->staging && plain_staging_applies(f)) ? launch_plain_staged(f, c->stream) : launch_plain(f, c->stream);
      break;
    }
    case CVR_METHOD_EXTINCTION: {
      if (params_size != sizeof(cvr_ext_params)) return fail(c, CVR_ERR_INVALID_ARG, "extinction params size");
      const cvr_ext_params* p = static_cast<const cvr_ext_params*>(params);
      if (!(p->step_size > 0.0f)) return fail(c, CVR_ERR_INVALID_ARG, "step_size must be > 0");
      ExtArgs a{};
      const ShadowBoxTable* table = nullptr;
      double no_compact = 0.0;  // the light cache reads the int64 table: no compact one to build
      cvr_status es = ext_args(c, p, light, f, &a, &table, c->lc_dims[0] > 0 ? &no_compact : nullptr);
      if (es != CVR_OK) return es;
      if (c->lc_dims[0] > 0) {  // object-space light cache, then the object-space marcher
        if (!c->sdw_table) c->sdw_table.reset(new ShadowBoxTable());
        const size_t cells = (size_t)c->lc_dims[0] * c->lc_dims[1] * c->lc_dims[2];
        CK(c, ensure(c->d_lcache, c->lcache_cap, cells * sizeof(float2)));
        e = launch_cache_extinction(f, a, table, *c->sdw_table, c->lc_dims, c->d_lcache, c->stream);
        if (e == cudaSuccess)
          e = launch_march_cached(f, c->d_lcache, c->lc_dims, p->apply_occlusion, p->apply_shadow, p->ka, p->kd,
                                  c->stream);
      } else {
        if (!c->sdw_table) c->sdw_table.reset(new ShadowBoxTable());
        e = launch_extinction(f, a, table, *c->sdw_table, c->stream);
      }
      break;
    }
    case CVR_METHOD_CONE_DOS: {
      if (params_size != sizeof(cvr_dos_params)) return fail(c, CVR_ERR_INVALID_ARG, "dos params size");
      const cvr_dos_params* p = static_cast<const cvr_dos_params*>(params);
      if (!(p->step_size > 0.0f)) return fail(c, CVR_ERR_INVALID_ARG, "step_size must be > 0");
      if (!c->pyr_ready) return fail(c, CVR_ERR_NOT_READY, "cvr_render: extinction pyramid not built");
      if (!c->cone_ready) return fail(c, CVR_ERR_NOT_READY, "cvr_render: cone tables not set");
      f.step = p->step_size;
      DosArgs a{};
      cvr_status ps = pyramid_view(c, &a.pyr);
      if (ps != CVR_OK) return ps;
      a.occ_sections = c->d_occ_sec; a.sdw_sections = c->d_sdw_sec;
      a.occ = c->occ; a.sdw = c->sdw;
      a.apply_occ = p->apply_occlusion; a.apply_sdw = p->apply_shadow; a.shadow_type = p->shadow_type;
      a.light_pos = make3(light->position); a.light_fwd = make3(light->forward);
      a.light_up = make3(light->up); a.light_right = make3(light->right);
      a.spot_cos_max = light->spot_cos_max;
      a.ka = p->ka; a.kd = p->kd;
      if (c->lc_dims[0] > 0) {  // object-space light cache, then the object-space marcher
        const size_t cells = (size_t)c->lc_dims[0] * c->lc_dims[1] * c->lc_dims[2];
        CK(c, ensure(c->d_lcache, c->lcache_cap, cells * sizeof(float2)));
        e = launch_cache_dos(f, a, c->lc_dims, c->d_lcache, c->stream);
        if (e == cudaSuccess)
          e = launch_march_cached(f, c->d_lcache, c->lc_dims, p->apply_occlusion, p->apply_shadow, p->ka, p->kd,
                                  c->stream);
      } else {
        bool tex = false;
        if (c->sampling & CVR_SAMPLING_TEX_PYRAMID) {
          cvr_status ts = ensure_pyramid_textures(c);
          if (ts != CVR_OK) return ts;
          for (int l = 0; l < c->tex.n_pyr; ++l) a.ptex[l] = c->tex.pyr[l].tex;
          tex = true;
        }
        e = launch_dos(f, a, tex, c->stream);
      }
      break;
    }
    case CVR_METHOD_GROUND_TRUTH: {
      if (params_size != sizeof(cvr_gt_params)) return fail(c, CVR_ERR_INVALID_ARG, "gt params size");
      const cvr_gt_params* p = static_cast<const cvr_gt_params*>(params);
      const float min_step = 1.0e-6f * std::sqrt(dot3(f.vol.grid, f.vol.grid));
      if (!(p->step_size > 0.0f) || !(p->light_ray_step_size >= min_step))
        return fail(c, CVR_ERR_INVALID_ARG, "step sizes must be >= 1e-6 * diagonal");
      if (!c->gt_ready) return fail(c, CVR_ERR_NOT_READY, "cvr_render: GT kernel vectors not set");
      f.step = p->step_size;
      GtArgs a{};
      a.occ_vec = c->d_occ_vec; a.sdw_vec = c->d_sdw_vec;
      a.n_occ = c->n_occ; a.n_sdw = c->n_sdw;
      a.gap = p->light_ray_initial_gap; a.lstep = p->light_ray_step_size;
      a.apply_occ = p->apply_occlusion; a.apply_sdw = p->apply_shadow; a.shadow_type = p->shadow_type;
      a.occ_dist = p->occ_distance; a.sdw_dist = p->sdw_distance;
      a.light_pos = make3(light->position); a.light_fwd = make3(light->forward);
      a.light_up = make3(light->up); a.light_right = make3(light->right);
      a.ka = p->ka; a.kd = p->kd;
      e = launch_gt(f, a, c->stream);
      break;
    }
    case CVR_METHOD_ISO: {
      if (params_size != sizeof(cvr_iso_params)) return fail(c, CVR_ERR_INVALID_ARG, "iso params size");
      const cvr_iso_params* p = static_cast<const cvr_iso_params*>(params);
      const float min_step = 1.0e-6f * std::sqrt(dot3(f.vol.grid, f.vol.grid));
      if (!(p->step_size_large >= min_step) || !std::isfinite(p->step_size_large) || !std::isfinite(p->isovalue) ||
          !std::isfinite(p->step_size_range) || !finite3(p->color) || !std::isfinite(p->color[3]))
        return fail(c, CVR_ERR_INVALID_ARG, "iso params: steps >= 1e-6 * diagonal, finite values");
      IsoArgs a;
      a.step_small = p->step_size_small; a.step_large = p->step_size_large;
      a.step_range = p->step_size_range; a.iso = p->isovalue;
      a.color = make_float4(p->color[0], p->color[1], p->color[2], p->color[3]);
      e = launch_iso(f, a, c->stream);
      break;
    }
    case CVR_METHOD_SURROGATE: {
      if (params_size != sizeof(cvr_gt_params)) return fail(c, CVR_ERR_INVALID_ARG, "surrogate params size");
      const cvr_gt_params* p = static_cast<const cvr_gt_params*>(params);
      f.step = p->step_size;
      cvr_status s = render_surrogate(c, f, p, light);
      if (s != CVR_OK) return s;
      break;
    }
    default:
      return fail(c, CVR_ERR_INVALID_ARG, "cvr_render: unknown method");
  }
  if (e != cudaSuccess) return cuda_fail(c, e, "render launch");
  if (stats) {
    CK(c, cudaEventRecord(c->ev[3], c->stream));
    unsigned long long hs[3];
    CK(c, cudaMemcpyAsync(hs, c->d_stats, sizeof hs, cudaMemcpyDeviceToHost, c->stream));
    CK(c, cudaStreamSynchronize(c->stream));
    float ms = 0.0f;
    CK(c, cudaEventElapsedTime(&ms, c->ev[2], c->ev[3]));
    stats->samples = hs[0];
    stats->shaded_samples = hs[1];
    stats->aux_fetches = hs[2];
    stats->kernel_ms = ms;
    if (method == CVR_METHOD_SURROGATE) return mlp_check_err(c);
  }
  return CVR_OK;
}

cvr_status cvr_render(cvr_ctx* c, int method, const cvr_camera* cam, const cvr_light* light, const void* params,
                      size_t params_size, float* out_dev, int w, int h, uint32_t* counts, cvr_frame_stats* stats) {
  return render_impl(c, method, cam, light, params, params_size, out_dev, w, h, counts, stats);
}

cvr_status cvr_render_host(cvr_ctx* c, int method, const cvr_camera* cam, const cvr_light* light, const void* params,
                           size_t params_size, float* out_host, int w, int h, cvr_frame_stats* stats) {
  if (!c || !out_host || w <= 0 || h <= 0) return fail(c, CVR_ERR_INVALID_ARG, "cvr_render_host: bad arguments");
  CK(c, cudaSetDevice(c->device));
  size_t bytes = (size_t)w * h * sizeof(float4);
  CK(c, ensure(c->d_out, c->out_cap, bytes));
  cvr_status s = render_impl(c, method, cam, light, params, params_size, reinterpret_cast<float*>(c->d_out), w, h,
                             nullptr, stats);
  if (s != CVR_OK) return s;
  CK(c, cudaMemcpyAsync(out_host, c->d_out, bytes, cudaMemcpyDeviceToHost, c->stream));
  CK(c, cudaStreamSynchronize(c->stream));
  return CVR_OK;
}

static bool tile_ok(int tile_w, int tile_h) {
  if (tile_w <= 0 || tile_h <= 0 || tile_w % 8 || tile_h % 4) return false;
  const int warps = (tile_w / 8) * (tile_h / 4);
  return warps == 2 || warps == 4 || warps == 8;
}

cvr_status cvr_set_walk_tables(cvr_ctx* c, int on) {
  if (!c) return CVR_ERR_INVALID_ARG;
  c->walk_tables = on != 0;
  return CVR_OK;
}

int cvr_get_walk_tables(const cvr_ctx* c) { return c && c->walk_tables ? 1 : 0; }

cvr_status cvr_set_brick_staging(cvr_ctx* c, int on) {
  if (!c) return CVR_ERR_INVALID_ARG;
  c->staging = on != 0;
  return CVR_OK;
}

int cvr_get_brick_staging(const cvr_ctx* c) { return c && c->staging ? 1 : 0; }

cvr_status cvr_set_ray_refill(cvr_ctx* c, int on) {
  if (!c) return CVR_ERR_INVALID_ARG;
  c->refill = on != 0;
  return CVR_OK;
}

int cvr_get_ray_refill(const cvr_ctx* c) { return c && c->refill ? 1 : 0; }

cvr_status cvr_set_tuning(cvr_ctx* c, int tile_w, int tile_h, int variant) {
  if (!c) return CVR_ERR_INVALID_ARG;
  if (!tile_ok(tile_w, tile_h) || variant < 0 || variant > 3)
    return fail(c, CVR_ERR_INVALID_ARG,
                "cvr_set_tuning: tile must be 2, 4 or 8 warps of 8x4 pixels (8x8 ... 32x8), variant 0..3");
  c->tile_w = tile_w;
  c->tile_h = tile_h;
  c->variant = variant;
  return CVR_OK;
}

cvr_status cvr_set_warp_shape(cvr_ctx* c, int warp_w) {
  if (!c) return CVR_ERR_INVALID_ARG;
  if (warp_w != 4 && warp_w != 8 && warp_w != 16)
    return fail(c, CVR_ERR_INVALID_ARG, "cvr_set_warp_shape: 4, 8 or 16 pixels per warp row");
  c->warp_w = warp_w;
  return CVR_OK;
}

int cvr_get_warp_shape(cvr_ctx* c) { return c ? c->warp_w : 8; }

cvr_status cvr_get_tuning(cvr_ctx* c, int* tile_w, int* tile_h, int* variant) {
  if (!c) return CVR_ERR_INVALID_ARG;
  if (tile_w) *tile_w = c->tile_w;
  if (tile_h) *tile_h = c->tile_h;
  if (variant) *variant = c->variant;
  return CVR_OK;
}

cvr_status cvr_set_compact_sat(cvr_ctx* c, int enable) {
  if (!c) return CVR_ERR_INVALID_ARG;
  c->compact_sat = enable != 0;
  return CVR_OK;
}

int cvr_get_compact_sat(cvr_ctx* c) { return c ? (int)c->compact_sat : 0; }

cvr_status cvr_set_light_cache(cvr_ctx* c, int w, int h, int d) {
  if (!c) return CVR_ERR_INVALID_ARG;
  const bool off = w == 0 && h == 0 && d == 0;
  if (!off && (w < 1 || h < 1 || d < 1 || w > 1024 || h > 1024 || d > 1024))
    return fail(c, CVR_ERR_INVALID_ARG, "cvr_set_light_cache: dims must be 0,0,0 (off) or 1..1024 each");
  c->lc_dims[0] = w; c->lc_dims[1] = h; c->lc_dims[2] = d;
  return CVR_OK;
}

cvr_status cvr_download_light_cache(cvr_ctx* c, float* host, size_t n_floats) {
  if (!c || !host) return CVR_ERR_INVALID_ARG;
  const size_t cells = (size_t)c->lc_dims[0] * c->lc_dims[1] * c->lc_dims[2];
  if (cells == 0 || !c->d_lcache) return fail(c, CVR_ERR_NOT_READY, "cvr_download_light_cache: no light cache");
  if (n_floats != 2 * cells) return fail(c, CVR_ERR_INVALID_ARG, "cvr_download_light_cache: need 2 floats per cell");
  CK(c, cudaSetDevice(c->device));
  CK(c, cudaMemcpyAsync(host, c->d_lcache, cells * sizeof(float2), cudaMemcpyDeviceToHost, c->stream));
  CK(c, cudaStreamSynchronize(c->stream));
  return CVR_OK;
}

cvr_status cvr_set_brick_size(cvr_ctx* c, int edge) {
  if (!c) return CVR_ERR_INVALID_ARG;
  int bs = edge == 0 ? 0 : (edge == 4 ? 2 : (edge == 8 ? 3 : (edge == 16 ? 4 : (edge == 32 ? 5 : -1))));
  if (bs < 0) return fail(c, CVR_ERR_INVALID_ARG, "cvr_set_brick_size: edge must be 0, 4, 8, 16 or 32");
  c->brick_bs = bs;
  return CVR_OK;
}

int cvr_get_brick_size(cvr_ctx* c) { return (c && c->brick_bs > 0) ? (1 << c->brick_bs) : 0; }

cvr_status cvr_set_volume_layout(cvr_ctx* c, int layout) {
  if (!c) return CVR_ERR_INVALID_ARG;
  if (layout != CVR_LAYOUT_PLAIN && layout != CVR_LAYOUT_QUADS)
    return fail(c, CVR_ERR_INVALID_ARG, "cvr_set_volume_layout: CVR_LAYOUT_PLAIN or CVR_LAYOUT_QUADS");
  c->quads = layout == CVR_LAYOUT_QUADS;
  return CVR_OK;
}

int cvr_get_volume_layout(cvr_ctx* c) { return (c && c->quads) ? CVR_LAYOUT_QUADS : CVR_LAYOUT_PLAIN; }

// Mean device time of reps frames of the current tuning (one untimed frame
// first, L2 flushed before each timed one).
static cvr_status time_config(cvr_ctx* c, int method, const cvr_camera* cam, const cvr_light* light,
                              const void* params, size_t params_size, float* frame, int w, int h, int reps,
                              float* mean_ms) {
  cvr_status s = render_impl(c, method, cam, light, params, params_size, frame, w, h, nullptr, nullptr);
  float total = 0.0f;
  for (int r = 0; r < reps && s == CVR_OK; ++r) {
    if ((s = cvr_flush_l2(c)) != CVR_OK) break;
    if ((s = cvr_timer_start(c)) != CVR_OK) break;
    if ((s = render_impl(c, method, cam, light, params, params_size, frame, w, h, nullptr, nullptr)) != CVR_OK) break;
    float ms = 0.0f;
    if ((s = cvr_timer_stop(c, &ms)) != CVR_OK) break;
    total += ms;
  }
  *mean_ms = total / (float)reps;
  return s;
}

cvr_status cvr_autotune(cvr_ctx* c, int method, const cvr_camera* cam, const cvr_light* light, const void* params,
                        size_t params_size, int w, int h, int reps, int* btw, int* bth, int* bv, float* bms) {
  if (!c || reps <= 0 || reps > 100) return fail(c, CVR_ERR_INVALID_ARG, "cvr_autotune: bad arguments");
  // Coordinate descent over three groups: ray tile (8x8 to 32x8: 2, 4 and 8
  // warps) x warp shape (4x8, 8x4, 16x2 pixels; the two interact: a warp
  // shape fits some tiles only), register variant, volume layout (plain,
  // bricks of 8^3, 16^3, 32^3, x-y quads; -1 stands for the quads).  Each
  // sweep times every member of a group with the other two fixed at the best
  // so far; the search stops after a sweep that changes nothing (at most
  // three).  Each configuration is timed once (memoised).
  static const int tiles[6][2] = {{8, 8}, {16, 8}, {32, 4}, {8, 16}, {32, 8}, {16, 16}};
  static const int bricks[5] = {0, 3, 4, 5, -1};
  static const int warps[3] = {8, 4, 16};
  float* frame = nullptr;
  cvr_status s = cvr_get_frame_buffer(c, w, h, &frame);
  if (s != CVR_OK) return s;
  const int keep_w = c->tile_w, keep_h = c->tile_h, keep_v = c->variant, keep_b = c->brick_bs;
  const bool keep_q = c->quads;
  const int keep_ww = c->warp_w;
  const bool keep_r = c->refill, keep_st = c->staging;
  c->refill = false;
  c->staging = false;
  // register variants: the extinction marchers have a fourth (<= 96 registers)
  const int n_variants = method == CVR_METHOD_EXTINCTION ? 4 : 3;
  float timed[6][4][3][5];
  for (auto& a : timed)
    for (auto& b : a)
      for (auto& d : b)
        for (float& x : d) x = -1.0f;
  int bt = 1, bvar = 0, bw = 0, bb = 0;  // indices into tiles, variants, warps, bricks
  float best = 1e30f;
  auto trial = [&](int t, int v, int wi, int k) {
    if (s != CVR_OK) return;
    float& ms = timed[t][v][wi][k];
    if (ms < 0.0f) {
      c->tile_w = tiles[t][0]; c->tile_h = tiles[t][1]; c->variant = v;
      c->warp_w = warps[wi];
      c->brick_bs = bricks[k] > 0 ? bricks[k] : 0;
      c->quads = bricks[k] < 0;
      float m = 0.0f;
      s = time_config(c, method, cam, light, params, params_size, frame, w, h, reps, &m);
      if (s != CVR_OK) return;
      ms = m;
    }
    if (ms < best) {
      best = ms;
      bt = t; bvar = v; bw = wi; bb = k;
    }
  };
  for (int sweep = 0; sweep < 3 && s == CVR_OK; ++sweep) {
    const int before[4] = {bt, bvar, bw, bb};
    for (int t = 0; t < 6; ++t)
      for (int wi = 0; wi < 3; ++wi)
        if (warp_fits(tiles[t][0], tiles[t][1], warps[wi])) trial(t, bvar, wi, bb);
    for (int v = 0; v < n_variants; ++v) trial(bt, v, bw, bb);
    for (int k = 0; k < 5; ++k) trial(bt, bvar, bw, k);
    if (before[0] == bt && before[1] == bvar && before[2] == bw && before[3] == bb) break;
  }
  // Single timings of configurations a few percent apart are within the
  // frames' noise: the five fastest are timed again in three interleaved
  // rounds (so that a drift of the clocks or caches hits all of them), and
  // the lowest median wins.
  if (s == CVR_OK) {
    struct Cand { float ms; int t, v, wi, k; float runs[3]; };
    std::vector<Cand> cands;
    for (int t = 0; t < 6; ++t)
      for (int v = 0; v < n_variants; ++v)
        for (int wi = 0; wi < 3; ++wi)
          for (int k = 0; k < 5; ++k)
            if (timed[t][v][wi][k] >= 0.0f) cands.push_back({timed[t][v][wi][k], t, v, wi, k, {0, 0, 0}});
    std::sort(cands.begin(), cands.end(), [](const Cand& a, const Cand& b) { return a.ms < b.ms; });
    if (cands.size() > 5) cands.resize(5);
    if (cands.size() > 1) {
      for (int round = 0; round < 3 && s == CVR_OK; ++round) {
        for (Cand& cd : cands) {
          c->tile_w = tiles[cd.t][0]; c->tile_h = tiles[cd.t][1]; c->variant = cd.v;
          c->warp_w = warps[cd.wi];
          c->brick_bs = bricks[cd.k] > 0 ? bricks[cd.k] : 0;
          c->quads = bricks[cd.k] < 0;
          s = time_config(c, method, cam, light, params, params_size, frame, w, h, reps, &cd.runs[round]);
          if (s != CVR_OK) break;
        }
      }
      if (s == CVR_OK) {
        best = 1e30f;
        for (Cand& cd : cands) {
          std::sort(cd.runs, cd.runs + 3);
          if (cd.runs[1] < best) {
            best = cd.runs[1];
            bt = cd.t; bvar = cd.v; bw = cd.wi; bb = cd.k;
          }
        }
      }
    }
  }
  if (s != CVR_OK) {
    c->tile_w = keep_w; c->tile_h = keep_h; c->variant = keep_v; c->brick_bs = keep_b; c->quads = keep_q;
    c->warp_w = keep_ww;
    c->refill = keep_r;
    c->staging = keep_st;
    return s;
  }
  c->tile_w = tiles[bt][0]; c->tile_h = tiles[bt][1]; c->variant = bvar;
  c->warp_w = warps[bw];
  c->brick_bs = bricks[bb] > 0 ? bricks[bb] : 0;
  c->quads = bricks[bb] < 0;
  const int bwt = tiles[bt][0], bht = tiles[bt][1];
  // the persistent ray-refill marcher at each register variant (the tile
  // shape does not apply to it)
  bool br = false;
  if (method == CVR_METHOD_PLAIN || method == CVR_METHOD_EXTINCTION || method == CVR_METHOD_CONE_DOS ||
      method == CVR_METHOD_GROUND_TRUTH) {
    for (int v = 0; v < n_variants && s == CVR_OK; ++v) {
      c->refill = true;
      c->variant = v;
      float ms = 0.0f;
      s = time_config(c, method, cam, light, params, params_size, frame, w, h, reps, &ms);
      if (s == CVR_OK && ms < best) {
        best = ms;
        br = true;
        bvar = v;
      }
    }
  }
  c->variant = bvar;
  c->refill = br;
  // the plain marcher with shared-memory brick staging (plain layout, its own tile)
  bool bst = false;
  if (method == CVR_METHOD_PLAIN && s == CVR_OK && !(c->sampling & CVR_SAMPLING_TEX_VOLUME)) {
    const int kb = c->brick_bs;
    const bool kq = c->quads, kr = c->refill;
    c->brick_bs = 0; c->quads = false; c->refill = false; c->staging = true;
    float ms = 0.0f;
    s = time_config(c, method, cam, light, params, params_size, frame, w, h, reps, &ms);
    if (s == CVR_OK && ms < best) {
      best = ms;
      bst = true;
      bb = 0;
      br = false;
    } else {
      c->brick_bs = kb; c->quads = kq; c->refill = kr;
    }
  }
  c->staging = bst;
  if (s != CVR_OK) {
    c->staging = keep_st;
    c->tile_w = keep_w; c->tile_h = keep_h; c->variant = keep_v; c->brick_bs = keep_b; c->quads = keep_q;
    c->warp_w = keep_ww;
    c->refill = keep_r;
    return s;
  }
  if (btw) *btw = bwt;
  if (bth) *bth = bht;
  if (bv) *bv = bvar;
  if (bms) *bms = best;
  return CVR_OK;
}

cvr_status cvr_get_frame_buffer(cvr_ctx* c, int w, int h, float** dev_out) {
  if (!c || !dev_out || w <= 0 || h <= 0 || w > 32768 || h > 32768)
    return fail(c, CVR_ERR_INVALID_ARG, "cvr_get_frame_buffer: bad arguments");
  CK(c, cudaSetDevice(c->device));
  CK(c, ensure(c->d_out, c->out_cap, (size_t)w * h * sizeof(float4)));
  *dev_out = reinterpret_cast<float*>(c->d_out);
  return CVR_OK;
}

cvr_status cvr_download_frame(cvr_ctx* c, const float* dev, int w, int h, float* host) {
  if (!c || !dev || !host || w <= 0 || h <= 0) return fail(c, CVR_ERR_INVALID_ARG, "cvr_download_frame: bad arguments");
  CK(c, cudaSetDevice(c->device));
  CK(c, cudaMemcpyAsync(host, dev, (size_t)w * h * sizeof(float4), cudaMemcpyDeviceToHost, c->stream));
  CK(c, cudaStreamSynchronize(c->stream));
  return CVR_OK;
}

cvr_status cvr_timer_start(cvr_ctx* c) {
  if (!c) return CVR_ERR_INVALID_ARG;
  CK(c, cudaEventRecord(c->ev[0], c->stream));
  return CVR_OK;
}

cvr_status cvr_timer_stop(cvr_ctx* c, float* ms) {
  if (!c || !ms) return CVR_ERR_INVALID_ARG;
  CK(c, cudaEventRecord(c->ev[1], c->stream));
  CK(c, cudaEventSynchronize(c->ev[1]));
  CK(c, cudaEventElapsedTime(ms, c->ev[0], c->ev[1]));
  return CVR_OK;
}

cvr_status cvr_flush_l2(cvr_ctx* c) {
  if (!c) return CVR_ERR_INVALID_ARG;
  CK(c, cudaSetDevice(c->device));
  if (!c->d_flush) {
    int l2 = 0;
    CK(c, cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, c->device));
    size_t bytes = std::max<size_t>((size_t)l2 * 2, 256u << 20);
    CK(c, cudaMalloc(&c->d_flush, bytes));
    c->flush_bytes = bytes;
  }
  CK(c, launch_fill(c->d_flush, c->flush_bytes, 0x5a5a5a5au, c->stream));
  return CVR_OK;
}

cvr_status cvr_host_alloc_pinned(size_t bytes, void** out) {
  if (!out || bytes == 0) return CVR_ERR_INVALID_ARG;
  cudaError_t e = cudaHostAlloc(out, bytes, cudaHostAllocDefault);
  if (e != cudaSuccess) {
    cudaGetLastError();
    *out = nullptr;
    g_create_err = std::string("cudaHostAlloc: ") + cudaGetErrorString(e);
    return e == cudaErrorMemoryAllocation ? CVR_ERR_OUT_OF_MEMORY : CVR_ERR_CUDA;
  }
  return CVR_OK;
}

void cvr_host_free_pinned(void* p) {
  if (p) cudaFreeHost(p);
}

}  // extern "C"
