// shade.cuh — the shading policies of the four renderers and the shared
// primary-ray loop (ShadeSample and main() of each reference shader).
// Included by march.cu (the marchers) and surrogate.cu (training targets and
// the surrogate-shaded marcher reuse the ground-truth light rays).
#pragma once

#include <algorithm>

#include <cuda_fp16.h>

#include "march.cuh"

namespace cvr {

// Iteration bounds of the secondary loops.  Validated parameters stay far
// below them (a cone walk has at most 0.75*diagonal/interval boxes, a light
// ray distance/step samples); they only stop a loop whose position stopped
// advancing from spinning forever.
constexpr int kMaxConeBoxes = 1 << 16;
constexpr int kMaxLightSteps = 1 << 20;

// ============================================= gradient Blinn-Phong terms
// texture(TexVolumeGradient, Tpos / VolumeGridSize).xyz: GL_LINEAR,
// clamp-to-edge on the voxel grid (the texture copy when there is one).
__device__ __forceinline__ float3 sample_gradient(const GradView& g, float3 p) {
  if (g.tex) {
    const float4 r = tex3D<float4>(g.tex, p.x * g.inv_grid.x, p.y * g.inv_grid.y, p.z * g.inv_grid.z);
    return f3(r.x, r.y, r.z);
  }
  const Tap a = axis_tap(fmaf(p.x, g.inv_spacing.x, -0.5f), g.nx);
  const Tap b = axis_tap(fmaf(p.y, g.inv_spacing.y, -0.5f), g.ny);
  const Tap c = axis_tap(fmaf(p.z, g.inv_spacing.z, -0.5f), g.nz);
  const size_t sy = (size_t)g.nx, sz = (size_t)g.nx * g.ny;
  auto at = [&](int x, int y, int z) {
    const uint2 q = __ldg(g.g + (size_t)x + sy * y + sz * z);
    const float2 xy = __half22float2(*reinterpret_cast<const __half2*>(&q.x));
    return f3(xy.x, xy.y, __low2float(*reinterpret_cast<const __half2*>(&q.y)));
  };
  auto lerp = [](float t, float3 u, float3 v) {
    return f3(fmaf(t, v.x - u.x, u.x), fmaf(t, v.y - u.y, u.y), fmaf(t, v.z - u.z, u.z));
  };
  const float3 c00 = lerp(a.t, at(a.i0, b.i0, c.i0), at(a.i1, b.i0, c.i0));
  const float3 c10 = lerp(a.t, at(a.i0, b.i1, c.i0), at(a.i1, b.i1, c.i0));
  const float3 c01 = lerp(a.t, at(a.i0, b.i0, c.i1), at(a.i1, b.i0, c.i1));
  const float3 c11 = lerp(a.t, at(a.i0, b.i1, c.i1), at(a.i1, b.i1, c.i1));
  return lerp(c.t, lerp(b.t, c00, c10), lerp(b.t, c01, c11));
}

// The terms every gradient branch shares (ray_marching_1p.comp:50-70 and its
// copies in the other shaders): false when the interpolated gradient is the
// zero vector, where the sample keeps its unshaded colour.
struct BlinnTerms {
  float diff;  // max(0, dot(N, L))
  float spec;  // pow(max(0, dot(H, N)), shininess)
};
__device__ __forceinline__ bool blinn_terms(const FrameArgs& f, float3 tx, BlinnTerms& t) {
  float3 n = sample_gradient(f.grad, tx);
  if (n.x == 0.0f && n.y == 0.0f && n.z == 0.0f) return false;
  n = normalize3(n);
  const float3 w = tx - f.vol.grid * 0.5f;
  const float3 l = normalize3(f.grad.light_pos - w);
  const float3 e = normalize3(f.cam.eye - w);
  const float3 hv = normalize3(e + l);
  t.diff = fmaxf(0.0f, dot3(n, l));
  // pow(x, N) = exp2(N log2 x) on the special-function unit (relative error
  // ~1e-6 for N = 30; 0 at x = 0 as GLSL's pow gives for N > 0)
  t.spec = __powf(fmaxf(0.0f, dot3(hv, n)), f.grad.shininess);
  return true;
}

// ShadeBlinnPhong (ray_marching_1p.comp:48-81):
// clr * (Ka + Kd * diff) + Ispecular * Ks * spec.
__device__ __forceinline__ float4 phong_plain(const FrameArgs& f, float4 L, float3 tx) {
  BlinnTerms t;
  if (!blinn_terms(f, tx, t)) return L;
  const float m = f.grad.ka + f.grad.kd * t.diff;
  const float s = f.grad.ks * t.spec;
  L.x = L.x * m + f.grad.ispec.x * s;
  L.y = L.y * m + f.grad.ispec.y * s;
  L.z = L.z * m + f.grad.ispec.z * s;
  return L;
}

// Extinction / light cache (ebs_ray_bbox_marching.comp:524-546,
// obj_ray_marching.comp:111-129):
// (1/(ka+kd)) * (L*Io*ka + Is*(L*kd*diff)) + Is*(ks*Ispecular*spec).
__device__ __forceinline__ float4 phong_ext(const FrameArgs& f, float4 L, float3 tx, float io, float ka, float is,
                                            float kd) {
  BlinnTerms t;
  if (!blinn_terms(f, tx, t)) return L;
  const float kk = 1.0f / (ka + kd);
  const float s = is * (f.grad.ks * t.spec);
  L.x = kk * (L.x * io * ka + is * (L.x * kd * t.diff)) + s * f.grad.ispec.x;
  L.y = kk * (L.y * io * ka + is * (L.y * kd * t.diff)) + s * f.grad.ispec.y;
  L.z = kk * (L.z * io * ka + is * (L.z * kd * t.diff)) + s * f.grad.ispec.z;
  return L;
}

// Cone and ground truth (ray_bbox_marching.comp:630-648, gt_ray_marching.comp:
// 277-295, whose specular colour is 1): L * ((1/(ka+kd)) * (Io*ka + Is*kd*diff))
// + Ispecular * (Is*ks*spec).
__device__ __forceinline__ float4 phong_cone(const FrameArgs& f, float4 L, float3 tx, float io, float ka, float is,
                                             float kd) {
  BlinnTerms t;
  if (!blinn_terms(f, tx, t)) return L;
  const float m = (1.0f / (ka + kd)) * (io * ka + is * kd * t.diff);
  const float s = is * f.grad.ks * t.spec;
  L.x = L.x * m + f.grad.ispec.x * s;
  L.y = L.y * m + f.grad.ispec.y * s;
  L.z = L.z * m + f.grad.ispec.z * s;
  return L;
}

// ============================================================ plain (rc1pass)
struct PlainShade {
  struct Ray {};
  __device__ __forceinline__ void begin(Ray&, float3) const {}
  // ShadeSample is the identity unless gradient shading is on
  // (ApplyGradientPhongShading, ray_marching_1p.comp:143-145).
  __device__ __forceinline__ float4 shade(float4 src, float3 tx, const Ray&, const FrameArgs& f, unsigned&) const {
    return f.grad.g ? phong_plain(f, src, tx) : src;
  }
};

// ====================================================== extinction (rc1pextbsd)
// COMPACT: the frame's SAT box queries read the 32-bit table (SatView::sat32).
// ALIGNED (with COMPACT): every AO box and every box of the directional
// shadow table has integer texel widths, so every query is the equal-fraction
// one (sat_box_aligned); the kernel then always has a table (ttx set).
template <bool COMPACT = false, bool ALIGNED = false>
struct ExtShadeT {
  static_assert(COMPACT || !ALIGNED, "the equal-fraction query reads the compact table");
  const ExtArgs* e;
  // Per-frame box table of a directional light (shared memory), or nullptr.
  const float4* tlo = nullptr;
  const float4* thi = nullptr;
  // the table's texel offsets and packed integer widths (compact table only), or nullptr
  const float4* ttx = nullptr;
  int tn = 0, tax = 0;
  float tiw = 0.0f, tvmin = 0.0f, tvmax = 0.0f;
  struct Ray {};
  __device__ __forceinline__ void begin(Ray&, float3) const {}

  // EvaluateAmbientOcclusionSAT3D (ebs_ray_bbox_marching.comp:102-110).
  __device__ __forceinline__ float ao_box(float3 p1, float3 p2, const FrameArgs& f) const {
    const SatView& S = e->sat;
    p1 = clamp3(p1 + f.vol.spacing, S.min_pos, S.max_pos);
    p2 = clamp3(p2 + f.vol.spacing, S.min_pos, S.max_pos);
    return sat_box<COMPACT>(S, p1, p2);
  }

  // ExtinctionAmbientOcclusion (ebs_ray_bbox_marching.comp:112-146), with the
  // shell radii taken from a list (reference: AmbOccRadius * (i + 1)).
  __device__ float ambient_occlusion(float3 tx, const FrameArgs& f) const {
    if constexpr (ALIGNED) {
      {
        // the box [tx - r, tx + r] (voxels) starts at texel coordinate
        // (tx + spacing) / spacing - 0.5 - r = g - r and is 2 r texels wide
        const SatView& S = e->sat;
        const float3 g = f3(fmaf(tx.x, S.inv_spacing.x, 0.5f), fmaf(tx.y, S.inv_spacing.y, 0.5f),
                            fmaf(tx.z, S.inv_spacing.z, 0.5f));
        float r0 = e->radii[0];
        int w0 = __float2int_rn(2.0f * r0);
        float sat0 = sat_box_aligned(S, f3(g.x - r0, g.y - r0, g.z - r0), w0, w0, w0);
        float t = sat0 * (1.0f / (r0 * r0));
        float sat_i = sat0;
        for (int i = 1; i < e->n_shells; ++i) {
          const float ri = e->radii[i];
          const int wi = __float2int_rn(2.0f * ri);
          const float sat_n = sat_box_aligned(S, f3(g.x - ri, g.y - ri, g.z - ri), wi, wi, wi);
          t = t + (sat_n - sat_i) * (1.0f / (ri * ri));
          sat_i = sat_n;
        }
        const float rk = e->radii[e->n_shells - 1];
        return expf(-((1.0f / (rk * rk)) * t));
      }
    }
    float3 sc = f.vol.spacing;
    float r0 = e->radii[0];
    float sat0 = ao_box(tx - sc * r0, tx + sc * r0, f);
    float t = sat0 * (1.0f / (r0 * r0));
    float sat_i = sat0;
    for (int i = 1; i < e->n_shells; ++i) {
      float ri = e->radii[i];
      float sat_n = ao_box(tx - sc * ri, tx + sc * ri, f);
      t = t + (sat_n - sat_i) * (1.0f / (ri * ri));
      sat_i = sat_n;
    }
    float rk = e->radii[e->n_shells - 1];
    float wa = 1.0f / (rk * rk);
    return expf(-(wa * t));
  }

  // EvaluateShadowSAT3D, texture() branch (ebs_ray_bbox_marching.comp:173-187).
  __device__ __forceinline__ float shadow_box(float3 p1, float3 p2, const FrameArgs& f) const {
    float3 sc = f.vol.spacing;
    float volq = (fabsf(p1.x - p2.x) / sc.x) * (fabsf(p1.y - p2.y) / sc.y) * (fabsf(p1.z - p2.z) / sc.z);
    const SatView& S = e->sat;
    p1 = clamp3(p1 + sc, S.min_pos, S.max_pos);
    p2 = clamp3(p2 + sc, S.min_pos, S.max_pos);
    return (sat_box<COMPACT>(S, p1, p2) / volq) * e->ui_weight;
  }

  // ConeZAxis (ebs_ray_bbox_marching.comp:190-270).
  __device__ float cone_z(float3 pos, float3 c, const FrameArgs& f, unsigned& aux) const {
    float3 sc = f.vol.spacing;
    float st = 0.0f;
    float signal = c.z < 0.0f ? -1.0f : 1.0f;
    float3 proj_y = normalize3(f3(0.0f, c.y, c.z));
    float3 proj_x = normalize3(f3(c.x, 0.0f, c.z));
    float p_cs = cosf(e->cone_angle), p_sn = sinf(e->cone_angle);
    float n_cs = cosf(-e->cone_angle), n_sn = sinf(-e->cone_angle);
    float3 pj_x1 = normalize3(f3(proj_x.x * n_cs - proj_x.z * n_sn, 0.0f, proj_x.x * n_sn + proj_x.z * n_cs));
    float3 pj_x2 = normalize3(f3(proj_x.x * p_cs - proj_x.z * p_sn, 0.0f, proj_x.x * p_sn + proj_x.z * p_cs));
    float3 pj_y1 = normalize3(f3(0.0f, proj_y.y * n_cs - proj_y.z * n_sn, proj_y.y * n_sn + proj_y.z * n_cs));
    float3 pj_y2 = normalize3(f3(0.0f, proj_y.y * p_cs - proj_y.z * p_sn, proj_y.y * p_sn + proj_y.z * p_cs));
    float interval = e->interval * signal * sc.z;
    float zp = e->initial * signal * sc.z;
    float vmin = sc.z * 0.5f, vmax = f.vol.grid.z - sc.z * 0.5f;
    for (int guard = 0; guard < kMaxConeBoxes && (zp / c.z) < e->max_dist &&
                        (pos.z + (zp + interval) > vmin && pos.z + (zp + interval) < vmax); ++guard) {
      float zm = fabsf(zp + interval * 0.5f);
      float px1 = pj_x1.x * (zm / fabsf(pj_x1.z)), px2 = pj_x2.x * (zm / fabsf(pj_x2.z));
      float py1 = pj_y1.y * (zm / fabsf(pj_y1.z)), py2 = pj_y2.y * (zm / fabsf(pj_y2.z));
      float x1 = fminf(px1, px2), x2 = fmaxf(px1, px2);
      float y1 = fminf(py1, py2), y2 = fmaxf(py1, py2);
      float xd = fabsf(x2 - x1), yd = fabsf(y2 - y1);
      float xs = (ceilf(xd / sc.x) - (xd / sc.x)) * 0.5f;
      float ys = (ceilf(yd / sc.y) - (yd / sc.y)) * 0.5f;
      x1 = x1 - xs * sc.x; x2 = x2 + xs * sc.x;
      y1 = y1 - ys * sc.y; y2 = y2 + ys * sc.y;
      float z1 = fminf(zp, zp + interval), z2 = fmaxf(zp, zp + interval);
      st += shadow_box(pos + f3(x1, y1, z1), pos + f3(x2, y2, z2), f);
      ++aux;
      zp = zp + interval;
    }
    return st;
  }

  // ConeYAxis (ebs_ray_bbox_marching.comp:272-350).
  __device__ float cone_y(float3 pos, float3 c, const FrameArgs& f, unsigned& aux) const {
    float3 sc = f.vol.spacing;
    float st = 0.0f;
    float signal = c.y < 0.0f ? -1.0f : 1.0f;
    float3 proj_x = normalize3(f3(c.x, c.y, 0.0f));
    float3 proj_z = normalize3(f3(0.0f, c.y, c.z));
    float p_cs = cosf(e->cone_angle), p_sn = sinf(e->cone_angle);
    float n_cs = cosf(-e->cone_angle), n_sn = sinf(-e->cone_angle);
    float3 pj_x1 = normalize3(f3(proj_x.x * n_cs - proj_x.y * n_sn, proj_x.x * n_sn + proj_x.y * n_cs, 0.0f));
    float3 pj_x2 = normalize3(f3(proj_x.x * p_cs - proj_x.y * p_sn, proj_x.x * p_sn + proj_x.y * p_cs, 0.0f));
    float3 pj_z1 = normalize3(f3(0.0f, proj_z.z * n_sn + proj_z.y * n_cs, proj_z.z * n_cs - proj_z.y * n_sn));
    float3 pj_z2 = normalize3(f3(0.0f, proj_z.z * p_sn + proj_z.y * p_cs, proj_z.z * p_cs - proj_z.y * p_sn));
    float interval = e->interval * signal * sc.y;
    float yp = e->initial * signal * sc.y;
    float vmin = sc.y * 0.5f, vmax = f.vol.grid.y - sc.y * 0.5f;
    for (int guard = 0; guard < kMaxConeBoxes && (yp / c.y) < e->max_dist &&
                        (pos.y + (yp + interval) > vmin && pos.y + (yp + interval) < vmax); ++guard) {
      float ym = fabsf(yp + interval * 0.5f);
      float px1 = pj_x1.x * (ym / fabsf(pj_x1.y)), px2 = pj_x2.x * (ym / fabsf(pj_x2.y));
      float pz1 = pj_z1.z * (ym / fabsf(pj_z1.y)), pz2 = pj_z2.z * (ym / fabsf(pj_z2.y));
      float x1 = fminf(px1, px2), x2 = fmaxf(px1, px2);
      float z1 = fminf(pz1, pz2), z2 = fmaxf(pz1, pz2);
      float xd = fabsf(x2 - x1), zd = fabsf(z2 - z1);
      float xs = (ceilf(xd / sc.x) - (xd / sc.x)) * 0.5f;
      float zs = (ceilf(zd / sc.z) - (zd / sc.z)) * 0.5f;
      x1 = x1 - xs * sc.x; x2 = x2 + xs * sc.x;
      z1 = z1 - zs * sc.z; z2 = z2 + zs * sc.z;
      float y1 = fminf(yp, yp + interval), y2 = fmaxf(yp, yp + interval);
      st += shadow_box(pos + f3(x1, y1, z1), pos + f3(x2, y2, z2), f);
      ++aux;
      yp = yp + interval;
    }
    return st;
  }

  // ConeXAxis (ebs_ray_bbox_marching.comp:352-430).
  __device__ float cone_x(float3 pos, float3 c, const FrameArgs& f, unsigned& aux) const {
    float3 sc = f.vol.spacing;
    float st = 0.0f;
    float signal = c.x < 0.0f ? -1.0f : 1.0f;
    float3 proj_y = normalize3(f3(c.x, c.y, 0.0f));
    float3 proj_z = normalize3(f3(c.x, 0.0f, c.z));
    float p_cs = cosf(e->cone_angle), p_sn = sinf(e->cone_angle);
    float n_cs = cosf(-e->cone_angle), n_sn = sinf(-e->cone_angle);
    float3 pj_y1 = normalize3(f3(proj_y.y * n_sn + proj_y.x * n_cs, proj_y.y * n_cs - proj_y.x * n_sn, 0.0f));
    float3 pj_y2 = normalize3(f3(proj_y.y * p_sn + proj_y.x * p_cs, proj_y.y * p_cs - proj_y.x * p_sn, 0.0f));
    float3 pj_z1 = normalize3(f3(proj_z.z * n_sn + proj_z.x * n_cs, 0.0f, proj_z.z * n_cs - proj_z.x * n_sn));
    float3 pj_z2 = normalize3(f3(proj_z.z * p_sn + proj_z.x * p_cs, 0.0f, proj_z.z * p_cs - proj_z.x * p_sn));
    float interval = e->interval * signal * sc.x;
    float xp = e->initial * signal * sc.x;
    float vmin = sc.x * 0.5f, vmax = f.vol.grid.x - sc.x * 0.5f;
    for (int guard = 0; guard < kMaxConeBoxes && (xp / c.x) < e->max_dist &&
                        (pos.x + (xp + interval) > vmin && pos.x + (xp + interval) < vmax); ++guard) {
      float xm = fabsf(xp + interval * 0.5f);
      float py1 = pj_y1.y * (xm / fabsf(pj_y1.x)), py2 = pj_y2.y * (xm / fabsf(pj_y2.x));
      float pz1 = pj_z1.z * (xm / fabsf(pj_z1.x)), pz2 = pj_z2.z * (xm / fabsf(pj_z2.x));
      float y1 = fminf(py1, py2), y2 = fmaxf(py1, py2);
      float z1 = fminf(pz1, pz2), z2 = fmaxf(pz1, pz2);
      float yd = fabsf(y2 - y1), zd = fabsf(z2 - z1);
      float ys = (ceilf(yd / sc.y) - (yd / sc.y)) * 0.5f;
      float zs = (ceilf(zd / sc.z) - (zd / sc.z)) * 0.5f;
      y1 = y1 - ys * sc.y; y2 = y2 + ys * sc.y;
      z1 = z1 - zs * sc.z; z2 = z2 + zs * sc.z;
      float x1 = fminf(xp, xp + interval), x2 = fmaxf(xp, xp + interval);
      st += shadow_box(pos + f3(x1, y1, z1), pos + f3(x2, y2, z2), f);
      ++aux;
      xp = xp + interval;
    }
    return st;
  }

  // The Cone*Axis walk over the precomputed boxes of a directional light:
  // same boxes, same CUT_WHEN_AWAY_FROM_VOLUME test, same sum.
  __device__ float shadow_table(float3 tx, const FrameArgs& f, unsigned& aux) const {
    const SatView& S = e->sat;
    const float3 sc = f.vol.spacing;
    const float pm = tax == 0 ? tx.x : (tax == 1 ? tx.y : tx.z);
    float st = 0.0f;
    if constexpr (ALIGNED) {
      const float3 g = f3(fmaf(tx.x, S.inv_spacing.x, 0.5f), fmaf(tx.y, S.inv_spacing.y, 0.5f),
                          fmaf(tx.z, S.inv_spacing.z, 0.5f));
      {  // every box has integer widths: the equal-fraction query
        for (int k = 0; k < tn; ++k) {
          const float nxt = pm + (tlo[k].w + tiw);
          if (!(nxt > tvmin && nxt < tvmax)) break;
          const float4 o = ttx[k];
          const int w = __float_as_int(o.w);
          const float3 u = f3(g.x + o.x, g.y + o.y, g.z + o.z);
          const float b = e->walk.oct ? sat_box_walk(S, e->walk, u, w & 1023, (w >> 10) & 1023, w >> 20)
                                      : sat_box_aligned(S, u, w & 1023, (w >> 10) & 1023, w >> 20);
          st = fmaf(b, thi[k].w, st);
          ++aux;
        }
        return expf(-st);
      }
    }
    for (int k = 0; k < tn; ++k) {
      const float4 lo = tlo[k];
      const float nxt = pm + (lo.w + tiw);
      if (!(nxt > tvmin && nxt < tvmax)) break;
      const float4 hi = thi[k];
      float3 p1 = clamp3(tx + f3(lo.x, lo.y, lo.z) + sc, S.min_pos, S.max_pos);
      float3 p2 = clamp3(tx + f3(hi.x, hi.y, hi.z) + sc, S.min_pos, S.max_pos);
      st = fmaf(sat_box<COMPACT>(S, p1, p2), hi.w, st);
      ++aux;
    }
    return expf(-st);
  }

  // ExtinctionDirectionalShadows (ebs_ray_bbox_marching.comp:432-456).
  __device__ float shadow(float3 tx, const FrameArgs& f, unsigned& aux) const {
    float3 realpos = tx - f.vol.grid * 0.5f;
    float3 c = (e->shadow_type == 0) ? normalize3(e->light_pos - realpos) : normalize3(e->light_fwd);
    float3 a = abs3(c);
    float st;
    if (a.z > a.x && a.z > a.y) st = cone_z(tx, c, f, aux);
    else if (a.y > a.x) st = cone_y(tx, c, f, aux);
    else st = cone_x(tx, c, f, aux);
    return expf(-st);
  }

  // ShadeSample (ebs_ray_bbox_marching.comp:500-551).
  __device__ __forceinline__ float4 shade(float4 src, float3 tx, const Ray&, const FrameArgs& f, unsigned& aux) const {
    float ka = 0.0f, kd = 0.0f, io = 0.0f, is = 0.0f;
    if (e->apply_occ) { ka = e->ka; io = ambient_occlusion(tx, f); aux += e->n_shells; }
    if (e->apply_sdw) {
      kd = e->kd;
      if constexpr (ALIGNED) is = shadow_table(tx, f, aux);
      else is = tlo ? shadow_table(tx, f, aux) : shadow(tx, f, aux);
    }
    if (f.grad.g) return phong_ext(f, src, tx, io, ka, is, kd);
    float k = 1.0f / (ka + kd);
    src.x = k * (src.x * io * ka + src.x * is * kd);
    src.y = k * (src.y * io * ka + src.y * is * kd);
    src.z = k * (src.z * io * ka + src.z * is * kd);
    return src;
  }
};
using ExtShade = ExtShadeT<false>;

// ==================================================== cone DOS (rc1pdosct)
// TEX: the pyramid taps through the texture unit (DosArgs::ptex).
template <bool TEX = false>
struct DosShadeT {
  const DosArgs* d;
  const float4* occ_tab;  // shared-memory copies of the section tables
  const float4* sdw_tab;
  struct Ray { float3 v_up, v_right; };

  // main(), ray_bbox_marching.comp:682-684.
  __device__ __forceinline__ void begin(Ray& r, float3 dir) const {
    r.v_right = normalize3(cross3(dir, f3(0.0f, 1.0f, 0.0f)));
    r.v_up = normalize3(cross3(-dir, r.v_right));
  }

  // GetGaussianExtinction with CONSIDER_BORDERS (ray_bbox_marching.comp:92-112).
  __device__ __forceinline__ float gauss_ext(float3 p, float level, const FrameArgs& f) const {
    float rg = TEX ? pyr_sample_tex(level, p) : pyr_sample(d->pyr, level, p);
    float3 S = f.vol.grid;
    if (p.x < 0.0f || p.x > S.x || p.y < 0.0f || p.y > S.y || p.z < 0.0f || p.z > S.z) {
      float sg = exp2f(level);
      float3 c = clamp3(p, f3(0.0f, 0.0f, 0.0f), S) - p;
      float dist = c.x * c.x + c.y * c.y + c.z * c.z;
      rg = rg * expf(-(dist) / (2.0f * sg * sg));
    }
    return rg;
  }

  // pyr_sample's GL_LINEAR_MIPMAP_LINEAR lookup on the level textures: hardware
  // trilinear within a level (normalised coordinates, all levels span the
  // grid), linear between the two levels of a fractional lod.
  __device__ __forceinline__ float pyr_sample_tex(float lod, float3 p) const {
    const PyramidView& P = d->pyr;
    lod = fminf(fmaxf(lod, 0.0f), float(P.n_levels - 1));
    const float fl = floorf(lod);
    const int l0 = int(fl);
    const float t = lod - fl;
    const float u = p.x * P.inv_grid.x, v = p.y * P.inv_grid.y, w = p.z * P.inv_grid.z;
    const float a = tex3D<float>(d->ptex[l0], u, v, w);
    if (t == 0.0f) return a;
    const float b = tex3D<float>(d->ptex[min(l0 + 1, P.n_levels - 1)], u, v, w);
    return fmaf(t, b - a, a);
  }

  // Cone1/3/7Ray{Occlusion,Shadow} (ray_bbox_marching.comp:124-322, 345-531):
  // the same three-stage integration for both cones, parameterised by table.
  __device__ float cone(const float4* tab, const ConeTableDev& T, float3 pos, float3 k, float3 u, float3 v,
                        const FrameArgs& f, unsigned& aux) const {
    aux += T.n1 + 3 * T.n3 + 7 * T.n7;
    float rays[7], last[7];
    float track = T.initial_step;
    rays[0] = 0.0f; last[0] = 0.0f;
    // Cone1Ray*: one sample per section.
    for (int i = 0; i < T.n1; ++i) {
      float4 s = tab[i];
      float tau = gauss_ext(pos + k * track, s.y, f);
      float amptau = tau * s.w;
      rays[0] += (last[0] + amptau) * s.z * T.ui_weight;
      last[0] = amptau;
      track += s.x;
    }
    if (T.n3 + T.n7 == 0) return expf(-rays[0]);
    // Cone3Ray*: transform 1 -> 3.
    rays[2] = rays[0]; rays[1] = rays[0];
    last[2] = last[0]; last[1] = last[0];
    {
      float3 vk[3];
#pragma unroll
      for (int r = 0; r < 3; ++r) vk[r] = k * T.axes[r].z + u * T.axes[r].y + v * T.axes[r].x;
      for (int i = 0; i < T.n3; ++i) {
        float4 s = tab[T.n1 + i];
#pragma unroll
        for (int r = 0; r < 3; ++r) {
          float tau = gauss_ext(pos + vk[r] * track, s.y, f);
          float amptau = tau * s.w;
          rays[r] += (last[r] + amptau) * s.z * T.ui_weight;
          last[r] = amptau;
        }
        track += s.x;
      }
    }
    if (T.n7 == 0) return (expf(-rays[0]) + expf(-rays[1]) + expf(-rays[2])) / 3.0f;
    // Cone7Ray*: transform 3 -> 7.
    rays[6] = rays[5] = rays[2];
    rays[4] = rays[3] = rays[1];
    float avg = (rays[2] + rays[1] + rays[0]) / 3.0f;
    rays[2] = rays[1] = rays[0];
    rays[0] = avg;
    last[6] = last[5] = last[2];
    last[4] = last[3] = last[1];
    float avgt = (last[2] + last[1] + last[0]) / 3.0f;
    last[2] = last[1] = last[0];
    last[0] = avgt;
    float3 vk[7];
#pragma unroll
    for (int r = 0; r < 7; ++r) vk[r] = k * T.axes[3 + r].z + u * T.axes[3 + r].y + v * T.axes[3 + r].x;
    int step0 = T.n1 + T.n3;
    for (int i = 0; i < T.n7; ++i) {
      float4 s = tab[step0 + i];
#pragma unroll
      for (int r = 0; r < 7; ++r) {
        float tau = gauss_ext(pos + vk[r] * track, s.y, f);
        float amptau = tau * s.w;
        rays[r] += (last[r] + amptau) * s.z * T.ui_weight;
        last[r] = amptau;
      }
      track += s.x;
    }
    return (expf(-rays[0]) + (expf(-rays[1]) + expf(-rays[2]) + expf(-rays[3]) + expf(-rays[4]) +
                              expf(-rays[5]) + expf(-rays[6])) * T.w7) / (1.0f + T.w7 * 6.0f);
  }

  // OcclusionEvaluationKernel (ray_bbox_marching.comp:324-333).
  __device__ __forceinline__ float occlusion(float3 tx, const Ray& r, const FrameArgs& f, unsigned& aux) const {
    float3 realpos = tx - f.vol.grid * 0.5f;
    float3 k = normalize3(f.cam.eye - realpos);
    return cone(occ_tab, d->occ, tx, k, r.v_up, r.v_right, f, aux);
  }

  // ShadowEvaluationKernel (ray_bbox_marching.comp:533-562).  Cone1RayShadow
  // declares its parameters as (pos, k, v, u) and is called with (pos, k, u, v),
  // so the shadow cone works in the swapped frame; that is kept.
  __device__ __forceinline__ float shadow(float3 tx, const FrameArgs& f, unsigned& aux) const {
    float3 k, u, v;
    if (d->shadow_type == 0 || d->shadow_type == 1) {
      k = normalize3(d->light_pos - (tx - f.vol.grid * 0.5f));
      u = normalize3(cross3(k, d->light_right));
      v = normalize3(cross3(k, u));
      if (d->shadow_type == 1 && dot3(k, d->light_fwd) < d->spot_cos_max) return 0.0f;
    } else {
      k = d->light_fwd; v = d->light_up; u = d->light_right;
    }
    return cone(sdw_tab, d->sdw, tx, k, v, u, f, aux);
  }

  // ShadeSample (ray_bbox_marching.comp:607-656).
  __device__ __forceinline__ float4 shade(float4 src, float3 tx, const Ray& r, const FrameArgs& f, unsigned& aux) const {
    float ka = 0.0f, kd = 0.0f, io = 0.0f, is = 0.0f;
    if (d->apply_occ) { ka = d->ka; io = occlusion(tx, r, f, aux); }
    if (d->apply_sdw) { kd = d->kd; is = shadow(tx, f, aux); }
    if (f.grad.g) return phong_cone(f, src, tx, io, ka, is, kd);
    float kk = 1.0f / (ka + kd);
    src.x = kk * (src.x * io * ka + src.x * is * kd);
    src.y = kk * (src.y * io * ka + src.y * is * kd);
    src.z = kk * (src.z * io * ka + src.z * is * kd);
    return src;
  }
};
using DosShade = DosShadeT<false>;


// ================================================= ground truth (rc1pcrtgt)
struct GtShade {
  const GtArgs* g;
  const float4* tf;
  int tf_n;
  const float3* occ_vec;  // shared-memory copies
  const float3* sdw_vec;
  struct Ray { float3 dir, v_up, v_right; };

  // main(), gt_ray_marching.comp:396-399.
  __device__ __forceinline__ void begin(Ray& r, float3 dir) const {
    r.dir = dir;
    r.v_right = normalize3(cross3(dir, f3(0.0f, 1.0f, 0.0f)));
    r.v_up = normalize3(cross3(-dir, r.v_right));
  }

  // One light ray of ConeOcclusion/ShadowsEvaluationRayCasting
  // (gt_ray_marching.comp:125-159 and 209-242): trapezoidal transmittance.
  __device__ float light_ray(float3 tx, float3 w, float dist, const FrameArgs& f, unsigned& aux) const {
    float vt = 1.0f;
    ++aux;
    float s = g->gap;
    float3 S = f.vol.grid;
    float st0 = tf_alpha(tf, tf_n, sample_volume(f.vol, tx + w * s));
    for (int guard = 0; guard < kMaxLightSteps && s < dist; ++guard) {
      float h = fminf(g->lstep, dist - s);
      float3 at = tx + w * (s + h);
      if (at.x < 0.0f || at.x > S.x || at.y < 0.0f || at.y > S.y || at.z < 0.0f || at.z > S.z) break;
      float st1 = tf_alpha(tf, tf_n, sample_volume(f.vol, at));
      ++aux;
      vt *= expf(-((st0 + st1) * 0.5f) * h);
      if ((1.0f - vt) > 0.99f) break;
      st0 = st1;
      s = s + h;
    }
    return vt;
  }

  // ConeOcclusionEvaluationRayCasting (gt_ray_marching.comp:109-169).
  __device__ float occlusion(float3 tx, const Ray& r, const FrameArgs& f, unsigned& aux) const {
    float socc = 0.0f, swgt = 0.0f;
    float3 vd = normalize3(-r.dir);
    for (int i = 0; i < g->n_occ; ++i) {
      float3 c = occ_vec[i];
      float3 w = normalize3(r.v_right * c.x + r.v_up * c.y + vd * c.z);
      float vt = light_ray(tx, w, g->occ_dist, f, aux);
      float rw = dot3(vd, w);
      socc += vt * rw;
      swgt += rw;
    }
    return socc / swgt;
  }

  // ConeShadowsEvaluationRayCasting (gt_ray_marching.comp:171-252).
  __device__ float shadow(float3 tx, const FrameArgs& f, unsigned& aux) const {
    float3 wpos = tx - f.vol.grid * 0.5f;
    float3 vd, vu, vr;
    if (g->shadow_type == 0 || g->shadow_type == 1) {
      vd = normalize3(g->light_pos - wpos);
      vu = normalize3(cross3(vd, g->light_right));
      vr = normalize3(cross3(vd, vu));
      // The reference compares a cosine against 30.0 here, so spot lights always return 0.
      if (g->shadow_type == 1 && dot3(vd, g->light_fwd) < 30.0f) return 0.0f;
    } else {
      vd = g->light_fwd; vu = g->light_up; vr = g->light_right;
    }
    float ssdw = 0.0f, swgt = 0.0f;
    for (int i = 0; i < g->n_sdw; ++i) {
      float3 c = sdw_vec[i];
      float3 w = normalize3(vr * c.x + vu * c.y + vd * c.z);
      float vt = light_ray(tx, w, g->sdw_dist, f, aux);
      float rw = dot3(vd, w);
      ssdw += vt * rw;
      swgt += rw;
    }
    return ssdw / swgt;
  }

  // ShadeSample (gt_ray_marching.comp:254-303).
  __device__ __forceinline__ float4 shade(float4 src, float3 tx, const Ray& r, const FrameArgs& f, unsigned& aux) const {
    float ka = 0.0f, kd = 0.0f, io = 0.0f, is = 0.0f;
    if (g->apply_occ) { ka = g->ka; io = occlusion(tx, r, f, aux); }
    if (g->apply_sdw) { kd = g->kd; is = shadow(tx, f, aux); }
    if (f.grad.g) return phong_cone(f, src, tx, io, ka, is, kd);
    float kk = 1.0f / (ka + kd);
    src.x = kk * (src.x * io * ka + src.x * is * kd);
    src.y = kk * (src.y * io * ka + src.y * is * kd);
    src.z = kk * (src.z * io * ka + src.z * is * kd);
    return src;
  }
};

// ============================================================ primary loop
// The warp's log2 width in pixels (warps of 4x8, 8x4 or 16x2 pixels).
__device__ __forceinline__ int warp_shift(int warp_w) { return warp_w == 4 ? 2 : (warp_w == 16 ? 4 : 3); }

__device__ __forceinline__ void pixel_of(const FrameArgs& f, int& px, int& py) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, wl = warp_shift(f.warp_w);
  const int warps_x = f.tile_w >> wl;
  px = blockIdx.x * f.tile_w + (warp % warps_x) * (1 << wl) + (lane & ((1 << wl) - 1));
  py = blockIdx.y * f.tile_h + (warp / warps_x) * (32 >> wl) + (lane >> wl);
}

__device__ __forceinline__ void add_stats(const FrameArgs& f, unsigned int n, unsigned int shaded, unsigned int aux) {
  unsigned long long a = n, b = shaded, c = aux;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_down_sync(0xffffffffu, a, o);
    b += __shfl_down_sync(0xffffffffu, b, o);
    c += __shfl_down_sync(0xffffffffu, c, o);
  }
  if ((threadIdx.x & 31) == 0 && f.stats) {
    atomicAdd(f.stats + 0, a);
    atomicAdd(f.stats + 1, b);
    atomicAdd(f.stats + 2, c);
  }
}

// The a5 loop (ray_marching_1p.comp:170-247): h = min(StepSize, D - s),
// sample at s + h/2, skip transparent samples, alpha = 1 - exp(-sigma h),
// front-to-back composite, stop once alpha > 0.99.
template <class Shade>
__device__ __forceinline__ void march_ray(const FrameArgs& f, const float4* tf, const Shade& sh, int px, int py) {
  bool inside = px < f.W && py < f.H;
  unsigned int n = 0, shaded = 0, aux = 0;
  if (inside) {
    float3 dir = primary_dir(f.cam, px, py, f.W, f.H);
    float tnear, tfar;
    float4 dst = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    if (ray_aabb(f.cam.eye, dir, f.vol.grid, tnear, tfar)) {
      typename Shade::Ray ray;
      sh.begin(ray, dir);
      float D = fabsf(tfar - tnear);
      float3 tex0 = f.cam.eye + dir * tnear + f.vol.grid * 0.5f;
      // Bound on the step count (never reached for validated step sizes):
      // keeps a loop whose s stops advancing from spinning forever.
      const unsigned max_iter = (unsigned)fminf(D / f.step, 1.0e9f) + 4u;
      for (float s = 0.0f; s < D && n < max_iter;) {
        float h = fminf(f.step, D - s);
        float3 p = tex0 + dir * (s + h * 0.5f);
        float density = sample_volume(f.vol, p);
        float4 src = tf_lookup(tf, f.tf_n, density);
        ++n;
        if (src.w > 0.0f) {
          ++shaded;
          src = sh.shade(src, p, ray, f, aux);
          src.w = 1.0f - expf(-src.w * h);
          src.x *= src.w; src.y *= src.w; src.z *= src.w;
          float r = 1.0f - dst.w;
          dst.x += r * src.x; dst.y += r * src.y; dst.z += r * src.z; dst.w += r * src.w;
          if (dst.w > 0.99f) break;
        }
        s = s + h;
      }
    }
    size_t o = (size_t)py * f.W + px;
    f.out[o] = dst;
    if (f.counts) f.counts[o] = n;
  }
  add_stats(f, n, shaded, aux);
}

// One CTA-tile pixel per thread (pixel_of).
template <class Shade>
__device__ __forceinline__ void march_pixel(const FrameArgs& f, const float4* tf, const Shade& sh) {
  int px, py;
  pixel_of(f, px, py);
  march_ray(f, tf, sh, px, py);
}

// ============================================ persistent marcher, ray refill
// Next ray index for every active lane of a warp with one atomic.
__device__ __forceinline__ unsigned take_ray(unsigned int* work) {
  const unsigned m = __activemask();
  const int lane = threadIdx.x & 31;
  const int leader = __ffs(m) - 1;
  unsigned base = 0;
  if (lane == leader) base = atomicAdd(work, (unsigned)__popc(m));
  base = __shfl_sync(m, base, leader);
  return base + (unsigned)__popc(m & ((1u << lane) - 1u));
}

// Square spiral of 8x4-pixel tiles around the tile (cx, cy): sequence number
// k -> ring r = ceil((sqrt(k+1) - 1) / 2), then the position on that ring.
// Tiles near the projected volume centre (the longest rays) come first and
// consecutive tiles are neighbours, so the CTAs' working sets overlap.
__device__ __forceinline__ void spiral_tile(unsigned k, int& dx, int& dy) {
  if (k == 0) { dx = dy = 0; return; }
  int r = (int)((sqrtf((float)k + 1.0f) - 1.0f) * 0.5f);
  while ((unsigned)(2 * r + 1) * (unsigned)(2 * r + 1) <= k) ++r;  // fix float rounding
  while (r > 0 && (unsigned)(2 * r - 1) * (unsigned)(2 * r - 1) > k) --r;
  const int m = (int)(k - (unsigned)(2 * r - 1) * (unsigned)(2 * r - 1));
  const int side = m / (2 * r), off = m % (2 * r);
  switch (side) {
    case 0: dx = r; dy = -r + 1 + off; break;
    case 1: dx = r - 1 - off; dy = r; break;
    case 2: dx = -r; dy = r - 1 - off; break;
    default: dx = -r + 1 + off; dy = -r; break;
  }
}


// Ray order of the persistent marchers: 8x4-pixel tiles in the square spiral
// around the tile of the projected volume centre (long rays first,
// neighbouring tiles together); total = 32 x the tiles of the spiral's
// bounding square (positions outside the image are skipped).
struct RayOrder {
  int cx, cy, tiles_x, tiles_y;
  unsigned total;
};

// The a5 loop with persistent ray refill and warp-ballot control flow: each
// lane advances its own ray to its next shaded sample, then the lanes with a
// pending sample run ShadeSample together (the expensive light integrals run
// with the warp's lanes aligned); a lane whose ray ends (front-to-back
// termination or the far side of the box) writes its pixel and takes the
// next ray of the frame from *work, so no lane idles until the longest ray of
// its tile ends.  The warp leaves when a ballot finds no lane with a ray.
// Same arithmetic per ray as march_ray.
template <class Shade>
__device__ __forceinline__ void march_refill(const FrameArgs& f, const float4* tf, const Shade& sh, unsigned* work,
                                             const RayOrder& o) {
  unsigned n_all = 0, shaded = 0, aux = 0;
  bool have = false, done = false;
  int px = 0, py = 0;
  float3 dir = f3(0.0f, 0.0f, 1.0f), tex0 = f3(0.0f, 0.0f, 0.0f);
  float D = 0.0f, s = 0.0f;
  float4 dst = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  unsigned n = 0, max_iter = 0;
  typename Shade::Ray ray;
  auto finish = [&]() {
    const size_t off = (size_t)py * f.W + px;
    f.out[off] = dst;
    if (f.counts) f.counts[off] = n;
    n_all += n;
    have = false;
  };
  for (;;) {
    // lanes without a ray take new ones; rays that miss the box are written at once
    while (!have && !done) {
      const unsigned idx = take_ray(work);
      if (idx >= o.total) { done = true; break; }
      int dx, dy;
      spiral_tile(idx >> 5, dx, dy);
      const int tx = o.cx + dx, ty = o.cy + dy;
      if (tx < 0 || ty < 0 || tx >= o.tiles_x || ty >= o.tiles_y) continue;
      px = tx * 8 + (int)(idx & 7u);
      py = ty * 4 + (int)((idx >> 3) & 3u);
      if (px >= f.W || py >= f.H) continue;
      dir = primary_dir(f.cam, px, py, f.W, f.H);
      dst = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
      n = 0;
      float tnear, tfar;
      if (!ray_aabb(f.cam.eye, dir, f.vol.grid, tnear, tfar)) {
        finish();
        continue;
      }
      sh.begin(ray, dir);
      D = fabsf(tfar - tnear);
      tex0 = f.cam.eye + dir * tnear + f.vol.grid * 0.5f;
      s = 0.0f;
      max_iter = (unsigned)fminf(D / f.step, 1.0e9f) + 4u;
      have = true;
    }
    if (__ballot_sync(0xffffffffu, have) == 0u) break;
    bool pending = false;
    float4 src = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    float3 p = f3(0.0f, 0.0f, 0.0f);
    float h = 0.0f;
    if (have) {
      while (s < D && n < max_iter) {
        h = fminf(f.step, D - s);
        p = tex0 + dir * (s + h * 0.5f);
        src = tf_lookup(tf, f.tf_n, sample_volume(f.vol, p));
        ++n;
        if (src.w > 0.0f) { pending = true; break; }
        s = s + h;
      }
      if (!pending) finish();
    }
    if (pending) {
      ++shaded;
      src = sh.shade(src, p, ray, f, aux);
      src.w = 1.0f - expf(-src.w * h);
      src.x *= src.w; src.y *= src.w; src.z *= src.w;
      const float r = 1.0f - dst.w;
      dst.x += r * src.x; dst.y += r * src.y; dst.z += r * src.z; dst.w += r * src.w;
      s = s + h;
      if (dst.w > 0.99f) finish();
    }
  }
  add_stats(f, n_all, shaded, aux);
}

// The spiral order of a frame: centred on the pixel where the volume centre
// projects (the frame centre when it projects behind or far off the camera).
inline RayOrder ray_order(const FrameArgs& f) {
  const float3 d = f3(0.0f, 0.0f, 0.0f) - f.cam.eye;
  const float zf = dot3(d, f.cam.f);
  int px = f.W / 2, py = f.H / 2;
  if (zf > 1e-6f) {
    const float xn = dot3(d, f.cam.s) / (zf * f.cam.tan_half_fovy * f.cam.aspect);
    const float yn = dot3(d, f.cam.u) / (zf * f.cam.tan_half_fovy);
    if (xn == xn && yn == yn && fabsf(xn) < 4.0f && fabsf(yn) < 4.0f) {
      px = (int)((xn * 0.5f + 0.5f) * (float)f.W);
      py = (int)((yn * 0.5f + 0.5f) * (float)f.H);
    }
  }
  RayOrder o;
  o.tiles_x = (f.W + 7) / 8;
  o.tiles_y = (f.H + 3) / 4;
  o.cx = px / 8 < 0 ? 0 : (px / 8 >= o.tiles_x ? o.tiles_x - 1 : px / 8);
  o.cy = py / 4 < 0 ? 0 : (py / 4 >= o.tiles_y ? o.tiles_y - 1 : py / 4);
  const int R = std::max(std::max(o.cx, o.tiles_x - 1 - o.cx), std::max(o.cy, o.tiles_y - 1 - o.cy));
  o.total = (unsigned)(2 * R + 1) * (unsigned)(2 * R + 1) * 32u;  // frames <= 32768^2: below 2^32
  return o;
}

// Loads the RGBt table into shared memory (n <= tf_smem_cap) and returns it.
__device__ __forceinline__ const float4* stage_tf(const FrameArgs& f, float4* smem) {
  for (int i = threadIdx.x; i < f.tf_n; i += blockDim.x) smem[i] = f.tf[i];
  return smem;
}

}  // namespace cvr
