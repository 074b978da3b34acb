// cvr_oracle.cpp — TEST INFRASTRUCTURE ONLY (the parity checker and the timed
// CPU baseline).  Nothing in the product links, loads or calls this file.
//
// A CPU restatement of the reference's rendering shaders and table builders,
// templated on the arithmetic type: T = double is the FP64 oracle every GPU
// image is compared with; T = float reproduces the shaders' single-precision
// arithmetic (and is the timed CPU baseline).  Texture fetches emulate OpenGL
// texture() on normalised coordinates: texel centres at (i+0.5)/n,
// clamp-to-edge, exact (tri)linear weights.  Not emulated: FP16 texture
// storage (R16F volume, RGBA16F tables, R16F pyramid) and 8-bit hardware
// filter weights.
//
// Parity pinning: the table builders this file relies on (TransferFunction1D
// tables, the extinction SAT, the cone section tables, the GT kernel vectors)
// are checked against the reference's own C++ compiled from its sources
// (oracle/build_ref.py) and against golden vectors generated from it.  The
// GLSL marching loops themselves cannot run here (no OpenGL on either
// machine), so the loops below are restatements of the shader text, cited per
// function.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "../include/cvr.h"

namespace {

template <class T>
struct V3 {
  T x, y, z;
};
template <class T> V3<T> v3(T x, T y, T z) { return V3<T>{x, y, z}; }
template <class T> V3<T> operator+(V3<T> a, V3<T> b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <class T> V3<T> operator-(V3<T> a, V3<T> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <class T> V3<T> operator-(V3<T> a) { return {-a.x, -a.y, -a.z}; }
template <class T> V3<T> operator*(V3<T> a, V3<T> b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
template <class T> V3<T> operator/(V3<T> a, V3<T> b) { return {a.x / b.x, a.y / b.y, a.z / b.z}; }
template <class T> V3<T> operator*(V3<T> a, T s) { return {a.x * s, a.y * s, a.z * s}; }
template <class T> T dot(V3<T> a, V3<T> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <class T> V3<T> cross(V3<T> a, V3<T> b) {
  return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
template <class T> V3<T> normalize(V3<T> a) { return a * (T(1) / std::sqrt(dot(a, a))); }
template <class T> V3<T> vmin(V3<T> a, V3<T> b) { return {std::min(a.x, b.x), std::min(a.y, b.y), std::min(a.z, b.z)}; }
template <class T> V3<T> vmax(V3<T> a, V3<T> b) { return {std::max(a.x, b.x), std::max(a.y, b.y), std::max(a.z, b.z)}; }
template <class T> V3<T> vclamp(V3<T> v, V3<T> lo, V3<T> hi) { return vmin(vmax(v, lo), hi); }
template <class T> V3<T> vabs(V3<T> a) { return {std::fabs(a.x), std::fabs(a.y), std::fabs(a.z)}; }
template <class T> V3<T> from(const float* p) { return {T(p[0]), T(p[1]), T(p[2])}; }

template <class T>
struct V4 {
  T r, g, b, a;
};

struct Scene {
  int nx = 0, ny = 0, nz = 0, dtype = 0;
  double sx = 1, sy = 1, sz = 1;
  std::vector<uint8_t> vox;
  std::vector<float> rgbt, rgba;
  int tf_n = 0;
  std::vector<double> sat64;  // restated GenerateExtinctionSAT3DTex (FP64)
  std::vector<float> sat32;   // the same downcast to float (the reference's R32F upload)
  bool sat_ready = false;
  int n_levels = 0;
  int ldims[16][3];
  size_t loff[16];
  std::vector<double> pyr64;
  std::vector<float> pyr32;
  bool pyr_ready = false;
  cvr_cone_table occ{}, sdw{};
  bool cone_ready = false;
  std::vector<float> occ_vec, sdw_vec;
  bool gt_ready = false;
  std::vector<float> mlp;  // surrogate network parameters (CVR_MLP_PARAMS floats)
  int lc[3] = {0, 0, 0};   // object-space light cache dims (0: off)
  std::vector<float> grad; // per-voxel gradient, 3 per voxel, FP16-rounded (the RGB16F texture)
  bool grad_ready = false;
  cvr_blinn_phong bp{0, 0.5f, 0.5f, 0.8f, 30.0f, {1.0f, 1.0f, 1.0f}};

  double vox_norm(size_t i) const {
    if (dtype == CVR_U8) return (double)vox[i] / 255.0;
    uint16_t v;
    std::memcpy(&v, &vox[2 * i], 2);
    return (double)v / 65535.0;
  }
};

// ------------------------------------------------------------ GL sampling
template <class T>
struct Tap {
  int i0, i1;
  T t;
};
template <class T> Tap<T> axis_tap(T u, int n) {
  T fl = std::floor(u);
  int i = (int)fl;
  Tap<T> r;
  r.t = u - fl;
  r.i0 = std::min(std::max(i, 0), n - 1);
  r.i1 = std::min(std::max(i + 1, 0), n - 1);
  return r;
}

// texture(TexVolume, p / VolumeGridSize).r; p in [0, S] world units.
template <class T> T sample_volume(const Scene& s, V3<T> p) {
  V3<T> grid = v3<T>(T(s.nx * s.sx), T(s.ny * s.sy), T(s.nz * s.sz));
  Tap<T> tx = axis_tap<T>(p.x / grid.x * T(s.nx) - T(0.5), s.nx);
  Tap<T> ty = axis_tap<T>(p.y / grid.y * T(s.ny) - T(0.5), s.ny);
  Tap<T> tz = axis_tap<T>(p.z / grid.z * T(s.nz) - T(0.5), s.nz);
  auto at = [&](int x, int y, int z) {
    return (T)s.vox_norm((size_t)x + (size_t)s.nx * ((size_t)y + (size_t)s.ny * z));
  };
  T c000 = at(tx.i0, ty.i0, tz.i0), c100 = at(tx.i1, ty.i0, tz.i0);
  T c010 = at(tx.i0, ty.i1, tz.i0), c110 = at(tx.i1, ty.i1, tz.i0);
  T c001 = at(tx.i0, ty.i0, tz.i1), c101 = at(tx.i1, ty.i0, tz.i1);
  T c011 = at(tx.i0, ty.i1, tz.i1), c111 = at(tx.i1, ty.i1, tz.i1);
  T c00 = c000 + tx.t * (c100 - c000), c10 = c010 + tx.t * (c110 - c010);
  T c01 = c001 + tx.t * (c101 - c001), c11 = c011 + tx.t * (c111 - c011);
  T c0 = c00 + ty.t * (c10 - c00), c1 = c01 + ty.t * (c11 - c01);
  return c0 + tz.t * (c1 - c0);
}

// texture(TexTransferFunc, density) on an n-entry RGBA table.
template <class T> V4<T> tf_lookup(const std::vector<float>& tf, int n, T d) {
  Tap<T> t = axis_tap<T>(d * T(n) - T(0.5), n);
  const float* a = &tf[4 * (size_t)t.i0];
  const float* b = &tf[4 * (size_t)t.i1];
  V4<T> r;
  r.r = T(a[0]) + t.t * (T(b[0]) - T(a[0]));
  r.g = T(a[1]) + t.t * (T(b[1]) - T(a[1]));
  r.b = T(a[2]) + t.t * (T(b[2]) - T(a[2]));
  r.a = T(a[3]) + t.t * (T(b[3]) - T(a[3]));
  return r;
}

// ------------------------------------------------------------ camera
template <class T>
struct Cam {
  V3<T> eye, s, u, f;
  T tanf, aspect;
};
// glm::lookAt(eye, center, up) (camera.cpp:281-284) and the row-vector product
// of ray_marching_1p.comp:170.
template <class T> Cam<T> make_cam(const cvr_camera& c, int w, int h) {
  Cam<T> k;
  k.eye = from<T>(c.eye);
  V3<T> f = normalize(from<T>(c.center) - k.eye);
  V3<T> s = normalize(cross(f, from<T>(c.up)));
  k.s = s; k.f = f; k.u = cross(s, f);
  k.tanf = (T)std::tan((double)c.fovy_deg * (3.14159265358979323846 / 180.0) / 2.0);
  k.aspect = c.aspect > 0.0f ? T(c.aspect) : T(float(w) / float(h));
  return k;
}
template <class T> V3<T> primary_dir(const Cam<T>& c, int x, int y, int W, int H) {
  T vx = ((T(x) + T(0.5)) / T(W)) * T(2) - T(1);
  T vy = ((T(y) + T(0.5)) / T(H)) * T(2) - T(1);
  return normalize(c.s * (vx * c.tanf * c.aspect) + c.u * (vy * c.tanf) + c.f);
}

// IntersectBox / RayAABBIntersection (ray_bbox_intersection.comp:18-52).
template <class T> bool ray_aabb(V3<T> o, V3<T> d, V3<T> grid, T& tnear, T& tfar) {
  V3<T> bmin = grid * T(-0.5), bmax = grid * T(0.5);
  V3<T> inv = v3<T>(T(1) / d.x, T(1) / d.y, T(1) / d.z);
  V3<T> t0 = inv * (bmin - o), t1 = inv * (bmax - o);
  V3<T> tmin = vmin(t0, t1), tmax = vmax(t0, t1);
  tnear = std::max(std::max(tmin.x, tmin.y), tmin.z);
  tfar = std::min(std::min(tmax.x, tmax.y), tmax.z);
  bool hit = tfar > tnear;
  tnear = std::max(tnear, T(0));
  return hit;
}

// ------------------------------------------------------------ frame state
template <class T>
struct Frame {
  const Scene* s;
  V3<T> spacing, grid;
  Cam<T> cam;
  T step;
};

// ------------------------------------------------------------ extinction
template <class T>
struct Ext {
  const cvr_ext_params* p;
  V3<T> light_pos, light_fwd;
  const T* sat;  // (nx+2)(ny+2)(nz+2) in T
  int sx, sy, sz;
};

// GetSummed3Density: texture(TexVolumeSAT3D, p * inv_vol_scaled) with
// inv_vol_scaled = 1 / (S + 2 spacing) (ebs_ray_bbox_marching.comp:73-83).
template <class T> T sat_fetch(const Frame<T>& f, const Ext<T>& e, V3<T> p) {
  V3<T> ext = f.grid + f.spacing * T(2);
  Tap<T> tx = axis_tap<T>(p.x / ext.x * T(e.sx) - T(0.5), e.sx);
  Tap<T> ty = axis_tap<T>(p.y / ext.y * T(e.sy) - T(0.5), e.sy);
  Tap<T> tz = axis_tap<T>(p.z / ext.z * T(e.sz) - T(0.5), e.sz);
  auto at = [&](int x, int y, int z) { return e.sat[(size_t)x + (size_t)e.sx * ((size_t)y + (size_t)e.sy * z)]; };
  T c000 = at(tx.i0, ty.i0, tz.i0), c100 = at(tx.i1, ty.i0, tz.i0);
  T c010 = at(tx.i0, ty.i1, tz.i0), c110 = at(tx.i1, ty.i1, tz.i0);
  T c001 = at(tx.i0, ty.i0, tz.i1), c101 = at(tx.i1, ty.i0, tz.i1);
  T c011 = at(tx.i0, ty.i1, tz.i1), c111 = at(tx.i1, ty.i1, tz.i1);
  T c00 = c000 + tx.t * (c100 - c000), c10 = c010 + tx.t * (c110 - c010);
  T c01 = c001 + tx.t * (c101 - c001), c11 = c011 + tx.t * (c111 - c011);
  T c0 = c00 + ty.t * (c10 - c00), c1 = c01 + ty.t * (c11 - c01);
  return c0 + tz.t * (c1 - c0);
}

// EvaluateSAT3D (ebs_ray_bbox_marching.comp:87-100).
template <class T> T eval_sat(const Frame<T>& f, const Ext<T>& e, V3<T> p1, V3<T> p2) {
  T V1 = sat_fetch(f, e, v3(p2.x, p2.y, p2.z));
  T V2 = sat_fetch(f, e, v3(p1.x, p2.y, p2.z));
  T V3_ = sat_fetch(f, e, v3(p2.x, p2.y, p1.z));
  T V4_ = sat_fetch(f, e, v3(p1.x, p2.y, p1.z));
  T V5 = sat_fetch(f, e, v3(p2.x, p1.y, p2.z));
  T V6 = sat_fetch(f, e, v3(p1.x, p1.y, p2.z));
  T V7 = sat_fetch(f, e, v3(p2.x, p1.y, p1.z));
  T V8 = sat_fetch(f, e, v3(p1.x, p1.y, p1.z));
  return (V1 - V2 - V3_ + V4_ - V5 + V6 + V7 - V8);
}

// EvaluateAmbientOcclusionSAT3D (:102-110).
template <class T> T ao_sat(const Frame<T>& f, const Ext<T>& e, V3<T> p1, V3<T> p2) {
  V3<T> mn = f.spacing * T(0.5), mx = f.grid + f.spacing * T(1.5);
  p1 = vclamp(p1 + f.spacing, mn, mx);
  p2 = vclamp(p2 + f.spacing, mn, mx);
  return eval_sat(f, e, p1, p2);
}

// ExtinctionAmbientOcclusion (:112-146) with shell radii from a list.
template <class T> T ext_ao(const Frame<T>& f, const Ext<T>& e, V3<T> tx) {
  T r0 = T(e.p->ao_radii[0]);
  T sat0 = ao_sat(f, e, tx - f.spacing * r0, tx + f.spacing * r0);
  T tsh = sat0 * (T(1) / (r0 * r0));
  T sat_i = sat0;
  for (int i = 1; i < e.p->ao_n_shells; ++i) {
    T ri = T(e.p->ao_radii[i]);
    T sat_n = ao_sat(f, e, tx - f.spacing * ri, tx + f.spacing * ri);
    tsh = tsh + (sat_n - sat_i) * (T(1) / (ri * ri));
    sat_i = sat_n;
  }
  T rk = T(e.p->ao_radii[e.p->ao_n_shells - 1]);
  T wa = T(1) / (rk * rk);
  return std::exp(-(wa * tsh));
}

// EvaluateShadowSAT3D, texture() branch (:173-187).
template <class T> T shadow_sat(const Frame<T>& f, const Ext<T>& e, V3<T> p1, V3<T> p2) {
  V3<T> sc = f.spacing;
  T volq = (std::fabs(p1.x - p2.x) / sc.x) * (std::fabs(p1.y - p2.y) / sc.y) * (std::fabs(p1.z - p2.z) / sc.z);
  V3<T> mn = sc * T(0.5), mx = f.grid + sc * T(1.5);
  p1 = vclamp(p1 + sc, mn, mx);
  p2 = vclamp(p2 + sc, mn, mx);
  return (eval_sat(f, e, p1, p2) / volq) * T(e.p->sdw_ui_weight);
}

// One cone walk along a dominant axis: ConeZAxis / ConeYAxis / ConeXAxis
// (:190-430).  'ax' is the marching axis; (a, b) are the two secondary axes in
// the order the reference names them (Z: x,y; Y: x,z; X: y,z), and the
// rotation formulas of the projected cone-boundary vectors follow each
// function's text.
template <class T> T cone_axis(const Frame<T>& f, const Ext<T>& e, V3<T> pos, V3<T> c, int ax) {
  auto comp = [](V3<T> v, int i) { return i == 0 ? v.x : (i == 1 ? v.y : v.z); };
  V3<T> sc = f.spacing;
  T st = 0;
  T ang = T(e.p->sdw_cone_angle_rad);
  T p_cs = std::cos(ang), p_sn = std::sin(ang), n_cs = std::cos(-ang), n_sn = std::sin(-ang);
  V3<T> pa1, pa2, pb1, pb2;  // projected boundary vectors of the two secondary axes
  int sa, sb;
  if (ax == 2) {  // ConeZAxis
    sa = 0; sb = 1;
    V3<T> proj_y = normalize(v3<T>(0, c.y, c.z)), proj_x = normalize(v3<T>(c.x, 0, c.z));
    pa1 = normalize(v3<T>(proj_x.x * n_cs - proj_x.z * n_sn, 0, proj_x.x * n_sn + proj_x.z * n_cs));
    pa2 = normalize(v3<T>(proj_x.x * p_cs - proj_x.z * p_sn, 0, proj_x.x * p_sn + proj_x.z * p_cs));
    pb1 = normalize(v3<T>(0, proj_y.y * n_cs - proj_y.z * n_sn, proj_y.y * n_sn + proj_y.z * n_cs));
    pb2 = normalize(v3<T>(0, proj_y.y * p_cs - proj_y.z * p_sn, proj_y.y * p_sn + proj_y.z * p_cs));
  } else if (ax == 1) {  // ConeYAxis
    sa = 0; sb = 2;
    V3<T> proj_x = normalize(v3<T>(c.x, c.y, 0)), proj_z = normalize(v3<T>(0, c.y, c.z));
    pa1 = normalize(v3<T>(proj_x.x * n_cs - proj_x.y * n_sn, proj_x.x * n_sn + proj_x.y * n_cs, 0));
    pa2 = normalize(v3<T>(proj_x.x * p_cs - proj_x.y * p_sn, proj_x.x * p_sn + proj_x.y * p_cs, 0));
    pb1 = normalize(v3<T>(0, proj_z.z * n_sn + proj_z.y * n_cs, proj_z.z * n_cs - proj_z.y * n_sn));
    pb2 = normalize(v3<T>(0, proj_z.z * p_sn + proj_z.y * p_cs, proj_z.z * p_cs - proj_z.y * p_sn));
  } else {  // ConeXAxis
    sa = 1; sb = 2;
    V3<T> proj_y = normalize(v3<T>(c.x, c.y, 0)), proj_z = normalize(v3<T>(c.x, 0, c.z));
    pa1 = normalize(v3<T>(proj_y.y * n_sn + proj_y.x * n_cs, proj_y.y * n_cs - proj_y.x * n_sn, 0));
    pa2 = normalize(v3<T>(proj_y.y * p_sn + proj_y.x * p_cs, proj_y.y * p_cs - proj_y.x * p_sn, 0));
    pb1 = normalize(v3<T>(proj_z.z * n_sn + proj_z.x * n_cs, 0, proj_z.z * n_cs - proj_z.x * n_sn));
    pb2 = normalize(v3<T>(proj_z.z * p_sn + proj_z.x * p_cs, 0, proj_z.z * p_cs - proj_z.x * p_sn));
  }
  T cm = comp(c, ax);
  T signal = cm < 0 ? T(-1) : T(1);
  T sca = comp(sc, sa), scb = comp(sc, sb), scm = comp(sc, ax);
  T interval = T(e.p->sdw_sample_interval) * signal * scm;
  T mp = T(e.p->sdw_initial_step) * signal * scm;
  T vmin_ = scm * T(0.5), vmax_ = comp(f.grid, ax) - scm * T(0.5);
  T pm = comp(pos, ax);
  while ((mp / cm) < T(e.p->sdw_max_distance) && (pm + (mp + interval) > vmin_ && pm + (mp + interval) < vmax_)) {
    T mean = std::fabs(mp + interval * T(0.5));
    T pa_1 = comp(pa1, sa) * (mean / std::fabs(comp(pa1, ax)));
    T pa_2 = comp(pa2, sa) * (mean / std::fabs(comp(pa2, ax)));
    T pb_1 = comp(pb1, sb) * (mean / std::fabs(comp(pb1, ax)));
    T pb_2 = comp(pb2, sb) * (mean / std::fabs(comp(pb2, ax)));
    T a1 = std::min(pa_1, pa_2), a2 = std::max(pa_1, pa_2);
    T b1 = std::min(pb_1, pb_2), b2 = std::max(pb_1, pb_2);
    T ad = std::fabs(a2 - a1), bd = std::fabs(b2 - b1);
    T as = (std::ceil(ad / sca) - (ad / sca)) * T(0.5);
    T bs = (std::ceil(bd / scb) - (bd / scb)) * T(0.5);
    a1 = a1 - as * sca; a2 = a2 + as * sca;
    b1 = b1 - bs * scb; b2 = b2 + bs * scb;
    T m1 = std::min(mp, mp + interval), m2 = std::max(mp, mp + interval);
    T lo[3], hi[3];
    lo[ax] = m1; hi[ax] = m2; lo[sa] = a1; hi[sa] = a2; lo[sb] = b1; hi[sb] = b2;
    st += shadow_sat(f, e, pos + v3(lo[0], lo[1], lo[2]), pos + v3(hi[0], hi[1], hi[2]));
    mp = mp + interval;
  }
  return st;
}

// ExtinctionDirectionalShadows (:432-456).
template <class T> T ext_shadow(const Frame<T>& f, const Ext<T>& e, V3<T> tx) {
  V3<T> realpos = tx - f.grid * T(0.5);
  V3<T> c = e.p->shadow_type == 0 ? normalize(e.light_pos - realpos) : normalize(e.light_fwd);
  V3<T> a = vabs(c);
  T st;
  if (a.z > a.x && a.z > a.y) st = cone_axis(f, e, tx, c, 2);
  else if (a.y > a.x) st = cone_axis(f, e, tx, c, 1);
  else st = cone_axis(f, e, tx, c, 0);
  return std::exp(-st);
}

// ------------------------------------------------------------ DOS cones
template <class T>
struct Dos {
  const cvr_dos_params* p;
  const Scene* s;
  const std::vector<T>* pyr;
  V3<T> light_pos, light_fwd, light_up, light_right;
  T spot_cos;
};

template <class T> T pyr_level(const Frame<T>& f, const Dos<T>& d, int l, V3<T> p) {
  const Scene& s = *d.s;
  const int* dm = s.ldims[l];
  Tap<T> tx = axis_tap<T>(p.x / f.grid.x * T(dm[0]) - T(0.5), dm[0]);
  Tap<T> ty = axis_tap<T>(p.y / f.grid.y * T(dm[1]) - T(0.5), dm[1]);
  Tap<T> tz = axis_tap<T>(p.z / f.grid.z * T(dm[2]) - T(0.5), dm[2]);
  const T* L = d.pyr->data() + s.loff[l];
  auto at = [&](int x, int y, int z) { return L[(size_t)x + (size_t)dm[0] * ((size_t)y + (size_t)dm[1] * z)]; };
  T c000 = at(tx.i0, ty.i0, tz.i0), c100 = at(tx.i1, ty.i0, tz.i0);
  T c010 = at(tx.i0, ty.i1, tz.i0), c110 = at(tx.i1, ty.i1, tz.i0);
  T c001 = at(tx.i0, ty.i0, tz.i1), c101 = at(tx.i1, ty.i0, tz.i1);
  T c011 = at(tx.i0, ty.i1, tz.i1), c111 = at(tx.i1, ty.i1, tz.i1);
  T c00 = c000 + tx.t * (c100 - c000), c10 = c010 + tx.t * (c110 - c010);
  T c01 = c001 + tx.t * (c101 - c001), c11 = c011 + tx.t * (c111 - c011);
  T c0 = c00 + ty.t * (c10 - c00), c1 = c01 + ty.t * (c11 - c01);
  return c0 + tz.t * (c1 - c0);
}
// textureLod with GL_LINEAR_MIPMAP_LINEAR: lod clamped to the chain, fractional
// lods blend two levels.
template <class T> T pyr_lod(const Frame<T>& f, const Dos<T>& d, T lod, V3<T> p) {
  T maxl = T(d.s->n_levels - 1);
  lod = std::min(std::max(lod, T(0)), maxl);
  T fl = std::floor(lod);
  int l0 = (int)fl;
  T t = lod - fl;
  T a = pyr_level(f, d, l0, p);
  if (t == T(0)) return a;
  T b = pyr_level(f, d, std::min(l0 + 1, d.s->n_levels - 1), p);
  return a + t * (b - a);
}
// GetGaussianExtinction with CONSIDER_BORDERS (ray_bbox_marching.comp:92-112).
template <class T> T gauss_ext(const Frame<T>& f, const Dos<T>& d, V3<T> p, T level) {
  T rg = pyr_lod(f, d, level, p);
  V3<T> S = f.grid;
  if (p.x < 0 || p.x > S.x || p.y < 0 || p.y > S.y || p.z < 0 || p.z > S.z) {
    T sg = std::pow(T(2), level);
    V3<T> c = vclamp(p, v3<T>(0, 0, 0), S) - p;
    T dist = c.x * c.x + c.y * c.y + c.z * c.z;
    rg = rg * std::exp(-(dist) / (T(2) * sg * sg));
  }
  return rg;
}

// Cone1Ray -> Cone3Ray -> Cone7Ray integration (ray_bbox_marching.comp:124-322
// for occlusion, 345-531 for shadows; identical arithmetic).
template <class T>
T cone_integrate(const Frame<T>& f, const Dos<T>& d, const cvr_cone_table& tab, V3<T> pos, V3<T> k, V3<T> u,
                 V3<T> v) {
  const int n1 = tab.integration_samples[0], n3 = tab.integration_samples[1], n7 = tab.integration_samples[2];
  const T uiw = T(tab.ui_weight);
  auto axis = [&](int i) { return v3<T>(T(tab.axes[i][0]), T(tab.axes[i][1]), T(tab.axes[i][2])); };
  T rays[7], last[7];
  T track = T(tab.initial_step);
  rays[0] = 0; last[0] = 0;
  for (int i = 0; i < n1; ++i) {
    const float* s = tab.sections[i];
    T tau = gauss_ext(f, d, pos + k * track, T(s[1]));
    T amptau = tau * T(s[3]);
    rays[0] += (last[0] + amptau) * T(s[2]) * uiw;
    last[0] = amptau;
    track += T(s[0]);
  }
  if (n3 + n7 == 0) return std::exp(-rays[0]);
  rays[2] = rays[0]; rays[1] = rays[0];
  last[2] = last[0]; last[1] = last[0];
  {
    V3<T> vk[3];
    for (int r = 0; r < 3; ++r) { V3<T> a = axis(r); vk[r] = k * a.z + u * a.y + v * a.x; }
    for (int i = 0; i < n3; ++i) {
      const float* s = tab.sections[n1 + i];
      for (int r = 0; r < 3; ++r) {
        T tau = gauss_ext(f, d, pos + vk[r] * track, T(s[1]));
        T amptau = tau * T(s[3]);
        rays[r] += (last[r] + amptau) * T(s[2]) * uiw;
        last[r] = amptau;
      }
      track += T(s[0]);
    }
  }
  if (n7 == 0) return (std::exp(-rays[0]) + std::exp(-rays[1]) + std::exp(-rays[2])) / T(3);
  rays[6] = rays[5] = rays[2];
  rays[4] = rays[3] = rays[1];
  T avg = (rays[2] + rays[1] + rays[0]) / T(3);
  rays[2] = rays[1] = rays[0];
  rays[0] = avg;
  last[6] = last[5] = last[2];
  last[4] = last[3] = last[1];
  T avgt = (last[2] + last[1] + last[0]) / T(3);
  last[2] = last[1] = last[0];
  last[0] = avgt;
  V3<T> vk[7];
  for (int r = 0; r < 7; ++r) { V3<T> a = axis(3 + r); vk[r] = k * a.z + u * a.y + v * a.x; }
  for (int i = 0; i < n7; ++i) {
    const float* s = tab.sections[n1 + n3 + i];
    for (int r = 0; r < 7; ++r) {
      T tau = gauss_ext(f, d, pos + vk[r] * track, T(s[1]));
      T amptau = tau * T(s[3]);
      rays[r] += (last[r] + amptau) * T(s[2]) * uiw;
      last[r] = amptau;
    }
    track += T(s[0]);
  }
  T w7 = T(tab.ray7_adj_weight);
  return (std::exp(-rays[0]) + (std::exp(-rays[1]) + std::exp(-rays[2]) + std::exp(-rays[3]) + std::exp(-rays[4]) +
                                std::exp(-rays[5]) + std::exp(-rays[6])) * w7) / (T(1) + w7 * T(6));
}

// ------------------------------------------------------------ ground truth
template <class T>
struct Gt {
  const cvr_gt_params* p;
  const Scene* s;
  V3<T> light_pos, light_fwd, light_up, light_right;
};

template <class T> T tf_alpha(const Scene& s, T d) { return tf_lookup<T>(s.rgbt, s.tf_n, d).a; }

// One light ray (gt_ray_marching.comp:125-159 / 209-242).
template <class T> T gt_light_ray(const Frame<T>& f, const Gt<T>& g, V3<T> tx, V3<T> w, T dist) {
  T vt = 1;
  T s = T(g.p->light_ray_initial_gap);
  V3<T> S = f.grid;
  T st0 = tf_alpha(*g.s, sample_volume(*g.s, tx + w * s));
  while (s < dist) {
    T h = std::min(T(g.p->light_ray_step_size), dist - s);
    V3<T> at = tx + w * (s + h);
    if (at.x < 0 || at.x > S.x || at.y < 0 || at.y > S.y || at.z < 0 || at.z > S.z) break;
    T st1 = tf_alpha(*g.s, sample_volume(*g.s, at));
    vt *= std::exp(-((st0 + st1) * T(0.5)) * h);
    if ((T(1) - vt) > T(0.99)) break;
    st0 = st1;
    s = s + h;
  }
  return vt;
}

template <class T> T gt_occlusion(const Frame<T>& f, const Gt<T>& g, V3<T> tx, V3<T> v_up, V3<T> v_right, V3<T> dir) {
  T socc = 0, swgt = 0;
  V3<T> vd = normalize(-dir);
  for (int i = 0; i < (int)g.s->occ_vec.size() / 3; ++i) {
    V3<T> c = from<T>(&g.s->occ_vec[3 * i]);
    V3<T> w = normalize(v_right * c.x + v_up * c.y + vd * c.z);
    T vt = gt_light_ray(f, g, tx, w, T(g.p->occ_distance));
    T rw = dot(vd, w);
    socc += vt * rw;
    swgt += rw;
  }
  return socc / swgt;
}

template <class T> T gt_shadow(const Frame<T>& f, const Gt<T>& g, V3<T> tx) {
  V3<T> wpos = tx - f.grid * T(0.5);
  V3<T> vd, vu, vr;
  if (g.p->shadow_type == 0 || g.p->shadow_type == 1) {
    vd = normalize(g.light_pos - wpos);
    vu = normalize(cross(vd, g.light_right));
    vr = normalize(cross(vd, vu));
    if (g.p->shadow_type == 1 && dot(vd, g.light_fwd) < T(30)) return 0;
  } else {
    vd = g.light_fwd; vu = g.light_up; vr = g.light_right;
  }
  T ssdw = 0, swgt = 0;
  for (int i = 0; i < (int)g.s->sdw_vec.size() / 3; ++i) {
    V3<T> c = from<T>(&g.s->sdw_vec[3 * i]);
    V3<T> w = normalize(vr * c.x + vu * c.y + vd * c.z);
    T vt = gt_light_ray(f, g, tx, w, T(g.p->sdw_distance));
    T rw = dot(vd, w);
    ssdw += vt * rw;
    swgt += rw;
  }
  return ssdw / swgt;
}

// ------------------------------------------------------------ surrogate
// The network's inputs (no reference counterpart; definition in cvr.h): six
// pyramid levels x seven taps of segment opacity around the shading point in
// the ground-truth occlusion frame (gt_ray_marching.comp:396-399), the light
// direction and the gradient of pyramid level 0 in that frame.
template <class T>
void sur_features(const Frame<T>& f, const Scene& s, const std::vector<T>& pyr, int shadow_type, V3<T> light_pos,
                  V3<T> light_fwd, T sdw_dist, V3<T> tx, V3<T> dir, T* x) {
  Dos<T> d{};
  d.s = &s;
  d.pyr = &pyr;
  const V3<T> S = f.grid;
  V3<T> n = normalize(-dir);
  V3<T> c = cross(dir, v3<T>(0, 1, 0));
  if (dot(c, c) < T(1e-12)) c = v3<T>(1, 0, 0);
  V3<T> r = normalize(c);
  V3<T> u = normalize(cross(-dir, r));
  V3<T> L = shadow_type == 2 ? light_fwd : normalize(light_pos - (tx - S * T(0.5)));
  auto tap = [&](int l, V3<T> q, T dl) -> T {
    if (q.x < 0 || q.x > S.x || q.y < 0 || q.y > S.y || q.z < 0 || q.z > S.z) return T(0);
    return T(1) - std::exp(-pyr_level(f, d, l, q) * dl);
  };
  auto sig = [&](int l, V3<T> q) -> T {  // extinction of level l, 0 outside the box
    if (q.x < 0 || q.x > S.x || q.y < 0 || q.y > S.y || q.z < 0 || q.z > S.z) return T(0);
    return pyr_level(f, d, l, q);
  };
  const T unit = T((s.sx + s.sy + s.sz) / 3.0);
  // the light ray's end: the box exit, at most the shadow-ray length
  T t_end = sdw_dist;
  const T Lc[3] = {L.x, L.y, L.z}, Tc[3] = {tx.x, tx.y, tx.z}, Sc[3] = {S.x, S.y, S.z};
  for (int ax = 0; ax < 3; ++ax) {
    if (Lc[ax] > 0) t_end = std::min(t_end, (Sc[ax] - Tc[ax]) / Lc[ax]);
    else if (Lc[ax] < 0) t_end = std::min(t_end, -Tc[ax] / Lc[ax]);
  }
  t_end = std::max(t_end, T(0));
  // optical depth of the light-ray segment [s0, s1] clipped to [0, t_end]
  auto seg_tau = [&](int l, T s0, T s1) -> T {
    s0 = std::max(s0, T(0));
    s1 = std::min(s1, t_end);
    if (!(s1 > s0)) return T(0);
    return pyr_level(f, d, l, tx + L * (T(0.5) * (s0 + s1))) * (s1 - s0);
  };
  auto far = [&](T d5) -> T {  // the rest of the light path, x[35]
    T tau = 0;
    const T s0 = T(4) * d5 - T(4) * unit;
    for (int j = 0; j < 8; ++j) {
      const T lo = s0 + T(j) * d5;
      if (!(lo < t_end)) break;
      tau += seg_tau(5, lo, lo + d5);
    }
    return T(1) - std::exp(-tau);
  };
  T dl = T((s.sx + s.sy + s.sz) / 3.0) * T(2);
  for (int l = 0; l < 6; ++l) {
    x[7 * l + 0] = l == 5 ? far(dl) : tap(l, tx, dl);
    // two consecutive light-ray segments of length dl (the twelve partition
    // [0, 252 unit]), clipped to the ray's end
    x[7 * l + 1] = T(1) - std::exp(-seg_tau(l, T(2) * dl - T(4) * unit, T(3) * dl - T(4) * unit));
    x[7 * l + 2] = T(1) - std::exp(-seg_tau(l, T(3) * dl - T(4) * unit, T(4) * dl - T(4) * unit));
    x[7 * l + 3] = tap(l, tx + n * dl, dl);
    x[7 * l + 4] = tap(l, tx + n * (T(3) * dl), dl);
    // the mean extinction of the taps at +- r dl (k = 5) and +- u dl (k = 6)
    x[7 * l + 5] = T(1) - std::exp(-(T(0.5) * (sig(l, tx + r * dl) + sig(l, tx - r * dl))) * dl);
    x[7 * l + 6] = T(1) - std::exp(-(T(0.5) * (sig(l, tx + u * dl) + sig(l, tx - u * dl))) * dl);
    dl = dl * T(2);
  }
  x[42] = dot(L, r);
  x[43] = dot(L, u);
  x[44] = dot(L, n);
  auto sg = [&](V3<T> q) { return pyr_level(f, d, 0, q); };  // level 0 of the pyramid
  V3<T> g;
  g.x = T(0.5) * f.spacing.x * (sg(tx + v3<T>(f.spacing.x, 0, 0)) - sg(tx - v3<T>(f.spacing.x, 0, 0)));
  g.y = T(0.5) * f.spacing.y * (sg(tx + v3<T>(0, f.spacing.y, 0)) - sg(tx - v3<T>(0, f.spacing.y, 0)));
  g.z = T(0.5) * f.spacing.z * (sg(tx + v3<T>(0, 0, f.spacing.z)) - sg(tx - v3<T>(0, 0, f.spacing.z)));
  x[45] = dot(g, r);
  x[46] = dot(g, u);
  x[47] = dot(g, n);
}

// Round to nearest even BF16 (the operand format of the tensor-core GEMMs).
inline double bf16(double v) {
  float f = (float)v;
  uint32_t b;
  std::memcpy(&b, &f, 4);
  b += 0x7FFFu + ((b >> 16) & 1u);
  b &= 0xFFFF0000u;
  std::memcpy(&f, &b, 4);
  return (double)f;
}

// 48 -> 64 -> 64 -> 2 with BF16 operands (inputs, weights, hidden
// activations) and exact accumulation; biases in FP32.
inline void mlp_forward_bf16(const std::vector<float>& P, const double* x, double* y) {
  const float* W1 = P.data();
  const float* b1 = W1 + 64 * 48;
  const float* W2 = b1 + 64;
  const float* b2 = W2 + 64 * 64;
  const float* W3 = b2 + 64;
  const float* b3 = W3 + 2 * 64;
  double xb[48], h1[64], h2[64];
  for (int k = 0; k < 48; ++k) xb[k] = bf16(x[k]);
  for (int o = 0; o < 64; ++o) {
    double a = 0;
    for (int k = 0; k < 48; ++k) a += xb[k] * bf16(W1[o * 48 + k]);
    h1[o] = bf16(std::max(a + (double)b1[o], 0.0));
  }
  for (int o = 0; o < 64; ++o) {
    double a = 0;
    for (int k = 0; k < 64; ++k) a += h1[k] * bf16(W2[o * 64 + k]);
    h2[o] = bf16(std::max(a + (double)b2[o], 0.0));
  }
  for (int o = 0; o < 2; ++o) {
    double a = 0;
    for (int k = 0; k < 64; ++k) a += h2[k] * bf16(W3[o * 64 + k]);
    y[o] = a + (double)b3[o];
  }
}

// ------------------------------------------------------------ gradient shading
// texture(TexVolumeGradient, Tpos / VolumeGridSize).xyz
template <class T> V3<T> sample_gradient(const Scene& s, V3<T> p) {
  V3<T> grid = v3<T>(T(s.nx * s.sx), T(s.ny * s.sy), T(s.nz * s.sz));
  Tap<T> tx = axis_tap<T>(p.x / grid.x * T(s.nx) - T(0.5), s.nx);
  Tap<T> ty = axis_tap<T>(p.y / grid.y * T(s.ny) - T(0.5), s.ny);
  Tap<T> tz = axis_tap<T>(p.z / grid.z * T(s.nz) - T(0.5), s.nz);
  T r[3];
  for (int ch = 0; ch < 3; ++ch) {
    auto at = [&](int x, int y, int z) {
      return (T)s.grad[3 * ((size_t)x + (size_t)s.nx * ((size_t)y + (size_t)s.ny * z)) + ch];
    };
    T c00 = at(tx.i0, ty.i0, tz.i0) + tx.t * (at(tx.i1, ty.i0, tz.i0) - at(tx.i0, ty.i0, tz.i0));
    T c10 = at(tx.i0, ty.i1, tz.i0) + tx.t * (at(tx.i1, ty.i1, tz.i0) - at(tx.i0, ty.i1, tz.i0));
    T c01 = at(tx.i0, ty.i0, tz.i1) + tx.t * (at(tx.i1, ty.i0, tz.i1) - at(tx.i0, ty.i0, tz.i1));
    T c11 = at(tx.i0, ty.i1, tz.i1) + tx.t * (at(tx.i1, ty.i1, tz.i1) - at(tx.i0, ty.i1, tz.i1));
    T c0 = c00 + ty.t * (c10 - c00), c1 = c01 + ty.t * (c11 - c01);
    r[ch] = c0 + tz.t * (c1 - c0);
  }
  return v3<T>(r[0], r[1], r[2]);
}

// The shared terms of the gradient branches (ray_marching_1p.comp:50-70):
// false for a zero gradient (the colour is left unshaded).
template <class T>
bool blinn_terms(const Scene& s, V3<T> grid, V3<T> eye, V3<T> tx, V3<T> light_pos, T& diff, T& spec) {
  V3<T> n = sample_gradient<T>(s, tx);
  if (n.x == T(0) && n.y == T(0) && n.z == T(0)) return false;
  n = normalize(n);
  V3<T> w = tx - grid * T(0.5);
  V3<T> l = normalize(light_pos - w);
  V3<T> e = normalize(eye - w);
  V3<T> hv = normalize(e + l);
  diff = std::max(T(0), dot(n, l));
  spec = std::pow(std::max(T(0), dot(hv, n)), T(s.bp.shininess));
  return true;
}

enum PhongKind { PHONG_PLAIN, PHONG_EXT, PHONG_CONE, PHONG_GT };

// The gradient branch of each ShadeSample:
//  plain  ShadeBlinnPhong (ray_marching_1p.comp:71-76): L*(Ka + Kd*diff) + Is*Ks*spec
//  ext    ebs_ray_bbox_marching.comp:540-542, obj_ray_marching.comp:127-128:
//         (1/(ka+kd))*(L*Io*ka + IS*(L*kd*diff)) + IS*(ks*Is*spec)
//  cone   ray_bbox_marching.comp:646-647: L*((1/(ka+kd))*(Io*ka + IS*kd*diff)) + Is*(IS*ks*spec)
//  gt     gt_ray_marching.comp:293-294: the cone form with specular colour 1
template <class T>
V4<T> phong(const Scene& s, const Frame<T>& f, V4<T> L, V3<T> tx, V3<T> light_pos, int kind, T io, T ka, T is, T kd) {
  T diff, spec;
  if (!blinn_terms<T>(s, f.grid, f.cam.eye, tx, light_pos, diff, spec)) return L;
  V3<T> isp = kind == PHONG_GT ? v3<T>(1, 1, 1) : from<T>(s.bp.specular);
  T ks = T(s.bp.ks);
  T* c[3] = {&L.r, &L.g, &L.b};
  T sp[3] = {isp.x, isp.y, isp.z};
  for (int i = 0; i < 3; ++i) {
    T& v = *c[i];
    if (kind == PHONG_PLAIN) v = v * (T(s.bp.ka) + T(s.bp.kd) * diff) + sp[i] * ks * spec;
    else if (kind == PHONG_EXT) v = (T(1) / (ka + kd)) * (v * io * ka + is * (v * kd * diff)) + is * (ks * sp[i] * spec);
    else v = v * ((T(1) / (ka + kd)) * (io * ka + is * kd * diff)) + sp[i] * (is * ks * spec);
  }
  return L;
}

// ------------------------------------------------------------ primary loop
// ray_marching_1p.comp:160-247 and the identical loops of the other shaders.
template <class T, class ShadeFn>
void march_rows(const Scene& s, const cvr_camera& camc, T step, int W, int H, int y0, int y1, double* out,
                uint32_t* counts, uint64_t* total, int threads, ShadeFn shade, bool gate = true) {
  Frame<T> f;
  f.s = &s;
  f.spacing = v3<T>(T(s.sx), T(s.sy), T(s.sz));
  f.grid = v3<T>(T(s.nx * s.sx), T(s.ny * s.sy), T(s.nz * s.sz));
  f.cam = make_cam<T>(camc, W, H);
  f.step = step;
  uint64_t acc = 0;
#pragma omp parallel for schedule(dynamic, 1) num_threads(threads) reduction(+ : acc)
  for (int y = y0; y < y1; ++y) {
    for (int x = 0; x < W; ++x) {
      V3<T> dir = primary_dir(f.cam, x, y, W, H);
      T tnear, tfar;
      V4<T> dst{0, 0, 0, 0};
      uint32_t n = 0;
      if (ray_aabb(f.cam.eye, dir, f.grid, tnear, tfar)) {
        T D = std::fabs(tfar - tnear);
        V3<T> tex0 = f.cam.eye + dir * tnear + f.grid * T(0.5);
        for (T st = 0; st < D;) {
          T h = std::min(step, D - st);
          V3<T> p = tex0 + dir * (st + h * T(0.5));
          T dens = sample_volume(s, p);
          V4<T> src = tf_lookup<T>(s.rgbt, s.tf_n, dens);
          ++n;
          if (src.a > T(0) && gate) {
            src = shade(f, src, p, dir);
            src.a = T(1) - std::exp(-src.a * h);
            src.r *= src.a; src.g *= src.a; src.b *= src.a;
            T r = T(1) - dst.a;
            dst.r += r * src.r; dst.g += r * src.g; dst.b += r * src.b; dst.a += r * src.a;
            if (dst.a > T(0.99)) break;
          }
          st = st + h;
        }
      }
      size_t o = (size_t)(y - y0) * W + x;
      out[4 * o + 0] = (double)dst.r; out[4 * o + 1] = (double)dst.g;
      out[4 * o + 2] = (double)dst.b; out[4 * o + 3] = (double)dst.a;
      if (counts) counts[o] = n;
      acc += n;
    }
  }
  if (total) *total = acc;
}

// ------------------------------------------------------------ isosurfaces
// main() of ray_marching_1p_iso_adapt.comp:84-172: the density at the entry
// point, adaptive steps (small within StepSizeRange of the isovalue), samples
// at interval ends, linear refinement of each crossing, constant colour
// (ShadeBlinnPhong when gradient shading is on), front-to-back until 0.99.
template <class T>
void iso_rows(const Scene& s, const cvr_camera& camc, const cvr_iso_params& p, const cvr_light& light, int W, int H,
              int y0, int y1, double* out, uint32_t* counts, uint64_t* total, int threads) {
  Frame<T> f;
  f.s = &s;
  f.spacing = v3<T>(T(s.sx), T(s.sy), T(s.sz));
  f.grid = v3<T>(T(s.nx * s.sx), T(s.ny * s.sy), T(s.nz * s.sz));
  f.cam = make_cam<T>(camc, W, H);
  f.step = T(p.step_size_small);
  const T iso = T(p.isovalue), small = T(p.step_size_small), large = T(p.step_size_large), range = T(p.step_size_range);
  const bool grad = s.bp.apply && s.grad_ready;
  const V3<T> lpos = from<T>(light.position);
  uint64_t acc = 0;
#pragma omp parallel for schedule(dynamic, 1) num_threads(threads) reduction(+ : acc)
  for (int y = y0; y < y1; ++y) {
    for (int x = 0; x < W; ++x) {
      V3<T> dir = primary_dir(f.cam, x, y, W, H);
      T tnear, tfar;
      V4<T> dst{0, 0, 0, 0};
      uint32_t n = 0;
      if (ray_aabb(f.cam.eye, dir, f.grid, tnear, tfar)) {
        T D = std::fabs(tfar - tnear);
        V3<T> tex0 = f.cam.eye + dir * tnear + f.grid * T(0.5);
        T prev = sample_volume(s, tex0);
        for (T st = 0; st < D;) {
          T h = std::min(std::fabs(prev - iso) < range ? small : large, D - st);
          T d = sample_volume(s, tex0 + dir * (st + h));
          ++n;
          if ((prev <= iso && iso < d) || (prev >= iso && iso > d)) {
            T t = (iso - prev) / (d - prev);
            V3<T> pos = tex0 + dir * (st + t * h);
            V4<T> src{T(p.color[0]), T(p.color[1]), T(p.color[2]), T(p.color[3])};
            if (grad) src = phong<T>(s, f, src, pos, lpos, PHONG_PLAIN, T(0), T(0), T(0), T(0));
            src.r *= src.a; src.g *= src.a; src.b *= src.a;
            T r = T(1) - dst.a;
            dst.r += r * src.r; dst.g += r * src.g; dst.b += r * src.b; dst.a += r * src.a;
            if (dst.a > T(0.99)) break;
          }
          prev = d;
          st = st + h;
        }
      }
      size_t o = (size_t)(y - y0) * W + x;
      out[4 * o + 0] = (double)dst.r; out[4 * o + 1] = (double)dst.g;
      out[4 * o + 2] = (double)dst.b; out[4 * o + 3] = (double)dst.a;
      if (counts) counts[o] = n;
      acc += n;
    }
  }
  if (total) *total = acc;
}

// ------------------------------------------------------------ light cache
// Object-space light cache: (occlusion, shadow) at the cell centres
// tex_pos = (cell + 0.5) * (VolumeScales * (VolumeDimensions / LightCacheDimensions))
// (rc1pextbsd/lightcachecomputation.comp:443-468, rc1pdosct/lightcachecomputation.comp:523-547).
template <class T, class CellFn>
std::vector<T> build_cache(const Scene& s, CellFn cell) {
  const int* d = s.lc;
  std::vector<T> c(2 * (size_t)d[0] * d[1] * d[2]);
#pragma omp parallel for schedule(dynamic, 1)
  for (int z = 0; z < d[2]; ++z)
    for (int y = 0; y < d[1]; ++y)
      for (int x = 0; x < d[0]; ++x) {
        V3<T> tx = v3<T>((T(x) + T(0.5)) * (T(s.sx) * (T(s.nx) / T(d[0]))),
                         (T(y) + T(0.5)) * (T(s.sy) * (T(s.ny) / T(d[1]))),
                         (T(z) + T(0.5)) * (T(s.sz) * (T(s.nz) / T(d[2]))));
        T io, is;
        cell(tx, io, is);
        size_t i = (size_t)x + (size_t)d[0] * ((size_t)y + (size_t)d[1] * z);
        c[2 * i] = io;
        c[2 * i + 1] = is;
      }
  return c;
}
// texture(TexVolumeLightCache, tx_pos / VolumeScaledSizes).rg
template <class T> void cache_lookup(const Scene& s, const std::vector<T>& c, V3<T> grid, V3<T> tx, T& io, T& is) {
  const int* d = s.lc;
  Tap<T> a = axis_tap<T>(tx.x / grid.x * T(d[0]) - T(0.5), d[0]);
  Tap<T> b = axis_tap<T>(tx.y / grid.y * T(d[1]) - T(0.5), d[1]);
  Tap<T> g = axis_tap<T>(tx.z / grid.z * T(d[2]) - T(0.5), d[2]);
  for (int ch = 0; ch < 2; ++ch) {
    auto at = [&](int x, int y, int z) { return c[2 * ((size_t)x + (size_t)d[0] * ((size_t)y + (size_t)d[1] * z)) + ch]; };
    T c00 = at(a.i0, b.i0, g.i0) + a.t * (at(a.i1, b.i0, g.i0) - at(a.i0, b.i0, g.i0));
    T c10 = at(a.i0, b.i1, g.i0) + a.t * (at(a.i1, b.i1, g.i0) - at(a.i0, b.i1, g.i0));
    T c01 = at(a.i0, b.i0, g.i1) + a.t * (at(a.i1, b.i0, g.i1) - at(a.i0, b.i0, g.i1));
    T c11 = at(a.i0, b.i1, g.i1) + a.t * (at(a.i1, b.i1, g.i1) - at(a.i0, b.i1, g.i1));
    T c0 = c00 + b.t * (c10 - c00), c1 = c01 + b.t * (c11 - c01);
    (ch == 0 ? io : is) = c0 + g.t * (c1 - c0);
  }
}

template <class T> V4<T> combine(V4<T> L, bool occ_on, T ka_in, T io, bool sdw_on, T kd_in, T is) {
  T ka = occ_on ? ka_in : T(0), kd = sdw_on ? kd_in : T(0);
  if (!occ_on) io = 0;
  if (!sdw_on) is = 0;
  T k = T(1) / (ka + kd);
  L.r = k * (L.r * io * ka + L.r * is * kd);
  L.g = k * (L.g * io * ka + L.g * is * kd);
  L.b = k * (L.b * io * ka + L.b * is * kd);
  return L;
}

// ShadeSample's final combination: the gradient branch when gradient shading
// is on (ApplyPhongShading), else combine().
template <class T>
V4<T> shade_mix(const Scene& s, const Frame<T>& f, V4<T> L, V3<T> tx, V3<T> light_pos, int kind, bool occ_on, T ka_in,
                T io, bool sdw_on, T kd_in, T is) {
  if (!(s.bp.apply && s.grad_ready)) return combine(L, occ_on, ka_in, io, sdw_on, kd_in, is);
  T ka = occ_on ? ka_in : T(0), kd = sdw_on ? kd_in : T(0);
  if (!occ_on) io = 0;
  if (!sdw_on) is = 0;
  return phong<T>(s, f, L, tx, light_pos, kind, io, ka, is, kd);
}

template <class T>
int render_t(Scene& s, int method, const cvr_camera& cam, const cvr_light& light, const void* params, int W, int H,
             int y0, int y1, double* out, uint32_t* counts, uint64_t* total, int threads) {
  switch (method) {
    case CVR_METHOD_PLAIN: {
      const cvr_plain_params* p = (const cvr_plain_params*)params;
      const bool grad = s.bp.apply && s.grad_ready;
      const V3<T> lpos = from<T>(light.position);
      march_rows<T>(s, cam, T(p->step_size), W, H, y0, y1, out, counts, total, threads,
                    [&](const Frame<T>& f, V4<T> src, V3<T> tx, V3<T>) {
                      return grad ? phong<T>(s, f, src, tx, lpos, PHONG_PLAIN, T(0), T(0), T(0), T(0)) : src;
                    });
      return 0;
    }
    case CVR_METHOD_EXTINCTION: {
      if (!s.sat_ready) return CVR_ERR_NOT_READY;
      const cvr_ext_params* p = (const cvr_ext_params*)params;
      Ext<T> e;
      e.p = p;
      e.light_pos = from<T>(light.position);
      e.light_fwd = from<T>(light.forward);
      if constexpr (sizeof(T) == 8) e.sat = s.sat64.data();
      else e.sat = s.sat32.data();
      e.sx = s.nx + 2; e.sy = s.ny + 2; e.sz = s.nz + 2;
      if (s.lc[0] > 0) {
        // obj_ray_marching.comp with the cache of lightcachecomputation.comp (rc1pextbsd)
        Frame<T> fc;
        fc.s = &s;
        fc.spacing = v3<T>(T(s.sx), T(s.sy), T(s.sz));
        fc.grid = v3<T>(T(s.nx * s.sx), T(s.ny * s.sy), T(s.nz * s.sz));
        std::vector<T> cache = build_cache<T>(s, [&](V3<T> tx, T& io, T& is) {
          io = p->apply_occlusion ? ext_ao(fc, e, tx) : T(1);
          is = p->apply_shadow ? ext_shadow(fc, e, tx) : T(1);
        });
        march_rows<T>(s, cam, T(p->step_size), W, H, y0, y1, out, counts, total, threads,
                      [&](const Frame<T>& f, V4<T> src, V3<T> tx, V3<T>) {
                        T io, is;
                        cache_lookup<T>(s, cache, f.grid, tx, io, is);
                        return shade_mix<T>(s, f, src, tx, e.light_pos, PHONG_EXT, p->apply_occlusion != 0, T(p->ka), io, p->apply_shadow != 0, T(p->kd),
                                       is);
                      },
                      p->apply_occlusion || p->apply_shadow);
        return 0;
      }
      march_rows<T>(s, cam, T(p->step_size), W, H, y0, y1, out, counts, total, threads,
                    [&](const Frame<T>& f, V4<T> src, V3<T> tx, V3<T>) {
                      T io = p->apply_occlusion ? ext_ao(f, e, tx) : T(0);
                      T is = p->apply_shadow ? ext_shadow(f, e, tx) : T(0);
                      return shade_mix<T>(s, f, src, tx, e.light_pos, PHONG_EXT, p->apply_occlusion != 0, T(p->ka), io, p->apply_shadow != 0, T(p->kd), is);
                    });
      return 0;
    }
    case CVR_METHOD_CONE_DOS: {
      if (!s.pyr_ready || !s.cone_ready) return CVR_ERR_NOT_READY;
      const cvr_dos_params* p = (const cvr_dos_params*)params;
      Dos<T> d;
      d.p = p; d.s = &s;
      if constexpr (sizeof(T) == 8) d.pyr = &s.pyr64;
      else d.pyr = &s.pyr32;
      d.light_pos = from<T>(light.position); d.light_fwd = from<T>(light.forward);
      d.light_up = from<T>(light.up); d.light_right = from<T>(light.right);
      d.spot_cos = T(light.spot_cos_max);
      // ShadowEvaluationKernel (:533-562); Cone1RayShadow's (k, v, u)
      // parameter order swaps u and v.
      auto dos_shadow = [&](const Frame<T>& f, V3<T> tx) -> T {
        V3<T> k, u, v;
        if (p->shadow_type == 0 || p->shadow_type == 1) {
          k = normalize(d.light_pos - (tx - f.grid * T(0.5)));
          u = normalize(cross(k, d.light_right));
          v = normalize(cross(k, u));
          if (p->shadow_type == 1 && dot(k, d.light_fwd) < d.spot_cos) return T(0);
        } else {
          k = d.light_fwd; v = d.light_up; u = d.light_right;
        }
        return cone_integrate(f, d, s.sdw, tx, k, v, u);
      };
      if (s.lc[0] > 0) {
        // obj_ray_marching.comp with the cache of lightcachecomputation.comp (rc1pdosct): the
        // occlusion cone's frame comes from the camera's up vector (:280-292)
        Frame<T> fc;
        fc.s = &s;
        fc.spacing = v3<T>(T(s.sx), T(s.sy), T(s.sz));
        fc.grid = v3<T>(T(s.nx * s.sx), T(s.ny * s.sy), T(s.nz * s.sz));
        fc.cam = make_cam<T>(cam, W, H);
        std::vector<T> cache = build_cache<T>(s, [&](V3<T> tx, T& io, T& is) {
          io = T(1);
          is = T(1);
          if (p->apply_occlusion) {
            V3<T> k = normalize(fc.cam.eye - (tx - fc.grid * T(0.5)));
            V3<T> v_right = normalize(cross(-k, fc.cam.u));
            V3<T> v_up = normalize(cross(k, v_right));
            io = cone_integrate(fc, d, s.occ, tx, k, v_up, v_right);
          }
          if (p->apply_shadow) is = dos_shadow(fc, tx);
        });
        march_rows<T>(s, cam, T(p->step_size), W, H, y0, y1, out, counts, total, threads,
                      [&](const Frame<T>& f, V4<T> src, V3<T> tx, V3<T>) {
                        T io, is;
                        cache_lookup<T>(s, cache, f.grid, tx, io, is);
                        return shade_mix<T>(s, f, src, tx, d.light_pos, PHONG_EXT, p->apply_occlusion != 0, T(p->ka), io, p->apply_shadow != 0, T(p->kd),
                                       is);
                      },
                      p->apply_occlusion || p->apply_shadow);
        return 0;
      }
      march_rows<T>(s, cam, T(p->step_size), W, H, y0, y1, out, counts, total, threads,
                    [&](const Frame<T>& f, V4<T> src, V3<T> tx, V3<T> dir) {
                      T io = 0, is = 0;
                      if (p->apply_occlusion) {
                        // OcclusionEvaluationKernel (:324-333), frame from main() (:682-684).
                        V3<T> v_right = normalize(cross(dir, v3<T>(0, 1, 0)));
                        V3<T> v_up = normalize(cross(-dir, v_right));
                        V3<T> k = normalize(f.cam.eye - (tx - f.grid * T(0.5)));
                        io = cone_integrate(f, d, s.occ, tx, k, v_up, v_right);
                      }
                      if (p->apply_shadow) {
                        // ShadowEvaluationKernel (:533-562); Cone1RayShadow's (k, v, u)
                        // parameter order swaps u and v.
                        V3<T> k, u, v;
                        bool dark = false;
                        if (p->shadow_type == 0 || p->shadow_type == 1) {
                          k = normalize(d.light_pos - (tx - f.grid * T(0.5)));
                          u = normalize(cross(k, d.light_right));
                          v = normalize(cross(k, u));
                          if (p->shadow_type == 1 && dot(k, d.light_fwd) < d.spot_cos) dark = true;
                        } else {
                          k = d.light_fwd; v = d.light_up; u = d.light_right;
                        }
                        is = dark ? T(0) : cone_integrate(f, d, s.sdw, tx, k, v, u);
                      }
                      return shade_mix<T>(s, f, src, tx, d.light_pos, PHONG_CONE, p->apply_occlusion != 0, T(p->ka), io, p->apply_shadow != 0, T(p->kd), is);
                    });
      return 0;
    }
    case CVR_METHOD_GROUND_TRUTH: {
      if (!s.gt_ready) return CVR_ERR_NOT_READY;
      const cvr_gt_params* p = (const cvr_gt_params*)params;
      Gt<T> g;
      g.p = p; g.s = &s;
      g.light_pos = from<T>(light.position); g.light_fwd = from<T>(light.forward);
      g.light_up = from<T>(light.up); g.light_right = from<T>(light.right);
      march_rows<T>(s, cam, T(p->step_size), W, H, y0, y1, out, counts, total, threads,
                    [&](const Frame<T>& f, V4<T> src, V3<T> tx, V3<T> dir) {
                      V3<T> v_right = normalize(cross(dir, v3<T>(0, 1, 0)));
                      V3<T> v_up = normalize(cross(-dir, v_right));
                      T io = p->apply_occlusion ? gt_occlusion(f, g, tx, v_up, v_right, dir) : T(0);
                      T is = p->apply_shadow ? gt_shadow(f, g, tx) : T(0);
                      return shade_mix<T>(s, f, src, tx, g.light_pos, PHONG_GT, p->apply_occlusion != 0, T(p->ka), io, p->apply_shadow != 0, T(p->kd), is);
                    });
      return 0;
    }
    case CVR_METHOD_ISO: {
      iso_rows<T>(s, cam, *(const cvr_iso_params*)params, light, W, H, y0, y1, out, counts, total, threads);
      return 0;
    }
    case CVR_METHOD_SURROGATE: {
      // The ground-truth ShadeSample (gt_ray_marching.comp:254-303) fed by the
      // network's (occlusion, shadow), clamped to [0, 1]; spot lights give
      // shadow 0 as the ground truth does.
      if (!s.pyr_ready || s.n_levels < 6 || s.mlp.size() != (size_t)CVR_MLP_PARAMS) return CVR_ERR_NOT_READY;
      const cvr_gt_params* p = (const cvr_gt_params*)params;
      const std::vector<T>* pyr;
      if constexpr (sizeof(T) == 8) pyr = &s.pyr64;
      else pyr = &s.pyr32;
      V3<T> lpos = from<T>(light.position), lfwd = from<T>(light.forward);
      march_rows<T>(s, cam, T(p->step_size), W, H, y0, y1, out, counts, total, threads,
                    [&](const Frame<T>& f, V4<T> src, V3<T> tx, V3<T> dir) {
                      T x[48];
                      sur_features(f, s, *pyr, p->shadow_type, lpos, lfwd, T(p->sdw_distance), tx, dir, x);
                      double xd[48], y[2];
                      for (int k = 0; k < 48; ++k) xd[k] = (double)x[k];
                      mlp_forward_bf16(s.mlp, xd, y);
                      T io = T(std::min(std::max(y[0], 0.0), 1.0));
                      T is = p->shadow_type == 1 ? T(0) : T(std::min(std::max(y[1], 0.0), 1.0));
                      return shade_mix<T>(s, f, src, tx, lpos, PHONG_GT, p->apply_occlusion != 0, T(p->ka), io, p->apply_shadow != 0, T(p->kd), is);
                    });
      return 0;
    }
  }
  return CVR_ERR_INVALID_ARG;
}

// ------------------------------------------------------------ pyramid
// gen_extcoefvol_anysize.comp / _mmlevel.comp / backtotau.comp restated in T.
template <class T> void build_pyramid_t(Scene& s, float s0f, std::vector<T>& out) {
  size_t total = s.loff[s.n_levels - 1] +
                 (size_t)s.ldims[s.n_levels - 1][0] * s.ldims[s.n_levels - 1][1] * s.ldims[s.n_levels - 1][2];
  out.assign(total, T(0));
  V3<T> grid = v3<T>(T(s.nx * s.sx), T(s.ny * s.sy), T(s.nz * s.sz));
  for (int l = 0; l < s.n_levels; ++l) {
    const int* dm = s.ldims[l];
    T sig = l == 0 ? T(s0f) : T(s0f * std::pow(2.0f, (float)l));
    V3<T> vs = grid / v3<T>(T(dm[0]), T(dm[1]), T(dm[2]));
    T* dst = out.data() + s.loff[l];
    const T* prev = l > 0 ? out.data() + s.loff[l - 1] : nullptr;
    const int* pd = l > 0 ? s.ldims[l - 1] : nullptr;
#pragma omp parallel for schedule(static)
    for (int z = 0; z < dm[2]; ++z) {
      for (int y = 0; y < dm[1]; ++y) {
        for (int x = 0; x < dm[0]; ++x) {
          V3<T> gp = v3<T>((T(x) + T(0.5)) * vs.x, (T(y) + T(0.5)) * vs.y, (T(z) + T(0.5)) * vs.z);
          T swc = 0, sw = 0;
          for (int ptx = -3; ptx < 4; ++ptx)
            for (int pty = -3; pty < 4; ++pty)
              for (int ptz = -3; ptz < 4; ++ptz) {
                T fx = T(ptx) * sig, fy = T(pty) * sig, fz = T(ptz) * sig;
                T wk = (sig * sig * sig) * std::exp(-(fx * fx + fy * fy + fz * fz) / (T(2) * sig * sig));
                V3<T> p = gp + v3(fx, fy, fz);
                V3<T> t = p / grid;
                T ck = 0;
                if (!(t.x < 0 || t.y < 0 || t.z < 0 || t.x > 1 || t.y > 1 || t.z > 1)) {
                  if (l == 0) {
                    ck = tf_lookup<T>(s.rgba, s.tf_n, sample_volume(s, p)).a;
                  } else {
                    Tap<T> tx = axis_tap<T>(t.x * T(pd[0]) - T(0.5), pd[0]);
                    Tap<T> ty = axis_tap<T>(t.y * T(pd[1]) - T(0.5), pd[1]);
                    Tap<T> tz = axis_tap<T>(t.z * T(pd[2]) - T(0.5), pd[2]);
                    auto at = [&](int a, int b, int c) {
                      return prev[(size_t)a + (size_t)pd[0] * ((size_t)b + (size_t)pd[1] * c)];
                    };
                    T c000 = at(tx.i0, ty.i0, tz.i0), c100 = at(tx.i1, ty.i0, tz.i0);
                    T c010 = at(tx.i0, ty.i1, tz.i0), c110 = at(tx.i1, ty.i1, tz.i0);
                    T c001 = at(tx.i0, ty.i0, tz.i1), c101 = at(tx.i1, ty.i0, tz.i1);
                    T c011 = at(tx.i0, ty.i1, tz.i1), c111 = at(tx.i1, ty.i1, tz.i1);
                    T c00 = c000 + tx.t * (c100 - c000), c10 = c010 + tx.t * (c110 - c010);
                    T c01 = c001 + tx.t * (c101 - c001), c11 = c011 + tx.t * (c111 - c011);
                    T c0 = c00 + ty.t * (c10 - c00), c1 = c01 + ty.t * (c11 - c01);
                    ck = c0 + tz.t * (c1 - c0);
                  }
                }
                swc += wk * ck;
                sw += wk;
              }
          dst[(size_t)x + (size_t)dm[0] * ((size_t)y + (size_t)dm[1] * z)] = swc / sw;
        }
      }
    }
  }
  for (auto& v : out) v = T(-1) * std::log(T(1) - v);
}

// float -> IEEE binary16 (round to nearest, ties to even) -> float: the
// RGB16F storage of the reference's gradient texture.
float to_half(float v) {
  if (!std::isfinite(v) || v == 0.0f) return v;
  const double a = std::fabs((double)v);
  if (a >= 65520.0) return std::copysign(INFINITY, v);
  int e;
  std::frexp(a, &e);                     // a = m 2^e, m in [0.5, 1)
  const int ue = std::max(e - 11, -24);  // 11 significant bits; subnormal spacing 2^-24
  const double r = std::nearbyint(std::ldexp(a, -ue));
  return (float)std::copysign(std::ldexp(r, ue), (double)v);
}

// DataManager::GenerateStructuredGradientTexture (datamanager.cpp:332-352):
// GenerateGradientTexture (utils.cpp:146-284) for finite differences,
// GenerateSobelFeldmanGradientTexture (utils.cpp:287-351) for both Sobel
// models (the compute-shader one, sobelfeldman_generator.comp, is the same
// stencil), in double, stored as float then FP16.
void build_gradient(Scene& s, const cvr_gradient_params& p) {
  const int W = s.nx, H = s.ny, D = s.nz;
  auto S = [&](int x, int y, int z) -> double {  // GetNormalizedSample (structuredgridvolume.cpp:121-150)
    if (x < 0 || y < 0 || z < 0 || x >= W || y >= H || z >= D) return 0.0;
    return s.vox_norm((size_t)x + (size_t)W * ((size_t)y + (size_t)H * z));
  };
  std::vector<V3<double>> g((size_t)W * H * D);
  for (int z = 0; z < D; ++z)
    for (int y = 0; y < H; ++y)
      for (int x = 0; x < W; ++x) {
        V3<double> r{0, 0, 0};
        if (p.model == CVR_GRADIENT_FINITE_DIFFERENCES) {
          const int n = p.sample_size;
          V3<double> s1{S(x - n, y, z), S(x, y - n, z), S(x, y, z - n)};
          V3<double> s2{S(x + n, y, z), S(x, y + n, z), S(x, y, z + n)};
          r = s2 - s1;
          if (p.normalized) r = normalize(r);
          else r = v3<double>(r.x / 2.0f * (float)n, r.y / 2.0f * (float)n, r.z / 2.0f * (float)n);
          if (r.x != r.x) r = v3<double>(0, 0, 0);
        } else {
          for (int v1 = -1; v1 <= 1; ++v1)
            for (int v2 = -1; v2 <= 1; ++v2) {
              const double w = 4.0 / std::pow(2.0, std::abs(v1) + std::abs(v2));
              r.z += S(x + v1, y + v2, z - 1) * w + S(x + v1, y + v2, z + 1) * -w;
              r.y += S(x + v1, y - 1, z + v2) * w + S(x + v1, y + 1, z + v2) * -w;
              r.x += S(x - 1, y + v2, z + v1) * w + S(x + 1, y + v2, z + v1) * -w;
            }
        }
        g[(size_t)x + (size_t)W * ((size_t)y + (size_t)H * z)] = r;
      }
  if (p.model == CVR_GRADIENT_FINITE_DIFFERENCES && p.filter_nxnxn > 0) {
    // utils.cpp:196-233: the window sums the centre's own gradient num times
    const int fn = (p.filter_nxnxn - 1) / 2;
    size_t index = 0;
    for (int z = 0; z < D; ++z)
      for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
          V3<double> avg{0, 0, 0};
          int num = 0;
          for (int k = z - fn; k <= z + fn; ++k)
            for (int j = y - fn; j <= y + fn; ++j)
              for (int i = x - fn; i <= x + fn; ++i)
                if (!(i < 0 || j < 0 || k < 0 || i >= W || j >= H || k >= D)) {
                  avg = avg + g[(size_t)x + (size_t)W * ((size_t)y + (size_t)H * z)];
                  ++num;
                }
          avg = v3<double>(avg.x / (double)num, avg.y / (double)num, avg.z / (double)num);
          if (avg.x != 0.0 && avg.y != 0.0 && avg.z != 0.0) avg = normalize(avg);
          g[index++] = avg;
        }
  }
  s.grad.resize(3 * g.size());
  for (size_t i = 0; i < g.size(); ++i) {
    s.grad[3 * i] = to_half((float)g[i].x);
    s.grad[3 * i + 1] = to_half((float)g[i].y);
    s.grad[3 * i + 2] = to_half((float)g[i].z);
  }
  s.grad_ready = true;
}

}  // namespace

extern "C" {

void* oracle_create(void) { return new Scene(); }
void oracle_destroy(void* h) { delete (Scene*)h; }

int oracle_set_volume(void* h, const void* vox, int w, int hh, int d, int dtype, double sx, double sy, double sz) {
  Scene& s = *(Scene*)h;
  if (!vox || w <= 0 || hh <= 0 || d <= 0 || (dtype != CVR_U8 && dtype != CVR_U16)) return CVR_ERR_INVALID_ARG;
  s.nx = w; s.ny = hh; s.nz = d; s.dtype = dtype;
  s.sx = sx; s.sy = sy; s.sz = sz;
  size_t n = (size_t)w * hh * d * (dtype == CVR_U8 ? 1 : 2);
  s.vox.assign((const uint8_t*)vox, (const uint8_t*)vox + n);
  s.sat_ready = s.pyr_ready = false;
  s.grad_ready = false;
  return 0;
}

int oracle_set_tf(void* h, const float* rgbt, const float* rgba, int n) {
  Scene& s = *(Scene*)h;
  if (!rgbt || !rgba || n < 2) return CVR_ERR_INVALID_ARG;
  s.rgbt.assign(rgbt, rgbt + 4 * (size_t)n);
  s.rgba.assign(rgba, rgba + 4 * (size_t)n);
  s.tf_n = n;
  return 0;
}

// GenerateExtinctionSAT3DTex (ebsrenderer.cpp:624-723): zero-border grid of the
// per-voxel extinction, then the 3D inclusive prefix sum in FP64 (the
// recurrence of SummedAreaTable3D::BuildSAT, summedareatable.h:218-280),
// then the FP32 copy the reference uploads.
int oracle_build_sat(void* h, const double* ext, int n_values) {
  Scene& s = *(Scene*)h;
  if (!ext || n_values != (s.dtype == CVR_U8 ? 256 : 65536)) return CVR_ERR_INVALID_ARG;
  const int W = s.nx + 2, H = s.ny + 2, D = s.nz + 2;
  std::vector<double>& a = s.sat64;
  a.assign((size_t)W * H * D, 0.0);
  for (int z = 1; z < D - 1; ++z)
    for (int y = 1; y < H - 1; ++y)
      for (int x = 1; x < W - 1; ++x) {
        size_t vi = (size_t)(x - 1) + (size_t)s.nx * ((size_t)(y - 1) + (size_t)s.ny * (z - 1));
        unsigned v = s.dtype == CVR_U8 ? s.vox[vi] : (unsigned)(s.vox[2 * vi] | (s.vox[2 * vi + 1] << 8));
        a[(size_t)x + (size_t)W * ((size_t)y + (size_t)H * z)] = ext[v];
      }
  auto G = [&](int x, int y, int z) -> double {
    if (x < 0 || y < 0 || z < 0) return 0.0;
    return a[(size_t)x + (size_t)W * ((size_t)y + (size_t)H * z)];
  };
  for (int z = 0; z < D; ++z)
    for (int y = 0; y < H; ++y)
      for (int x = 0; x < W; ++x) {
        double v = G(x, y, z) + G(x - 1, y - 1, z - 1) + G(x, y, z - 1) + G(x, y - 1, z) + G(x - 1, y, z) -
                   G(x - 1, y - 1, z) - G(x, y - 1, z - 1) - G(x - 1, y, z - 1);
        a[(size_t)x + (size_t)W * ((size_t)y + (size_t)H * z)] = v;
      }
  s.sat32.assign(a.begin(), a.end());
  s.sat_ready = true;
  return 0;
}

int oracle_get_sat(void* h, double* out) {
  Scene& s = *(Scene*)h;
  if (!s.sat_ready || !out) return CVR_ERR_NOT_READY;
  std::memcpy(out, s.sat64.data(), s.sat64.size() * sizeof(double));
  return 0;
}

// Exact integer SAT of q[voxel] with the zero border (the fixed-point form the
// GPU builds), computed by separable prefix sums.
int oracle_sat_i64(const void* vox, int nx, int ny, int nz, int dtype, const int64_t* q, int64_t* out) {
  const int W = nx + 2, H = ny + 2, D = nz + 2;
  std::memset(out, 0, sizeof(int64_t) * (size_t)W * H * D);
  for (int z = 1; z < D - 1; ++z)
    for (int y = 1; y < H - 1; ++y)
      for (int x = 1; x < W - 1; ++x) {
        size_t vi = (size_t)(x - 1) + (size_t)nx * ((size_t)(y - 1) + (size_t)ny * (z - 1));
        unsigned v = dtype == CVR_U8 ? ((const uint8_t*)vox)[vi] : ((const uint16_t*)vox)[vi];
        out[(size_t)x + (size_t)W * ((size_t)y + (size_t)H * z)] = q[v];
      }
  for (int z = 0; z < D; ++z)
    for (int y = 0; y < H; ++y)
      for (int x = 1; x < W; ++x) out[(size_t)x + (size_t)W * ((size_t)y + (size_t)H * z)] += out[(size_t)(x - 1) + (size_t)W * ((size_t)y + (size_t)H * z)];
  for (int z = 0; z < D; ++z)
    for (int y = 1; y < H; ++y)
      for (int x = 0; x < W; ++x) out[(size_t)x + (size_t)W * ((size_t)y + (size_t)H * z)] += out[(size_t)x + (size_t)W * ((size_t)(y - 1) + (size_t)H * z)];
  for (int z = 1; z < D; ++z)
    for (int y = 0; y < H; ++y)
      for (int x = 0; x < W; ++x) out[(size_t)x + (size_t)W * ((size_t)y + (size_t)H * z)] += out[(size_t)x + (size_t)W * ((size_t)y + (size_t)H * (z - 1))];
  return 0;
}

int oracle_build_pyramid(void* h, const cvr_pyramid_params* p) {
  Scene& s = *(Scene*)h;
  if (!p || s.tf_n == 0 || s.vox.empty()) return CVR_ERR_NOT_READY;
  int maxdim = std::max(p->base_dims[0], std::max(p->base_dims[1], p->base_dims[2]));
  int chain = 1;
  while ((maxdim >> chain) > 0) ++chain;
  int levels = p->n_levels > 0 ? std::min(p->n_levels, chain) : chain;
  levels = std::min(levels, 16);
  size_t off = 0;
  for (int l = 0; l < levels; ++l) {
    for (int a = 0; a < 3; ++a) s.ldims[l][a] = std::max(1, p->base_dims[a] >> l);
    s.loff[l] = off;
    off += (size_t)s.ldims[l][0] * s.ldims[l][1] * s.ldims[l][2];
  }
  s.n_levels = levels;
  build_pyramid_t<double>(s, p->sigma0, s.pyr64);
  build_pyramid_t<float>(s, p->sigma0, s.pyr32);
  s.pyr_ready = true;
  return levels;
}

int oracle_get_pyramid_level(void* h, int precision, int level, double* out) {
  Scene& s = *(Scene*)h;
  if (!s.pyr_ready || level < 0 || level >= s.n_levels) return CVR_ERR_INVALID_ARG;
  size_t n = (size_t)s.ldims[level][0] * s.ldims[level][1] * s.ldims[level][2];
  for (size_t i = 0; i < n; ++i)
    out[i] = precision == 64 ? s.pyr64[s.loff[level] + i] : (double)s.pyr32[s.loff[level] + i];
  return 0;
}

int oracle_set_cone_tables(void* h, const cvr_cone_table* occ, const cvr_cone_table* sdw) {
  Scene& s = *(Scene*)h;
  if (!occ || !sdw) return CVR_ERR_INVALID_ARG;
  s.occ = *occ;
  s.sdw = *sdw;
  s.cone_ready = true;
  return 0;
}

int oracle_set_gt_kernels(void* h, const float* occ, int n_occ, const float* sdw, int n_sdw) {
  Scene& s = *(Scene*)h;
  s.occ_vec.assign(occ, occ + 3 * (size_t)n_occ);
  s.sdw_vec.assign(sdw, sdw + 3 * (size_t)n_sdw);
  s.gt_ready = true;
  return 0;
}

int oracle_set_light_cache(void* h, int w, int hh, int d) {
  Scene& s = *(Scene*)h;
  if (w < 0 || hh < 0 || d < 0) return CVR_ERR_INVALID_ARG;
  s.lc[0] = w; s.lc[1] = hh; s.lc[2] = d;
  return 0;
}

int oracle_build_gradient(void* h, const cvr_gradient_params* p) {
  Scene& s = *(Scene*)h;
  s.grad_ready = false;
  s.grad.clear();
  if (!p || p->model == CVR_GRADIENT_NONE) return 0;
  if (p->model < 0 || p->model > CVR_GRADIENT_NONE || s.vox.empty()) return CVR_ERR_INVALID_ARG;
  if (p->model == CVR_GRADIENT_FINITE_DIFFERENCES && p->sample_size < 1) return CVR_ERR_INVALID_ARG;
  build_gradient(s, *p);
  return 0;
}

int oracle_get_gradient(void* h, float* out) {
  Scene& s = *(Scene*)h;
  if (!s.grad_ready) return CVR_ERR_NOT_READY;
  std::memcpy(out, s.grad.data(), sizeof(float) * s.grad.size());
  return 0;
}

int oracle_set_blinn_phong(void* h, const cvr_blinn_phong* bp) {
  if (!bp) return CVR_ERR_INVALID_ARG;
  ((Scene*)h)->bp = *bp;
  return 0;
}

int oracle_set_mlp(void* h, const float* params, int n) {
  Scene& s = *(Scene*)h;
  if (!params || n != CVR_MLP_PARAMS) return CVR_ERR_INVALID_ARG;
  s.mlp.assign(params, params + n);
  return 0;
}

// Network inputs (n x 48) of n points (n x 6: texture-space position, primary
// direction) and, when y_out is given and parameters are set, the network's
// outputs (n x 2) on the FP64 features.
int oracle_sur_features(void* h, int precision, const cvr_light* light, int shadow_type, double sdw_dist,
                        const float* pts, int n, double* x_out, double* y_out) {
  Scene& s = *(Scene*)h;
  if (!light || !pts || !x_out || n < 0) return CVR_ERR_INVALID_ARG;
  if (!s.pyr_ready || s.n_levels < 6) return CVR_ERR_NOT_READY;
  if (y_out && s.mlp.size() != (size_t)CVR_MLP_PARAMS) return CVR_ERR_NOT_READY;
  auto run = [&](auto zero) {
    using T = decltype(zero);
    Frame<T> f;
    f.s = &s;
    f.spacing = v3<T>(T(s.sx), T(s.sy), T(s.sz));
    f.grid = v3<T>(T(s.nx * s.sx), T(s.ny * s.sy), T(s.nz * s.sz));
    const std::vector<T>* pyr;
    if constexpr (sizeof(T) == 8) pyr = &s.pyr64;
    else pyr = &s.pyr32;
    for (int i = 0; i < n; ++i) {
      const float* q = pts + 6 * (size_t)i;
      T x[48];
      sur_features<T>(f, s, *pyr, shadow_type, from<T>(light->position), from<T>(light->forward), T(sdw_dist),
                      from<T>(q), from<T>(q + 3), x);
      double* xo = x_out + 48 * (size_t)i;
      for (int k = 0; k < 48; ++k) xo[k] = (double)x[k];
      if (y_out) mlp_forward_bf16(s.mlp, xo, y_out + 2 * (size_t)i);
    }
  };
  if (precision == 64) run(0.0);
  else run(0.0f);
  return 0;
}

// Ground-truth (occlusion, shadow) of n points (n x 6), the integrator of
// gt_ray_marching.comp:109-252 with the scene's kernel vectors.
int oracle_gt_points(void* h, const cvr_light* light, const cvr_gt_params* p, const float* pts, int n, double* out) {
  Scene& s = *(Scene*)h;
  if (!light || !p || !pts || !out || n < 0) return CVR_ERR_INVALID_ARG;
  if (!s.gt_ready) return CVR_ERR_NOT_READY;
  Frame<double> f;
  f.s = &s;
  f.spacing = v3<double>(s.sx, s.sy, s.sz);
  f.grid = v3<double>(s.nx * s.sx, s.ny * s.sy, s.nz * s.sz);
  Gt<double> g;
  g.p = p; g.s = &s;
  g.light_pos = from<double>(light->position); g.light_fwd = from<double>(light->forward);
  g.light_up = from<double>(light->up); g.light_right = from<double>(light->right);
  for (int i = 0; i < n; ++i) {
    const float* q = pts + 6 * (size_t)i;
    V3<double> tx = from<double>(q), dir = from<double>(q + 3);
    V3<double> v_right = normalize(cross(dir, v3<double>(0, 1, 0)));
    V3<double> v_up = normalize(cross(-dir, v_right));
    out[2 * (size_t)i] = gt_occlusion(f, g, tx, v_up, v_right, dir);
    out[2 * (size_t)i + 1] = gt_shadow(f, g, tx);
  }
  return 0;
}

// Renders rows [y0, y1) of a W x H frame in FP64 (precision 64) or FP32 (32).
int oracle_render(void* h, int precision, int method, const cvr_camera* cam, const cvr_light* light,
                  const void* params, int W, int H, int y0, int y1, double* out, uint32_t* counts, uint64_t* total,
                  int threads) {
  Scene& s = *(Scene*)h;
  if (!cam || !params || !out || W <= 0 || H <= 0 || y0 < 0 || y1 > H || y0 >= y1) return CVR_ERR_INVALID_ARG;
  if (s.vox.empty() || s.tf_n == 0) return CVR_ERR_NO_VOLUME;
  cvr_light dl{};
  const cvr_light& L = light ? *light : dl;
  if (threads <= 0) threads = 1;
  if (precision == 64) return render_t<double>(s, method, *cam, L, params, W, H, y0, y1, out, counts, total, threads);
  return render_t<float>(s, method, *cam, L, params, W, H, y0, y1, out, counts, total, threads);
}

}  // extern "C"
