// surrogate.cuh — the learned stand-in for the ground-truth light integrals of
// RC1PConeLightGroundTruthSteps (gt_ray_marching.comp:109-252): a feature
// vector of multi-level extinction samples around a shading point, the light
// direction and the local extinction gradient, mapped by the MLP of mlp.cuh
// to (ambient occlusion, shadow).
//
// Features at a shading point tx (texture-space position in [0, S]) of a
// primary ray with direction dir:
//   frame  n = -dir, r = normalize(dir x (0,1,0)), u = normalize(-dir x r)
//          (the (v_right, v_up, -dir) frame of the ground-truth occlusion
//          kernel, gt_ray_marching.comp:396-399)
//   light  L = normalize(light_pos - world(tx)) for point and spot lights,
//          L = light forward vector for directional lights
//   taps   for level l = 0..5, d_l = unit * 2^(l+1) (unit = mean voxel
//          spacing): x[7l + k] = 1 - exp(-sigma_l(tx + offset_k) * d_l), where
//          sigma_l is level l of the Gaussian extinction pyramid (trilinear
//          within the level) and 0 outside the volume box, with offsets
//            k = 0: 0 (the centre)
//            k = 3, 4: n * d_l, n * 3 d_l;  k = 5: +-r * d_l and k = 6:
//                   +-u * d_l, each the mean extinction of the two taps
//                   (1 - exp(-(sigma_l(tx + o) + sigma_l(tx - o)) d_l / 2))
//          except the light taps k = 1, 2: the segments [2 d_l - 4 unit,
//          3 d_l - 4 unit] and [3 d_l - 4 unit, 4 d_l - 4 unit] of the light ray
//          tx + L s (the twelve partition [0, 252 unit] into segments of
//          doubling length), each clipped to the ray's end t_end = min(box exit,
//          shadow-ray length): 1 - exp(-sigma_l(midpoint) * clipped length), 0
//          when nothing is left; and x[35] (level 5, centre): the rest of the
//          light ray, 1 - exp(-sum_j sigma_5(midpoint_j) * length_j) over the
//          segments [(4 + j) d_5 - 4 unit, (5 + j) d_5 - 4 unit], j = 0..7
//          (252 ... 764 unit), clipped the same way
//   x[42..44] = (L.r, L.u, L.n)
//   x[45..47] = (g.r, g.u, g.n), g = central differences of pyramid level 0
//               at +-1 voxel, times the voxel length (the level-0 taps are
//               in cache: no second copy of the volume is read)
// The same routine produces training inputs and the marcher's inputs.
#pragma once

#include "march.cuh"
#include "mlp.cuh"

namespace cvr {

constexpr int kSurLevels = 6;
constexpr int kSurTaps = 7;
constexpr int kSurTapFeatures = kSurLevels * kSurTaps;  // 42
// Pyramid taps per shading point: 9 per level (centre, 2 light-ray segments,
// 2 along n, the +-r and +-u pairs) on levels 0-4, the far path's 8 and 8 on
// level 5, and the gradient's 6 on level 0.
constexpr int kSurPyramidTaps = 5 * 9 + 8 + 8 + 6;  // 67

struct SurArgs {
  PyramidView pyr;  // at least kSurLevels levels
  cudaTextureObject_t ptex[kSurLevels];  // texture-unit copies of the first levels (tex sampling)
  const uint8_t* packed;  // packed network image (mlp.cuh)
  int apply_occ, apply_sdw, shadow_type;
  float3 light_pos, light_fwd;
  float ka, kd;
  float unit;      // world length of one voxel (mean spacing)
  float sdw_dist;  // shadow-ray length of the integrator the network stands in for
};

struct SurFrame { float3 n, r, u, L; };

__device__ __forceinline__ SurFrame sur_frame(const SurArgs& a, float3 tx, float3 dir, float3 grid) {
  SurFrame F;
  F.n = normalize3(-dir);
  float3 c = cross3(dir, f3(0.0f, 1.0f, 0.0f));
  // A ray parallel to y has no right vector; any perpendicular frame will do.
  if (dot3(c, c) < 1.0e-12f) c = f3(1.0f, 0.0f, 0.0f);
  F.r = normalize3(c);
  F.u = normalize3(cross3(-dir, F.r));
  F.L = a.shadow_type == 2 ? a.light_fwd : normalize3(a.light_pos - (tx - grid * 0.5f));
  return F;
}

// Extinction of pyramid level l at texture-space q: FP32 trilinear, or the
// texture unit's trilinear (8-bit interpolation weights).
template <bool TEX>
__device__ __forceinline__ float sur_sigma(const SurArgs& a, int l, float3 q) {
  if constexpr (TEX) {
    return tex3D<float>(a.ptex[l], q.x * a.pyr.inv_grid.x, q.y * a.pyr.inv_grid.y, q.z * a.pyr.inv_grid.z);
  } else {
    return pyr_sample_level(a.pyr, l, q);
  }
}

// Extinction of level l at q, 0 outside the box.
template <bool TEX>
__device__ __forceinline__ float sur_sigma_box(const SurArgs& a, int l, float3 q, float3 S) {
  if (q.x < 0.0f || q.x > S.x || q.y < 0.0f || q.y > S.y || q.z < 0.0f || q.z > S.z) return 0.0f;
  return sur_sigma<TEX>(a, l, q);
}

// Segment opacity 1 - exp(-sigma_l(q) d) of one tap; 0 outside the box.
template <bool TEX>
__device__ __forceinline__ float sur_tap(const SurArgs& a, int l, float3 q, float d, float3 S) {
  if (q.x < 0.0f || q.x > S.x || q.y < 0.0f || q.y > S.y || q.z < 0.0f || q.z > S.z) return 0.0f;
  return 1.0f - __expf(-sur_sigma<TEX>(a, l, q) * d);
}

// The same for the mean extinction of the taps at c + o and c - o.
template <bool TEX>
__device__ __forceinline__ float sur_tap_pair(const SurArgs& a, int l, float3 c, float3 o, float d, float3 S) {
  const float s2 = sur_sigma_box<TEX>(a, l, c + o, S) + sur_sigma_box<TEX>(a, l, c - o, S);
  return 1.0f - __expf(-(0.5f * s2) * d);
}

// Length of the light ray tx + L s inside the box [0, S] (tx inside) and
// within the shadow-ray length: the end of the light path the taps cover.
__device__ __forceinline__ float sur_ray_end(const SurArgs& a, float3 tx, float3 L, float3 S) {
  float t = a.sdw_dist;
  if (L.x > 0.0f) t = fminf(t, (S.x - tx.x) / L.x); else if (L.x < 0.0f) t = fminf(t, -tx.x / L.x);
  if (L.y > 0.0f) t = fminf(t, (S.y - tx.y) / L.y); else if (L.y < 0.0f) t = fminf(t, -tx.y / L.y);
  if (L.z > 0.0f) t = fminf(t, (S.z - tx.z) / L.z); else if (L.z < 0.0f) t = fminf(t, -tx.z / L.z);
  return fmaxf(t, 0.0f);
}

// Optical depth sigma_l(midpoint) * length of the light-ray segment [s0, s1]
// clipped to [0, t_end] (0 when nothing is left).
template <bool TEX>
__device__ __forceinline__ float sur_seg_tau(const SurArgs& a, int l, float3 tx, float3 L, float s0, float s1,
                                             float t_end) {
  s0 = fmaxf(s0, 0.0f);
  s1 = fminf(s1, t_end);
  if (!(s1 > s0)) return 0.0f;
  return sur_sigma<TEX>(a, l, tx + L * (0.5f * (s0 + s1))) * (s1 - s0);
}

// The rest of the light path: level-5 optical depth of the eight segments
// beyond the twelve light taps.
template <bool TEX>
__device__ __forceinline__ float sur_far(const SurArgs& a, float3 tx, float3 L, float d5, float t_end) {
  float tau = 0.0f;
  const float s0 = fmaf(4.0f, d5, -4.0f * a.unit);
#pragma unroll 1
  for (int j = 0; j < 8; ++j) {
    const float lo = fmaf((float)j, d5, s0);
    if (!(lo < t_end)) break;
    tau += sur_seg_tau<TEX>(a, kSurLevels - 1, tx, L, lo, lo + d5, t_end);
  }
  return 1.0f - __expf(-tau);
}

// The 48 features of one shading point (layout above), handed to out(k, v)
// in order k = 0..47.
template <bool TEX, class Sink>
__device__ __forceinline__ void sur_features(const SurArgs& a, const VolumeView& vol, const float4* tf, int tf_n,
                                             float3 tx, float3 dir, Sink& out) {
  const float3 S = vol.grid;
  SurFrame F = sur_frame(a, tx, dir, S);
  const float t_end = sur_ray_end(a, tx, F.L, S);
  const float u4 = 4.0f * a.unit;
  float d = a.unit * 2.0f;
#pragma unroll
  for (int l = 0; l < kSurLevels; ++l) {
    out(7 * l + 0, l == kSurLevels - 1 ? sur_far<TEX>(a, tx, F.L, d, t_end) : sur_tap<TEX>(a, l, tx, d, S));
    const float s0 = fmaf(2.0f, d, -u4), s1 = fmaf(3.0f, d, -u4), s2 = fmaf(4.0f, d, -u4);
    out(7 * l + 1, 1.0f - __expf(-sur_seg_tau<TEX>(a, l, tx, F.L, s0, s1, t_end)));
    out(7 * l + 2, 1.0f - __expf(-sur_seg_tau<TEX>(a, l, tx, F.L, s1, s2, t_end)));
    out(7 * l + 3, sur_tap<TEX>(a, l, tx + F.n * d, d, S));
    out(7 * l + 4, sur_tap<TEX>(a, l, tx + F.n * (3.0f * d), d, S));
    out(7 * l + 5, sur_tap_pair<TEX>(a, l, tx, F.r * d, d, S));
    out(7 * l + 6, sur_tap_pair<TEX>(a, l, tx, F.u * d, d, S));
    d *= 2.0f;
  }
  out(42, dot3(F.L, F.r));
  out(43, dot3(F.L, F.u));
  out(44, dot3(F.L, F.n));
  const float3 sp = vol.spacing;
  float3 g;
  g.x = 0.5f * sp.x * (sur_sigma<TEX>(a, 0, tx + f3(sp.x, 0.0f, 0.0f)) - sur_sigma<TEX>(a, 0, tx - f3(sp.x, 0.0f, 0.0f)));
  g.y = 0.5f * sp.y * (sur_sigma<TEX>(a, 0, tx + f3(0.0f, sp.y, 0.0f)) - sur_sigma<TEX>(a, 0, tx - f3(0.0f, sp.y, 0.0f)));
  g.z = 0.5f * sp.z * (sur_sigma<TEX>(a, 0, tx + f3(0.0f, 0.0f, sp.z)) - sur_sigma<TEX>(a, 0, tx - f3(0.0f, 0.0f, sp.z)));
  out(45, dot3(g, F.r));
  out(46, dot3(g, F.u));
  out(47, dot3(g, F.n));
}

// Shading of the ground-truth renderer with the network's outputs in place of
// the light integrals (ShadeSample, gt_ray_marching.comp:254-303).  Spot
// lights shadow everything there (the cosine is compared against 30.0), so
// the shadow term is 0 for them here as well.
__device__ __forceinline__ float4 sur_shade(const SurArgs& a, float4 src, float ao, float sdw) {
  float ka = 0.0f, kd = 0.0f, io = 0.0f, is = 0.0f;
  if (a.apply_occ) { ka = a.ka; io = fminf(fmaxf(ao, 0.0f), 1.0f); }
  if (a.apply_sdw) { kd = a.kd; is = a.shadow_type == 1 ? 0.0f : fminf(fmaxf(sdw, 0.0f), 1.0f); }
  float kk = 1.0f / (ka + kd);
  src.x = kk * (src.x * io * ka + src.x * is * kd);
  src.y = kk * (src.y * io * ka + src.y * is * kd);
  src.z = kk * (src.z * io * ka + src.z * is * kd);
  return src;
}

// Shading points of primary rays: each shaded sample (the samples that reach
// ShadeSample) is kept with probability 'rate' (a hash of seed, pixel and step),
// appended as {position, 0}, {direction, 0}.  *count is the number kept
// (it may exceed cap; only the first cap are written).
cudaError_t launch_sur_collect(const FrameArgs& f, float rate, unsigned long long seed, float4* pts, int cap,
                               unsigned int* count, cudaStream_t st);

// Features (n x 48), ground-truth targets (n x 2: GtShade occlusion and
// shadow) and, when dos_out is given, the cone method's (occlusion, shadow)
// of n points.  f supplies the volume and transfer function.
cudaError_t launch_sur_label(const float4* pts, int n, const FrameArgs& f, const SurArgs& a, bool tex,
                             const GtArgs* g, const DosArgs* d, float* x_out, float* t_out, float* dos_out,
                             cudaStream_t st);

// One job of a batch of surrogate frames (device table entry).  f.stats points
// at the job's three counters; f.tf / f.tf_n and a.packed of a launch's first
// job serve all its jobs (one transfer function and network per batch).
struct SurJob {
  FrameArgs f;
  SurArgs a;
  unsigned first_tile;  // batch-wide index of the job's first spiral position
  int cx, cy;           // the job's spiral centre tile
  int tiles_x, tiles_y;
};

// Ray order of a surrogate frame: 8x4-pixel tiles in the square spiral around
// the tile of the projected volume centre (long rays first, neighbouring
// tiles together); positions = the tiles of the spiral's bounding square
// (those outside the image are skipped).
struct SurSpiral {
  int cx, cy;
  unsigned long long positions;
};
SurSpiral sur_spiral(const FrameArgs& f);

// One persistent launch of a batch's surrogate jobs: up to kSurLaunchJobs
// jobs whose descriptors are the launch's parameters (the constant bank, read
// as the single-frame marcher reads its own), ordered by first_tile (relative
// to the launch), each job's rays in its spiral order; total = 32 x the
// spiral positions of its jobs.
constexpr int kSurLaunchJobs = 32;
struct SurLaunch {
  int n_jobs;
  unsigned total;
  SurJob jobs[kSurLaunchJobs];
};
static_assert(sizeof(SurLaunch) <= 32000, "kernel parameters are limited to 32764 bytes");

// Rays taken from *work (zeroed before the launch).
cudaError_t launch_batch_surrogate(const SurLaunch& L, int tf_n, bool tex, int variant, unsigned int* work, int* err,
                                   cudaStream_t st);

// The surrogate-shaded marcher: persistent CTAs take rays from *work (zeroed
// before the launch) in 8x4-pixel tiles in the frame's spiral order; every
// round, each thread advances its ray to the next shaded sample, the CTA
// evaluates the network for its 128 samples on the tensor cores, and each
// thread composites its sample.
cudaError_t launch_surrogate(const FrameArgs& f, const SurArgs& a, bool tex, const SurSpiral& order,
                             unsigned int* work, int* err, cudaStream_t st);

}  // namespace cvr
