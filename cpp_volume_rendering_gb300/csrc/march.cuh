// march.cuh — kernel argument blocks shared by march.cu and the context code.
#pragma once

#include "cvr_device.cuh"

#include <mutex>
#include <tuple>
#include <vector>

namespace cvr {

#define CVR_MAX_GT_RAYS 256

// Gradient Blinn-Phong shading (the ApplyPhongShading / ApplyGradientPhongShading
// branches of the four ShadeSample functions): the per-voxel gradient of
// cvr_build_gradient, the light position and the Blinn-Phong constants.
struct GradView {
  const uint2* g;             // 4 halves per voxel (gx, gy, gz, 0), x fastest; nullptr: shading off
  cudaTextureObject_t tex;    // texture copy (hardware trilinear) or 0: the array with FP32 weights
  int nx, ny, nz;
  float3 inv_grid;            // 1 / VolumeGridSize (texture coordinates)
  float3 inv_spacing;         // 1 / VolumeScales (texel coordinates)
  float3 light_pos;           // LightSourcePosition / WorldLightingPos
  float3 ispec;               // BlinnPhongIspecular / Ispecular
  float ka, kd;               // BlinnPhongKa / Kd (the plain renderer's; the others bring theirs)
  float ks, shininess;        // BlinnPhongKs / Kspecular, BlinnPhongShininess / Nshininess
};

// Launch geometry: each CTA covers a tile_w x tile_h block of pixels; each
// warp covers an 8x4 sub-tile so the 32 rays of a warp stay spatially
// coherent (they walk neighbouring voxels, which keeps gathers in L1).
struct FrameArgs {
  VolumeView vol;
  CameraView cam;
  const float4* tf;      // RGBt table (alpha = extinction)
  int tf_n;
  float step;            // StepSize
  int W, H;
  int tile_w, tile_h;    // pixels per CTA: (tile_w/8) x (tile_h/4) warps of 8x4 pixels (2, 4 or 8 warps)
  int warp_w;            // pixels per warp row: 4, 8 or 16 (warps of warp_w x 32/warp_w; other values: 8)
  int variant;           // register / occupancy variant of the kernel (0, 1, 2)
  float4* out;
  uint32_t* counts;                // per-pixel step count, nullable
  unsigned long long* stats;       // [0] samples, [1] shaded samples, [2] secondary fetches
  GradView grad;                   // gradient shading (grad.g == nullptr: off)
  // Ray counter of the persistent ray-refill marchers (zeroed before the
  // launch), or nullptr: one CTA per tile_w x tile_h block of pixels.
  unsigned* work;
};

struct ExtArgs {
  SatView sat;
  int apply_occ, apply_sdw;
  int n_shells;
  float radii[32];
  float cone_angle, interval, initial, ui_weight, max_dist;
  int shadow_type;
  float3 light_pos, light_fwd;
  float ka, kd;
  // every AO box has integer texel widths (2 r): the compact table's
  // equal-fraction query applies (sat_box_aligned)
  int ao_aligned;
  // the directional shadow's walk table (walk.oct nullptr: none)
  WalkView walk;
};

// Boxes of the SAT shadow cone of a directional light.  The cone direction is
// the same for every sample, so the box offsets of ConeZAxis / ConeYAxis /
// ConeXAxis (ebs_ray_bbox_marching.comp:190-430) depend only on the box index
// and are computed once per frame; each sample keeps its own
// CUT_WHEN_AWAY_FROM_VOLUME test.
#define CVR_MAX_SDW_BOXES 512
struct ShadowBoxTable {
  int n;           // boxes passing the max-distance test
  int axis;        // dominant axis of the light direction
  float interval;  // signed box step along the axis (world units)
  float vmin, vmax;
  float4 lo[CVR_MAX_SDW_BOXES];  // xyz: low corner offset, w: position along the axis
  float4 hi[CVR_MAX_SDW_BOXES];  // xyz: high corner offset, w: UI weight / box volume in voxels
  // Every box has integer texel widths below 1024 on all three axes (the
  // cross-sections are rounded up to whole voxels; the walk axis has the
  // sample interval): tx holds, per box, the low corner offset in texel units
  // (xyz) and the widths packed as wx | wy << 10 | wz << 20 (w, as int bits),
  // for the compact table's equal-fraction query.  0: tx is unused.
  int aligned;
  float4 tx[CVR_MAX_SDW_BOXES];
};

struct ConeTableDev {
  int n_sections;
  int n1, n3, n7;
  float3 axes[10];
  float initial_step, w7, ui_weight;
};

struct DosArgs {
  PyramidView pyr;
  // FP16 texture copies of the levels (the reference's R16F pyramid, sampled
  // by the texture unit) when CVR_SAMPLING_TEX_PYRAMID is set, else unused
  cudaTextureObject_t ptex[CVR_MAX_LEVELS];
  const float4* occ_sections;  // device, n_sections entries
  const float4* sdw_sections;
  ConeTableDev occ, sdw;
  int apply_occ, apply_sdw, shadow_type;
  float3 light_pos, light_fwd, light_up, light_right;
  float spot_cos_max;
  float ka, kd;
};

struct GtArgs {
  const float3* occ_vec;  // device
  const float3* sdw_vec;
  int n_occ, n_sdw;
  float gap, lstep;
  int apply_occ, apply_sdw, shadow_type;
  float occ_dist, sdw_dist;
  float3 light_pos, light_fwd, light_up, light_right;
  float ka, kd;
};

// Isosurface ray casting with adaptive steps (ray_marching_1p_iso_adapt.comp).
struct IsoArgs {
  float step_small, step_large, step_range, iso;
  float4 color;
};

// CTAs of kern that fit on one SM at once, from its shared memory (dynamic +
// static + the per-block reservation) and registers (allocated per warp in
// units of 8 per thread).  Persistent launches size their grids with it.
template <class K>
cudaError_t resident_ctas(K kern, int threads, size_t dyn_smem, int* out) {
  int dev = 0, smem_sm = 0, reserved = 0, regs_sm = 0, threads_sm = 0;
  cudaError_t e;
  if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
  if ((e = cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev)) != cudaSuccess) return e;
  if ((e = cudaDeviceGetAttribute(&reserved, cudaDevAttrReservedSharedMemoryPerBlock, dev)) != cudaSuccess) return e;
  if ((e = cudaDeviceGetAttribute(&regs_sm, cudaDevAttrMaxRegistersPerMultiprocessor, dev)) != cudaSuccess) return e;
  if ((e = cudaDeviceGetAttribute(&threads_sm, cudaDevAttrMaxThreadsPerMultiProcessor, dev)) != cudaSuccess) return e;
  cudaFuncAttributes fa{};
  if ((e = cudaFuncGetAttributes(&fa, kern)) != cudaSuccess) return e;
  int n = smem_sm / (int)(dyn_smem + fa.sharedSizeBytes + (size_t)reserved);
  const int regs_cta = ((fa.numRegs + 7) / 8) * 8 * threads;
  if (regs_cta > 0) n = n < regs_sm / regs_cta ? n : regs_sm / regs_cta;
  n = n < threads_sm / threads ? n : threads_sm / threads;
  *out = n < 1 ? 1 : n;
  return cudaSuccess;
}

// Shared-memory carveout of kern sized to the CTAs resident_ctas lets reside,
// so that the rest of the SM's unified L1 / shared storage serves as L1 cache
// (with no preference the driver reserves shared memory for as many CTAs as
// the shared memory alone would allow, e.g. 100 KB where the registers let 4
// CTAs of 11.6 KB reside).  Set once per device, kernel and size.
template <class K>
cudaError_t carve_l1(K kern, int threads, size_t dyn_smem) {
  static std::mutex mu;
  static std::vector<std::tuple<int, const void*, size_t>> done;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  const auto key = std::make_tuple(dev, reinterpret_cast<const void*>(kern), dyn_smem);
  std::lock_guard<std::mutex> lock(mu);
  for (const auto& k : done)
    if (k == key) return cudaSuccess;
  int n = 0, smem_sm = 0, reserved = 0;
  if ((e = resident_ctas(kern, threads, dyn_smem, &n)) != cudaSuccess) return e;
  if ((e = cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev)) != cudaSuccess) return e;
  if ((e = cudaDeviceGetAttribute(&reserved, cudaDevAttrReservedSharedMemoryPerBlock, dev)) != cudaSuccess) return e;
  cudaFuncAttributes fa{};
  if ((e = cudaFuncGetAttributes(&fa, kern)) != cudaSuccess) return e;
  const size_t need = (size_t)n * (dyn_smem + fa.sharedSizeBytes + (size_t)reserved);
  int pct = (int)((need * 100 + (size_t)smem_sm - 1) / (size_t)smem_sm);
  pct = pct < 1 ? 1 : (pct > 100 ? 100 : pct);
  if ((e = cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, pct)) != cudaSuccess) return e;
  if (done.size() >= 1024) done.clear();
  done.push_back(key);
  return cudaSuccess;
}

// One job of a batch of extinction frames (device table entry).  f.stats
// points at the job's three counters; f.tile_w / tile_h are the batch's tile.
struct BatchExtJob {
  FrameArgs f;
  ExtArgs e;
  const float4* tlo;  // directional shadow-box table in global memory, or null
  const float4* thi;
  const float4* ttx;  // the table's texel offsets and widths (ShadowBoxTable::tx), or null
  int tn, tax;
  float tiw, tvmin, tvmax;
  unsigned first_block;  // first batch-wide tile index of the job
  unsigned blocks_x;     // tiles per image row
};

// Persistent launch over all tiles of all jobs (jobs ordered by first_block):
// each CTA takes tiles from *counter (zeroed before the launch).  variant as
// in FrameArgs; max_table = the largest shadow table of the jobs; compact:
// every job reads its compact SAT (ExtArgs::sat.sat32); aligned: every job
// has an aligned shadow table (ttx) and aligned AO boxes (or AO off).
cudaError_t launch_batch_extinction(const BatchExtJob* jobs, int n_jobs, unsigned total_blocks, unsigned* counter,
                                    int tf_n, int max_table, int tile_threads, int variant, bool compact,
                                    bool aligned, cudaStream_t st);

// Object-space light cache (lightcache.cu).  Cells of dims[0] x dims[1] x
// dims[2], x fastest, float2 (occlusion, shadow).  table: the directional
// shadow-box table or null (storage: any table object, passed when null).
cudaError_t launch_cache_extinction(const FrameArgs& f, const ExtArgs& e, const ShadowBoxTable* table,
                                    const ShadowBoxTable& storage, const int dims[3], float2* out, cudaStream_t st);
cudaError_t launch_cache_dos(const FrameArgs& f, const DosArgs& d, const int dims[3], float2* out, cudaStream_t st);
cudaError_t launch_march_cached(const FrameArgs& f, const float2* cache, const int dims[3], int apply_occ,
                                int apply_sdw, float ka, float kd, cudaStream_t st);

cudaError_t launch_plain(const FrameArgs& f, cudaStream_t st);
// The plain marcher with shared-memory brick staging (staged.cu): plain
// volume layout, FP32 samples only (plain_staging_applies).
bool plain_staging_applies(const FrameArgs& f);
cudaError_t launch_plain_staged(const FrameArgs& f, cudaStream_t st);
cudaError_t launch_iso(const FrameArgs& f, const IsoArgs& a, cudaStream_t st);
// table == nullptr: per-sample cone geometry (point lights, or too many boxes);
// storage: any table object (the persistent variant's argument when table is null).
cudaError_t launch_extinction(const FrameArgs& f, const ExtArgs& e, const ShadowBoxTable* table,
                              const ShadowBoxTable& storage, cudaStream_t st);
// tex_pyramid: the pyramid taps read d.ptex (FP16 level textures).
cudaError_t launch_dos(const FrameArgs& f, const DosArgs& d, bool tex_pyramid, cudaStream_t st);
cudaError_t launch_gt(const FrameArgs& f, const GtArgs& g, cudaStream_t st);

}  // namespace cvr
