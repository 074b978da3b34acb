// lightcache.cu — object-space light cache (PreIlluminationStructuredVolume,
// cppvolrend/utils/preillumination.h:15-47): the occlusion and shadow terms
// evaluated once per frame at the centres of a coarse grid
// (rc1pextbsd/lightcachecomputation.comp:443-468,
// rc1pdosct/lightcachecomputation.comp:523-547), then the object-space
// marcher (_common_shaders/obj_ray_marching.comp:264-333) shades every sample
// from a trilinear lookup of that grid.
#include "shade.cuh"

namespace cvr {

// tex_pos = (cell + 0.5) * (VolumeScales * (VolumeDimensions / LightCacheDimensions))
__device__ __forceinline__ float3 cache_cell_pos(const FrameArgs& f, const int* dims, int x, int y, int z) {
  const float3 sc = f.vol.spacing;
  return f3((float(x) + 0.5f) * (sc.x * (float(f.vol.nx) / float(dims[0]))),
            (float(y) + 0.5f) * (sc.y * (float(f.vol.ny) / float(dims[1]))),
            (float(z) + 0.5f) * (sc.z * (float(f.vol.nz) / float(dims[2]))));
}

struct CacheDims { int d[3]; };

// Extinction cache: ExtinctionAmbientOcclusion and ExtinctionDirectionalShadows
// at the cell centre (1 where a term is off), the same functions as per sample.
__global__ void __launch_bounds__(128) k_cache_extinction(FrameArgs f, ExtArgs e, CacheDims cd, int table_n,
                                                          const __grid_constant__ ShadowBoxTable t,
                                                          float2* __restrict__ out) {
  extern __shared__ float4 sm_lc[];
  for (int i = threadIdx.x; i < table_n; i += blockDim.x) {
    sm_lc[i] = t.lo[i];
    sm_lc[table_n + i] = t.hi[i];
  }
  __syncthreads();
  const long long n = (long long)cd.d[0] * cd.d[1] * cd.d[2];
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int x = (int)(i % cd.d[0]), y = (int)((i / cd.d[0]) % cd.d[1]), z = (int)(i / ((long long)cd.d[0] * cd.d[1]));
  const float3 tx = cache_cell_pos(f, cd.d, x, y, z);
  ExtShade sh{&e};
  if (table_n > 0) {
    sh.tlo = sm_lc; sh.thi = sm_lc + table_n; sh.tn = table_n; sh.tax = t.axis;
    sh.tiw = t.interval; sh.tvmin = t.vmin; sh.tvmax = t.vmax;
  }
  unsigned aux = 0;
  const float ao = e.apply_occ ? sh.ambient_occlusion(tx, f) : 1.0f;
  const float sd = e.apply_sdw ? (table_n > 0 ? sh.shadow_table(tx, f, aux) : sh.shadow(tx, f, aux)) : 1.0f;
  out[i] = make_float2(ao, sd);
}

// Cone cache: OcclusionEvaluationKernel with the occlusion cone's frame from
// the camera's up vector (EyeCamUp, rc1pdosct/lightcachecomputation.comp:280-292)
// and ShadowEvaluationKernel, the same cone integration as per sample.
__global__ void __launch_bounds__(128) k_cache_dos(FrameArgs f, DosArgs d, CacheDims cd, float2* __restrict__ out) {
  extern __shared__ float4 sm_lcd[];
  float4* occ = sm_lcd;
  float4* sdw = occ + d.occ.n_sections;
  for (int i = threadIdx.x; i < d.occ.n_sections; i += blockDim.x) occ[i] = d.occ_sections[i];
  for (int i = threadIdx.x; i < d.sdw.n_sections; i += blockDim.x) sdw[i] = d.sdw_sections[i];
  __syncthreads();
  const long long n = (long long)cd.d[0] * cd.d[1] * cd.d[2];
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int x = (int)(i % cd.d[0]), y = (int)((i / cd.d[0]) % cd.d[1]), z = (int)(i / ((long long)cd.d[0] * cd.d[1]));
  const float3 tx = cache_cell_pos(f, cd.d, x, y, z);
  DosShade ds{&d, occ, sdw};
  unsigned aux = 0;
  float io = 1.0f, is = 1.0f;
  if (d.apply_occ) {
    const float3 realpos = tx - f.vol.grid * 0.5f;
    const float3 k = normalize3(f.cam.eye - realpos);
    const float3 v_right = normalize3(cross3(-k, f.cam.u));
    const float3 v_up = normalize3(cross3(k, v_right));
    io = ds.cone(occ, d.occ, tx, k, v_up, v_right, f, aux);
  }
  if (d.apply_sdw) is = ds.shadow(tx, f, aux);
  out[i] = make_float2(io, is);
}

// texture(TexVolumeLightCache, tx_pos / VolumeScaledSizes).rg: trilinear,
// texel centres, clamp-to-edge.
__device__ __forceinline__ float2 cache_lookup(const float2* __restrict__ c, const CacheDims& cd, float3 tx,
                                               float3 inv_grid) {
  Tap a = axis_tap(fmaf(tx.x * inv_grid.x, float(cd.d[0]), -0.5f), cd.d[0]);
  Tap b = axis_tap(fmaf(tx.y * inv_grid.y, float(cd.d[1]), -0.5f), cd.d[1]);
  Tap g = axis_tap(fmaf(tx.z * inv_grid.z, float(cd.d[2]), -0.5f), cd.d[2]);
  auto at = [&](int x, int y, int z) {
    return __ldg(c + (size_t)x + (size_t)cd.d[0] * ((size_t)y + (size_t)cd.d[1] * z));
  };
  float2 c000 = at(a.i0, b.i0, g.i0), c100 = at(a.i1, b.i0, g.i0), c010 = at(a.i0, b.i1, g.i0),
         c110 = at(a.i1, b.i1, g.i0), c001 = at(a.i0, b.i0, g.i1), c101 = at(a.i1, b.i0, g.i1),
         c011 = at(a.i0, b.i1, g.i1), c111 = at(a.i1, b.i1, g.i1);
  auto lerp2 = [](float t, float2 p, float2 q) { return make_float2(fmaf(t, q.x - p.x, p.x), fmaf(t, q.y - p.y, p.y)); };
  float2 c00 = lerp2(a.t, c000, c100), c10 = lerp2(a.t, c010, c110), c01 = lerp2(a.t, c001, c101),
         c11 = lerp2(a.t, c011, c111);
  float2 c0 = lerp2(b.t, c00, c10), c1 = lerp2(b.t, c01, c11);
  return lerp2(g.t, c0, c1);
}

// obj_ray_marching.comp main() + ShadeSample (both branches): the a5
// loop, but a sample is composited only when occlusion or shadow is on (the
// reference's `src.a > 0.0 && Shade`), its light terms read from the cache.
__global__ void __launch_bounds__(128) k_march_cached(FrameArgs f, CacheDims cd, const float2* __restrict__ cache,
                                                      int apply_occ, int apply_sdw, float ka_in, float kd_in) {
  extern __shared__ float4 sm_mc[];
  const float4* tf = stage_tf(f, sm_mc);
  __syncthreads();
  int px, py;
  pixel_of(f, px, py);
  const bool inside = px < f.W && py < f.H;
  unsigned n = 0, shaded = 0;
  if (inside) {
    const float3 dir = primary_dir(f.cam, px, py, f.W, f.H);
    float4 dst = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    float tnear, tfar;
    if (ray_aabb(f.cam.eye, dir, f.vol.grid, tnear, tfar)) {
      const bool shade = apply_occ || apply_sdw;
      const float ka = apply_occ ? ka_in : 0.0f, kd = apply_sdw ? kd_in : 0.0f;
      const float kk = 1.0f / (ka + kd);
      const float3 inv_grid = f3(1.0f / f.vol.grid.x, 1.0f / f.vol.grid.y, 1.0f / f.vol.grid.z);
      const float D = fabsf(tfar - tnear);
      const float3 tex0 = f.cam.eye + dir * tnear + f.vol.grid * 0.5f;
      const unsigned max_iter = (unsigned)fminf(D / f.step, 1.0e9f) + 4u;
      for (float s = 0.0f; s < D && n < max_iter;) {
        const float h = fminf(f.step, D - s);
        const float3 p = tex0 + dir * (s + h * 0.5f);
        float4 src = tf_lookup(tf, f.tf_n, sample_volume(f.vol, p));
        ++n;
        if (src.w > 0.0f && shade) {
          ++shaded;
          const float2 IaIs = cache_lookup(cache, cd, p, inv_grid);
          const float io = apply_occ ? IaIs.x : 0.0f, is = apply_sdw ? IaIs.y : 0.0f;
          if (f.grad.g) {
            src = phong_ext(f, src, p, io, ka, is, kd);
          } else {
            src.x = kk * (src.x * io * ka + src.x * is * kd);
            src.y = kk * (src.y * io * ka + src.y * is * kd);
            src.z = kk * (src.z * io * ka + src.z * is * kd);
          }
          src.w = 1.0f - expf(-src.w * h);
          src.x *= src.w; src.y *= src.w; src.z *= src.w;
          const float r = 1.0f - dst.w;
          dst.x += r * src.x; dst.y += r * src.y; dst.z += r * src.z; dst.w += r * src.w;
          if (dst.w > 0.99f) break;
        }
        s = s + h;
      }
    }
    const size_t o = (size_t)py * f.W + px;
    f.out[o] = dst;
    if (f.counts) f.counts[o] = n;
  }
  add_stats(f, n, shaded, shaded);
}

cudaError_t launch_cache_extinction(const FrameArgs& f, const ExtArgs& e, const ShadowBoxTable* t,
                                    const ShadowBoxTable& storage, const int dims[3], float2* out, cudaStream_t st) {
  CacheDims cd{{dims[0], dims[1], dims[2]}};
  const long long n = (long long)dims[0] * dims[1] * dims[2];
  const int tn = t ? t->n : 0;
  k_cache_extinction<<<(unsigned)((n + 127) / 128), 128, sizeof(float4) * 2 * tn, st>>>(f, e, cd, tn, t ? *t : storage,
                                                                                        out);
  return cudaGetLastError();
}

cudaError_t launch_cache_dos(const FrameArgs& f, const DosArgs& d, const int dims[3], float2* out, cudaStream_t st) {
  CacheDims cd{{dims[0], dims[1], dims[2]}};
  const long long n = (long long)dims[0] * dims[1] * dims[2];
  const size_t sm = sizeof(float4) * (d.occ.n_sections + d.sdw.n_sections);
  if (sm > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(k_cache_dos, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return e;
  }
  k_cache_dos<<<(unsigned)((n + 127) / 128), 128, sm, st>>>(f, d, cd, out);
  return cudaGetLastError();
}

cudaError_t launch_march_cached(const FrameArgs& f, const float2* cache, const int dims[3], int apply_occ,
                                int apply_sdw, float ka, float kd, cudaStream_t st) {
  CacheDims cd{{dims[0], dims[1], dims[2]}};
  FrameArgs g = f;
  g.tile_w = 16;  // 128-thread CTAs of 8x4-pixel warps
  g.tile_h = 8;
  dim3 grid((f.W + 15) / 16, (f.H + 7) / 8, 1);
  k_march_cached<<<grid, 128, sizeof(float4) * f.tf_n, st>>>(g, cd, cache, apply_occ, apply_sdw, ka, kd);
  return cudaGetLastError();
}

}  // namespace cvr
