// surrogate.cu — shading-point collection, feature/target labelling and the
// surrogate-shaded marcher (network inference fused into the ray loop).
#include "mlp_tile.cuh"
#include "shade.cuh"
#include "surrogate.cuh"

namespace cvr {

// ---------------------------------------------------------------- collection
__device__ __forceinline__ float keep_hash(unsigned long long seed, unsigned pixel, unsigned step) {
  unsigned long long z = seed + 0x9E3779B97F4A7C15ull * ((unsigned long long)pixel * 0x100000001ull + step + 1ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  z ^= z >> 31;
  return (float)(z >> 40) * (1.0f / 16777216.0f);
}

// The a5 loop of march_pixel with the opacity composite only (shading does
// not change alpha, so the same samples are reached and the same ray stops).
__global__ void __launch_bounds__(128) k_sur_collect(FrameArgs f, float rate, unsigned long long seed, float4* pts,
                                                     int cap, unsigned int* count) {
  extern __shared__ float4 sm_col[];
  float4* tf = sm_col;
  for (int i = threadIdx.x; i < f.tf_n; i += blockDim.x) tf[i] = f.tf[i];
  __syncthreads();
  int px, py;
  pixel_of(f, px, py);
  if (px >= f.W || py >= f.H) return;
  float3 dir = primary_dir(f.cam, px, py, f.W, f.H);
  float tnear, tfar;
  if (!ray_aabb(f.cam.eye, dir, f.vol.grid, tnear, tfar)) return;
  const unsigned pixel = (unsigned)(py * f.W + px);
  float D = fabsf(tfar - tnear);
  float3 tex0 = f.cam.eye + dir * tnear + f.vol.grid * 0.5f;
  const unsigned max_iter = (unsigned)fminf(D / f.step, 1.0e9f) + 4u;
  float dw = 0.0f;
  unsigned n = 0;
  for (float s = 0.0f; s < D && n < max_iter;) {
    float h = fminf(f.step, D - s);
    float3 p = tex0 + dir * (s + h * 0.5f);
    float4 src = tf_lookup(tf, f.tf_n, sample_volume(f.vol, p));
    ++n;
    if (src.w > 0.0f) {
      if (keep_hash(seed, pixel, n) < rate) {
        unsigned idx = atomicAdd(count, 1u);
        if (idx < (unsigned)cap) {
          pts[2 * (size_t)idx] = make_float4(p.x, p.y, p.z, 0.0f);
          pts[2 * (size_t)idx + 1] = make_float4(dir.x, dir.y, dir.z, 0.0f);
        }
      }
      float a = 1.0f - expf(-src.w * h);
      float r = 1.0f - dw;
      dw += r * a;
      if (dw > 0.99f) break;
    }
    s = s + h;
  }
}

cudaError_t launch_sur_collect(const FrameArgs& f, float rate, unsigned long long seed, float4* pts, int cap,
                               unsigned int* count, cudaStream_t st) {
  dim3 grid((f.W + f.tile_w - 1) / f.tile_w, (f.H + f.tile_h - 1) / f.tile_h, 1);
  k_sur_collect<<<grid, 128, sizeof(float4) * f.tf_n, st>>>(f, rate, seed, pts, cap, count);
  return cudaGetLastError();
}

// ---------------------------------------------------------------- labelling
// Writes feature k of one point as FP32 to global memory.
struct GlobalSink {
  float* row;
  __device__ __forceinline__ void operator()(int k, float v) { row[k] = v; }
};

template <bool TEX>
__global__ void __launch_bounds__(128) k_sur_label(const float4* __restrict__ pts, int n, FrameArgs f, SurArgs a,
                                                   GtArgs g, DosArgs d, int want_gt, int want_dos,
                                                   float* __restrict__ x_out, float* __restrict__ t_out,
                                                   float* __restrict__ dos_out) {
  extern __shared__ float4 sm_lab[];
  float4* tf = sm_lab;
  float4* occ_tab = tf + f.tf_n;
  float4* sdw_tab = occ_tab + (want_dos ? d.occ.n_sections : 0);
  float3* ov = reinterpret_cast<float3*>(sdw_tab + (want_dos ? d.sdw.n_sections : 0));
  float3* sv = ov + (want_gt ? g.n_occ : 0);
  for (int i = threadIdx.x; i < f.tf_n; i += blockDim.x) tf[i] = f.tf[i];
  if (want_dos) {
    for (int i = threadIdx.x; i < d.occ.n_sections; i += blockDim.x) occ_tab[i] = d.occ_sections[i];
    for (int i = threadIdx.x; i < d.sdw.n_sections; i += blockDim.x) sdw_tab[i] = d.sdw_sections[i];
  }
  if (want_gt) {
    for (int i = threadIdx.x; i < g.n_occ; i += blockDim.x) ov[i] = g.occ_vec[i];
    for (int i = threadIdx.x; i < g.n_sdw; i += blockDim.x) sv[i] = g.sdw_vec[i];
  }
  __syncthreads();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float4 P = pts[2 * (size_t)i], Q = pts[2 * (size_t)i + 1];
  float3 tx = f3(P.x, P.y, P.z), dir = f3(Q.x, Q.y, Q.z);
  if (x_out) {
    GlobalSink out{x_out + (size_t)i * kMlpIn};
    sur_features<TEX>(a, f.vol, tf, f.tf_n, tx, dir, out);
  }
  unsigned aux = 0;
  if (want_gt) {
    GtShade sh{&g, tf, f.tf_n, ov, sv};
    GtShade::Ray r;
    sh.begin(r, dir);
    t_out[2 * (size_t)i] = sh.occlusion(tx, r, f, aux);
    t_out[2 * (size_t)i + 1] = sh.shadow(tx, f, aux);
  }
  if (want_dos) {
    // The cone method aims its occlusion cone at the eye; any eye on the ray
    // behind the point gives the same axis.
    FrameArgs fl = f;
    fl.cam.eye = (tx - f.vol.grid * 0.5f) - dir;
    DosShade ds{&d, occ_tab, sdw_tab};
    DosShade::Ray r;
    ds.begin(r, dir);
    dos_out[2 * (size_t)i] = ds.occlusion(tx, r, fl, aux);
    dos_out[2 * (size_t)i + 1] = ds.shadow(tx, fl, aux);
  }
}

cudaError_t launch_sur_label(const float4* pts, int n, const FrameArgs& f, const SurArgs& a, bool tex,
                             const GtArgs* g, const DosArgs* d, float* x_out, float* t_out, float* dos_out,
                             cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  GtArgs gg = g ? *g : GtArgs{};
  DosArgs dd = d ? *d : DosArgs{};
  const int want_gt = g && t_out ? 1 : 0, want_dos = d && dos_out ? 1 : 0;
  size_t sm = sizeof(float4) * f.tf_n;
  if (want_dos) sm += sizeof(float4) * (dd.occ.n_sections + dd.sdw.n_sections);
  if (want_gt) sm += sizeof(float3) * (gg.n_occ + gg.n_sdw);
  auto kern = tex ? k_sur_label<true> : k_sur_label<false>;
  if (sm > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return e;
  }
  kern<<<(n + 127) / 128, 128, sm, st>>>(pts, n, f, a, gg, dd, want_gt, want_dos, x_out, t_out, dos_out);
  return cudaGetLastError();
}

// ---------------------------------------------------------------- fused marcher
struct SurRay {
  float3 dir, tex0;
  float D, s;
  float4 dst;
  unsigned n, max_iter;
  int px, py;
  int job;
};

// Where a marcher thread's rays come from.  SingleSource: one frame, tiles
// in the square spiral around (cx, cy) (positions outside the image are
// skipped: px = -1).  BatchSource: the jobs of one batch launch, each a run
// of spiral positions of one counter (jobs ordered by first position), each
// in the square spiral around its own centre tile.
struct SingleSource {
  const FrameArgs& f0;
  const SurArgs& a0;
  int cx, cy, tiles_x, tiles_y;
  unsigned total;
  __device__ __forceinline__ const FrameArgs& f(int) const { return f0; }
  __device__ __forceinline__ const SurArgs& a(int) const { return a0; }
  __device__ __forceinline__ void locate(unsigned idx, SurRay& r) const {
    int dx, dy;
    spiral_tile(idx >> 5, dx, dy);
    const int tx = cx + dx, ty = cy + dy, within = (int)(idx & 31u);
    r.job = 0;
    if (tx < 0 || ty < 0 || tx >= tiles_x || ty >= tiles_y) { r.px = -1; r.py = -1; return; }
    r.px = tx * 8 + (within & 7);
    r.py = ty * 4 + (within >> 3);
  }
};

struct BatchSource {
  const SurJob* jobs;
  int n_jobs;
  unsigned total;
  __device__ __forceinline__ const FrameArgs& f(int j) const { return jobs[j].f; }
  __device__ __forceinline__ const SurArgs& a(int j) const { return jobs[j].a; }
  __device__ __forceinline__ bool holds(int j, unsigned tile) const {
    return jobs[j].first_tile <= tile && (j + 1 == n_jobs || jobs[j + 1].first_tile > tile);
  }
  // r.job on entry: the job of the thread's previous ray.  Rays are taken in
  // increasing order, so the position is almost always in that job or the
  // next; else a binary search for the last job whose first position is <= tile.
  __device__ __forceinline__ void locate(unsigned idx, SurRay& r) const {
    const unsigned tile = idx >> 5;
    int j = r.job < 0 || r.job >= n_jobs ? 0 : r.job;
    if (!holds(j, tile)) {
      if (j + 1 < n_jobs && holds(j + 1, tile)) {
        ++j;
      } else {
        int lo = 0, hi = n_jobs - 1;
        while (lo < hi) {
          const int mid = (lo + hi + 1) >> 1;
          if (jobs[mid].first_tile <= tile) lo = mid;
          else hi = mid - 1;
        }
        j = lo;
      }
    }
    const SurJob& J = jobs[j];
    int dx, dy;
    spiral_tile(tile - J.first_tile, dx, dy);
    const int tx = J.cx + dx, ty = J.cy + dy, within = (int)(idx & 31u);
    r.job = j;
    if (tx < 0 || ty < 0 || tx >= J.tiles_x || ty >= J.tiles_y) { r.px = -1; r.py = -1; return; }
    r.px = tx * 8 + (within & 7);
    r.py = ty * 4 + (within >> 3);
  }
};

// Step counts of the rays a thread finished, flushed to the job's counters
// when the thread moves to another job and at the end.
struct SurCounts {
  int job = -1;
  unsigned n = 0, shaded = 0;
  __device__ __forceinline__ void flush(unsigned long long* stats) {
    if (job >= 0 && stats && (n | shaded)) {
      atomicAdd(stats + 0, (unsigned long long)n);
      atomicAdd(stats + 1, (unsigned long long)shaded);
      atomicAdd(stats + 2, (unsigned long long)shaded * (unsigned long long)kSurPyramidTaps);
    }
    n = shaded = 0;
  }
};

// sur_shade's light terms through the ground truth's gradient branch
// (gt_ray_marching.comp:277-295) when gradient shading is on.
__device__ __forceinline__ float4 sur_phong(const SurArgs& a, const FrameArgs& f, float4 src, float3 p, float ao,
                                            float sdw) {
  float ka = 0.0f, kd = 0.0f, io = 0.0f, is = 0.0f;
  if (a.apply_occ) { ka = a.ka; io = fminf(fmaxf(ao, 0.0f), 1.0f); }
  if (a.apply_sdw) { kd = a.kd; is = a.shadow_type == 1 ? 0.0f : fminf(fmaxf(sdw, 0.0f), 1.0f); }
  return phong_cone(f, src, p, io, ka, is, kd);
}

__device__ __forceinline__ void sur_finish(const FrameArgs& f, const SurRay& r) {
  size_t o = (size_t)r.py * f.W + r.px;
  f.out[o] = r.dst;
  if (f.counts) f.counts[o] = r.n;
}

// Packs features pairwise to BF16 and stores each 8-feature chunk of this
// thread's row of the input tile as soon as it is complete.
struct TileSink {
  uint8_t* tile;
  int row;
  uint32_t w[4];
  float lo;
  __device__ __forceinline__ void operator()(int k, float v) {
    if (k & 1) {
      w[(k >> 1) & 3] = pack_bf16(lo, v);
      if ((k & 7) == 7) store_chunk(tile, row, k >> 3, w[0], w[1], w[2], w[3]);
    } else {
      lo = v;
    }
  }
};

constexpr uint32_t kSurTmemCols = 64;

// The marcher body for either source.  tf_src / tf_n: the transfer function
// (shared by all jobs), packed: the network image.
template <bool TEX, bool BATCH, class Src>
__device__ __forceinline__ void sur_march(const Src& src_rays, const float4* tf_src, int tf_n, const uint8_t* packed,
                                          unsigned int* work, int* err) {
  extern __shared__ __align__(1024) uint8_t sm_sur[];
  uint8_t* w = sm_sur;
  uint8_t* xt = w + kPkFwdBytes;  // input tile, then the hidden activations of the same tile
  float4* tf = reinterpret_cast<float4*>(xt + kRowTile);
  uint64_t* bar = reinterpret_cast<uint64_t*>(tf + tf_n);
  uint32_t* tslot = reinterpret_cast<uint32_t*>(bar + 1);
  mlp_cta_begin(w, packed, bar, tslot, kSurTmemCols, kPkFwdBytes);
  for (int i = threadIdx.x; i < tf_n; i += blockDim.x) tf[i] = tf_src[i];
  fence_async_smem();
  __syncthreads();
  MlpSmem ms{w, xt, xt, bar, *tslot, 0u};

  const unsigned total = src_rays.total;
  SurRay ray{};
  bool has_ray = false, pending = false, no_work = false;
  float4 src = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  float3 p = f3(0.0f, 0.0f, 0.0f);
  float h = 0.0f;
  SurCounts cnt;
  while (true) {
    // Advance this thread's ray to its next shaded sample, taking new rays
    // as rays end, until a sample is pending or no rays are left.
    while (!pending && !no_work) {
      if (!has_ray) {
        unsigned idx = take_ray(work);
        if (idx >= total) { no_work = true; break; }
        src_rays.locate(idx, ray);
        const FrameArgs& f = src_rays.f(ray.job);
        if (ray.px < 0 || ray.px >= f.W || ray.py >= f.H) continue;
        if (ray.job != cnt.job) {
          if (BATCH) cnt.flush(src_rays.f(cnt.job < 0 ? 0 : cnt.job).stats);
          cnt.job = ray.job;
        }
        ray.dir = primary_dir(f.cam, ray.px, ray.py, f.W, f.H);
        ray.dst = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        ray.n = 0;
        float tnear, tfar;
        if (!ray_aabb(f.cam.eye, ray.dir, f.vol.grid, tnear, tfar)) {
          sur_finish(f, ray);
          continue;
        }
        ray.D = fabsf(tfar - tnear);
        ray.tex0 = f.cam.eye + ray.dir * tnear + f.vol.grid * 0.5f;
        ray.s = 0.0f;
        ray.max_iter = (unsigned)fminf(ray.D / f.step, 1.0e9f) + 4u;
        has_ray = true;
      }
      {
        const FrameArgs& f = src_rays.f(ray.job);
        while (ray.s < ray.D && ray.n < ray.max_iter) {
          h = fminf(f.step, ray.D - ray.s);
          p = ray.tex0 + ray.dir * (ray.s + h * 0.5f);
          src = tf_lookup(tf, tf_n, sample_volume(f.vol, p));
          ++ray.n;
          if (src.w > 0.0f) { pending = true; break; }
          ray.s = ray.s + h;
        }
        if (!pending) {
          sur_finish(f, ray);
          cnt.n += ray.n;
          has_ray = false;
        }
      }
    }
    if (!__syncthreads_or(pending)) break;
    // A row's outputs depend on that row's inputs alone, so the rows of
    // threads without a pending sample keep whatever the tile holds (their
    // outputs are not used): only the threads with a sample store features,
    // which halves the partial-warp stores of every chunk.
    if (pending) {
      TileSink out{xt, (int)threadIdx.x};
      sur_features<TEX>(src_rays.a(ray.job), src_rays.f(ray.job).vol, tf, tf_n, p, ray.dir, out);
    }
    // K padding (inputs 48..63): the previous round's hidden layers wrote there
    store_chunk(xt, threadIdx.x, 6, 0u, 0u, 0u, 0u);
    store_chunk(xt, threadIdx.x, 7, 0u, 0u, 0u, 0u);
    sync_tiles();
    float y[2];
    bool ok = mlp_forward_tile(ms, y);
    if (__syncthreads_or(!ok)) {
      if (threadIdx.x == 0) atomicExch(err, 1);
      break;
    }
    if (pending) {
      ++cnt.shaded;
      pending = false;
      const FrameArgs& fj = src_rays.f(ray.job);
      src = fj.grad.g ? sur_phong(src_rays.a(ray.job), fj, src, p, y[0], y[1])
                      : sur_shade(src_rays.a(ray.job), src, y[0], y[1]);
      src.w = 1.0f - expf(-src.w * h);
      src.x *= src.w; src.y *= src.w; src.z *= src.w;
      float r = 1.0f - ray.dst.w;
      ray.dst.x += r * src.x; ray.dst.y += r * src.y; ray.dst.z += r * src.z; ray.dst.w += r * src.w;
      if (ray.dst.w > 0.99f) {
        sur_finish(src_rays.f(ray.job), ray);
        cnt.n += ray.n;
        has_ray = false;
      } else {
        ray.s = ray.s + h;
      }
    }
  }
  if (BATCH) {
    cnt.flush(src_rays.f(cnt.job < 0 ? 0 : cnt.job).stats);
  } else {
    add_stats(src_rays.f(0), cnt.n, cnt.shaded, cnt.shaded * (unsigned)kSurPyramidTaps);
  }
  mlp_cta_end(ms.tmem, kSurTmemCols);
}

// MINB: resident CTAs per SM the register budget is cut for (5: at most 96
// registers; 4: at most 128).  The single-frame marcher runs at 5 for every
// variant (measured faster than 4 at the 4-CTA variant); the batch marcher,
// which keeps its job's descriptor fields live, takes 4 where 5 would spill.
template <bool TEX, int MINB>
__global__ void __launch_bounds__(128, MINB) k_march_surrogate(FrameArgs f, SurArgs a, int cx, int cy, unsigned total,
                                                               unsigned int* work, int* err) {
  SingleSource s{f, a, cx, cy, (f.W + 7) >> 3, (f.H + 3) >> 2, total};
  sur_march<TEX, false>(s, f.tf, f.tf_n, a.packed, work, err);
}

template <bool TEX, int MINB>
__global__ void __launch_bounds__(128, MINB) k_batch_surrogate(const __grid_constant__ SurLaunch L, unsigned int* work,
                                                               int* err) {
  BatchSource s{L.jobs, L.n_jobs, L.total};
  sur_march<TEX, true>(s, L.jobs[0].f.tf, L.jobs[0].f.tf_n, L.jobs[0].a.packed, work, err);
}

// Persistent grid.  CTAs per SM: at most 4 for variant 0, the most that fit
// (shared memory, registers, at most 512 / 64 by TMEM) for variant 1, at most
// 3 for variant 2.  The shared-memory carveout is sized to those CTAs,
// so the rest of the SM's 256 KB serves as L1 / texture cache for the
// network inputs (fewer CTAs: less latency hiding, more cache).
template <class K>
static cudaError_t surrogate_grid(K kern, size_t smem, unsigned rays, int variant, unsigned* ctas) {
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  int dev = 0, sms = 0, per_sm = 0, smem_sm = 0, reserved = 0;
  if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
  if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
  if ((e = cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev)) != cudaSuccess) return e;
  if ((e = cudaDeviceGetAttribute(&reserved, cudaDevAttrReservedSharedMemoryPerBlock, dev)) != cudaSuccess) return e;
  if ((e = resident_ctas(kern, 128, smem, &per_sm)) != cudaSuccess) return e;
  per_sm = per_sm > (int)(512 / kSurTmemCols) ? (int)(512 / kSurTmemCols) : per_sm;
  if (variant == 0 && per_sm > 4) per_sm = 4;
  if (variant == 2 && per_sm > 3) per_sm = 3;
  cudaFuncAttributes fa{};
  if ((e = cudaFuncGetAttributes(&fa, kern)) != cudaSuccess) return e;
  const size_t need = (size_t)per_sm * (smem + fa.sharedSizeBytes + (size_t)reserved);
  int pct = (int)((need * 100 + (size_t)smem_sm - 1) / (size_t)smem_sm);
  pct = pct < 1 ? 1 : (pct > 100 ? 100 : pct);
  if ((e = cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, pct)) != cudaSuccess) return e;
  unsigned long long n = (unsigned long long)sms * (unsigned long long)per_sm, groups = (rays + 127ull) / 128ull;
  if (n > groups) n = groups;
  *ctas = n < 1 ? 1u : (unsigned)n;
  return cudaSuccess;
}

cudaError_t launch_batch_surrogate(const SurLaunch& L, int tf_n, bool tex, int variant, unsigned int* work, int* err,
                                   cudaStream_t st) {
  const size_t smem = kPkFwdBytes + kRowTile + sizeof(float4) * tf_n + 16;
  // texture-unit features: 124 registers without spills at MINB 4 (at 5 they
  // spill and the launch ran at 0.7x the single frames), so every variant takes 4
  const bool wide = variant == 1 || variant == 3;
  auto kern = tex ? k_batch_surrogate<true, 4> : (wide ? k_batch_surrogate<false, 5> : k_batch_surrogate<false, 4>);
  unsigned ctas = 0;
  cudaError_t e = surrogate_grid(kern, smem, L.total, variant, &ctas);
  if (e != cudaSuccess) return e;
  kern<<<ctas, 128, smem, st>>>(L, work, err);
  return cudaGetLastError();
}

SurSpiral sur_spiral(const FrameArgs& f) {
  // pixel of the projected volume centre (the box is centred on the origin)
  const float3 d = f3(0.0f, 0.0f, 0.0f) - f.cam.eye;
  const float zf = dot3(d, f.cam.f);
  int px = f.W / 2, py = f.H / 2;
  if (zf > 1e-6f) {
    const float xn = dot3(d, f.cam.s) / (zf * f.cam.tan_half_fovy * f.cam.aspect);
    const float yn = dot3(d, f.cam.u) / (zf * f.cam.tan_half_fovy);
    if (std::isfinite(xn) && std::isfinite(yn) && std::fabs(xn) < 4.0f && std::fabs(yn) < 4.0f) {
      px = (int)((xn * 0.5f + 0.5f) * (float)f.W);
      py = (int)((yn * 0.5f + 0.5f) * (float)f.H);
    }
  }
  const int tiles_x = (f.W + 7) / 8, tiles_y = (f.H + 3) / 4;
  SurSpiral o;
  o.cx = std::min(std::max(px / 8, 0), tiles_x - 1);
  o.cy = std::min(std::max(py / 4, 0), tiles_y - 1);
  const int R = std::max(std::max(o.cx, tiles_x - 1 - o.cx), std::max(o.cy, tiles_y - 1 - o.cy));
  o.positions = (unsigned long long)(2 * R + 1) * (unsigned long long)(2 * R + 1);
  return o;
}

cudaError_t launch_surrogate(const FrameArgs& f, const SurArgs& a, bool tex, const SurSpiral& order,
                             unsigned int* work, int* err, cudaStream_t st) {
  const size_t smem = kPkFwdBytes + kRowTile + sizeof(float4) * f.tf_n + 16;
  auto kern = tex ? k_march_surrogate<true, 5> : k_march_surrogate<false, 5>;
  const unsigned long long spiral = order.positions * 32ull;
  if (spiral > 0xFFFFFFF0ull) return cudaErrorInvalidValue;
  const unsigned rays = (unsigned)((f.W + 7) / 8) * (unsigned)((f.H + 3) / 4) * 32u;
  unsigned ctas = 0;
  cudaError_t e = surrogate_grid(kern, smem, rays, f.variant, &ctas);
  if (e != cudaSuccess) return e;
  kern<<<ctas, 128, smem, st>>>(f, a, order.cx, order.cy, (unsigned)spiral, work, err);
  return cudaGetLastError();
}

}  // namespace cvr
