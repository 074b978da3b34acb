// march.cu — the single-pass ray marchers of the four renderers.
//
// One templated primary-ray loop restates the loop that all four reference
// shaders share (ray_marching_1p.comp:160-247, ebs_ray_bbox_marching.comp:553-627,
// ray_bbox_marching.comp:658-734, gt_ray_marching.comp:371-482); the
// per-method ShadeSample() functions are the shading policies below.
#include "shade.cuh"

namespace cvr {

template <int NT>
__global__ void __launch_bounds__(NT) k_march_plain(FrameArgs f) {
  extern __shared__ float4 sm_tf[];
  const float4* tf = stage_tf(f, sm_tf);
  __syncthreads();
  march_pixel(f, tf, PlainShade{});
}

// NT: threads per CTA (64, 128 or 256: tiles of 2, 4 or 8 warps of 8x4
// pixels).  MINB: minimum resident CTAs per SM requested from the register
// allocator, from the tuner's register variant (0: no cap, 1: <= 128, 2: <= 80
// registers per thread).
// C: the SAT queries read the compact 32-bit table.
template <int NT, int MINB, bool C>
__global__ void __launch_bounds__(NT, MINB) k_march_extinction(FrameArgs f, ExtArgs e) {
  extern __shared__ float4 sm_tf[];
  const float4* tf = stage_tf(f, sm_tf);
  __syncthreads();
  ExtShadeT<C> sh{&e};
  march_pixel(f, tf, sh);
}

// Directional light: the shadow boxes come from the per-frame table, staged
// in shared memory after the transfer function.  A: every box (AO and
// shadow) has integer texel widths, so every query is the compact table's
// equal-fraction one (the host selects it; it needs C).
template <int NT, int MINB, bool C, bool A>
__global__ void __launch_bounds__(NT, MINB) k_march_extinction_dir(FrameArgs f, ExtArgs e,
                                                                    const __grid_constant__ ShadowBoxTable t) {
  extern __shared__ float4 sm_tf[];
  const float4* tf = stage_tf(f, sm_tf);
  float4* lo = sm_tf + f.tf_n;
  float4* hi = lo + t.n;
  float4* tx = hi + t.n;
  for (int i = threadIdx.x; i < t.n; i += blockDim.x) {
    lo[i] = t.lo[i];
    hi[i] = t.hi[i];
    if (A) tx[i] = t.tx[i];
  }
  __syncthreads();
  ExtShadeT<C, A> sh{&e};
  sh.tlo = lo; sh.thi = hi; sh.tn = t.n; sh.tax = t.axis;
  if (A) sh.ttx = tx;
  sh.tiw = t.interval; sh.tvmin = t.vmin; sh.tvmax = t.vmax;
  march_pixel(f, tf, sh);
}

// MINB: the tuner's register variant, as for the extinction marcher.
template <int NT, int MINB, bool TEX>
__global__ void __launch_bounds__(NT, MINB) k_march_dos(DosArgs d, FrameArgs f) {
  extern __shared__ float4 sm[];
  float4* tf = sm;
  float4* occ = sm + f.tf_n;
  float4* sdw = occ + d.occ.n_sections;
  for (int i = threadIdx.x; i < f.tf_n; i += blockDim.x) tf[i] = f.tf[i];
  for (int i = threadIdx.x; i < d.occ.n_sections; i += blockDim.x) occ[i] = d.occ_sections[i];
  for (int i = threadIdx.x; i < d.sdw.n_sections; i += blockDim.x) sdw[i] = d.sdw_sections[i];
  __syncthreads();
  DosShadeT<TEX> sh{&d, occ, sdw};
  march_pixel(f, tf, sh);
}

template <int NT>
__global__ void __launch_bounds__(NT) k_march_gt(GtArgs g, FrameArgs f) {
  extern __shared__ float4 sm[];
  float4* tf = sm;
  float3* ov = reinterpret_cast<float3*>(sm + f.tf_n);
  float3* sv = ov + g.n_occ;
  for (int i = threadIdx.x; i < f.tf_n; i += blockDim.x) tf[i] = f.tf[i];
  for (int i = threadIdx.x; i < g.n_occ; i += blockDim.x) ov[i] = g.occ_vec[i];
  for (int i = threadIdx.x; i < g.n_sdw; i += blockDim.x) sv[i] = g.sdw_vec[i];
  __syncthreads();
  GtShade sh{&g, tf, f.tf_n, ov, sv};
  march_pixel(f, tf, sh);
}

// ---- persistent ray-refill variants (FrameArgs::work set): 128 threads,
// as many CTAs as fit on the GPU, rays from the frame's counter (march_refill)
template <int MINB>
__global__ void __launch_bounds__(128, MINB) k_march_plain_refill(FrameArgs f, RayOrder o) {
  extern __shared__ float4 sm_tf[];
  const float4* tf = stage_tf(f, sm_tf);
  __syncthreads();
  march_refill(f, tf, PlainShade{}, f.work, o);
}

template <int MINB, bool C, bool A>
__global__ void __launch_bounds__(128, MINB) k_march_extinction_refill(FrameArgs f, ExtArgs e, RayOrder o,
                                                                      const __grid_constant__ ShadowBoxTable t,
                                                                      int has_table) {
  extern __shared__ float4 sm_tf[];
  const float4* tf = stage_tf(f, sm_tf);
  const int tn = has_table ? t.n : 0;
  float4* lo = sm_tf + f.tf_n;
  float4* hi = lo + tn;
  float4* tx = hi + tn;
  for (int i = threadIdx.x; i < tn; i += blockDim.x) {
    lo[i] = t.lo[i];
    hi[i] = t.hi[i];
    if (A) tx[i] = t.tx[i];
  }
  __syncthreads();
  ExtShadeT<C, A> sh{&e};
  if (tn > 0) {
    sh.tlo = lo; sh.thi = hi; sh.tn = tn; sh.tax = t.axis;
    sh.tiw = t.interval; sh.tvmin = t.vmin; sh.tvmax = t.vmax;
    if (A) sh.ttx = tx;
  }
  march_refill(f, tf, sh, f.work, o);
}

template <int MINB, bool TEX>
__global__ void __launch_bounds__(128, MINB) k_march_dos_refill(DosArgs d, FrameArgs f, RayOrder o) {
  extern __shared__ float4 sm[];
  float4* tf = sm;
  float4* occ = sm + f.tf_n;
  float4* sdw = occ + d.occ.n_sections;
  for (int i = threadIdx.x; i < f.tf_n; i += blockDim.x) tf[i] = f.tf[i];
  for (int i = threadIdx.x; i < d.occ.n_sections; i += blockDim.x) occ[i] = d.occ_sections[i];
  for (int i = threadIdx.x; i < d.sdw.n_sections; i += blockDim.x) sdw[i] = d.sdw_sections[i];
  __syncthreads();
  DosShadeT<TEX> sh{&d, occ, sdw};
  march_refill(f, tf, sh, f.work, o);
}

template <int MINB>
__global__ void __launch_bounds__(128, MINB) k_march_gt_refill(GtArgs g, FrameArgs f, RayOrder o) {
  extern __shared__ float4 sm[];
  float4* tf = sm;
  float3* ov = reinterpret_cast<float3*>(sm + f.tf_n);
  float3* sv = ov + g.n_occ;
  for (int i = threadIdx.x; i < f.tf_n; i += blockDim.x) tf[i] = f.tf[i];
  for (int i = threadIdx.x; i < g.n_occ; i += blockDim.x) ov[i] = g.occ_vec[i];
  for (int i = threadIdx.x; i < g.n_sdw; i += blockDim.x) sv[i] = g.sdw_vec[i];
  __syncthreads();
  GtShade sh{&g, tf, f.tf_n, ov, sv};
  march_refill(f, tf, sh, f.work, o);
}

// Persistent launch: every SM filled with as many CTAs of kern as fit.
template <class K, class... Args>
static cudaError_t launch_persistent(K kern, size_t smem, cudaStream_t st, Args... args) {
  cudaError_t e;
  if (smem > 48 * 1024 &&
      (e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)) != cudaSuccess)
    return e;
  if ((e = carve_l1(kern, 128, smem)) != cudaSuccess) return e;
  int dev = 0, sms = 0, per_sm = 0;
  if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
  if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
  if ((e = resident_ctas(kern, 128, smem, &per_sm)) != cudaSuccess) return e;
  kern<<<(unsigned)(sms * per_sm), 128, smem, st>>>(args...);
  return cudaGetLastError();
}

static dim3 grid_of(const FrameArgs& f) {
  return dim3((f.W + f.tile_w - 1) / f.tile_w, (f.H + f.tile_h - 1) / f.tile_h, 1);
}
static int threads_of(const FrameArgs& f) { return (f.tile_w / 8) * (f.tile_h / 4) * 32; }

template <int V>
constexpr int minb128() {
  return V == 1 ? 65536 / (128 * 128) : (V == 2 ? 65536 / (128 * 80) : (V == 3 ? 65536 / (128 * 96) : 1));
}

cudaError_t launch_plain(const FrameArgs& f, cudaStream_t st) {
  size_t sm = sizeof(float4) * f.tf_n;
  if (f.work) {
    const RayOrder o = ray_order(f);
    switch (f.variant) {
      case 1: return launch_persistent(k_march_plain_refill<minb128<1>()>, sm, st, f, o);
      case 2: return launch_persistent(k_march_plain_refill<minb128<2>()>, sm, st, f, o);
      default: return launch_persistent(k_march_plain_refill<1>, sm, st, f, o);
    }
  }
  switch (threads_of(f)) {
    case 64: k_march_plain<64><<<grid_of(f), 64, sm, st>>>(f); break;
    case 256: k_march_plain<256><<<grid_of(f), 256, sm, st>>>(f); break;
    default: k_march_plain<128><<<grid_of(f), 128, sm, st>>>(f); break;
  }
  return cudaGetLastError();
}

// Batched extinction frames: persistent CTAs take tiles of all jobs from one
// counter; the job descriptor, transfer function and shadow table are staged
// in shared memory whenever a CTA moves to another job.
// A: every job has a shadow table and integer box widths (the equal-fraction
// query; needs C).
template <int NT, int MINB, bool C, bool A>
__global__ void __launch_bounds__(NT, MINB) k_batch_extinction(const BatchExtJob* __restrict__ jobs, int n_jobs,
                                                                unsigned total, unsigned* counter) {
  __shared__ BatchExtJob J;
  __shared__ unsigned s_blk;
  __shared__ int s_job;
  extern __shared__ float4 sm_bt[];
  int cur = -1;
  while (true) {
    if (threadIdx.x == 0) {
      const unsigned b = atomicAdd(counter, 1u);
      s_blk = b;
      if (b < total) {
        int lo = 0, hi = n_jobs - 1;  // last job whose first tile is <= b
        while (lo < hi) {
          const int mid = (lo + hi + 1) >> 1;
          if (jobs[mid].first_block <= b) lo = mid;
          else hi = mid - 1;
        }
        s_job = lo;
      }
    }
    __syncthreads();
    const unsigned b = s_blk;
    if (b >= total) break;
    const int j = s_job;
    if (j != cur) {
      const int* src = reinterpret_cast<const int*>(jobs + j);
      int* dst = reinterpret_cast<int*>(&J);
      for (int i = threadIdx.x; i < (int)(sizeof(BatchExtJob) / sizeof(int)); i += blockDim.x) dst[i] = src[i];
      __syncthreads();
      for (int i = threadIdx.x; i < J.f.tf_n; i += blockDim.x) sm_bt[i] = J.f.tf[i];
      for (int i = threadIdx.x; i < J.tn; i += blockDim.x) {
        sm_bt[J.f.tf_n + i] = J.tlo[i];
        sm_bt[J.f.tf_n + J.tn + i] = J.thi[i];
        if (A) sm_bt[J.f.tf_n + 2 * J.tn + i] = J.ttx[i];
      }
      cur = j;
      __syncthreads();
    }
    const unsigned local = b - J.first_block;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, wl = warp_shift(J.f.warp_w);
    const int warps_x = J.f.tile_w >> wl;
    const int px = (int)(local % J.blocks_x) * J.f.tile_w + (warp % warps_x) * (1 << wl) + (lane & ((1 << wl) - 1));
    const int py = (int)(local / J.blocks_x) * J.f.tile_h + (warp / warps_x) * (32 >> wl) + (lane >> wl);
    ExtShadeT<C, A> sh{&J.e};
    if (J.tn > 0) {
      sh.tlo = sm_bt + J.f.tf_n; sh.thi = sm_bt + J.f.tf_n + J.tn; sh.tn = J.tn; sh.tax = J.tax;
      if (A) sh.ttx = sm_bt + J.f.tf_n + 2 * J.tn;
      sh.tiw = J.tiw; sh.tvmin = J.tvmin; sh.tvmax = J.tvmax;
    }
    march_ray(J.f, sm_bt, sh, px, py);
    __syncthreads();  // J and the staged tables are reused by the next tile
  }
}

template <int NT, int MINB>
static cudaError_t launch_batch_t(const BatchExtJob* jobs, int n_jobs, unsigned total_blocks, unsigned* counter,
                                  size_t smem, bool compact, bool aligned, cudaStream_t st) {
  auto kern = compact ? (aligned ? k_batch_extinction<NT, MINB, true, true> : k_batch_extinction<NT, MINB, true, false>)
                      : k_batch_extinction<NT, MINB, false, false>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  if ((e = carve_l1(kern, NT, smem)) != cudaSuccess) return e;
  int dev = 0, sms = 0, per_sm = 0;
  if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
  if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
  if ((e = resident_ctas(kern, NT, smem, &per_sm)) != cudaSuccess) return e;
  unsigned ctas = (unsigned)sms * (unsigned)per_sm;
  if (ctas > total_blocks) ctas = total_blocks;
  if (ctas == 0) return cudaSuccess;
  kern<<<ctas, NT, smem, st>>>(jobs, n_jobs, total_blocks, counter);
  return cudaGetLastError();
}

// Register variants as minimum resident CTAs: caps of 128 and 80 registers.
template <int NT>
constexpr int minb_of(int variant) {
  return variant == 1 ? 65536 / (NT * 128) : (variant == 2 ? 65536 / (NT * 80) : (variant == 3 ? 65536 / (NT * 96) : 1));
}

cudaError_t launch_batch_extinction(const BatchExtJob* jobs, int n_jobs, unsigned total_blocks, unsigned* counter,
                                    int tf_n, int max_table, int tile_threads, int variant, bool compact,
                                    bool aligned, cudaStream_t st) {
  const size_t smem = sizeof(float4) * (tf_n + 3 * max_table);
  aligned = aligned && compact;
#define CVR_BATCH(NT)                                                                                         \
  switch (variant) {                                                                                         \
    case 1:                                                                                                  \
      return launch_batch_t<NT, minb_of<NT>(1)>(jobs, n_jobs, total_blocks, counter, smem, compact, aligned, st); \
    case 2:                                                                                                  \
      return launch_batch_t<NT, minb_of<NT>(2)>(jobs, n_jobs, total_blocks, counter, smem, compact, aligned, st); \
    case 3:                                                                                                  \
      return launch_batch_t<NT, minb_of<NT>(3)>(jobs, n_jobs, total_blocks, counter, smem, compact, aligned, st); \
    default: return launch_batch_t<NT, 1>(jobs, n_jobs, total_blocks, counter, smem, compact, aligned, st);      \
  }
  if (tile_threads == 64) { CVR_BATCH(64) }
  if (tile_threads == 256) { CVR_BATCH(256) }
  CVR_BATCH(128)
#undef CVR_BATCH
}

template <int NT, int MINB>
static cudaError_t launch_extinction_t(const FrameArgs& f, const ExtArgs& e, const ShadowBoxTable* table,
                                       cudaStream_t st) {
  const bool c = e.sat.sat32 != nullptr;
  if (table) {
    size_t sm = sizeof(float4) * (f.tf_n + 3 * table->n);
    const bool a = c && table->aligned && (e.ao_aligned || !e.apply_occ);
    auto kern = a ? k_march_extinction_dir<NT, MINB, true, true>
                  : (c ? k_march_extinction_dir<NT, MINB, true, false> : k_march_extinction_dir<NT, MINB, false, false>);
    const cudaError_t err = carve_l1(kern, NT, sm);
    if (err != cudaSuccess) return err;
    kern<<<grid_of(f), NT, sm, st>>>(f, e, *table);
  } else {
    size_t sm = sizeof(float4) * f.tf_n;
    auto kern = c ? k_march_extinction<NT, MINB, true> : k_march_extinction<NT, MINB, false>;
    const cudaError_t err = carve_l1(kern, NT, sm);
    if (err != cudaSuccess) return err;
    kern<<<grid_of(f), NT, sm, st>>>(f, e);
  }
  return cudaGetLastError();
}

template <int NT>
static cudaError_t launch_extinction_nt(const FrameArgs& f, const ExtArgs& e, const ShadowBoxTable* table,
                                        cudaStream_t st) {
  switch (f.variant) {
    case 1: return launch_extinction_t<NT, minb_of<NT>(1)>(f, e, table, st);
    case 2: return launch_extinction_t<NT, minb_of<NT>(2)>(f, e, table, st);
    case 3: return launch_extinction_t<NT, minb_of<NT>(3)>(f, e, table, st);
    default: return launch_extinction_t<NT, 1>(f, e, table, st);
  }
}

template <int MINB>
static cudaError_t launch_extinction_refill(const FrameArgs& f, const ExtArgs& e, const ShadowBoxTable* table,
                                           const ShadowBoxTable& storage, cudaStream_t st) {
  const RayOrder o = ray_order(f);
  const bool c = e.sat.sat32 != nullptr;
  const bool a = c && table && table->aligned && (e.ao_aligned || !e.apply_occ);
  const ShadowBoxTable& t = table ? *table : storage;
  const int has = table ? 1 : 0;
  const size_t sm = sizeof(float4) * (f.tf_n + (table ? 3 * table->n : 0));
  if (a) return launch_persistent(k_march_extinction_refill<MINB, true, true>, sm, st, f, e, o, t, has);
  if (c) return launch_persistent(k_march_extinction_refill<MINB, true, false>, sm, st, f, e, o, t, has);
  return launch_persistent(k_march_extinction_refill<MINB, false, false>, sm, st, f, e, o, t, has);
}

cudaError_t launch_extinction(const FrameArgs& f, const ExtArgs& e, const ShadowBoxTable* table,
                              const ShadowBoxTable& storage, cudaStream_t st) {
  if (!e.sat.sat32 && !e.sat.sat) return cudaErrorInvalidValue;  // no table to read
  if (f.work) {
    switch (f.variant) {
      case 1: return launch_extinction_refill<minb128<1>()>(f, e, table, storage, st);
      case 2: return launch_extinction_refill<minb128<2>()>(f, e, table, storage, st);
      case 3: return launch_extinction_refill<minb128<3>()>(f, e, table, storage, st);
      default: return launch_extinction_refill<1>(f, e, table, storage, st);
    }
  }
  switch (threads_of(f)) {
    case 64: return launch_extinction_nt<64>(f, e, table, st);
    case 256: return launch_extinction_nt<256>(f, e, table, st);
    default: return launch_extinction_nt<128>(f, e, table, st);
  }
}

static cudaError_t launch_dos_k(void (*kern)(DosArgs, FrameArgs), int nt, const FrameArgs& f, const DosArgs& d,
                                size_t sm, cudaStream_t st) {
  if (sm > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return e;
  }
  cudaError_t e = carve_l1(kern, nt, sm);
  if (e != cudaSuccess) return e;
  kern<<<grid_of(f), nt, sm, st>>>(d, f);
  return cudaGetLastError();
}

template <int NT>
static cudaError_t launch_dos_nt(const FrameArgs& f, const DosArgs& d, bool tex, size_t sm, cudaStream_t st) {
  void (*kern)(DosArgs, FrameArgs);
  switch (f.variant) {
    case 1: kern = tex ? k_march_dos<NT, minb_of<NT>(1), true> : k_march_dos<NT, minb_of<NT>(1), false>; break;
    case 2: kern = tex ? k_march_dos<NT, minb_of<NT>(2), true> : k_march_dos<NT, minb_of<NT>(2), false>; break;
    default: kern = tex ? k_march_dos<NT, 1, true> : k_march_dos<NT, 1, false>; break;
  }
  return launch_dos_k(kern, NT, f, d, sm, st);
}

cudaError_t launch_dos(const FrameArgs& f, const DosArgs& d, bool tex_pyramid, cudaStream_t st) {
  size_t sm = sizeof(float4) * (f.tf_n + d.occ.n_sections + d.sdw.n_sections);
  if (f.work) {
    const RayOrder o = ray_order(f);
    switch (f.variant) {
      case 1:
        return tex_pyramid ? launch_persistent(k_march_dos_refill<minb128<1>(), true>, sm, st, d, f, o)
                           : launch_persistent(k_march_dos_refill<minb128<1>(), false>, sm, st, d, f, o);
      case 2:
        return tex_pyramid ? launch_persistent(k_march_dos_refill<minb128<2>(), true>, sm, st, d, f, o)
                           : launch_persistent(k_march_dos_refill<minb128<2>(), false>, sm, st, d, f, o);
      default:
        return tex_pyramid ? launch_persistent(k_march_dos_refill<1, true>, sm, st, d, f, o)
                           : launch_persistent(k_march_dos_refill<1, false>, sm, st, d, f, o);
    }
  }
  switch (threads_of(f)) {
    case 64: return launch_dos_nt<64>(f, d, tex_pyramid, sm, st);
    case 256: return launch_dos_nt<256>(f, d, tex_pyramid, sm, st);
    default: return launch_dos_nt<128>(f, d, tex_pyramid, sm, st);
  }
}

template <int NT>
static cudaError_t launch_gt_t(const FrameArgs& f, const GtArgs& g, size_t sm, cudaStream_t st) {
  if (sm > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(k_march_gt<NT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return e;
  }
  cudaError_t e = carve_l1(k_march_gt<NT>, NT, sm);
  if (e != cudaSuccess) return e;
  k_march_gt<NT><<<grid_of(f), NT, sm, st>>>(g, f);
  return cudaGetLastError();
}

cudaError_t launch_gt(const FrameArgs& f, const GtArgs& g, cudaStream_t st) {
  size_t sm = sizeof(float4) * f.tf_n + sizeof(float3) * (g.n_occ + g.n_sdw);
  if (f.work) {
    const RayOrder o = ray_order(f);
    switch (f.variant) {
      case 1: return launch_persistent(k_march_gt_refill<minb128<1>()>, sm, st, g, f, o);
      case 2: return launch_persistent(k_march_gt_refill<minb128<2>()>, sm, st, g, f, o);
      default: return launch_persistent(k_march_gt_refill<1>, sm, st, g, f, o);
    }
  }
  switch (threads_of(f)) {
    case 64: return launch_gt_t<64>(f, g, sm, st);
    case 256: return launch_gt_t<256>(f, g, sm, st);
    default: return launch_gt_t<128>(f, g, sm, st);
  }
}

}  // namespace cvr
