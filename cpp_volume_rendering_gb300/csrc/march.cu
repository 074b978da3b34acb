// march.cu — the single-pass ray marchers of the four renderers.
//
// One templated primary-ray loop restates the loop that all four reference
// shaders share (ray_marching_1p.comp:160-247, ebs_ray_bbox_marching.comp:553-627,
// ray_bbox_marching.comp:658-734, gt_ray_marching.comp:371-482); the
// per-method ShadeSample() functions are the shading policies below.
#include "march_ext.cuh"

namespace cvr {

// the extinction marchers of each CTA size: march_ext{64,128,256}.cu
CVR_EXTINCTION_EXTERN(64)
CVR_EXTINCTION_EXTERN(128)
CVR_EXTINCTION_EXTERN(256)

template <int NT>
__global__ void __launch_bounds__(NT) k_march_plain(FrameArgs f) {
  extern __shared__ float4 sm_tf[];
  const float4* tf = stage_tf(f, sm_tf);
  __syncthreads();
  march_pixel(f, tf, PlainShade{});
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

cudaError_t launch_batch_extinction(const BatchExtJob* jobs, int n_jobs, unsigned total_blocks, unsigned* counter,
                                    int tf_n, int max_table, int tile_threads, int variant, bool compact,
                                    bool aligned, cudaStream_t st) {
  const size_t smem = sizeof(float4) * (tf_n + 3 * max_table);
  aligned = aligned && compact;
  switch (tile_threads) {
    case 64: return launch_batch_nt<64>(jobs, n_jobs, total_blocks, counter, smem, variant, compact, aligned, st);
    case 256: return launch_batch_nt<256>(jobs, n_jobs, total_blocks, counter, smem, variant, compact, aligned, st);
    default: return launch_batch_nt<128>(jobs, n_jobs, total_blocks, counter, smem, variant, compact, aligned, st);
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
