// march_ext.cuh — the extinction marchers (single frames and batches) and
// their launch templates.  Each CTA size (64, 128, 256 threads) is
// instantiated in its own translation unit (march_ext64.cu, march_ext128.cu,
// march_ext256.cu), so that the many register-variant instantiations compile
// in parallel; march.cu dispatches to them.
#pragma once

#include "shade.cuh"

namespace cvr {

// Persistent launch: every SM filled with as many CTAs of kern as fit.
template <class K, class... Args>
cudaError_t launch_persistent(K kern, size_t smem, cudaStream_t st, Args... args) {
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

inline dim3 grid_of(const FrameArgs& f) {
  return dim3((f.W + f.tile_w - 1) / f.tile_w, (f.H + f.tile_h - 1) / f.tile_h, 1);
}
inline int threads_of(const FrameArgs& f) { return (f.tile_w / 8) * (f.tile_h / 4) * 32; }

template <int V>
constexpr int minb128() {
  return V == 1 ? 65536 / (128 * 128) : (V == 2 ? 65536 / (128 * 80) : (V == 3 ? 65536 / (128 * 96) : 1));
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
cudaError_t launch_batch_t(const BatchExtJob* jobs, int n_jobs, unsigned total_blocks, unsigned* counter,
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

// The batch launch of one CTA size at the tuner's register variant.
template <int NT>
cudaError_t launch_batch_nt(const BatchExtJob* jobs, int n_jobs, unsigned total_blocks, unsigned* counter,
                            size_t smem, int variant, bool compact, bool aligned, cudaStream_t st) {
  switch (variant) {
    case 1: return launch_batch_t<NT, minb_of<NT>(1)>(jobs, n_jobs, total_blocks, counter, smem, compact, aligned, st);
    case 2: return launch_batch_t<NT, minb_of<NT>(2)>(jobs, n_jobs, total_blocks, counter, smem, compact, aligned, st);
    case 3: return launch_batch_t<NT, minb_of<NT>(3)>(jobs, n_jobs, total_blocks, counter, smem, compact, aligned, st);
    default: return launch_batch_t<NT, 1>(jobs, n_jobs, total_blocks, counter, smem, compact, aligned, st);
  }
}

template <int NT, int MINB>
cudaError_t launch_extinction_t(const FrameArgs& f, const ExtArgs& e, const ShadowBoxTable* table,
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
cudaError_t launch_extinction_nt(const FrameArgs& f, const ExtArgs& e, const ShadowBoxTable* table,
                                        cudaStream_t st) {
  switch (f.variant) {
    case 1: return launch_extinction_t<NT, minb_of<NT>(1)>(f, e, table, st);
    case 2: return launch_extinction_t<NT, minb_of<NT>(2)>(f, e, table, st);
    case 3: return launch_extinction_t<NT, minb_of<NT>(3)>(f, e, table, st);
    default: return launch_extinction_t<NT, 1>(f, e, table, st);
  }
}

// Instantiated once per CTA size in its own translation unit.
#define CVR_EXTINCTION_INSTANCES(NT)                                                                       \
  template cudaError_t launch_extinction_nt<NT>(const FrameArgs&, const ExtArgs&, const ShadowBoxTable*,   \
                                                cudaStream_t);                                              \
  template cudaError_t launch_batch_nt<NT>(const BatchExtJob*, int, unsigned, unsigned*, size_t, int, bool, \
                                           bool, cudaStream_t);
#define CVR_EXTINCTION_EXTERN(NT)                                                                          \
  extern template cudaError_t launch_extinction_nt<NT>(const FrameArgs&, const ExtArgs&,                   \
                                                       const ShadowBoxTable*, cudaStream_t);               \
  extern template cudaError_t launch_batch_nt<NT>(const BatchExtJob*, int, unsigned, unsigned*, size_t, int, \
                                                  bool, bool, cudaStream_t);

}  // namespace cvr
