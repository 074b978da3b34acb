// staged.cu — the plain marcher (ray_marching_1p.comp:170-247) with
// shared-memory brick staging.
//
// A CTA renders one 16x8-pixel tile slab by slab along the ray parameter t.
// For each slab it loads into shared memory the box of voxels the tile's rays
// cross in it (the axis-aligned box of the tile frustum's four corner rays at
// the slab's two depths, one voxel of margin on every side for the trilinear
// taps and the curvature of the ray fan), then every thread takes the samples
// of its ray that fall in the slab from shared memory.  A tap outside the box
// (single-precision rounding at a slab edge) is read from the volume instead,
// so every sample is the same trilinear lookup as sample_volume's.  The slab
// depth starts at 8 voxels and halves until the box fits the staging buffer;
// a slab whose box never fits is sampled from the volume.
#include "shade.cuh"

namespace cvr {

namespace {

constexpr int kStageW = 16, kStageH = 8, kStageThreads = kStageW * kStageH;
constexpr int kStageBytes = 40 * 1024;

struct StageBox {
  int ox, oy, oz;   // voxel origin of the box
  int bx, by, bz;   // extent (0: this slab reads the volume)
  float t1;         // the slab's end (ray parameter)
};

template <class T>
__device__ __forceinline__ float staged_trilinear(const T* box, const StageBox& B, const VolumeView& v, float3 p) {
  const Tap tx = axis_tap(fmaf(p.x, v.inv_spacing.x, -0.5f), v.nx);
  const Tap ty = axis_tap(fmaf(p.y, v.inv_spacing.y, -0.5f), v.ny);
  const Tap tz = axis_tap(fmaf(p.z, v.inv_spacing.z, -0.5f), v.nz);
  const int x0 = tx.i0 - B.ox, x1 = tx.i1 - B.ox, y0 = ty.i0 - B.oy, y1 = ty.i1 - B.oy;
  const int z0 = tz.i0 - B.oz, z1 = tz.i1 - B.oz;
  const bool inside = (unsigned)x0 < (unsigned)B.bx && (unsigned)x1 < (unsigned)B.bx &&
                      (unsigned)y0 < (unsigned)B.by && (unsigned)y1 < (unsigned)B.by &&
                      (unsigned)z0 < (unsigned)B.bz && (unsigned)z1 < (unsigned)B.bz;
  if (!inside) return sample_volume(v, p);
  const int sy = B.bx, sz = B.bx * B.by;
  const float c000 = box[x0 + y0 * sy + z0 * sz], c100 = box[x1 + y0 * sy + z0 * sz];
  const float c010 = box[x0 + y1 * sy + z0 * sz], c110 = box[x1 + y1 * sy + z0 * sz];
  const float c001 = box[x0 + y0 * sy + z1 * sz], c101 = box[x1 + y0 * sy + z1 * sz];
  const float c011 = box[x0 + y1 * sy + z1 * sz], c111 = box[x1 + y1 * sy + z1 * sz];
  const float c00 = fmaf(tx.t, c100 - c000, c000), c10 = fmaf(tx.t, c110 - c010, c010);
  const float c01 = fmaf(tx.t, c101 - c001, c001), c11 = fmaf(tx.t, c111 - c011, c011);
  const float c0 = fmaf(ty.t, c10 - c00, c00), c1 = fmaf(ty.t, c11 - c01, c01);
  return fmaf(tz.t, c1 - c0, c0) * v.norm;
}

// The voxel box of the tile's rays over [t0, t0 + dt): extent 0 when it does
// not fit the staging buffer.
__device__ __forceinline__ StageBox stage_box(const FrameArgs& f, const float3 dirs[4], float t0, float dt) {
  const VolumeView& v = f.vol;
  float3 lo = f3(3.0e38f, 3.0e38f, 3.0e38f), hi = f3(-3.0e38f, -3.0e38f, -3.0e38f);
#pragma unroll
  for (int c = 0; c < 4; ++c) {
#pragma unroll
    for (int e = 0; e < 2; ++e) {
      const float3 w = f.cam.eye + dirs[c] * (t0 + (e ? dt : 0.0f)) + v.grid * 0.5f;
      const float3 u = f3(fmaf(w.x, v.inv_spacing.x, -0.5f), fmaf(w.y, v.inv_spacing.y, -0.5f),
                          fmaf(w.z, v.inv_spacing.z, -0.5f));
      lo = fmin3(lo, u);
      hi = fmax3(hi, u);
    }
  }
  StageBox B;
  B.t1 = t0 + dt;
  // texel coordinates beyond +-2^30 are outside any volume: the box is empty there
  lo = fmax3(lo, f3(-1.0e9f, -1.0e9f, -1.0e9f));
  hi = fmin3(hi, f3(1.0e9f, 1.0e9f, 1.0e9f));
  const int lx = max((int)floorf(lo.x) - 1, 0), ly = max((int)floorf(lo.y) - 1, 0), lz = max((int)floorf(lo.z) - 1, 0);
  const int hx = min((int)floorf(hi.x) + 2, v.nx - 1), hy = min((int)floorf(hi.y) + 2, v.ny - 1),
            hz = min((int)floorf(hi.z) + 2, v.nz - 1);
  B.ox = lx; B.oy = ly; B.oz = lz;
  B.bx = hx - lx + 1; B.by = hy - ly + 1; B.bz = hz - lz + 1;
  const long long cells = (long long)max(B.bx, 0) * max(B.by, 0) * max(B.bz, 0);
  const int esz = v.dtype == 1 ? 1 : 2;
  if (B.bx <= 0 || B.by <= 0 || B.bz <= 0 || cells * esz > kStageBytes) B.bx = B.by = B.bz = 0;
  return B;
}

template <class T>
__global__ void __launch_bounds__(kStageThreads) k_march_plain_staged(FrameArgs f) {
  extern __shared__ float4 sm_tf[];
  __shared__ __align__(16) T box[kStageBytes / sizeof(T)];
  __shared__ StageBox B;
  __shared__ unsigned s_tmin, s_tmax;
  const float4* tf = stage_tf(f, sm_tf);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  // warps of 8x4 pixels, 2 x 2 of them per 16x8 tile
  const int px = blockIdx.x * kStageW + (warp & 1) * 8 + (lane & 7);
  const int py = blockIdx.y * kStageH + (warp >> 1) * 4 + (lane >> 3);
  if (threadIdx.x == 0) { s_tmin = 0x7f7fffffu; s_tmax = 0u; }
  __syncthreads();
  const bool inside = px < f.W && py < f.H;
  float3 dir = f3(0.0f, 0.0f, 1.0f), tex0 = f3(0.0f, 0.0f, 0.0f);
  float tnear = 0.0f, tfar = 0.0f, D = 0.0f, s = 0.0f;
  float4 dst = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  unsigned n = 0, shaded = 0, max_iter = 0;
  bool active = false;
  if (inside) {
    dir = primary_dir(f.cam, px, py, f.W, f.H);
    if (ray_aabb(f.cam.eye, dir, f.vol.grid, tnear, tfar)) {
      D = fabsf(tfar - tnear);
      tex0 = f.cam.eye + dir * tnear + f.vol.grid * 0.5f;
      max_iter = (unsigned)fminf(D / f.step, 1.0e9f) + 4u;
      active = D > 0.0f;
      // non-negative floats order like their bit patterns
      if (active) {
        atomicMin(&s_tmin, __float_as_uint(tnear));
        atomicMax(&s_tmax, __float_as_uint(tnear + D));
      }
    }
  }
  // the tile's corner rays (clamped to the image)
  float3 dirs[4];
  {
    const int x0 = blockIdx.x * kStageW, y0 = blockIdx.y * kStageH;
    const int x1 = min(x0 + kStageW - 1, f.W - 1), y1 = min(y0 + kStageH - 1, f.H - 1);
    dirs[0] = primary_dir(f.cam, x0, y0, f.W, f.H);
    dirs[1] = primary_dir(f.cam, x1, y0, f.W, f.H);
    dirs[2] = primary_dir(f.cam, x0, y1, f.W, f.H);
    dirs[3] = primary_dir(f.cam, x1, y1, f.W, f.H);
  }
  __syncthreads();
  const float t_start = __uint_as_float(s_tmin), t_stop = __uint_as_float(s_tmax);
  const float vox = fminf(f.vol.spacing.x, fminf(f.vol.spacing.y, f.vol.spacing.z));
  float t0 = t_start;
  // every slab is at least a quarter voxel deep: a bounded number of slabs
  const int max_slabs = t_stop >= t_start ? (int)fminf((t_stop - t_start) / (0.25f * vox), 1.0e6f) + 2 : 0;
  for (int slab = 0; slab < max_slabs && __syncthreads_or(active); ++slab) {
    if (threadIdx.x == 0) {
      float dt = 8.0f * vox;
      StageBox b = stage_box(f, dirs, t0, dt);
      while (b.bx == 0 && dt * 0.5f >= 0.25f * vox) {
        dt *= 0.5f;
        b = stage_box(f, dirs, t0, dt);
      }
      if (b.bx == 0) b.t1 = t0 + dt;  // sampled from the volume
      B = b;
    }
    __syncthreads();
    const StageBox sb = B;
    const int cells = sb.bx * sb.by * sb.bz;
    for (int i = threadIdx.x; i < cells; i += kStageThreads) {
      const int x = i % sb.bx, r = i / sb.bx, y = r % sb.by, z = r / sb.by;
      const size_t g =
          (size_t)(sb.ox + x) + (size_t)f.vol.nx * ((size_t)(sb.oy + y) + (size_t)f.vol.ny * (size_t)(sb.oz + z));
      box[i] = __ldg(static_cast<const T*>(f.vol.voxels) + g);
    }
    __syncthreads();
    // this ray's samples in [t0, t1)
    while (active && s < D && n < max_iter) {
      const float h = fminf(f.step, D - s);
      if (tnear + (s + h * 0.5f) >= sb.t1) break;
      const float3 p = tex0 + dir * (s + h * 0.5f);
      const float density = sb.bx ? staged_trilinear(box, sb, f.vol, p) : sample_volume(f.vol, p);
      float4 src = tf_lookup(tf, f.tf_n, density);
      ++n;
      if (src.w > 0.0f) {
        ++shaded;
        if (f.grad.g) src = phong_plain(f, src, p);
        src.w = 1.0f - expf(-src.w * h);
        src.x *= src.w; src.y *= src.w; src.z *= src.w;
        const float rr = 1.0f - dst.w;
        dst.x += rr * src.x; dst.y += rr * src.y; dst.z += rr * src.z; dst.w += rr * src.w;
        if (dst.w > 0.99f) { active = false; break; }
      }
      s = s + h;
    }
    if (!(s < D && n < max_iter)) active = false;
    t0 = sb.t1;
  }
  if (inside) {
    const size_t o = (size_t)py * f.W + px;
    f.out[o] = dst;
    if (f.counts) f.counts[o] = n;
  }
  add_stats(f, n, shaded, 0u);
}

}  // namespace

// plain layout, FP32 samples, and the transfer function and the staging
// buffer within the 48 KB of shared memory a CTA gets without opting in
bool plain_staging_applies(const FrameArgs& f) {
  return f.vol.bs == 0 && !f.vol.quad && !f.vol.tex && sizeof(float4) * f.tf_n + kStageBytes + 256 <= 48 * 1024;
}

cudaError_t launch_plain_staged(const FrameArgs& f, cudaStream_t st) {
  const dim3 grid((f.W + kStageW - 1) / kStageW, (f.H + kStageH - 1) / kStageH);
  const size_t sm = sizeof(float4) * f.tf_n;
  if (f.vol.dtype == 1) k_march_plain_staged<uint8_t><<<grid, kStageThreads, sm, st>>>(f);
  else k_march_plain_staged<uint16_t><<<grid, kStageThreads, sm, st>>>(f);
  return cudaGetLastError();
}

}  // namespace cvr
