// gradient.cu — per-voxel gradients for gradient Blinn-Phong shading
// (DataManager::GenerateStructuredGradientTexture,
// libs/volvis_utils/datamanager.cpp:332-352) built on the device, and the
// per-frame gradient-shading arguments of the marchers.
//
// The reference computes the gradient on the host in double precision
// (utils.cpp:146-351) and uploads it as RGB16F; here the same stencils are
// formed from the integer voxel values (exact), scaled once in FP32 and
// stored as four FP16 values (x, y, z, 0: one 8-byte load per tap).
#include <cuda.h>  // CUtensorMap (encoded through the runtime's driver entry point)
#include <cudaTypedefs.h>
#include <cuda_fp16.h>

#include "ctx.cuh"
#include "tc.cuh"  // mbarrier helpers

using namespace cvr::ctxutil;
using cvr::tc::mbar_init;
using cvr::tc::mbar_wait;
using cvr::tc::smem_u32;

namespace {

// GetNormalizedSample's integer numerator: the voxel, 0 outside the grid
// (structuredgridvolume.cpp:121-128).
template <class T>
__device__ __forceinline__ int vox(const T* __restrict__ v, int nx, int ny, int nz, int x, int y, int z) {
  if (x < 0 || y < 0 || z < 0 || x >= nx || y >= ny || z >= nz) return 0;
  return (int)__ldg(v + (size_t)x + (size_t)nx * ((size_t)y + (size_t)ny * z));
}

struct GradBuild {
  int model, n, filter, normalized;
  float inv_max;  // 1/255 or 1/65535
};

// GenerateGradientTexture's per-voxel result from the integer differences
// s2 - s1 (utils.cpp:156-193), its filter step (utils.cpp:196-233), and the
// FP16 store.
__device__ __forceinline__ void fd_finish(const GradBuild& b, float dx, float dy, float dz, float& gx, float& gy,
                                          float& gz) {
  if (b.normalized) {
    // normalize(s2 - s1) is normalize of the integer differences (the common
    // 1/255 scale cancels); the zero vector gives NaN there, then 0.
    // glm::normalize: v * inversesqrt(dot(v, v))
    const float l2 = dx * dx + dy * dy + dz * dz;
    if (l2 > 0.0f) {
      const float il = __frsqrt_rn(l2);  // correctly rounded 1/sqrt
      gx = dx * il; gy = dy * il; gz = dz * il;
    } else {
      gx = gy = gz = 0.0f;
    }
  } else {
    // s2s1 / 2.0f * (float)gradient_sample_size
    const float k = b.inv_max * 0.5f * float(b.n);
    gx = dx * k; gy = dy * k; gz = dz * k;
  }
  if (b.filter > 0 && gx != 0.0f && gy != 0.0f && gz != 0.0f) {
    // The filter sums gradients[x, y, z] -- the centre, not the neighbour --
    // over the in-bounds window and divides by the count, so the average is
    // the centre itself; it is then normalised when no component is zero.
    const float il = __frsqrt_rn(gx * gx + gy * gy + gz * gz);
    gx *= il; gy *= il; gz *= il;
  }
}

__device__ __forceinline__ void store_grad(uint2* __restrict__ out, size_t i, float gx, float gy, float gz) {
  const __half2 xy = __floats2half2_rn(gx, gy);
  const __half2 zw = __floats2half2_rn(gz, 0.0f);
  uint2 o;
  o.x = *reinterpret_cast<const unsigned int*>(&xy);
  o.y = *reinterpret_cast<const unsigned int*>(&zw);
  out[i] = o;
}

// Any model and sample size: one thread per voxel, neighbours straight from
// global memory (finite differences with gradient_sample_size > 1 reach n
// voxels away).
template <class T>
__global__ void __launch_bounds__(256) k_gradient(const T* __restrict__ v, int nx, int ny, int nz, GradBuild b,
                                                  uint2* __restrict__ out) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  const int z = blockIdx.z * blockDim.z + threadIdx.z;
  if (x >= nx || y >= ny || z >= nz) return;
  float gx, gy, gz;
  if (b.model == CVR_GRADIENT_FINITE_DIFFERENCES) {
    const int n = b.n;
    const float dx = float(vox(v, nx, ny, nz, x + n, y, z) - vox(v, nx, ny, nz, x - n, y, z));
    const float dy = float(vox(v, nx, ny, nz, x, y + n, z) - vox(v, nx, ny, nz, x, y - n, z));
    const float dz = float(vox(v, nx, ny, nz, x, y, z + n) - vox(v, nx, ny, nz, x, y, z - n));
    fd_finish(b, dx, dy, dz, gx, gy, gz);
  } else {
    // Sobel-Feldman (utils.cpp:295-321, sobelfeldman_generator.comp:37-60):
    // weights 4 / 2^(|v1|+|v2|) on the planes at -1 minus those at +1.
    int sx = 0, sy = 0, sz = 0;
#pragma unroll
    for (int v1 = -1; v1 <= 1; ++v1) {
#pragma unroll
      for (int v2 = -1; v2 <= 1; ++v2) {
        const int w = 4 >> ((v1 < 0 ? -v1 : v1) + (v2 < 0 ? -v2 : v2));
        sz += w * (vox(v, nx, ny, nz, x + v1, y + v2, z - 1) - vox(v, nx, ny, nz, x + v1, y + v2, z + 1));
        sy += w * (vox(v, nx, ny, nz, x + v1, y - 1, z + v2) - vox(v, nx, ny, nz, x + v1, y + 1, z + v2));
        sx += w * (vox(v, nx, ny, nz, x - 1, y + v2, z + v1) - vox(v, nx, ny, nz, x + 1, y + v2, z + v1));
      }
    }
    gx = float(sx) * b.inv_max; gy = float(sy) * b.inv_max; gz = float(sz) * b.inv_max;
  }
  store_grad(out, (size_t)x + (size_t)nx * ((size_t)y + (size_t)ny * z), gx, gy, gz);
}

// The 3x3x3 stencils (Sobel-Feldman, finite differences of sample size 1),
// HBM-bound form: a CTA owns a 32 x 8 column of voxels and walks kGradZ
// planes along z with the planes z-1, z, z+1 of its tile (plus a one-voxel
// halo, 0 outside the grid) in a shared-memory ring, so each voxel is read
// from memory about once and the 8-byte results stream out coalesced.  The
// (x, y) part of every load address and bounds test is computed once per
// thread; a plane costs each thread one or two loads.
constexpr int kGradTX = 32, kGradTY = 8, kGradZ = 32;
constexpr int kGradPW = kGradTX + 2, kGradPH = kGradTY + 2;
constexpr int kGradHalo = kGradPW * kGradPH - kGradTX * kGradTY;  // 84 halo cells

template <class T>
__global__ void __launch_bounds__(kGradTX * kGradTY) k_gradient_tiled(const T* __restrict__ v, int nx, int ny, int nz,
                                                                      GradBuild b, uint2* __restrict__ out) {
  __shared__ int ring[3][kGradPH][kGradPW];
  const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * kGradTX + tx;
  const int x0 = blockIdx.x * kGradTX, y0 = blockIdx.y * kGradTY, z0 = blockIdx.z * kGradZ;
  const int z1 = min(z0 + kGradZ, nz);
  const size_t plane = (size_t)nx * ny;
  // this thread's interior cell and, for the first kGradHalo threads, one halo cell
  const int x = x0 + tx, y = y0 + ty;
  const bool in_xy = x < nx && y < ny;
  const size_t off_xy = in_xy ? (size_t)x + (size_t)nx * y : 0;
  int hx = 0, hy = 0;
  bool h_on = false, h_xy = false;
  size_t h_off = 0;
  if (tid < kGradHalo) {
    // halo ring of the (kGradPW x kGradPH) tile: top row, bottom row, then the side columns
    if (tid < kGradPW) { hx = tid; hy = 0; }
    else if (tid < 2 * kGradPW) { hx = tid - kGradPW; hy = kGradPH - 1; }
    else { const int k = tid - 2 * kGradPW; hx = (k & 1) ? kGradPW - 1 : 0; hy = 1 + (k >> 1); }
    h_on = true;
    const int gx = x0 + hx - 1, gy = y0 + hy - 1;
    h_xy = gx >= 0 && gy >= 0 && gx < nx && gy < ny;
    h_off = h_xy ? (size_t)gx + (size_t)nx * gy : 0;
  }
  // a plane's two cells of this thread: fetched into registers one plane
  // ahead, so the loads are in flight while the current plane is computed
  int pv = 0, ph = 0;
  auto fetch = [&](int z) {
    const bool zin = z >= 0 && z < nz;
    const size_t zo = zin ? plane * (size_t)z : 0;
    pv = (zin && in_xy) ? (int)__ldg(v + zo + off_xy) : 0;
    ph = (zin && h_xy) ? (int)__ldg(v + zo + h_off) : 0;
  };
  auto put = [&](int slot) {
    ring[slot][ty + 1][tx + 1] = pv;
    if (h_on) ring[slot][hy][hx] = ph;
  };
  int s0 = 0, sm = 1, sp = 2;  // ring slots of the planes z - 1, z, z + 1
  fetch(z0 - 1);
  put(s0);
  fetch(z0);
  put(sm);
  fetch(z0 + 1);
  const bool sobel = b.model != CVR_GRADIENT_FINITE_DIFFERENCES;
  const int cx = tx + 1, cy = ty + 1;
  uint2* o = out + off_xy + plane * (size_t)z0;
  for (int z = z0; z < z1; ++z, o += plane) {
    put(sp);         // plane z + 1
    fetch(z + 2);    // lands during this plane's stencil
    __syncthreads();
    if (in_xy) {
      float gx, gy, gz;
      if (sobel) {
        int sx = 0, sy = 0, sz = 0;
#pragma unroll
        for (int v1 = -1; v1 <= 1; ++v1) {
#pragma unroll
          for (int v2 = -1; v2 <= 1; ++v2) {
            const int w = 4 >> ((v1 < 0 ? -v1 : v1) + (v2 < 0 ? -v2 : v2));
            const int pz = v2 < 0 ? s0 : (v2 > 0 ? sp : sm);  // plane z + v2
            const int qz = v1 < 0 ? s0 : (v1 > 0 ? sp : sm);  // plane z + v1
            sz += w * (ring[s0][cy + v2][cx + v1] - ring[sp][cy + v2][cx + v1]);
            sy += w * (ring[pz][cy - 1][cx + v1] - ring[pz][cy + 1][cx + v1]);
            sx += w * (ring[qz][cy + v2][cx - 1] - ring[qz][cy + v2][cx + 1]);
          }
        }
        gx = float(sx) * b.inv_max; gy = float(sy) * b.inv_max; gz = float(sz) * b.inv_max;
      } else {
        const float dx = float(ring[sm][cy][cx + 1] - ring[sm][cy][cx - 1]);
        const float dy = float(ring[sm][cy + 1][cx] - ring[sm][cy - 1][cx]);
        const float dz = float(ring[sp][cy][cx] - ring[s0][cy][cx]);
        fd_finish(b, dx, dy, dz, gx, gy, gz);
      }
      store_grad(o, 0, gx, gy, gz);
    }
    __syncthreads();  // the next iteration overwrites the slot of z - 1
    const int t = s0; s0 = sm; sm = sp; sp = t;
  }
}

// The 3x3x3 stencils with the planes brought in by the tensor memory
// accelerator: a CTA owns a 32 x 16 column of voxels over zc planes; one
// thread keeps kTmaBuf plane tiles (the column plus a one-voxel halo, read
// from an x origin rounded down to 16 bytes; the copy engine writes 0 outside
// the grid, which is GetNormalizedSample's 0) in flight, each completing on
// its own mbarrier.  Every thread computes two voxels (rows y, y + 1) and
// keeps, per voxel, three separable in-plane partial sums of the last three
// planes in registers, so a plane costs it 12 shared-memory reads for both
// voxels.  Sobel-Feldman's weights 4 / 2^(|v1|+|v2|) are (2 >> |v1|)(2 >> |v2|):
//   sx = sum_z w_z D[z],  D = sum_y w_y (P(x-1) - P(x+1))
//   sy = sum_z w_z E[z],  E = Sx(y-1) - Sx(y+1),   Sx = P(x-1) + 2 P(x) + P(x+1)
//   sz = Q[z-1] - Q[z+1], Q = sum_y w_y Sx
// -- the same integers as the direct 27-tap sums.  Needs the row pitch
// (nx x voxel bytes) to be a multiple of 16 bytes.  A CTA walks zc planes
// (32, or 16 / 8 when that is needed for two waves of CTAs on a small volume).
constexpr int kTmaTX = 32, kTmaTY = 16, kTmaBuf = 4;
constexpr int kTmaRows = kTmaTY + 2;
constexpr int kTmaPitch = 96;                        // bytes of a tile row: 64 u8 or 48 u16 voxels
constexpr int kTmaBufStride = 1792;                  // 128-byte aligned slots
static_assert(kTmaPitch * kTmaRows <= kTmaBufStride && kTmaBufStride % 128 == 0, "plane slot");
constexpr int kGradErrTma = 1;                       // d_kerr: a plane copy did not complete
constexpr uint32_t kTmaPolls = 1u << 22;             // bound of every plane wait

template <class T>
struct TmaGeom {
  static constexpr int OX = 16 / (int)sizeof(T);                 // x origin offset (16 bytes)
  static constexpr int BW = (sizeof(T) == 1) ? 64 : 48;          // box width in voxels (>= OX + 32 + 1)
  static constexpr unsigned kBytes = (unsigned)(BW * kTmaRows * sizeof(T));
  static_assert(BW * sizeof(T) <= kTmaPitch && (BW * sizeof(T)) % 16 == 0 && BW >= OX + kTmaTX + 1, "tile box");
};

template <class T, bool SOBEL>
__global__ void __launch_bounds__(256) k_gradient_tma(const __grid_constant__ CUtensorMap vol, int nx, int ny, int nz,
                                                      int zc, GradBuild b, uint2* __restrict__ out,
                                                      int* __restrict__ err) {
  using G = TmaGeom<T>;
  __shared__ __align__(128) uint8_t tiles[kTmaBuf][kTmaBufStride];
  __shared__ __align__(8) uint64_t bars[kTmaBuf];
  const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * kTmaTX + tx;
  const int x0 = blockIdx.x * kTmaTX, y0 = blockIdx.y * kTmaTY, z0 = blockIdx.z * zc;
  const int z1 = min(z0 + zc, nz);
  const int n_planes = z1 - z0 + 2;  // planes z0 - 1 .. z1
  if (tid == 0) {
#pragma unroll
    for (int i = 0; i < kTmaBuf; ++i) mbar_init(&bars[i], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  auto issue = [&](int i) {  // plane z0 - 1 + i into slot i % kTmaBuf
    const uint32_t bar = smem_u32(&bars[i % kTmaBuf]);
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(G::kBytes) : "memory");
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
        "[%5];" ::"r"(smem_u32(tiles[i % kTmaBuf])),
        "l"(reinterpret_cast<uint64_t>(&vol)), "r"(x0 - G::OX), "r"(y0 - 1), "r"(z0 - 1 + i), "r"(bar)
        : "memory");
  };
  if (tid == 0)
    for (int i = 0; i < kTmaBuf && i < n_planes; ++i) issue(i);

  const int x = x0 + tx, ya = y0 + 2 * ty;
  const bool on_a = x < nx && ya < ny, on_b = x < nx && ya + 1 < ny;
  const int c = tx + G::OX;  // tile column of x
  // per voxel (a, b) and plane: the three partial sums (Sobel: D, E, Q;
  // finite differences: P(x+1) - P(x-1), P(y+1) - P(y-1), P) of the planes
  // z - 1 (p0), z (p1), z + 1 (p2)
  int p0[2][3] = {}, p1[2][3] = {}, p2[2][3] = {};
  const size_t plane = (size_t)nx * ny;
  uint2* o = out + (size_t)x + (size_t)nx * ya + plane * (size_t)z0;
  for (int i = 0; i < n_planes; ++i) {
    const bool ok = mbar_wait(&bars[i % kTmaBuf], (uint32_t)((i / kTmaBuf) & 1), kTmaPolls);
    const T* t = reinterpret_cast<const T*>(tiles[i % kTmaBuf]) + (size_t)(2 * ty) * G::BW + c;
#pragma unroll
    for (int j = 0; j < 2; ++j)
#pragma unroll
      for (int k = 0; k < 3; ++k) { p0[j][k] = p1[j][k]; p1[j][k] = p2[j][k]; }
    if (SOBEL) {
      int sx[4], df[4];
#pragma unroll
      for (int r = 0; r < 4; ++r) {  // tile rows of y - 1 .. y + 2
        const int l = t[r * G::BW - 1], m = t[r * G::BW], h = t[r * G::BW + 1];
        sx[r] = l + 2 * m + h;
        df[r] = l - h;
      }
#pragma unroll
      for (int j = 0; j < 2; ++j) {
        p2[j][0] = df[j] + 2 * df[j + 1] + df[j + 2];
        p2[j][1] = sx[j] - sx[j + 2];
        p2[j][2] = sx[j] + 2 * sx[j + 1] + sx[j + 2];
      }
    } else {
      int ctr[4];
#pragma unroll
      for (int r = 0; r < 4; ++r) ctr[r] = t[r * G::BW];
#pragma unroll
      for (int j = 0; j < 2; ++j) {
        p2[j][0] = (int)t[(j + 1) * G::BW + 1] - (int)t[(j + 1) * G::BW - 1];
        p2[j][1] = ctr[j + 2] - ctr[j];
        p2[j][2] = ctr[j + 1];
      }
    }
    // one barrier per plane: every thread has read slot i and seen its copy
    // complete (or the CTA gives up together)
    if (__syncthreads_or(!ok)) {
      if (tid == 0) {
        atomicExch(err, kGradErrTma);
        // wait (bounded) for the copies still in flight before leaving
        for (int k = i; k < n_planes && k < i + kTmaBuf; ++k)
          mbar_wait(&bars[k % kTmaBuf], (uint32_t)((k / kTmaBuf) & 1), kTmaPolls);
      }
      return;
    }
    if (tid == 0 && i + kTmaBuf < n_planes) issue(i + kTmaBuf);
    if (i >= 2) {  // p0, p1, p2 hold the planes z - 1, z, z + 1 of z = z0 + i - 2
#pragma unroll
      for (int j = 0; j < 2; ++j) {
        if (!(j ? on_b : on_a)) continue;
        float gx, gy, gz;
        if (SOBEL) {
          gx = float(p0[j][0] + 2 * p1[j][0] + p2[j][0]) * b.inv_max;
          gy = float(p0[j][1] + 2 * p1[j][1] + p2[j][1]) * b.inv_max;
          gz = float(p0[j][2] - p2[j][2]) * b.inv_max;
        } else {
          fd_finish(b, float(p1[j][0]), float(p1[j][1]), float(p2[j][2] - p0[j][2]), gx, gy, gz);
        }
        store_grad(o, j ? (size_t)nx : 0, gx, gy, gz);
      }
      o += plane;
    }
  }
}

using EncodeTiled = PFN_cuTensorMapEncodeTiled_v12000;

EncodeTiled encode_tiled() {
  static EncodeTiled fn = [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      p = nullptr;
    return reinterpret_cast<EncodeTiled>(p);
  }();
  return fn;
}

// The volume's tensor map for k_gradient_tma: false when the layout does not
// allow one (row pitch not a multiple of 16 bytes, or no encoder).
template <class T>
bool volume_tensor_map(const void* vol, int nx, int ny, int nz, CUtensorMap* m) {
  using G = TmaGeom<T>;
  const cuuint64_t pitch = (cuuint64_t)nx * sizeof(T);
  if (pitch % 16 != 0 || (reinterpret_cast<uintptr_t>(vol) & 15) != 0) return false;
  EncodeTiled enc = encode_tiled();
  if (!enc) return false;
  const cuuint64_t dims[3] = {(cuuint64_t)nx, (cuuint64_t)ny, (cuuint64_t)nz};
  const cuuint64_t strides[2] = {pitch, pitch * (cuuint64_t)ny};
  const cuuint32_t box[3] = {(cuuint32_t)G::BW, (cuuint32_t)kTmaRows, 1};
  const cuuint32_t estr[3] = {1, 1, 1};
  return enc(m, sizeof(T) == 1 ? CU_TENSOR_MAP_DATA_TYPE_UINT8 : CU_TENSOR_MAP_DATA_TYPE_UINT16, 3,
             const_cast<void*>(vol), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
             CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
             CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

template <class T>
bool launch_gradient_tma(const void* vol, int nx, int ny, int nz, const GradBuild& b, uint2* out, int* err,
                         cudaStream_t st) {
  CUtensorMap m;
  if (!volume_tensor_map<T>(vol, nx, ny, nz, &m)) return false;
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    sms = 152;
  const long long xy = (long long)((nx + kTmaTX - 1) / kTmaTX) * ((ny + kTmaTY - 1) / kTmaTY);
  int zc = 32;
  while (zc > 8 && xy * ((nz + zc - 1) / zc) < 16LL * sms) zc /= 2;
  const dim3 block(kTmaTX, kTmaTY / 2, 1);
  const dim3 grid((nx + kTmaTX - 1) / kTmaTX, (ny + kTmaTY - 1) / kTmaTY, (nz + zc - 1) / zc);
  if (b.model == CVR_GRADIENT_FINITE_DIFFERENCES)
    k_gradient_tma<T, false><<<grid, block, 0, st>>>(m, nx, ny, nz, zc, b, out, err);
  else
    k_gradient_tma<T, true><<<grid, block, 0, st>>>(m, nx, ny, nz, zc, b, out, err);
  return true;
}

__global__ void k_gradient_to_float(const uint2* __restrict__ g, float* __restrict__ out, long long n) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint2 q = g[i];
  const float2 xy = __half22float2(*reinterpret_cast<const __half2*>(&q.x));
  const float2 zw = __half22float2(*reinterpret_cast<const __half2*>(&q.y));
  out[3 * i] = xy.x;
  out[3 * i + 1] = xy.y;
  out[3 * i + 2] = zw.x;
}

cvr_status check_gradient_params(cvr_ctx* c, const cvr_gradient_params& p) {
  if (p.model < 0 || p.model > CVR_GRADIENT_NONE) return fail(c, CVR_ERR_INVALID_ARG, "gradient: unknown model");
  if (p.model == CVR_GRADIENT_FINITE_DIFFERENCES && (p.sample_size < 1 || p.sample_size > 32768 || p.filter_nxnxn < 0))
    return fail(c, CVR_ERR_INVALID_ARG, "gradient: sample_size must be in [1, 32768], filter_nxnxn >= 0");
  return CVR_OK;
}

// Builds the current volume's gradient with c->grad_params.
cvr_status build_gradient(cvr_ctx* c) {
  const cvr_gradient_params& p = c->grad_params;
  const size_t n = (size_t)c->nx * c->ny * c->nz;
  CK(c, ensure(c->d_grad, c->grad_cap, n * sizeof(uint2)));
  GradBuild b{p.model, p.sample_size, p.filter_nxnxn, p.normalized, c->dtype == CVR_U8 ? 1.0f / 255.0f : 1.0f / 65535.0f};
  const bool u8 = c->dtype == CVR_U8;
  const bool stencil = p.model != CVR_GRADIENT_FINITE_DIFFERENCES || p.sample_size == 1;
  const int kern = stencil ? c->grad_kernel : CVR_GRADIENT_KERNEL_GENERIC;
  bool done = false;
  if (kern == CVR_GRADIENT_KERNEL_AUTO) {
    done = u8 ? launch_gradient_tma<uint8_t>(c->d_vol, c->nx, c->ny, c->nz, b, c->d_grad, c->d_kerr, c->stream)
              : launch_gradient_tma<uint16_t>(c->d_vol, c->nx, c->ny, c->nz, b, c->d_grad, c->d_kerr, c->stream);
  }
  c->grad_last = done ? CVR_GRADIENT_KERNEL_TMA : kern == CVR_GRADIENT_KERNEL_GENERIC ? kern : CVR_GRADIENT_KERNEL_TILED;
  if (done) {
    // nothing else to launch
  } else if (kern != CVR_GRADIENT_KERNEL_GENERIC) {
    const dim3 block(kGradTX, kGradTY, 1);
    const dim3 grid((c->nx + kGradTX - 1) / kGradTX, (c->ny + kGradTY - 1) / kGradTY, (c->nz + kGradZ - 1) / kGradZ);
    if (u8)
      k_gradient_tiled<uint8_t><<<grid, block, 0, c->stream>>>(static_cast<const uint8_t*>(c->d_vol), c->nx, c->ny,
                                                               c->nz, b, c->d_grad);
    else
      k_gradient_tiled<uint16_t><<<grid, block, 0, c->stream>>>(static_cast<const uint16_t*>(c->d_vol), c->nx, c->ny,
                                                                c->nz, b, c->d_grad);
  } else {
    const dim3 block(32, 4, 2);
    const dim3 grid((c->nx + 31) / 32, (c->ny + 3) / 4, (c->nz + 1) / 2);
    if (u8)
      k_gradient<uint8_t><<<grid, block, 0, c->stream>>>(static_cast<const uint8_t*>(c->d_vol), c->nx, c->ny, c->nz,
                                                         b, c->d_grad);
    else
      k_gradient<uint16_t><<<grid, block, 0, c->stream>>>(static_cast<const uint16_t*>(c->d_vol), c->nx, c->ny,
                                                          c->nz, b, c->d_grad);
  }
  CK(c, cudaGetLastError());
  if (done) {
    // a copy that never completed leaves the flag set: checked here unless
    // the stream is being captured (then by cvr_download_gradient)
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    CK(c, cudaStreamIsCapturing(c->stream, &cs));
    if (cs == cudaStreamCaptureStatusNone) {
      cvr_status s = check_kernel_flag(c, "gradient build: a plane copy did not complete");
      if (s != CVR_OK) return s;
    }
  }
  c->grad_ready = true;
  c->tex.grad_valid = false;
  return CVR_OK;
}

}  // namespace

namespace cvr {
namespace ctxutil {

cvr_status grad_args(cvr_ctx* c, int method, const cvr_light* light, FrameArgs* f) {
  f->grad = GradView{};
  if (!c->bp.apply || c->grad_params.model == CVR_GRADIENT_NONE) return CVR_OK;
  if (!light) return fail(c, CVR_ERR_INVALID_ARG, "gradient shading needs a light (its position)");
  if (!finite3(light->position)) return fail(c, CVR_ERR_INVALID_ARG, "gradient shading: non-finite light position");
  if (!c->grad_ready) {
    cvr_status s = build_gradient(c);
    if (s != CVR_OK) return s;
  }
  GradView& g = f->grad;
  g.g = c->d_grad;
  g.tex = 0;
  if (c->sampling & CVR_SAMPLING_TEX_VOLUME) {
    cvr_status s = ensure_gradient_texture(c);
    if (s != CVR_OK) return s;
    g.tex = c->tex.grad.tex;
  }
  g.nx = c->nx; g.ny = c->ny; g.nz = c->nz;
  g.inv_grid = f->vol.inv_grid;
  g.inv_spacing = f->vol.inv_spacing;
  g.light_pos = make3(light->position);
  // the ground truth's (and so the surrogate's) specular colour is vec3(1)
  // (gt_ray_marching.comp:293-294)
  const bool unit = method == CVR_METHOD_GROUND_TRUTH || method == CVR_METHOD_SURROGATE;
  g.ispec = unit ? f3(1.0f, 1.0f, 1.0f) : make3(c->bp.specular);
  g.ka = c->bp.ka; g.kd = c->bp.kd;
  g.ks = c->bp.ks; g.shininess = c->bp.shininess;
  return CVR_OK;
}

}  // namespace ctxutil
}  // namespace cvr

extern "C" {

cvr_status cvr_build_gradient(cvr_ctx* c, const cvr_gradient_params* p) {
  if (!c) return CVR_ERR_INVALID_ARG;
  cvr_gradient_params q = p ? *p : cvr_gradient_params{CVR_GRADIENT_NONE, 1, 0, 1};
  cvr_status s = check_gradient_params(c, q);
  if (s != CVR_OK) return s;
  CK(c, cudaSetDevice(c->device));
  c->grad_params = q;
  c->grad_ready = false;
  c->tex.grad_valid = false;
  if (q.model == CVR_GRADIENT_NONE) return CVR_OK;
  if (!c->has_volume) return fail(c, CVR_ERR_NO_VOLUME, "cvr_build_gradient: no volume");
  return build_gradient(c);
}

cvr_status cvr_set_gradient_kernel(cvr_ctx* c, int kernel) {
  if (!c) return CVR_ERR_INVALID_ARG;
  if (kernel < CVR_GRADIENT_KERNEL_AUTO || kernel > CVR_GRADIENT_KERNEL_GENERIC)
    return fail(c, CVR_ERR_INVALID_ARG, "cvr_set_gradient_kernel: AUTO, TILED or GENERIC");
  c->grad_kernel = kernel;
  return CVR_OK;
}

int cvr_get_gradient_kernel(cvr_ctx* c) { return c ? c->grad_last : -1; }

cvr_status cvr_download_gradient(cvr_ctx* c, float* host, size_t n_floats) {
  if (!c || !host) return CVR_ERR_INVALID_ARG;
  if (!c->grad_ready) return fail(c, CVR_ERR_NOT_READY, "cvr_download_gradient: no gradient built");
  const long long n = (long long)c->nx * c->ny * c->nz;
  if (n_floats < 3 * (size_t)n) return fail(c, CVR_ERR_INVALID_ARG, "cvr_download_gradient: buffer too small");
  CK(c, cudaSetDevice(c->device));
  cvr_status ks = check_kernel_flag(c, "gradient build: a plane copy did not complete");
  if (ks != CVR_OK) return ks;
  float* tmp = nullptr;
  CK(c, cudaMalloc((void**)&tmp, sizeof(float) * 3 * (size_t)n));
  k_gradient_to_float<<<(unsigned)((n + 255) / 256), 256, 0, c->stream>>>(c->d_grad, tmp, n);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpyAsync(host, tmp, sizeof(float) * 3 * (size_t)n, cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  cudaFree(tmp);
  if (e != cudaSuccess) return cuda_fail(c, e, "cvr_download_gradient");
  return CVR_OK;
}

cvr_status cvr_set_blinn_phong(cvr_ctx* c, const cvr_blinn_phong* bp) {
  if (!c || !bp) return CVR_ERR_INVALID_ARG;
  const float v[] = {bp->ka, bp->kd, bp->ks, bp->shininess, bp->specular[0], bp->specular[1], bp->specular[2]};
  for (float x : v)
    if (!std::isfinite(x)) return fail(c, CVR_ERR_INVALID_ARG, "cvr_set_blinn_phong: non-finite value");
  c->bp = *bp;
  return CVR_OK;
}

cvr_status cvr_get_blinn_phong(cvr_ctx* c, cvr_blinn_phong* out) {
  if (!c || !out) return CVR_ERR_INVALID_ARG;
  *out = c->bp;
  return CVR_OK;
}

}  // extern "C"
