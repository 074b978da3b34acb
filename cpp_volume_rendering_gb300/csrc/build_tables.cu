// build_tables.cu — device builders for the two illumination tables:
//  * the extinction summed-area table of RC1PExtinctionBasedShading
//    (GenerateExtinctionSAT3DTex, ebsrenderer.cpp:624-723, and
//    SummedAreaTable3D<double>::BuildSAT, libs/vis_utils/summedareatable.h:218-280),
//  * the Gaussian extinction mip pyramid of RC1PConeTracingDirOcclusionShading
//    (ExtinctionCoefficientVolume::GenerateExtinctionCoefficientVolumeAnySize,
//    extcoefvolumegenerator.cpp:230-408, gen_extcoefvol_anysize*.comp, backtotau.comp).
#include "build_tables.cuh"

#include <algorithm>
#include <cmath>

namespace cvr {

// ------------------------------------------------------------------ SAT
// Pass 1: fill + x-scan.  One warp per SAT row (y, z).  Interior cells take
// lut[voxel(x-1, y-1, z-1)] (the extinction of that voxel value in fixed
// point); the one-cell border is zero (ebsrenderer.cpp:651-659).
// W: long long (exact int64 prefix sums) or unsigned (sums modulo 2^32).
template <class W>
__global__ void k_sat_fill_xscan(const void* vox, int dtype, int nx, int ny, int nz,
                                 const W* __restrict__ lut, W* __restrict__ sat) {
  const int sx = nx + 2, sy = ny + 2, sz = nz + 2;
  int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int lane = threadIdx.x & 31;
  if (warp >= sy * sz) return;
  int y = warp % sy, z = warp / sy;
  W* row = sat + ((size_t)z * sy + y) * (size_t)sx;
  bool border_row = (y == 0 || z == 0 || y == sy - 1 || z == sz - 1);
  size_t vrow = border_row ? 0 : ((size_t)(z - 1) * ny + (y - 1)) * (size_t)nx;
  W carry = 0;
  for (int base = 0; base < sx; base += 32) {
    int x = base + lane;
    W v = 0;
    if (!border_row && x > 0 && x < sx - 1) {
      unsigned int q = (dtype == 1) ? (unsigned int)__ldg(static_cast<const uint8_t*>(vox) + vrow + (x - 1))
                                    : (unsigned int)__ldg(static_cast<const uint16_t*>(vox) + vrow + (x - 1));
      v = __ldg(lut + q);
    }
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      W n = __shfl_up_sync(0xffffffffu, v, o);
      if (lane >= o) v += n;
    }
    v += carry;
    if (x < sx) row[x] = v;
    carry = __shfl_sync(0xffffffffu, v, 31);
  }
}

// Pass 2 / 3: inclusive scan along y (stride sx) or z (stride sx*sy).  One
// thread per line; consecutive threads own consecutive x, so every step is a
// coalesced 256-byte warp access.
template <class W>
__global__ void k_sat_scan_lines(W* __restrict__ sat, int sx, int n_lines_inner, int n_lines_outer,
                                 size_t line_stride_inner, size_t line_stride_outer, size_t step, int len) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  int total = sx * n_lines_inner * n_lines_outer;
  if (t >= total) return;
  int x = t % sx;
  int r = t / sx;
  int a = r % n_lines_inner, b = r / n_lines_inner;
  W* p = sat + (size_t)x + (size_t)a * line_stride_inner + (size_t)b * line_stride_outer;
  W acc = 0;
  int i = 0;
  for (; i + 4 <= len; i += 4) {
    W v0 = p[(size_t)(i + 0) * step], v1 = p[(size_t)(i + 1) * step];
    W v2 = p[(size_t)(i + 2) * step], v3 = p[(size_t)(i + 3) * step];
    acc += v0; p[(size_t)(i + 0) * step] = acc;
    acc += v1; p[(size_t)(i + 1) * step] = acc;
    acc += v2; p[(size_t)(i + 2) * step] = acc;
    acc += v3; p[(size_t)(i + 3) * step] = acc;
  }
  for (; i < len; ++i) {
    acc += p[(size_t)i * step];
    p[(size_t)i * step] = acc;
  }
}

// ---- blocked builder: x-y prefix of every plane in shared memory, then a
// z-scan (in place for the int64 table; fused with the quad layout for the
// compact one).  Two passes over the table instead of three.

// Pass 1: one CTA per z plane, in chunks of R <= kSatChunkRows rows.  Phase A: a
// thread per column (or per few columns) carries the column's running
// y-prefix from chunk to chunk (in shared memory); the voxel loads and table
// lookups of the chunk's rows are issued before the adds, and each row's
// prefix goes to shared memory.  Phase B: a warp per row
// scans it along x (shuffles, carried across 32-cell segments) and writes
// the plane's row out (coalesced).  The y-then-x order gives the same 2D
// prefix sums (integer adds).  Interior cells take lut[voxel(x-1, y-1, z-1)];
// the one-cell border is zero.
constexpr int kSatPlaneThreads = 512;
constexpr int kSatChunkRows = 16;
template <class W>
__global__ void __launch_bounds__(kSatPlaneThreads, 2) k_sat_planes(const void* vox, int dtype, int nx, int ny,
                                                                     int nz, const W* __restrict__ lut,
                                                                     W* __restrict__ out, int R) {
  extern __shared__ __align__(16) unsigned char sm_sat[];
  const int sx = nx + 2, sy = ny + 2, sz = nz + 2;
  W* chunk = reinterpret_cast<W*>(sm_sat);  // R x sx
  W* carry = chunk + (size_t)R * sx;        // sx running column sums
  const int z = blockIdx.x;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, warps = blockDim.x >> 5;
  const bool border_plane = z == 0 || z == sz - 1;
  W* plane = out + (size_t)z * sx * sy;
  for (int x = threadIdx.x; x < sx; x += blockDim.x) carry[x] = 0;
  for (int y0 = 0; y0 < sy; y0 += R) {
    const int rows = min(R, sy - y0);
#pragma unroll 1
    for (int x = threadIdx.x; x < sx; x += blockDim.x) {
      const bool col = !border_plane && x > 0 && x < sx - 1;
      unsigned q[kSatChunkRows];
#pragma unroll
      for (int r = 0; r < kSatChunkRows; ++r) {
        const int y = y0 + r;
        q[r] = 0xffffffffu;
        if (col && r < rows && y > 0 && y < sy - 1) {
          const size_t i = ((size_t)(z - 1) * ny + (y - 1)) * (size_t)nx + (x - 1);
          q[r] = dtype == 1 ? (unsigned)__ldg(static_cast<const uint8_t*>(vox) + i)
                            : (unsigned)__ldg(static_cast<const uint16_t*>(vox) + i);
        }
      }
      W v[kSatChunkRows];
#pragma unroll
      for (int r = 0; r < kSatChunkRows; ++r) v[r] = q[r] != 0xffffffffu ? __ldg(lut + q[r]) : W(0);
      W run = carry[x];
#pragma unroll
      for (int r = 0; r < kSatChunkRows; ++r) {
        if (r >= rows) break;
        run += v[r];
        chunk[(size_t)r * sx + x] = run;
      }
      carry[x] = run;
    }
    __syncthreads();
    for (int r = warp; r < rows; r += warps) {
      W run = 0;
      W* dst = plane + (size_t)(y0 + r) * sx;
      const W* src = chunk + (size_t)r * sx;
      for (int base = 0; base < sx; base += 32) {
        const int x = base + lane;
        W t = x < sx ? src[x] : W(0);
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const W n = __shfl_up_sync(0xffffffffu, t, o);
          if (lane >= o) t += n;
        }
        t += run;
        if (x < sx) dst[x] = t;
        run = __shfl_sync(0xffffffffu, t, 31);
      }
    }
    __syncthreads();  // the chunk is read before the next one is written
  }
}

// Pass 2 (int64 table): in-place running sum along z of every (x, y) column,
// a thread per column (coalesced along x), 16 planes loaded before they are
// summed so that enough loads are in flight to stream at HBM rate.
template <class W>
__global__ void __launch_bounds__(256) k_sat_zscan(W* __restrict__ sat, long long columns, int sz) {
  const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= columns) return;
  W* p = sat + c;
  W run = 0;
  constexpr int B = 16;
  for (int z0 = 0; z0 < sz; z0 += B) {
    W v[B];
#pragma unroll
    for (int k = 0; k < B; ++k) v[k] = z0 + k < sz ? p[(size_t)(z0 + k) * columns] : W(0);
#pragma unroll
    for (int k = 0; k < B; ++k) {
      run += v[k];
      if (z0 + k < sz) p[(size_t)(z0 + k) * columns] = run;
    }
  }
}

// Pass 2 (compact table): the z-scan of 32 x 8 columns and of their low halo
// (x0 - 1, y0 - 1) per CTA, writing the predecessor quads of each plane
// (S at (x-1, y-1), (x, y-1), (x-1, y), (x, y), coordinates clamped to the
// table) from shared-memory tiles of the planes' running sums.  Two groups of
// kQuadGroup tiles alternate, so one barrier serves kQuadGroup planes: a
// group is rewritten only after the barrier that follows the reads of its
// previous planes.
constexpr int kQuadTileX = 32, kQuadTileY = 8, kQuadHaloCols = (kQuadTileX + 1) * (kQuadTileY + 1);
constexpr int kQuadThreads = ((kQuadHaloCols + 31) / 32) * 32;
constexpr int kQuadGroup = 4;
__global__ void __launch_bounds__(kQuadThreads) k_sat_zscan_quads(const unsigned* __restrict__ P, uint4* __restrict__ out,
                                                                  int sx, int sy, int sz) {
  __shared__ unsigned tile[2][kQuadGroup][kQuadTileY + 1][kQuadTileX + 1];
  const int x0 = blockIdx.x * kQuadTileX, y0 = blockIdx.y * kQuadTileY;
  const int t = threadIdx.x;
  const bool owner = t < kQuadHaloCols;
  const int hx = t % (kQuadTileX + 1), hy = t / (kQuadTileX + 1);
  const int gx = min(max(x0 - 1 + hx, 0), sx - 1), gy = min(max(y0 - 1 + hy, 0), sy - 1);
  const size_t sxy = (size_t)sx * sy;
  const unsigned* col = P + (size_t)gy * sx + gx;
  const int lx = t % kQuadTileX, ly = t / kQuadTileX;
  const int ox = x0 + lx, oy = y0 + ly;
  const bool writer = t < kQuadTileX * kQuadTileY && ox < sx && oy < sy;
  uint4* dst = out + (size_t)oy * sx + ox;
  unsigned run = 0;
  constexpr int B = 16;  // planes loaded per round (a multiple of kQuadGroup)
  int grp = 0;
  for (int z0 = 0; z0 < sz; z0 += B) {
    unsigned v[B];
#pragma unroll
    for (int k = 0; k < B; ++k) v[k] = (owner && z0 + k < sz) ? __ldg(col + (size_t)(z0 + k) * sxy) : 0u;
#pragma unroll
    for (int k0 = 0; k0 < B; k0 += kQuadGroup) {
      if (z0 + k0 >= sz) break;
#pragma unroll
      for (int j = 0; j < kQuadGroup; ++j) {
        run += v[k0 + j];
        if (owner) tile[grp][j][hy][hx] = run;
      }
      __syncthreads();
      if (writer) {
#pragma unroll
        for (int j = 0; j < kQuadGroup; ++j) {
          const int z = z0 + k0 + j;
          if (z < sz)
            dst[(size_t)z * sxy] = make_uint4(tile[grp][j][ly][lx], tile[grp][j][ly][lx + 1], tile[grp][j][ly + 1][lx],
                                              tile[grp][j][ly + 1][lx + 1]);
        }
      }
      grp ^= 1;
    }
  }
}

// Rows per chunk of k_sat_planes for rows of sx cells of type W: the chunk
// and the column sums within 200 KB of shared memory (0: fewer than 4 rows
// fit; the line-scan builder below is used).
template <class W>
static int sat_plane_rows(int sx) {
  const long long r = (long long)(200 * 1024 / sizeof(W)) / sx - 1;
  return r >= 4 ? (int)std::min<long long>(r, kSatChunkRows) : 0;
}

template <class W>
static cudaError_t sat_planes(const void* vox, int dtype, int nx, int ny, int nz, const W* lut, W* out, int R,
                              cudaStream_t st) {
  const int sx = nx + 2, sz = nz + 2;
  const size_t smem = sizeof(W) * (size_t)(R + 1) * sx;
  cudaError_t e = cudaFuncSetAttribute(k_sat_planes<W>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  k_sat_planes<W><<<sz, kSatPlaneThreads, smem, st>>>(vox, dtype, nx, ny, nz, lut, out, R);
  return cudaGetLastError();
}

// The previous builder (three passes: fill + x-scan, y-scan, z-scan), kept
// for planes too wide for shared memory.
template <class W>
static cudaError_t sat_build_lines(const void* vox, int dtype, int nx, int ny, int nz, const W* lut, W* sat,
                                   cudaStream_t st) {
  const int sx = nx + 2, sy = ny + 2, sz = nz + 2;
  {
    long long rows = (long long)sy * sz;
    int threads = 256;
    long long blocks = (rows * 32 + threads - 1) / threads;
    k_sat_fill_xscan<W><<<(unsigned)blocks, threads, 0, st>>>(vox, dtype, nx, ny, nz, lut, sat);
  }
  {
    // y-scan: lines indexed by (x, z); stride along y = sx.
    int total = sx * sz;
    k_sat_scan_lines<W><<<(total + 255) / 256, 256, 0, st>>>(sat, sx, 1, sz, 0, (size_t)sx * sy, (size_t)sx, sy);
  }
  {
    // z-scan: lines indexed by (x, y); stride along z = sx*sy.
    int total = sx * sy;
    k_sat_scan_lines<W><<<(total + 255) / 256, 256, 0, st>>>(sat, sx, sy, 1, (size_t)sx, 0, (size_t)sx * sy, sz);
  }
  return cudaGetLastError();
}

cudaError_t launch_sat_build(const void* vox, int dtype, int nx, int ny, int nz, const long long* lut,
                             long long* sat, cudaStream_t st) {
  const int sx = nx + 2, sy = ny + 2, sz = nz + 2;
  const int R = sat_plane_rows<long long>(sx);
  if (R == 0) return sat_build_lines(vox, dtype, nx, ny, nz, lut, sat, st);
  cudaError_t e = sat_planes(vox, dtype, nx, ny, nz, lut, sat, R, st);
  if (e != cudaSuccess) return e;
  const long long columns = (long long)sx * sy;
  k_sat_zscan<long long><<<(unsigned)((columns + 255) / 256), 256, 0, st>>>(sat, columns, sz);
  return cudaGetLastError();
}

cudaError_t launch_sat_build_quads(const void* vox, int dtype, int nx, int ny, int nz, const unsigned* lut,
                                   unsigned* scratch, uint4* out, cudaStream_t st) {
  const int sx = nx + 2, sy = ny + 2, sz = nz + 2;
  const int R = sat_plane_rows<unsigned>(sx);
  cudaError_t e = R == 0 ? sat_build_lines(vox, dtype, nx, ny, nz, lut, scratch, st) : cudaSuccess;
  if (e != cudaSuccess) return e;
  if (R > 0) {
    // x-y plane prefixes only: the quad pass below adds them up along z
    e = sat_planes(vox, dtype, nx, ny, nz, lut, scratch, R, st);
    if (e != cudaSuccess) return e;
    dim3 grid((sx + kQuadTileX - 1) / kQuadTileX, (sy + kQuadTileY - 1) / kQuadTileY);
    k_sat_zscan_quads<<<grid, kQuadThreads, 0, st>>>(scratch, out, sx, sy, sz);
    return cudaGetLastError();
  }
  return launch_sat_quads(scratch, out, sx, sy, sz, st);  // the line builder made the whole table
}

// x-y quads of the volume: cell (x, y, z) = the voxels at (x, y), (x', y),
// (x, y'), (x', y') of plane z, with the successors clamped to the volume.
template <class T, class Q>
__global__ void k_quad_volume(const T* __restrict__ v, Q* __restrict__ out, int nx, int ny, long long n) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int x = (int)(i % nx), y = (int)((i / nx) % ny);
  const long long dx = x + 1 < nx ? 1 : 0, dy = y + 1 < ny ? nx : 0;
  Q q;
  q.x = v[i]; q.y = v[i + dx]; q.z = v[i + dy]; q.w = v[i + dy + dx];
  out[i] = q;
}

cudaError_t launch_quad_volume(const void* src, void* dst, int dtype, int nx, int ny, int nz, cudaStream_t st) {
  const long long n = (long long)nx * ny * nz;
  const unsigned blocks = (unsigned)((n + 255) / 256);
  if (dtype == 1)
    k_quad_volume<uint8_t, uchar4><<<blocks, 256, 0, st>>>(static_cast<const uint8_t*>(src), static_cast<uchar4*>(dst),
                                                           nx, ny, n);
  else
    k_quad_volume<uint16_t, ushort4><<<blocks, 256, 0, st>>>(static_cast<const uint16_t*>(src),
                                                             static_cast<ushort4*>(dst), nx, ny, n);
  return cudaGetLastError();
}

// x-y quads of every pyramid level (successors clamped within the level).
__global__ void k_quad_pyramid(const float* __restrict__ src, float4* __restrict__ dst, int dx, int dy,
                               long long n) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int x = (int)(i % dx), y = (int)((i / dx) % dy);
  const long long ox = x + 1 < dx ? 1 : 0, oy = y + 1 < dy ? dx : 0;
  dst[i] = make_float4(src[i], src[i + ox], src[i + oy], src[i + oy + ox]);
}

cudaError_t launch_pyramid_quads(const PyramidView& P, const float* data, float4* dst, cudaStream_t st) {
  for (int l = 0; l < P.n_levels; ++l) {
    const long long n = (long long)P.dims[l][0] * P.dims[l][1] * P.dims[l][2];
    k_quad_pyramid<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(data + P.offset[l], dst + P.offset[l], P.dims[l][0],
                                                                P.dims[l][1], n);
  }
  return cudaGetLastError();
}

// x-y predecessor quads of a table: out[(x, y, z)] = s at (x-1, y-1),
// (x, y-1), (x-1, y), (x, y) of plane z, the predecessors clamped to 0.
__global__ void k_sat_quads(const unsigned* __restrict__ s, uint4* __restrict__ out, int sx, int sy,
                            long long cells) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= cells) return;
  const int x = (int)(i % sx), y = (int)((i / sx) % sy);
  const long long dx = x > 0 ? 1 : 0, dy = y > 0 ? sx : 0;
  out[i] = make_uint4(s[i - dy - dx], s[i - dy], s[i - dx], s[i]);
}

// Walk table (WalkView) from the predecessor-quad table: the oct of cell
// (x, y, z) is D = S(shifted) - S at the clamped coordinates (x-1..x, y-1..y,
// z-1..z), read as four quads: planes z-1 and z of the cell (S at the x-y
// pairs) and the same two shifted by w along the walk axis (clamped to the
// table).  Along the walk axis this uses the predecessor of the shifted
// coordinate, which equals the shift of the clamped predecessor except at
// walk coordinate 0, a cell no query reads (a box reaching below the table
// on the walk axis takes the quad query); past the high face S repeats.
__global__ void k_sat_walk(const uint4* __restrict__ q, uint4* __restrict__ out, int sx, int sy, int sz, int axis,
                           int w, long long cells) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= cells) return;
  const int x = (int)(i % sx), y = (int)((i / sx) % sy), z = (int)(i / ((long long)sx * sy));
  const size_t sxy = (size_t)sx * sy;
  auto Q = [&](int X, int Y, int Z) {
    X = min(max(X, 0), sx - 1); Y = min(max(Y, 0), sy - 1); Z = min(max(Z, 0), sz - 1);
    return __ldg(&q[(size_t)X + (size_t)sx * Y + sxy * Z]);
  };
  const int z0 = max(z - 1, 0);
  const uint4 lo0 = Q(x, y, z0), lo1 = Q(x, y, z);
  const int dx = axis == 0 ? w : 0, dy = axis == 1 ? w : 0;
  const uint4 up0 = Q(x + dx, y + dy, axis == 2 ? z0 + w : z0), up1 = Q(x + dx, y + dy, axis == 2 ? z + w : z);
  out[2 * i] = make_uint4(up0.x - lo0.x, up0.y - lo0.y, up0.z - lo0.z, up0.w - lo0.w);
  out[2 * i + 1] = make_uint4(up1.x - lo1.x, up1.y - lo1.y, up1.z - lo1.z, up1.w - lo1.w);
}

cudaError_t launch_sat_walk(const uint4* quads, uint4* out, int sx, int sy, int sz, int axis, int w,
                            cudaStream_t st) {
  const long long cells = (long long)sx * sy * sz;
  k_sat_walk<<<(unsigned)((cells + 255) / 256), 256, 0, st>>>(quads, out, sx, sy, sz, axis, w, cells);
  return cudaGetLastError();
}

cudaError_t launch_sat_quads(const unsigned* sat, uint4* out, int sx, int sy, int sz, cudaStream_t st) {
  const long long cells = (long long)sx * sy * sz;
  k_sat_quads<<<(unsigned)((cells + 255) / 256), 256, 0, st>>>(sat, out, sx, sy, cells);
  return cudaGetLastError();
}

// --------------------------------------------------------------- pyramid
// gen_extcoefvol_anysize.comp: base level voxel (i,j,k) holds the normalised
// 7x7x7 Gaussian average (sigma S0, taps at integer multiples of S0) of the
// TF opacity of the trilinearly sampled volume; samples outside the grid
// count as 0 opacity but keep their weight.
// The 7^3 Gaussian weights s^3 exp(-|f|^2 / (2 s^2)) of the tap offsets f =
// (ptx, pty, ptz) * s, in the loops' order, and their sum in the same order:
// the same values for every output voxel, computed once per CTA.
__device__ __forceinline__ float stage_gauss(float s, float* w) {
  for (int k = threadIdx.x; k < 343; k += blockDim.x) {
    const int ptx = k / 49 - 3, pty = (k / 7) % 7 - 3, ptz = k % 7 - 3;
    const float fx = float(ptx) * s, fy = float(pty) * s, fz = float(ptz) * s;
    w[k] = (s * s * s) * expf(-(fx * fx + fy * fy + fz * fz) / (2.0f * s * s));
  }
  __syncthreads();
  float sum_w = 0.0f;
  for (int k = 0; k < 343; ++k) sum_w += w[k];
  return sum_w;
}

// Inside the grid: t = p / S in [0, 1] on every axis, which for a correctly
// rounded division is p in [0, S].
__device__ __forceinline__ bool in_grid(float3 p, float3 g) {
  return !(p.x < 0.0f || p.y < 0.0f || p.z < 0.0f || p.x > g.x || p.y > g.y || p.z > g.z);
}

__global__ void k_pyr_base(VolumeView vol, const float4* __restrict__ tf_rgba, int tf_n, int bx, int by, int bz,
                           float s0, float* __restrict__ out) {
  __shared__ float sm_w[343];
  extern __shared__ float4 sm_tf[];
  for (int i = threadIdx.x; i < tf_n; i += blockDim.x) sm_tf[i] = tf_rgba[i];
  const float sum_w = stage_gauss(s0, sm_w);
  long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  long long total = (long long)bx * by * bz;
  if (idx >= total) return;
  int x = int(idx % bx), y = int((idx / bx) % by), z = int(idx / ((long long)bx * by));
  float3 vs = f3(vol.grid.x / float(bx), vol.grid.y / float(by), vol.grid.z / float(bz));
  float3 gp = f3((float(x) + 0.5f) * vs.x, (float(y) + 0.5f) * vs.y, (float(z) + 0.5f) * vs.z);
  float sum_wc = 0.0f;
  int k = 0;
  for (int ptx = -3; ptx < 4; ++ptx) {
    for (int pty = -3; pty < 4; ++pty) {
      for (int ptz = -3; ptz < 4; ++ptz, ++k) {
        const float3 p = gp + f3(float(ptx) * s0, float(pty) * s0, float(ptz) * s0);
        float ck = 0.0f;
        if (in_grid(p, vol.grid)) ck = tf_alpha(sm_tf, tf_n, sample_volume(vol, p));
        sum_wc += sm_w[k] * ck;
      }
    }
  }
  out[idx] = sum_wc / sum_w;
}

// gen_extcoefvol_anysize_mmlevel.comp: level l from level l-1 with sigma
// Si = S0 * 2^l, sampling level l-1 trilinearly (textureLod at an integer lod).
__global__ void k_pyr_level(PyramidView P, int l, float si, float* __restrict__ out) {
  __shared__ float sm_w[343];
  const float sum_w = stage_gauss(si, sm_w);
  const int* d = P.dims[l];
  long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  long long total = (long long)d[0] * d[1] * d[2];
  if (idx >= total) return;
  int x = int(idx % d[0]), y = int((idx / d[0]) % d[1]), z = int(idx / ((long long)d[0] * d[1]));
  float3 lvs = P.grid / f3(float(d[0]), float(d[1]), float(d[2]));
  float3 gp = f3((float(x) + 0.5f) * lvs.x, (float(y) + 0.5f) * lvs.y, (float(z) + 0.5f) * lvs.z);
  float sum_wc = 0.0f;
  int k = 0;
  for (int ptx = -3; ptx < 4; ++ptx) {
    for (int pty = -3; pty < 4; ++pty) {
      for (int ptz = -3; ptz < 4; ++ptz, ++k) {
        const float3 p = gp + f3(float(ptx) * si, float(pty) * si, float(ptz) * si);
        float ck = 0.0f;
        if (in_grid(p, P.grid)) ck = pyr_sample_level(P, l - 1, p);
        sum_wc += sm_w[k] * ck;
      }
    }
  }
  out[idx] = sum_wc / sum_w;
}

// backtotau.comp: opacity -> extinction, -log(1 - opacity), every level.
__global__ void k_pyr_backtotau(float* data, long long n) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) data[i] = -1.0f * logf(1.0f - data[i]);
}

// ---- separable form of the two level builders
// Where a level's cells and taps fall on one lattice of input texel
// coordinates with a constant fraction on every axis -- m input texels per
// output cell and t per tap step, both whole numbers (the reference's base
// 128^3 of a 256^3 volume with S0 = 1 voxel; every level from the one below it
// when the dimensions halve) -- the Gaussian weights factor per axis
// (exp(-|k|^2 / 2) = product of exp(-k_a^2 / 2)), so a level is one pass that
// takes every lattice sample once (the TF opacity of the trilinear volume for
// the base, the trilinear level below for the others; 0 outside the box, as
// in_grid) and three 7-tap passes, instead of 343 samples per cell.  Cell i,
// tap k reads lattice point i m + (k + 3) t, at texel coordinate j0 + q + f.
struct PyrAxis {
  int m, t;   // texels per cell, per tap step
  int j0, g;  // lattice start (integer part) and size
  int n_out;  // cells
  float f;    // the constant fraction
};
struct PyrWeights { float w[7]; };

static bool pyr_axis(int n_in, int n_out, double tap_texels, PyrAxis* a) {
  if (n_out < 1 || n_in % n_out) return false;
  const double t = std::nearbyint(tap_texels);
  if (!(t >= 1.0) || std::fabs(tap_texels - t) > 1e-9 * t) return false;
  a->m = n_in / n_out;
  a->t = (int)t;
  const double c0 = 0.5 * a->m - 0.5;  // texel coordinate of cell 0, tap 0
  a->f = (float)(c0 - std::floor(c0));
  a->j0 = (int)std::floor(c0) - 3 * a->t;
  a->g = (n_out - 1) * a->m + 6 * a->t + 1;
  a->n_out = n_out;
  return a->g <= 65535;  // a grid dimension of the lattice and pass launches
}

// The plan of level l (l = 0: from the volume): false when it has no separable form.
static bool pyr_plan(const VolumeView& vol, const PyramidView& P, int l, float s0, PyrAxis ax[3]) {
  const int in[3] = {l == 0 ? vol.nx : P.dims[l - 1][0], l == 0 ? vol.ny : P.dims[l - 1][1],
                     l == 0 ? vol.nz : P.dims[l - 1][2]};
  const double grid[3] = {P.grid.x, P.grid.y, P.grid.z};
  const double sigma = (double)s0 * std::ldexp(1.0, l);
  for (int a = 0; a < 3; ++a)
    if (!pyr_axis(in[a], P.dims[l][a], sigma * in[a] / grid[a], &ax[a])) return false;
  return true;
}

static long long pyr_scratch(const PyrAxis ax[3]) {
  return (long long)ax[0].g * ax[1].g * ax[2].g + (long long)ax[0].n_out * ax[1].g * ax[2].g +
         (long long)ax[0].n_out * ax[1].n_out * ax[2].g;
}

long long pyramid_scratch_floats(const VolumeView& vol, const PyramidView& P, float s0) {
  long long need = 0;
  PyrAxis ax[3];
  for (int l = 0; l < P.n_levels; ++l)
    if (pyr_plan(vol, P, l, s0, ax)) need = std::max(need, pyr_scratch(ax));
  return need;
}

// Lattice point (qx, qy, qz) of a launch whose grid is (x blocks, g_y, g_z).
__device__ __forceinline__ bool pyr_lattice_point(const PyrAxis* A, const int n_in[3], int qx, int qy, int qz,
                                                  float3& u) {
  u = f3((float)(A[0].j0 + qx) + A[0].f, (float)(A[1].j0 + qy) + A[1].f, (float)(A[2].j0 + qz) + A[2].f);
  // inside the box [0, S]: texel coordinates in [-0.5, n - 0.5]
  return u.x >= -0.5f && u.y >= -0.5f && u.z >= -0.5f && u.x <= (float)n_in[0] - 0.5f &&
         u.y <= (float)n_in[1] - 0.5f && u.z <= (float)n_in[2] - 0.5f;
}

struct PyrAxes { PyrAxis a[3]; };

// The lattice and pass kernels run on (x blocks, y, z) grids: no division of
// a flat index per element.
__global__ void k_pyr_lattice_base(VolumeView vol, const float4* __restrict__ tf_rgba, int tf_n, PyrAxes A,
                                   float* __restrict__ G) {
  extern __shared__ float4 sm_tf[];
  for (int i = threadIdx.x; i < tf_n; i += blockDim.x) sm_tf[i] = tf_rgba[i];
  __syncthreads();
  const int qx = blockIdx.x * blockDim.x + threadIdx.x, qy = blockIdx.y, qz = blockIdx.z;
  if (qx >= A.a[0].g) return;
  const size_t idx = ((size_t)qz * A.a[1].g + qy) * A.a[0].g + qx;
  const int n_in[3] = {vol.nx, vol.ny, vol.nz};
  float3 u;
  const bool inside = pyr_lattice_point(A.a, n_in, qx, qy, qz, u);
  const float3 p = f3((u.x + 0.5f) * vol.spacing.x, (u.y + 0.5f) * vol.spacing.y, (u.z + 0.5f) * vol.spacing.z);
  G[idx] = inside ? tf_alpha(sm_tf, tf_n, sample_volume(vol, p)) : 0.0f;
}

__global__ void k_pyr_lattice_level(PyramidView P, int l_in, PyrAxes A, float* __restrict__ G) {
  const int qx = blockIdx.x * blockDim.x + threadIdx.x, qy = blockIdx.y, qz = blockIdx.z;
  if (qx >= A.a[0].g) return;
  const size_t idx = ((size_t)qz * A.a[1].g + qy) * A.a[0].g + qx;
  const int* n_in = P.dims[l_in];
  float3 u;
  const bool inside = pyr_lattice_point(A.a, n_in, qx, qy, qz, u);
  const float3 p = f3((u.x + 0.5f) * (P.grid.x / (float)n_in[0]), (u.y + 0.5f) * (P.grid.y / (float)n_in[1]),
                      (u.z + 0.5f) * (P.grid.z / (float)n_in[2]));
  G[idx] = inside ? pyr_sample_level(P, l_in, p) : 0.0f;
}

// One 7-tap pass along axis ax of an (nx, ny, nz) array: out has n_out cells
// along that axis, out[i] = sum_k w[k] in[i m + (k + 3) t].  Grid: (x blocks
// of the output's x extent, its y extent, its z extent).
__global__ void k_pyr_pass(const float* __restrict__ in, int nx, int ny, int nz, int ax, PyrAxis a, PyrWeights w,
                           float* __restrict__ out) {
  const int ox = ax == 0 ? a.n_out : nx, oy = ax == 1 ? a.n_out : ny;
  const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y, z = blockIdx.z;
  if (x >= ox) return;
  const size_t idx = ((size_t)z * oy + y) * ox + x;
  const int i = ax == 0 ? x : (ax == 1 ? y : z);
  const long long stride = ax == 0 ? 1 : (ax == 1 ? (long long)nx : (long long)nx * ny);
  const long long base = (ax == 0 ? 0 : x) + (ax == 1 ? 0 : (long long)y * nx) + (ax == 2 ? 0 : (long long)z * nx * ny);
  float acc = 0.0f;
#pragma unroll
  for (int k = 0; k < 7; ++k) acc = fmaf(w.w[k], __ldg(in + base + (long long)(i * a.m + k * a.t) * stride), acc);
  out[idx] = acc;
}

static cudaError_t pyr_separable(const PyrAxis A[3], float* G, float* T1, float* T2, float* out, cudaStream_t st) {
  PyrWeights w;
  double sum = 0.0;
  for (int k = -3; k <= 3; ++k) sum += std::exp(-0.5 * k * k);
  for (int k = -3; k <= 3; ++k) w.w[k + 3] = (float)(std::exp(-0.5 * k * k) / sum);
  const unsigned bx_n = (unsigned)(A[0].n_out + 127) / 128;  // every pass's output has n_out along x
  k_pyr_pass<<<dim3(bx_n, A[1].g, A[2].g), 128, 0, st>>>(G, A[0].g, A[1].g, A[2].g, 0, A[0], w, T1);
  k_pyr_pass<<<dim3(bx_n, A[1].n_out, A[2].g), 128, 0, st>>>(T1, A[0].n_out, A[1].g, A[2].g, 1, A[1], w, T2);
  k_pyr_pass<<<dim3(bx_n, A[1].n_out, A[2].n_out), 128, 0, st>>>(T2, A[0].n_out, A[1].n_out, A[2].g, 2, A[2], w, out);
  return cudaGetLastError();
}

cudaError_t launch_pyramid_build(const VolumeView& vol, const float4* tf_rgba, int tf_n, float s0,
                                 PyramidView& P, float* data, float* scratch, long long scratch_floats,
                                 cudaStream_t st) {
  const int threads = 128;
  long long n0 = (long long)P.dims[0][0] * P.dims[0][1] * P.dims[0][2];
  size_t sm = sizeof(float4) * tf_n;
  if (sm > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(k_pyr_base, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(k_pyr_lattice_base, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return e;
  }
  PyrAxes A;
  if (scratch && pyr_plan(vol, P, 0, s0, A.a) && pyr_scratch(A.a) <= scratch_floats) {
    const long long g = (long long)A.a[0].g * A.a[1].g * A.a[2].g;
    float* T1 = scratch + g;
    float* T2 = T1 + (long long)A.a[0].n_out * A.a[1].g * A.a[2].g;
    k_pyr_lattice_base<<<dim3((A.a[0].g + 127) / 128, A.a[1].g, A.a[2].g), 128, sm, st>>>(vol, tf_rgba, tf_n, A,
                                                                                          scratch);
    cudaError_t e = pyr_separable(A.a, scratch, T1, T2, data + P.offset[0], st);
    if (e != cudaSuccess) return e;
  } else {
    k_pyr_base<<<(unsigned)((n0 + threads - 1) / threads), threads, sm, st>>>(
        vol, tf_rgba, tf_n, P.dims[0][0], P.dims[0][1], P.dims[0][2], s0, data + P.offset[0]);
  }
  P.data = data;
  for (int l = 1; l < P.n_levels; ++l) {
    long long nl = (long long)P.dims[l][0] * P.dims[l][1] * P.dims[l][2];
    float si = s0 * powf(2.0f, float(l));
    if (scratch && pyr_plan(vol, P, l, s0, A.a) && pyr_scratch(A.a) <= scratch_floats) {
      const long long g = (long long)A.a[0].g * A.a[1].g * A.a[2].g;
      float* T1 = scratch + g;
      float* T2 = T1 + (long long)A.a[0].n_out * A.a[1].g * A.a[2].g;
      k_pyr_lattice_level<<<dim3((A.a[0].g + 127) / 128, A.a[1].g, A.a[2].g), 128, 0, st>>>(P, l - 1, A, scratch);
      cudaError_t e = pyr_separable(A.a, scratch, T1, T2, data + P.offset[l], st);
      if (e != cudaSuccess) return e;
    } else {
      k_pyr_level<<<(unsigned)((nl + threads - 1) / threads), threads, 0, st>>>(P, l, si, data + P.offset[l]);
    }
  }
  long long total = P.offset[P.n_levels - 1] +
                    (long long)P.dims[P.n_levels - 1][0] * P.dims[P.n_levels - 1][1] * P.dims[P.n_levels - 1][2];
  k_pyr_backtotau<<<(unsigned)((total + 255) / 256), 256, 0, st>>>(data, total);
  return cudaGetLastError();
}

// ----------------------------------------------------------- L2 flush
// ---------------------------------------------------------------- bricks
// Copies a plain x-fastest volume into bricks of 2^bs voxels per edge
// (brick-local x fastest, bricks x fastest); voxels past the volume's edge
// inside the last bricks are zero and never read.
template <class T>
__global__ void k_brick(const T* __restrict__ src, T* __restrict__ dst, int nx, int ny, int nz, int bs,
                        long long total) {
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= total) return;
  const int m = (1 << bs) - 1;
  const int local = (int)(e & ((1ll << (3 * bs)) - 1));
  const long long brick = e >> (3 * bs);
  const int bx = (nx + m) >> bs, by = (ny + m) >> bs;
  const int x = (int)(brick % bx) * (m + 1) + (local & m);
  const int y = (int)((brick / bx) % by) * (m + 1) + ((local >> bs) & m);
  const int z = (int)(brick / ((long long)bx * by)) * (m + 1) + (local >> (2 * bs));
  dst[e] = (x < nx && y < ny && z < nz) ? src[(size_t)x + (size_t)nx * ((size_t)y + (size_t)ny * z)] : T(0);
}

long long brick_elements(int nx, int ny, int nz, int bs) {
  const int m = (1 << bs) - 1;
  return (long long)((nx + m) >> bs) * ((ny + m) >> bs) * ((nz + m) >> bs) << (3 * bs);
}

cudaError_t launch_brick_volume(const void* src, void* dst, int dtype, int nx, int ny, int nz, int bs,
                                cudaStream_t st) {
  const long long total = brick_elements(nx, ny, nz, bs);
  const unsigned blocks = (unsigned)((total + 255) / 256);
  if (dtype == 1)
    k_brick<<<blocks, 256, 0, st>>>(static_cast<const uint8_t*>(src), static_cast<uint8_t*>(dst), nx, ny, nz, bs, total);
  else
    k_brick<<<blocks, 256, 0, st>>>(static_cast<const uint16_t*>(src), static_cast<uint16_t*>(dst), nx, ny, nz, bs,
                                    total);
  return cudaGetLastError();
}

__global__ void k_fill(uint4* p, size_t n, unsigned int v) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  size_t stride = (size_t)gridDim.x * blockDim.x;
  for (; i < n; i += stride) p[i] = make_uint4(v, v, v, v);
}
cudaError_t launch_fill(void* p, size_t bytes, unsigned int v, cudaStream_t st) {
  size_t n = bytes / sizeof(uint4);
  k_fill<<<152 * 8, 256, 0, st>>>(static_cast<uint4*>(p), n, v);
  return cudaGetLastError();
}

}  // namespace cvr
