// cvr_device.cuh — device-side building blocks shared by every marcher.
//
// Each function states the reference shader code it restates.  All sampling
// follows OpenGL texture() semantics on normalised coordinates: texel centres
// at (i + 0.5) / n, clamp-to-edge, (tri)linear weights computed exactly in
// FP32 (the reference's FP16 texture storage is not reproduced: voxels are
// read as exact u8/u16 values and normalised by 255 / 65535).
#pragma once

#include <cstdint>
#include <type_traits>
#include <cuda_runtime.h>

namespace cvr {

// ---------------------------------------------------------------- float3 math
__host__ __device__ __forceinline__ float3 f3(float x, float y, float z) { return make_float3(x, y, z); }
__host__ __device__ __forceinline__ float3 operator+(float3 a, float3 b) { return f3(a.x + b.x, a.y + b.y, a.z + b.z); }
__host__ __device__ __forceinline__ float3 operator-(float3 a, float3 b) { return f3(a.x - b.x, a.y - b.y, a.z - b.z); }
__host__ __device__ __forceinline__ float3 operator-(float3 a) { return f3(-a.x, -a.y, -a.z); }
__host__ __device__ __forceinline__ float3 operator*(float3 a, float3 b) { return f3(a.x * b.x, a.y * b.y, a.z * b.z); }
__host__ __device__ __forceinline__ float3 operator*(float3 a, float s) { return f3(a.x * s, a.y * s, a.z * s); }
__host__ __device__ __forceinline__ float3 operator*(float s, float3 a) { return f3(a.x * s, a.y * s, a.z * s); }
__host__ __device__ __forceinline__ float3 operator/(float3 a, float3 b) { return f3(a.x / b.x, a.y / b.y, a.z / b.z); }
__host__ __device__ __forceinline__ float dot3(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__host__ __device__ __forceinline__ float3 cross3(float3 a, float3 b) {
  return f3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ float3 normalize3(float3 a) {
  float inv = rsqrtf(dot3(a, a));
  return a * inv;
}
__device__ __forceinline__ float3 fmin3(float3 a, float3 b) { return f3(fminf(a.x, b.x), fminf(a.y, b.y), fminf(a.z, b.z)); }
__device__ __forceinline__ float3 fmax3(float3 a, float3 b) { return f3(fmaxf(a.x, b.x), fmaxf(a.y, b.y), fmaxf(a.z, b.z)); }
__device__ __forceinline__ float3 clamp3(float3 v, float3 lo, float3 hi) { return fmin3(fmax3(v, lo), hi); }
__device__ __forceinline__ float3 abs3(float3 a) { return f3(fabsf(a.x), fabsf(a.y), fabsf(a.z)); }
__host__ __device__ __forceinline__ float3 make3(const float* p) { return f3(p[0], p[1], p[2]); }

// ---------------------------------------------------------------- state
// Volume as uploaded by cvr_set_volume: u8/u16, x fastest.
struct VolumeView {
  const void* voxels;
  int dtype;            // 1 = u8, 2 = u16
  int nx, ny, nz;
  float3 spacing;       // VolumeScales
  float3 inv_spacing;
  float3 grid;          // VolumeGridSize = dims * spacing
  float norm;           // 1/255 or 1/65535
  // Storage: bricks of B = 2^bs voxels per edge, each brick x-fastest inside,
  // bricks x-fastest; bs = 0 is the plain x-fastest layout.  stride[a] is the
  // element distance between neighbouring bricks along axis a (plain layout:
  // 1, nx, nx*ny).
  int bs;
  long long stride[3];
  // Texture-unit copy (hardware trilinear, 8-bit weights), or 0: when set,
  // sample_volume reads it instead of the array (CVR_SAMPLING_TEX_VOLUME).
  cudaTextureObject_t tex;
  float3 inv_grid;
  // 1: voxels hold the x-y quad layout (cell (x, y, z) = the voxels at (x, y),
  // (x', y), (x, y'), (x', y') of plane z, x' = min(x + 1, nx - 1), y' likewise;
  // uchar4 / ushort4): a trilinear sample is two loads (planes z0 and z1).
  int quad;
};

// Per-frame camera frame (glm::lookAt rows s, u, f) and projection terms.
struct CameraView {
  float3 eye;
  float3 s, u, f;       // right, up, forward
  float tan_half_fovy;
  float aspect;
};

// ---------------------------------------------------------------- camera ray
// ray_marching_1p.comp:160-170: VerPos = ((x+0.5)/W, (y+0.5)/H)*2-1,
// camera_dir = normalize(vec3(X*tan*aspect, Y*tan, -1) * mat3(LookAt)).
// Row-vector times the lookAt 3x3 equals X*tan*aspect*s + Y*tan*u + f.
__device__ __forceinline__ float3 primary_dir(const CameraView& c, int px, int py, int W, int H) {
  float vx = ((float(px) + 0.5f) / float(W)) * 2.0f - 1.0f;
  float vy = ((float(py) + 0.5f) / float(H)) * 2.0f - 1.0f;
  float a = vx * c.tan_half_fovy * c.aspect;
  float b = vy * c.tan_half_fovy;
  return normalize3(c.s * a + c.u * b + c.f);
}

// ray_bbox_intersection.comp:18-52 (IntersectBox + RayAABBIntersection):
// slab test against [-S/2, S/2], tnear clamped to 0, hit iff tfar > tnear.
__device__ __forceinline__ bool ray_aabb(float3 origin, float3 dir, float3 grid, float& tnear, float& tfar) {
  float3 bmin = grid * -0.5f;
  float3 bmax = grid * 0.5f;
  float3 inv = f3(1.0f / dir.x, 1.0f / dir.y, 1.0f / dir.z);
  float3 t0 = inv * (bmin - origin);
  float3 t1 = inv * (bmax - origin);
  float3 tmin = fmin3(t0, t1);
  float3 tmax = fmax3(t0, t1);
  tnear = fmaxf(fmaxf(tmin.x, tmin.y), tmin.z);
  tfar = fminf(fminf(tmax.x, tmax.y), tmax.z);
  bool hit = tfar > tnear;
  tnear = fmaxf(tnear, 0.0f);
  return hit;
}

// ---------------------------------------------------------------- sampling
// Element offset of coordinate i along axis a (offsets of the three axes add).
__device__ __forceinline__ long long voxel_term(const VolumeView& v, int a, int i) {
  const int m = (1 << v.bs) - 1;
  return (long long)(i >> v.bs) * v.stride[a] + (long long)((i & m) << (a * v.bs));
}
__device__ __forceinline__ float voxel_at(const VolumeView& v, long long i) {
  if (v.dtype == 1) return float(__ldg(static_cast<const uint8_t*>(v.voxels) + i));
  return float(__ldg(static_cast<const uint16_t*>(v.voxels) + i));
}
__device__ __forceinline__ float voxel(const VolumeView& v, int x, int y, int z) {
  return voxel_at(v, voxel_term(v, 0, x) + voxel_term(v, 1, y) + voxel_term(v, 2, z));
}

// One axis of a GL_LINEAR clamp-to-edge lookup at texel coordinate u.
struct Tap {
  int i0, i1;
  float t;
};
__device__ __forceinline__ Tap axis_tap(float u, int n) {
  float fl = floorf(u);
  int i = int(fl);
  Tap r;
  r.t = u - fl;
  r.i0 = min(max(i, 0), n - 1);
  r.i1 = min(max(i + 1, 0), n - 1);
  return r;
}

// texture(TexVolume, tex_pos / VolumeGridSize).r with tex_pos in [0, S]:
// texel coordinate = tex_pos / spacing - 0.5.
__device__ __forceinline__ float sample_volume(const VolumeView& v, float3 tex_pos) {
  if (v.tex) return tex3D<float>(v.tex, tex_pos.x * v.inv_grid.x, tex_pos.y * v.inv_grid.y, tex_pos.z * v.inv_grid.z);
  if (v.quad) {
    // Texel coordinates below 0 (the half texel at the low faces) are raised
    // to 0 so the successor taps are the quad's; both read voxel 0 there.
    const Tap tx = axis_tap(fmaxf(fmaf(tex_pos.x, v.inv_spacing.x, -0.5f), 0.0f), v.nx);
    const Tap ty = axis_tap(fmaxf(fmaf(tex_pos.y, v.inv_spacing.y, -0.5f), 0.0f), v.ny);
    const Tap tz = axis_tap(fmaf(tex_pos.z, v.inv_spacing.z, -0.5f), v.nz);
    // 32-bit cell numbers (the quad copy is only made below 2^31 cells)
    const unsigned cell = (unsigned)tx.i0 + (unsigned)v.nx * (unsigned)ty.i0;
    const unsigned plane = (unsigned)v.nx * (unsigned)v.ny;
    const unsigned k0 = cell + plane * (unsigned)tz.i0, k1 = cell + plane * (unsigned)tz.i1;
    float c000, c100, c010, c110, c001, c101, c011, c111;
    if (v.dtype == 1) {
      const uchar4* q = static_cast<const uchar4*>(v.voxels);
      const uchar4 a = __ldg(q + k0), b = __ldg(q + k1);
      c000 = a.x; c100 = a.y; c010 = a.z; c110 = a.w;
      c001 = b.x; c101 = b.y; c011 = b.z; c111 = b.w;
    } else {
      const ushort4* q = static_cast<const ushort4*>(v.voxels);
      const ushort4 a = __ldg(q + k0), b = __ldg(q + k1);
      c000 = a.x; c100 = a.y; c010 = a.z; c110 = a.w;
      c001 = b.x; c101 = b.y; c011 = b.z; c111 = b.w;
    }
    const float c00 = fmaf(tx.t, c100 - c000, c000), c10 = fmaf(tx.t, c110 - c010, c010);
    const float c01 = fmaf(tx.t, c101 - c001, c001), c11 = fmaf(tx.t, c111 - c011, c011);
    const float c0 = fmaf(ty.t, c10 - c00, c00), c1 = fmaf(ty.t, c11 - c01, c01);
    return fmaf(tz.t, c1 - c0, c0) * v.norm;
  }
  Tap tx = axis_tap(fmaf(tex_pos.x, v.inv_spacing.x, -0.5f), v.nx);
  Tap ty = axis_tap(fmaf(tex_pos.y, v.inv_spacing.y, -0.5f), v.ny);
  Tap tz = axis_tap(fmaf(tex_pos.z, v.inv_spacing.z, -0.5f), v.nz);
  const long long x0 = voxel_term(v, 0, tx.i0), x1 = voxel_term(v, 0, tx.i1);
  const long long y0 = voxel_term(v, 1, ty.i0), y1 = voxel_term(v, 1, ty.i1);
  const long long z0 = voxel_term(v, 2, tz.i0), z1 = voxel_term(v, 2, tz.i1);
  float c000 = voxel_at(v, x0 + y0 + z0), c100 = voxel_at(v, x1 + y0 + z0);
  float c010 = voxel_at(v, x0 + y1 + z0), c110 = voxel_at(v, x1 + y1 + z0);
  float c001 = voxel_at(v, x0 + y0 + z1), c101 = voxel_at(v, x1 + y0 + z1);
  float c011 = voxel_at(v, x0 + y1 + z1), c111 = voxel_at(v, x1 + y1 + z1);
  float c00 = fmaf(tx.t, c100 - c000, c000), c10 = fmaf(tx.t, c110 - c010, c010);
  float c01 = fmaf(tx.t, c101 - c001, c001), c11 = fmaf(tx.t, c111 - c011, c011);
  float c0 = fmaf(ty.t, c10 - c00, c00), c1 = fmaf(ty.t, c11 - c01, c01);
  return fmaf(tz.t, c1 - c0, c0) * v.norm;
}

// texture(TexTransferFunc, density): 1D GL_LINEAR, clamp-to-edge over n entries.
__device__ __forceinline__ float4 tf_lookup(const float4* tf, int n, float density) {
  Tap t = axis_tap(fmaf(density, float(n), -0.5f), n);
  float4 a = tf[t.i0], b = tf[t.i1];
  return make_float4(fmaf(t.t, b.x - a.x, a.x), fmaf(t.t, b.y - a.y, a.y),
                     fmaf(t.t, b.z - a.z, a.z), fmaf(t.t, b.w - a.w, a.w));
}
__device__ __forceinline__ float tf_alpha(const float4* tf, int n, float density) {
  Tap t = axis_tap(fmaf(density, float(n), -0.5f), n);
  float a = tf[t.i0].w, b = tf[t.i1].w;
  return fmaf(t.t, b - a, a);
}

// ---------------------------------------------------------------- SAT query
// The extinction SAT is stored as exact int64 fixed point (value * 2^F).
// The reference evaluates a box as V1-V2-V3+V4-V5+V6+V7-V8 over eight
// trilinear SAT fetches (ebs_ray_bbox_marching.comp:74-100).  That is the
// tensor product, over the three axes, of the 1-D functional
//   L(S) = [(1-th) S[b0] + th S[b1]] - [(1-tl) S[a0] + tl S[a1]]
// over the taps a0, a1 (low corner, weight tl) and b0, b1 (high corner, th).
// Written as consecutive differences along the tap sequence (a0, a1, b0, b1),
//   L(S) = (1-tl) (S[a1]-S[a0]) + (S[b0]-S[a1]) + th (S[b1]-S[b0]).
// Applying the three integer differences along every axis gives 27 exact
// sub-box sums (a 3x3x3 split of the filtered box into faces, edges, corners
// and core); only those are converted to float and weighted, so the query has
// no cancellation however large the SAT entries are.  Planes are streamed in
// tap order, so one previous plane (9 int64) is live at a time.
struct SatView {
  const long long* sat;  // (nx+2)(ny+2)(nz+2), x fastest
  // The compact copy for frames whose boxes are all small enough: the same
  // prefix sums of round(sigma * 2^F32) modulo 2^32 (F32 chosen so that every
  // sub-box sum of the frame's boxes is below 2^31, which makes their
  // wrapped 32-bit differences exact), stored as x-y "predecessor" quads:
  // cell (x, y) holds S at (x-1, y-1), (x, y-1), (x-1, y), (x, y), each
  // coordinate clamped to the table.  A GL_LINEAR lookup whose taps start at
  // texel a reads the pair (S[clamp(a)], S[clamp(a+1)]) from cell
  // clamp(a + 1): exact for every a, because S is 0 at x = 0 and y = 0 (the
  // zero border) and repeats at the last cell, so clamping the cell equals
  // clamping each tap.  The four taps of a plane are one 16-byte load;
  // nullptr: frames use the int64 table.
  const uint4* sat32;
  float inv_scale32;     // 2^-F32
  int sx, sy, sz;        // SAT dims = volume dims + 2
  unsigned sxy;          // sx * sy (cells of the compact table: < 2^31)
  float inv_scale;       // 2^-F
  float3 inv_spacing;
  float3 min_pos;        // MinSATPosition = spacing*0.5
  float3 max_pos;        // MaxSATPosition = grid + spacing*1.5
};

struct BoxAxis {
  int s[4];    // tap sequence a0, a1, b0, b1
  float w[3];  // weights of the consecutive differences: 1-tl, 1, th
};
__device__ __forceinline__ BoxAxis box_axis(float lo, float hi, int n) {
  Tap l = axis_tap(lo, n), h = axis_tap(hi, n);
  BoxAxis b;
  b.s[0] = l.i0; b.s[1] = l.i1; b.s[2] = h.i0; b.s[3] = h.i1;
  b.w[0] = 1.0f - l.t; b.w[1] = 1.0f; b.w[2] = h.t;
  return b;
}
// The same axis for the compact quad table: s[0] and s[2] are the quad cells
// clamp(floor(u) + 1) holding the low and the high tap pair.
__device__ __forceinline__ BoxAxis box_axis_quad(float lo, float hi, int n) {
  const float fl = floorf(lo), fh = floorf(hi);
  BoxAxis b;
  b.s[0] = min(max(int(fl) + 1, 0), n - 1);
  b.s[2] = min(max(int(fh) + 1, 0), n - 1);
  b.s[1] = b.s[0]; b.s[3] = b.s[2];
  b.w[0] = 1.0f - (lo - fl); b.w[1] = 1.0f; b.w[2] = hi - fh;
  return b;
}

// int64 -> float without the FP64 pipe (where the hardware converts 64-bit
// integers, at the FP64 rate, which is low on this part): |v| as two 32-bit
// halves converted on the FP32 side, recombined by one FMA (at most one
// rounding step more than a direct conversion), then the sign.
__device__ __forceinline__ float ll_to_float(long long v) {
  const unsigned long long s = (unsigned long long)(v >> 63);  // 0 or all ones
  const unsigned long long a = ((unsigned long long)v ^ s) - s;
  const float f = fmaf(__uint2float_rn((unsigned)(a >> 32)), 4294967296.0f, __uint2float_rn((unsigned)a));
  return __uint_as_float(__float_as_uint(f) | ((unsigned)s & 0x80000000u));
}

// Exact box sums: W = long long (the int64 table) or unsigned (the compact
// table, differences wrapping modulo 2^32 and read as signed at the end).
template <class W>
struct D3 { W d[3]; };  // consecutive x-differences of one row
__device__ __forceinline__ D3<long long> row_diffs(const long long* row, const BoxAxis& X) {
  const long long v0 = __ldg(row + X.s[0]), v1 = __ldg(row + X.s[1]);
  const long long v2 = __ldg(row + X.s[2]), v3 = __ldg(row + X.s[3]);
  D3<long long> r;
  r.d[0] = v1 - v0; r.d[1] = v2 - v1; r.d[2] = v3 - v2;
  return r;
}
__device__ __forceinline__ D3<unsigned> x_diffs(unsigned v0, unsigned v1, unsigned v2, unsigned v3) {
  D3<unsigned> r;
  r.d[0] = v1 - v0; r.d[1] = v2 - v1; r.d[2] = v3 - v2;
  return r;
}
template <class W>
struct D9 { D3<W> y[3]; };  // consecutive y-differences of x-differenced rows
// The quad table: the 16 taps of a plane from four 16-byte loads; X.s[0] and
// X.s[2] (Y likewise) are the quad cells of the low and high tap pairs
// (box_axis_quad).
__device__ __forceinline__ D9<unsigned> plane_diffs_quad(const uint4* sat, const SatView& S, int z,
                                                         const BoxAxis& X, const BoxAxis& Y) {
  // 32-bit cell numbers (the compact table has fewer than 2^31 cells)
  const unsigned zo = (unsigned)z * S.sxy;
  const unsigned r0 = zo + (unsigned)Y.s[0] * (unsigned)S.sx, r2 = zo + (unsigned)Y.s[2] * (unsigned)S.sx;
  const uint4 q00 = __ldg(sat + (r0 + (unsigned)X.s[0])), q01 = __ldg(sat + (r0 + (unsigned)X.s[2]));
  const uint4 q10 = __ldg(sat + (r2 + (unsigned)X.s[0])), q11 = __ldg(sat + (r2 + (unsigned)X.s[2]));
  const D3<unsigned> rows[4] = {x_diffs(q00.x, q00.y, q01.x, q01.y), x_diffs(q00.z, q00.w, q01.z, q01.w),
                                x_diffs(q10.x, q10.y, q11.x, q11.y), x_diffs(q10.z, q10.w, q11.z, q11.w)};
  D9<unsigned> r;
#pragma unroll
  for (int b = 0; b < 3; ++b)
#pragma unroll
    for (int a = 0; a < 3; ++a) r.y[b].d[a] = rows[b + 1].d[a] - rows[b].d[a];
  return r;
}
__device__ __forceinline__ D9<long long> plane_diffs(const long long* sat, const SatView& S, int z,
                                                     const BoxAxis& X, const BoxAxis& Y) {
  const long long* plane = sat + (size_t)z * (size_t)S.sx * (size_t)S.sy;
  D9<long long> r;
  D3<long long> prev = row_diffs(plane + (size_t)Y.s[0] * S.sx, X);
#pragma unroll
  for (int b = 0; b < 3; ++b) {
    D3<long long> cur = row_diffs(plane + (size_t)Y.s[b + 1] * S.sx, X);
#pragma unroll
    for (int a = 0; a < 3; ++a) r.y[b].d[a] = cur.d[a] - prev.d[a];
    prev = cur;
  }
  return r;
}
__device__ __forceinline__ float box_to_float(long long v) { return ll_to_float(v); }
__device__ __forceinline__ float box_to_float(unsigned v) { return __int2float_rn((int)v); }
// sum over y-op and x-op of wy * wx * (cur - prev), the z-difference of two planes
template <class W>
__device__ __forceinline__ float weigh9(const D9<W>& cur, const D9<W>& prev, const BoxAxis& X, const BoxAxis& Y) {
  float acc = 0.0f;
#pragma unroll
  for (int b = 0; b < 3; ++b) {
    float row = 0.0f;
#pragma unroll
    for (int a = 0; a < 3; ++a) row = fmaf(X.w[a], box_to_float(cur.y[b].d[a] - prev.y[b].d[a]), row);
    acc = fmaf(Y.w[b], row, acc);
  }
  return acc;
}

// EvaluateSAT3D(p1, p2) on already offset + clamped world positions; COMPACT
// reads the 32-bit table.
template <bool COMPACT>
__device__ __forceinline__ float sat_box(const SatView& S, float3 p1, float3 p2) {
  using W = typename std::conditional<COMPACT, unsigned, long long>::type;
  using T = typename std::conditional<COMPACT, uint4, long long>::type;
  const T* sat;
  if constexpr (COMPACT) sat = S.sat32; else sat = S.sat;
  const float lx = fmaf(p1.x, S.inv_spacing.x, -0.5f), hx = fmaf(p2.x, S.inv_spacing.x, -0.5f);
  const float ly = fmaf(p1.y, S.inv_spacing.y, -0.5f), hy = fmaf(p2.y, S.inv_spacing.y, -0.5f);
  BoxAxis X = COMPACT ? box_axis_quad(lx, hx, S.sx) : box_axis(lx, hx, S.sx);
  BoxAxis Y = COMPACT ? box_axis_quad(ly, hy, S.sy) : box_axis(ly, hy, S.sy);
  BoxAxis Z = box_axis(fmaf(p1.z, S.inv_spacing.z, -0.5f), fmaf(p2.z, S.inv_spacing.z, -0.5f), S.sz);
  auto plane = [&](int z) {
    if constexpr (COMPACT) return plane_diffs_quad(sat, S, z, X, Y);
    else return plane_diffs(sat, S, z, X, Y);
  };
  float acc = 0.0f;
  D9<W> prev = plane(Z.s[0]);
#pragma unroll
  for (int g = 0; g < 3; ++g) {
    D9<W> cur = plane(Z.s[g + 1]);
    acc = fmaf(Z.w[g], weigh9(cur, prev, X, Y), acc);
    prev = cur;
  }
  return acc * (COMPACT ? S.inv_scale32 : S.inv_scale);
}

// A box whose two corners sit at the same fractional texel offset on every
// axis (integer widths w): low corner texel coordinate u, high corner u + w.
// With equal fractions t the reference's 1-D functional
//   (1-t) S[b0] + t S[b1] - (1-t) S[a0] - t S[a1],  b = a + w,
// is (1-t) (S[a+w] - S[a]) + t (S[a+1+w] - S[a+1]), so the eight trilinear
// corner fetches reduce to eight exact integer sums of boxes of width w
// (offset by 0 or 1 cell per axis), weighted by the trilinear weights of t.
// The 64 texels are the same; the integer work is 56 wrapped differences and
// 8 conversions (the general query above: 165 and 27).  Coordinates need no
// clamp: the quad cells are clamped (exact, see SatView::sat32), which equals
// the reference's clamp of the corner positions.  Compact (quad) table only.
__device__ __forceinline__ float sat_box_aligned(const SatView& S, float3 u, int wx, int wy, int wz) {
  const float fx = floorf(u.x), fy = floorf(u.y), fz = floorf(u.z);
  const float tx = u.x - fx, ty = u.y - fy, tz = u.z - fz;
  const int ax = int(fx), ay = int(fy), az = int(fz);
  const unsigned x0 = (unsigned)min(max(ax + 1, 0), S.sx - 1), x1 = (unsigned)min(max(ax + 1 + wx, 0), S.sx - 1);
  const unsigned y0 = (unsigned)min(max(ay + 1, 0), S.sy - 1), y1 = (unsigned)min(max(ay + 1 + wy, 0), S.sy - 1);
  const unsigned sx = (unsigned)S.sx;
  // 32-bit cell numbers (the compact table has fewer than 2^31 cells)
  const unsigned c00 = y0 * sx + x0, c01 = y0 * sx + x1, c10 = y1 * sx + x0, c11 = y1 * sx + x1;
  const uint4* __restrict__ q = S.sat32;
  // rectangle sums of the four (x, y) sub-boxes in plane z: component c of a
  // quad is sub-box (c & 1, c >> 1)
  auto rect = [&](int z) {
    const unsigned zo = (unsigned)min(max(z, 0), S.sz - 1) * S.sxy;
    const uint4 a = __ldg(q + (zo + c00)), b = __ldg(q + (zo + c01));
    const uint4 c = __ldg(q + (zo + c10)), d = __ldg(q + (zo + c11));
    return make_uint4(d.x - c.x - b.x + a.x, d.y - c.y - b.y + a.y, d.z - c.z - b.z + a.z, d.w - c.w - b.w + a.w);
  };
  // z-offset 0 (planes az, az + wz) and 1 (az + 1, az + wz + 1), one pair at a
  // time: eight 16-byte loads in flight instead of sixteen
  uint4 d0 = make_uint4(0u, 0u, 0u, 0u), d1 = d0;
#pragma unroll 1
  for (int o = 0; o < 2; ++o) {
    const uint4 lo = rect(az + o), hi = rect(az + wz + o);
    const uint4 dz = make_uint4(hi.x - lo.x, hi.y - lo.y, hi.z - lo.z, hi.w - lo.w);
    if (o == 0) d0 = dz;
    else d1 = dz;
  }
  // sub-box sums (below 2^31 by the compact table's fixed point): z-offset 0 and 1
  const float b00 = (float)(int)d0.x, b10 = (float)(int)d0.y;
  const float b01 = (float)(int)d0.z, b11 = (float)(int)d0.w;
  const float e00 = (float)(int)d1.x, e10 = (float)(int)d1.y;
  const float e01 = (float)(int)d1.z, e11 = (float)(int)d1.w;
  const float z00 = fmaf(tz, e00 - b00, b00), z10 = fmaf(tz, e10 - b10, b10);
  const float z01 = fmaf(tz, e01 - b01, b01), z11 = fmaf(tz, e11 - b11, b11);
  const float y0v = fmaf(ty, z01 - z00, z00), y1v = fmaf(ty, z11 - z10, z10);
  return fmaf(tx, y1v - y0v, y0v) * S.inv_scale32;
}

// Walk table of a directional light's shadow cone: the compact table's sums
// differenced along the walk axis by the boxes' common depth w (texels),
//   D(p) = S(clamp(p + w e_walk)) - S(p)   (p a clamped table coordinate),
// stored as predecessor octs: cell (x, y, z) holds D at (x-1..x, y-1..y,
// z-1..z), coordinates clamped, component dx + 2 dy + 4 dz (32 bytes).
struct WalkView {
  const uint4* oct;  // two uint4 per cell, or nullptr: no walk table
  int axis;          // the walk axis (0, 1, 2)
  int w;             // box depth along it, texels
};

__device__ __forceinline__ void load_oct(const uint4* p, unsigned (&v)[8]) {
  asm("ld.global.nc.v8.u32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
      : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7])
      : "l"(p));
}

// The equal-fraction query (sat_box_aligned) of a box of the walk, whose
// depth along the walk axis is the table's w: the eight sub-box sums are
// rectangle sums of D over the two lateral axes, four 32-byte loads (the
// walk-axis differences are in the table).  The walk-axis taps of every box
// of the walk lie inside the table (the walk stops where the next box would
// leave the volume), where D of a clamped tap is the clamped difference;
// a box reaching below the table on that axis takes sat_box_aligned.
// walk_fetch issues the four loads (always of clamped, valid cells) and
// walk_sum turns them into the box value.  (Fetching the next box before
// summing this one measured slower: the extra 32 registers cost occupancy.)
struct WalkFetch {
  unsigned q00[8], q10[8], q01[8], q11[8];
};

__device__ __forceinline__ void walk_fetch(const SatView& S, const WalkView& Wk, float3 u, int wx, int wy, int wz,
                                           WalkFetch& F) {
  const int ax = int(floorf(u.x)), ay = int(floorf(u.y)), az = int(floorf(u.z));
  const unsigned sx = (unsigned)S.sx, sxy = S.sxy;
  const unsigned x0 = (unsigned)min(max(ax + 1, 0), S.sx - 1), x1 = (unsigned)min(max(ax + 1 + wx, 0), S.sx - 1);
  const unsigned y0 = (unsigned)min(max(ay + 1, 0), S.sy - 1), y1 = (unsigned)min(max(ay + 1 + wy, 0), S.sy - 1);
  const unsigned z0 = (unsigned)min(max(az + 1, 0), S.sz - 1), z1 = (unsigned)min(max(az + 1 + wz, 0), S.sz - 1);
  // the walk axis contributes its low cell only; the lateral axes a (lower
  // index) and b contribute a low and a high cell each
  unsigned pw, pa0, pa1, pb0, pb1;
  if (Wk.axis == 0) { pw = x0; pa0 = y0 * sx; pa1 = y1 * sx; pb0 = z0 * sxy; pb1 = z1 * sxy; }
  else if (Wk.axis == 1) { pw = y0 * sx; pa0 = x0; pa1 = x1; pb0 = z0 * sxy; pb1 = z1 * sxy; }
  else { pw = z0 * sxy; pa0 = x0; pa1 = x1; pb0 = y0 * sx; pb1 = y1 * sx; }
  // 32-bit cell numbers (the compact table has fewer than 2^31 cells)
  load_oct(Wk.oct + 2u * (pw + pa0 + pb0), F.q00);
  load_oct(Wk.oct + 2u * (pw + pa1 + pb0), F.q10);
  load_oct(Wk.oct + 2u * (pw + pa0 + pb1), F.q01);
  load_oct(Wk.oct + 2u * (pw + pa1 + pb1), F.q11);
}

__device__ __forceinline__ float walk_sum(const SatView& S, const WalkView& Wk, float3 u, int wx, int wy, int wz,
                                          const WalkFetch& F) {
  const float fx = floorf(u.x), fy = floorf(u.y), fz = floorf(u.z);
  const int aw = Wk.axis == 0 ? int(fx) : (Wk.axis == 1 ? int(fy) : int(fz));
  if (aw < 0) return sat_box_aligned(S, u, wx, wy, wz);
  const float tx = u.x - fx, ty = u.y - fy, tz = u.z - fz;
  float b[8];  // sub-box sums (below 2^31 by the compact table's fixed point)
#pragma unroll
  for (int c = 0; c < 8; ++c) b[c] = (float)(int)(F.q11[c] - F.q01[c] - F.q10[c] + F.q00[c]);
  // component c = dx + 2 dy + 4 dz: trilinear weights of the fractions, in
  // sat_box_aligned's order (z, y, x), so both queries give the same bits
  const float z00 = fmaf(tz, b[4] - b[0], b[0]), z10 = fmaf(tz, b[5] - b[1], b[1]);
  const float z01 = fmaf(tz, b[6] - b[2], b[2]), z11 = fmaf(tz, b[7] - b[3], b[3]);
  const float y0v = fmaf(ty, z01 - z00, z00), y1v = fmaf(ty, z11 - z10, z10);
  return fmaf(tx, y1v - y0v, y0v) * S.inv_scale32;
}

__device__ __forceinline__ float sat_box_walk(const SatView& S, const WalkView& Wk, float3 u, int wx, int wy,
                                              int wz) {
  WalkFetch F;
  walk_fetch(S, Wk, u, wx, wy, wz, F);
  return walk_sum(S, Wk, u, wx, wy, wz, F);
}

// ---------------------------------------------------------------- pyramid
// Gaussian extinction pyramid, float32 levels concatenated, x fastest.
#define CVR_MAX_LEVELS 16
struct PyramidView {
  const float* data;
  // x-y quads of every level (cell (x, y, z) = the values at (x, y), (x', y),
  // (x, y'), (x', y') of its level, successors clamped), same offsets; or nullptr
  const float4* quads;
  int n_levels;
  int dims[CVR_MAX_LEVELS][3];
  long long offset[CVR_MAX_LEVELS];
  float3 grid;         // VolumeScaledSizes
  float3 inv_grid;
};

// textureLod(pyr, tex_pos / S, level) at an integer level: trilinear in that
// level.  32-bit element numbers: pyramids hold fewer than 2^31 values.
__device__ __forceinline__ float pyr_sample_level(const PyramidView& P, int l, float3 tex_pos) {
  const int* d = P.dims[l];
  const Tap tz = axis_tap(fmaf(tex_pos.z * P.inv_grid.z, float(d[2]), -0.5f), d[2]);
  const unsigned d0 = (unsigned)d[0], d01 = (unsigned)d[0] * (unsigned)d[1];
  if (P.quads) {
    // Texel coordinates below 0 raised to 0 so the successor taps are the
    // quad's (both taps read the edge value there, as without the raise).
    const Tap qx = axis_tap(fmaxf(fmaf(tex_pos.x * P.inv_grid.x, float(d[0]), -0.5f), 0.0f), d[0]);
    const Tap qy = axis_tap(fmaxf(fmaf(tex_pos.y * P.inv_grid.y, float(d[1]), -0.5f), 0.0f), d[1]);
    const unsigned cell = (unsigned)P.offset[l] + (unsigned)qx.i0 + d0 * (unsigned)qy.i0;
    const float4 a = __ldg(P.quads + (cell + d01 * (unsigned)tz.i0));
    const float4 e = __ldg(P.quads + (cell + d01 * (unsigned)tz.i1));
    const float c00 = fmaf(qx.t, a.y - a.x, a.x), c10 = fmaf(qx.t, a.w - a.z, a.z);
    const float c01 = fmaf(qx.t, e.y - e.x, e.x), c11 = fmaf(qx.t, e.w - e.z, e.z);
    const float c0 = fmaf(qy.t, c10 - c00, c00), c1 = fmaf(qy.t, c11 - c01, c01);
    return fmaf(tz.t, c1 - c0, c0);
  }
  const Tap tx = axis_tap(fmaf(tex_pos.x * P.inv_grid.x, float(d[0]), -0.5f), d[0]);
  const Tap ty = axis_tap(fmaf(tex_pos.y * P.inv_grid.y, float(d[1]), -0.5f), d[1]);
  const unsigned b = (unsigned)P.offset[l] + (unsigned)tx.i0 + d0 * (unsigned)ty.i0 + d01 * (unsigned)tz.i0;
  const unsigned dx = (unsigned)(tx.i1 - tx.i0), dy = (unsigned)(ty.i1 - ty.i0) * d0,
                 dz = (unsigned)(tz.i1 - tz.i0) * d01;
  const float* q = P.data;
  float c000 = __ldg(q + b), c100 = __ldg(q + (b + dx));
  float c010 = __ldg(q + (b + dy)), c110 = __ldg(q + (b + dy + dx));
  float c001 = __ldg(q + (b + dz)), c101 = __ldg(q + (b + dz + dx));
  float c011 = __ldg(q + (b + dz + dy)), c111 = __ldg(q + (b + dz + dy + dx));
  float c00 = fmaf(tx.t, c100 - c000, c000), c10 = fmaf(tx.t, c110 - c010, c010);
  float c01 = fmaf(tx.t, c101 - c001, c001), c11 = fmaf(tx.t, c111 - c011, c011);
  float c0 = fmaf(ty.t, c10 - c00, c00), c1 = fmaf(ty.t, c11 - c01, c01);
  return fmaf(tz.t, c1 - c0, c0);
}
// GL_LINEAR_MIPMAP_LINEAR with an explicit lod: levels clamped to the
// pyramid, fractional lods blend the two neighbouring levels.
__device__ __forceinline__ float pyr_sample(const PyramidView& P, float lod, float3 tex_pos) {
  float maxl = float(P.n_levels - 1);
  lod = fminf(fmaxf(lod, 0.0f), maxl);
  float fl = floorf(lod);
  int l0 = int(fl);
  float t = lod - fl;
  float a = pyr_sample_level(P, l0, tex_pos);
  if (t == 0.0f) return a;
  float b = pyr_sample_level(P, min(l0 + 1, P.n_levels - 1), tex_pos);
  return fmaf(t, b - a, a);
}

}  // namespace cvr
