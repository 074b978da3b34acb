// build_tables.cuh — launchers of the SAT / pyramid builders and utilities.
#pragma once

#include "cvr_device.cuh"

namespace cvr {

// Builds the (nx+2)(ny+2)(nz+2) int64 SAT of lut[voxel] with a zero border.
cudaError_t launch_sat_build(const void* vox, int dtype, int nx, int ny, int nz, const long long* lut,
                             long long* sat, cudaStream_t st);
// The compact table: the same prefix sums of a 32-bit lut, wrapping modulo
// 2^32, in the x-y predecessor-quad layout (SatView::sat32) in out;
// scratch holds (nx+2)(ny+2)(nz+2) 32-bit values (the plane prefixes).
cudaError_t launch_sat_build_quads(const void* vox, int dtype, int nx, int ny, int nz, const unsigned* lut,
                                   unsigned* scratch, uint4* out, cudaStream_t st);
// The walk table of a directional shadow cone (WalkView: 32 bytes per cell)
// along axis, box depth w, from the compact predecessor-quad table.
cudaError_t launch_sat_walk(const uint4* quads, uint4* out, int sx, int sy, int sz, int axis, int w,
                            cudaStream_t st);
// The x-y predecessor-quad layout of a finished plain (sx, sy, sz) table.
cudaError_t launch_sat_quads(const unsigned* sat, uint4* out, int sx, int sy, int sz, cudaStream_t st);

// Builds every level of P (dims/offsets/grid filled by the caller) into data;
// levels with a separable form use scratch (scratch_floats floats; see
// pyramid_scratch_floats), the others the direct 343-tap kernels.
cudaError_t launch_pyramid_build(const VolumeView& vol, const float4* tf_rgba, int tf_n, float s0,
                                 PyramidView& P, float* data, float* scratch, long long scratch_floats,
                                 cudaStream_t st);
// Floats of scratch the separable levels of P need (0: none is separable).
long long pyramid_scratch_floats(const VolumeView& vol, const PyramidView& P, float s0);

// Grid-stride fill of a device buffer (used to flush L2 between timed frames).
cudaError_t launch_fill(void* p, size_t bytes, unsigned int v, cudaStream_t st);
// The x-y quad copy of every pyramid level (float4 per value, same offsets).
cudaError_t launch_pyramid_quads(const PyramidView& P, const float* data, float4* dst, cudaStream_t st);
// The x-y quad copy of a plain volume (uchar4 / ushort4 per voxel).
cudaError_t launch_quad_volume(const void* src, void* dst, int dtype, int nx, int ny, int nz, cudaStream_t st);
// Bricked copy of a plain volume (bricks of 2^bs voxels per edge); the copy
// holds brick_elements(...) elements.
long long brick_elements(int nx, int ny, int nz, int bs);
cudaError_t launch_brick_volume(const void* src, void* dst, int dtype, int nx, int ny, int nz, int bs,
                                cudaStream_t st);

}  // namespace cvr
