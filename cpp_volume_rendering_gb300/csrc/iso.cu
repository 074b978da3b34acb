// iso.cu — the adaptive-step isosurface ray caster (RayCasting1PassIsoAdapt,
// cppvolrend/structured/rc1pisoadapt/ray_marching_1p_iso_adapt.comp:84-172).
#include "shade.cuh"

namespace cvr {

// main() of ray_marching_1p_iso_adapt.comp: the density at the entry point,
// then steps of StepSizeSmall where |previous density - Isovalue| <
// StepSizeRange (else StepSizeLarge), each sample at the end of its interval;
// a crossing (prev <= iso < d or prev >= iso > d) is placed at the linear
// root inside the interval, shaded with the constant colour (ShadeBlinnPhong
// when gradient shading is on) and composited front to back until alpha > 0.99.
template <int NT>
__global__ void __launch_bounds__(NT) k_march_iso(FrameArgs f, IsoArgs a) {
  int px, py;
  pixel_of(f, px, py);
  const bool inside = px < f.W && py < f.H;
  unsigned n = 0, hits = 0;
  if (inside) {
    const float3 dir = primary_dir(f.cam, px, py, f.W, f.H);
    float4 dst = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    float tnear, tfar;
    if (ray_aabb(f.cam.eye, dir, f.vol.grid, tnear, tfar)) {
      const float D = fabsf(tfar - tnear);
      const float3 tex0 = f.cam.eye + dir * tnear + f.vol.grid * 0.5f;
      float prev = sample_volume(f.vol, tex0);
      // bound on the step count (never reached for validated step sizes)
      const unsigned max_iter = (unsigned)fminf(D / a.step_small, 1.0e9f) + 4u;
      for (float s = 0.0f; s < D && n < max_iter;) {
        const float step = fabsf(prev - a.iso) < a.step_range ? a.step_small : a.step_large;
        const float h = fminf(step, D - s);
        const float d = sample_volume(f.vol, tex0 + dir * (s + h));
        ++n;
        if ((prev <= a.iso && a.iso < d) || (prev >= a.iso && a.iso > d)) {
          ++hits;
          const float t = (a.iso - prev) / (d - prev);
          const float3 p = tex0 + dir * (s + t * h);
          float4 src = a.color;
          if (f.grad.g) src = phong_plain(f, src, p);
          src.x *= src.w; src.y *= src.w; src.z *= src.w;
          const float r = 1.0f - dst.w;
          dst.x += r * src.x; dst.y += r * src.y; dst.z += r * src.z; dst.w += r * src.w;
          if (dst.w > 0.99f) break;
        }
        prev = d;
        s = s + h;
      }
    }
    const size_t o = (size_t)py * f.W + px;
    f.out[o] = dst;
    if (f.counts) f.counts[o] = n;
  }
  add_stats(f, n, hits, 0u);
}

cudaError_t launch_iso(const FrameArgs& f, const IsoArgs& a, cudaStream_t st) {
  const dim3 grid((f.W + f.tile_w - 1) / f.tile_w, (f.H + f.tile_h - 1) / f.tile_h, 1);
  switch ((f.tile_w / 8) * (f.tile_h / 4) * 32) {
    case 64: k_march_iso<64><<<grid, 64, 0, st>>>(f, a); break;
    case 256: k_march_iso<256><<<grid, 256, 0, st>>>(f, a); break;
    default: k_march_iso<128><<<grid, 128, 0, st>>>(f, a); break;
  }
  return cudaGetLastError();
}

}  // namespace cvr
