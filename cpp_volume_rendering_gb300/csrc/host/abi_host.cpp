// abi_host.cpp — the host-only entry points of cvr.h (no GPU needed):
// transfer-function tables, file readers, cone tables, GT kernel vectors and
// the seeded synthetic volumes of the benchmark configurations.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <random>
#include <string>
#include <vector>

#include "../../../include/cvr.h"
#include "cone_sampler.hpp"
#include "tf1d.hpp"
#include "volume.hpp"

namespace {

vis::TransferFunction1D make_tf(int max_density, int n_rgb, const double* rgb, int n_alpha, const double* alpha,
                                int extinction_input) {
  vis::TransferFunction1D tf(max_density);
  tf.SetExtinctionCoefficientInput(extinction_input != 0);
  for (int i = 0; i < n_rgb; ++i)
    tf.AddRGBControlPoint(vis::TransferControlPoint::RGB(rgb[4 * i], rgb[4 * i + 1], rgb[4 * i + 2],
                                                         (int)rgb[4 * i + 3]));
  for (int i = 0; i < n_alpha; ++i)
    tf.AddAlphaControlPoint(vis::TransferControlPoint::Alpha(alpha[2 * i], (int)alpha[2 * i + 1]));
  return tf;
}

bool tf_args_ok(int max_density, int n_rgb, const double* rgb, int n_alpha, const double* alpha) {
  if (max_density < 1 || max_density > (1 << 16)) return false;
  if (n_rgb < 0 || n_alpha < 0 || (n_rgb && !rgb) || (n_alpha && !alpha)) return false;
  return true;
}

// splitmix64: the seeded generator behind every synthetic volume.
struct SplitMix {
  uint64_t s;
  uint64_t next() {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  }
  double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
  double uniform(double a, double b) { return a + (b - a) * uniform(); }
};

uint64_t hash3(uint64_t seed, int64_t x, int64_t y, int64_t z) {
  SplitMix m{seed ^ ((uint64_t)x * 0x8CB92BA72F3D8DD7ull) ^ ((uint64_t)y * 0x9E3779B97F4A7C15ull) ^
             ((uint64_t)z * 0xC2B2AE3D27D4EB4Full)};
  m.next();
  return m.next();
}

void store_voxel(void* out, size_t i, int dtype, double v01) {
  v01 = std::min(1.0, std::max(0.0, v01));
  if (dtype == CVR_U8) static_cast<uint8_t*>(out)[i] = (uint8_t)std::lround(v01 * 255.0);
  else static_cast<uint16_t*>(out)[i] = (uint16_t)std::lround(v01 * 65535.0);
}

}  // namespace

extern "C" {

cvr_status cvr_tf_build_linear(int max_density, int n_rgb, const double* rgb, int n_alpha, const double* alpha,
                               int extinction_input, float* rgbt_out, float* rgba_out) {
  if (!tf_args_ok(max_density, n_rgb, rgb, n_alpha, alpha)) return CVR_ERR_INVALID_ARG;
  vis::TransferFunction1D tf = make_tf(max_density, n_rgb, rgb, n_alpha, alpha, extinction_input);
  if (rgbt_out) {
    std::vector<float> t = tf.TableRGBt();
    std::memcpy(rgbt_out, t.data(), t.size() * sizeof(float));
  }
  if (rgba_out) {
    std::vector<float> t = tf.TableRGBA();
    std::memcpy(rgba_out, t.data(), t.size() * sizeof(float));
  }
  return CVR_OK;
}

// GenerateExtinctionSAT3DTex's per-voxel value: tf->GetExtN(vol->GetNormalizedSample(...))
// (ebsrenderer.cpp:655), tabulated for every possible voxel value.
cvr_status cvr_tf_ext_per_value(int max_density, int n_rgb, const double* rgb, int n_alpha, const double* alpha,
                                int extinction_input, int dtype, double* out) {
  if (!tf_args_ok(max_density, n_rgb, rgb, n_alpha, alpha) || !out) return CVR_ERR_INVALID_ARG;
  if (dtype != CVR_U8 && dtype != CVR_U16) return CVR_ERR_INVALID_ARG;
  vis::TransferFunction1D tf = make_tf(max_density, n_rgb, rgb, n_alpha, alpha, extinction_input);
  int n = dtype == CVR_U8 ? 256 : 65536;
  double denom = dtype == CVR_U8 ? (256.0 - 1.0) : (65536.0 - 1.0);
  for (int v = 0; v < n; ++v) out[v] = (double)tf.GetExtN((double)v / denom);
  return CVR_OK;
}

cvr_status cvr_read_tf1d(const char* path, int* max_density, int* extinction_input, int* n_rgb, double* rgb_points,
                         int max_rgb, int* n_alpha, double* alpha_points, int max_alpha) {
  if (!path) return CVR_ERR_INVALID_ARG;
  // Parse through the TransferFunction1D reader, then re-read the points.
  vis::TransferFunction1D tf;
  std::string err;
  if (!vis::ReadTransferFunction1D(path, &tf, &err)) {
    FILE* f = std::fopen(path, "r");
    if (!f) return CVR_ERR_IO;
    std::fclose(f);
    return CVR_ERR_FORMAT;
  }
  // The reader validated the structure; extract the raw control points.
  std::FILE* f = std::fopen(path, "r");
  if (!f) return CVR_ERR_IO;
  char line[4096];
  if (!std::fgets(line, sizeof line, f)) { std::fclose(f); return CVR_ERR_FORMAT; }
  int init = 0, md = 255, ext = 0;
  if (std::fscanf(f, "%d", &init) != 1) { std::fclose(f); return CVR_ERR_FORMAT; }
  if (init == 2) { if (std::fscanf(f, "%d %d", &md, &ext) != 2) { std::fclose(f); return CVR_ERR_FORMAT; } }
  else if (init == 1) { if (std::fscanf(f, "%d", &md) != 1) { std::fclose(f); return CVR_ERR_FORMAT; } }
  int nr = 0;
  if (std::fscanf(f, "%d", &nr) != 1 || nr > max_rgb) { std::fclose(f); return nr > max_rgb ? CVR_ERR_INVALID_ARG : CVR_ERR_FORMAT; }
  for (int i = 0; i < nr; ++i) {
    double r, g, b; int iso;
    if (std::fscanf(f, "%lf %lf %lf %d", &r, &g, &b, &iso) != 4) { std::fclose(f); return CVR_ERR_FORMAT; }
    rgb_points[4 * i] = r; rgb_points[4 * i + 1] = g; rgb_points[4 * i + 2] = b; rgb_points[4 * i + 3] = iso;
  }
  int na = 0;
  if (std::fscanf(f, "%d", &na) != 1 || na > max_alpha) { std::fclose(f); return na > max_alpha ? CVR_ERR_INVALID_ARG : CVR_ERR_FORMAT; }
  for (int i = 0; i < na; ++i) {
    double a; int iso;
    if (std::fscanf(f, "%lf %d", &a, &iso) != 2) { std::fclose(f); return CVR_ERR_FORMAT; }
    alpha_points[2 * i] = a; alpha_points[2 * i + 1] = iso;
  }
  std::fclose(f);
  if (max_density) *max_density = md;
  if (extinction_input) *extinction_input = (init == 2 && ext == 1) ? 1 : 0;
  if (n_rgb) *n_rgb = nr;
  if (n_alpha) *n_alpha = na;
  return CVR_OK;
}

cvr_status cvr_read_volume_info(const char* path, int dims[3], int* dtype, float spacing[3]) {
  if (!path || !dims || !dtype) return CVR_ERR_INVALID_ARG;
  std::string p(path);
  size_t dot = p.find_last_of('.');
  std::string ext = dot == std::string::npos ? "" : p.substr(dot + 1);
  if (ext == "raw") {
    int w, h, d, b;
    if (!vis::ParseRawName(p, &w, &h, &d, &b)) return CVR_ERR_FORMAT;
    FILE* f = std::fopen(path, "rb");
    if (!f) return CVR_ERR_IO;
    std::fclose(f);
    dims[0] = w; dims[1] = h; dims[2] = d;
    *dtype = b == 2 ? CVR_U16 : CVR_U8;
  } else if (ext == "syn") {
    FILE* f = std::fopen(path, "r");
    if (!f) return CVR_ERR_IO;
    int w, h, d;
    int ok = std::fscanf(f, "%d %d %d", &w, &h, &d);
    std::fclose(f);
    if (ok != 3 || w <= 0 || h <= 0 || d <= 0) return CVR_ERR_FORMAT;
    dims[0] = w; dims[1] = h; dims[2] = d;
    *dtype = CVR_U8;
  } else if (ext == "pvm" || ext == "pvmold" || ext == "nrrd" || ext == "nhrd" || ext == "dat") {
    // the header of a DDS-compressed .pvm sits inside the compressed stream: read it whole
    vis::StructuredGridVolume v;
    std::string err;
    if (!vis::ReadStructuredVolume(p, &v, &err)) {
      FILE* f = std::fopen(path, "rb");
      if (!f) return CVR_ERR_IO;
      std::fclose(f);
      return (err.find("short") != std::string::npos || err.find("opening") != std::string::npos) ? CVR_ERR_IO
                                                                                                     : CVR_ERR_FORMAT;
    }
    dims[0] = v.GetWidth(); dims[1] = v.GetHeight(); dims[2] = v.GetDepth();
    *dtype = v.GetStorage() == vis::DataStorageSize::_16_BITS ? CVR_U16 : CVR_U8;
    if (spacing) {
      spacing[0] = (float)v.GetScaleX(); spacing[1] = (float)v.GetScaleY(); spacing[2] = (float)v.GetScaleZ();
    }
    return CVR_OK;
  } else {
    return CVR_ERR_UNSUPPORTED;
  }
  if (spacing) spacing[0] = spacing[1] = spacing[2] = 1.0f;  // readraw / readsyn SetScale(1,1,1)
  return CVR_OK;
}

cvr_status cvr_read_volume(const char* path, void* host_out, size_t out_bytes) {
  if (!path || !host_out) return CVR_ERR_INVALID_ARG;
  vis::StructuredGridVolume v;
  std::string err;
  if (!vis::ReadStructuredVolume(path, &v, &err)) {
    FILE* f = std::fopen(path, "rb");
    if (!f) return CVR_ERR_IO;
    std::fclose(f);
    return (err.find("short") != std::string::npos || err.find("opening") != std::string::npos) ? CVR_ERR_IO
                                                                                                   : CVR_ERR_FORMAT;
  }
  size_t n = v.GetNumVoxels() * v.GetBytesPerVoxel();
  if (out_bytes < n) return CVR_ERR_INVALID_ARG;
  std::memcpy(host_out, v.GetArrayData(), n);
  return CVR_OK;
}

cvr_status cvr_cone_sampler_build(float cone_half_angle_deg, int max_packing, float covered_distance,
                                  float initial_step, float ui_weight, double min_sigma, cvr_cone_table* out) {
  if (!out || max_packing < 0 || max_packing > 2 || !(min_sigma > 0.0)) return CVR_ERR_INVALID_ARG;
  cvrhost::ConeGaussianSampler s;
  s.SetConeHalfAngle(cone_half_angle_deg);
  s.SetMaxGaussianPacking(max_packing);
  s.SetCoveredDistanceUnclamped(covered_distance);
  s.SetInitialStep(initial_step);
  s.SetUIWeightPercentage(ui_weight);
  if (!s.ComputeConeIntegrationSteps(min_sigma)) return CVR_ERR_INVALID_ARG;
  int n = (int)s.sections.size();
  if (n > CVR_MAX_CONE_SECTIONS) return CVR_ERR_UNSUPPORTED;
  std::memset(out, 0, sizeof(*out));
  out->n_sections = n;
  // GetConeSectionsInfoTex (conegaussiansampler.cpp:179-205): the interval
  // distance of section i comes from the interval list, the rest from the section.
  for (int i = 0; i < n; ++i) {
    out->sections[i][0] = (float)s.intervals[i].s_distance;
    out->sections[i][1] = (float)s.sections[i].mip_map_level;
    out->sections[i][2] = (float)s.sections[i].d_integral;
    out->sections[i][3] = (float)s.sections[i].amplitude;
  }
  out->integration_samples[0] = s.gaussian_samples_1;
  out->integration_samples[1] = s.gaussian_samples_3;
  out->integration_samples[2] = s.gaussian_samples_7;
  for (int i = 0; i < 3; ++i) { out->axes[i][0] = s.ray3_axis[i].x; out->axes[i][1] = s.ray3_axis[i].y; out->axes[i][2] = s.ray3_axis[i].z; }
  for (int i = 0; i < 7; ++i) { out->axes[3 + i][0] = s.ray7_axis[i].x; out->axes[3 + i][1] = s.ray7_axis[i].y; out->axes[3 + i][2] = s.ray7_axis[i].z; }
  out->initial_step = s.initial_step;
  out->ray7_adj_weight = (float)s.ray7_adj_weight;
  out->ui_weight = s.ui_weight;
  return CVR_OK;
}

// crtgtrenderer.cpp:131-187: theta = U*aperture, phi = U*360 deg, rotate (0,0,1)
// about y by theta and then about z by phi; all in single precision.
cvr_status cvr_gt_kernel_vectors(int n_occ, float occ_aperture_deg, int n_sdw, float sdw_aperture_deg,
                                 unsigned int seed, float* occ_xyz, float* sdw_xyz) {
  if (n_occ < 0 || n_sdw < 0 || (n_occ && !occ_xyz) || (n_sdw && !sdw_xyz)) return CVR_ERR_INVALID_ARG;
  std::default_random_engine gen(seed);
  std::uniform_real_distribution<float> dist(0.0, 1.0);
  const float pi = 3.14159265358979323846f;
  const cvrhost::Vec3f gtray{0, 0, 1}, yax{0, 1, 0};
  for (int i = 0; i < n_occ; ++i) {
    float theta = dist(gen) * (pi * (occ_aperture_deg / 180.f));
    float phi = dist(gen) * (pi * (360.f / 180.f));
    cvrhost::Vec3f v = cvrhost::RodriguesRotation(gtray, theta, yax);
    v = cvrhost::RodriguesRotation(v, phi, gtray);
    occ_xyz[3 * i] = v.x; occ_xyz[3 * i + 1] = v.y; occ_xyz[3 * i + 2] = v.z;
  }
  for (int i = 0; i < n_sdw; ++i) {
    float theta = dist(gen) * (pi * (sdw_aperture_deg / 180.f));
    float phi = dist(gen) * (pi * (360.f / 180.f));
    cvrhost::Vec3f v = cvrhost::RodriguesRotation(gtray, theta, yax);
    v = cvrhost::RodriguesRotation(v, phi, gtray);
    sdw_xyz[3 * i] = v.x; sdw_xyz[3 * i + 1] = v.y; sdw_xyz[3 * i + 2] = v.z;
  }
  return CVR_OK;
}

// Sum of n isotropic Gaussian blobs in the unit cube (centres U[0.2,0.8]^3,
// sigma U[0.05,0.15], amplitude U[0.5,1]) evaluated at voxel centres, clamped
// to [0,1], plus optional uniform background noise of up to noise_max (in
// units of the u8 range, i.e. noise_max/255 of full scale).
cvr_status cvr_synth_blobs(void* out, int w, int h, int d, int dtype, int n_blobs, uint64_t seed, float noise_max) {
  if (!out || w <= 0 || h <= 0 || d <= 0 || n_blobs < 0 || (dtype != CVR_U8 && dtype != CVR_U16))
    return CVR_ERR_INVALID_ARG;
  SplitMix rng{seed};
  std::vector<double> cx(n_blobs), cy(n_blobs), cz(n_blobs), inv2s2(n_blobs), amp(n_blobs);
  for (int b = 0; b < n_blobs; ++b) {
    cx[b] = rng.uniform(0.2, 0.8); cy[b] = rng.uniform(0.2, 0.8); cz[b] = rng.uniform(0.2, 0.8);
    double s = rng.uniform(0.05, 0.15);
    inv2s2[b] = 1.0 / (2.0 * s * s);
    amp[b] = rng.uniform(0.5, 1.0);
  }
  const uint64_t nseed = seed ^ 0x6A09E667F3BCC909ull;
#pragma omp parallel for schedule(static)
  for (int z = 0; z < d; ++z) {
    for (int y = 0; y < h; ++y) {
      for (int x = 0; x < w; ++x) {
        double px = (x + 0.5) / w, py = (y + 0.5) / h, pz = (z + 0.5) / d;
        double v = 0.0;
        for (int b = 0; b < n_blobs; ++b) {
          double dx = px - cx[b], dy = py - cy[b], dz = pz - cz[b];
          v += amp[b] * std::exp(-(dx * dx + dy * dy + dz * dz) * inv2s2[b]);
        }
        v = std::min(1.0, std::max(0.0, v));
        if (noise_max > 0.0f) {
          double u = (double)(hash3(nseed, x, y, z) >> 11) * (1.0 / 9007199254740992.0);
          v = std::min(1.0, v + u * (double)noise_max / 255.0);
        }
        store_voxel(out, (size_t)x + (size_t)w * ((size_t)y + (size_t)h * z), dtype, v);
      }
    }
  }
  return CVR_OK;
}

// Fractal value noise (lattice values from a hash, smoothstep-weighted
// trilinear interpolation, base frequency 4 cells per side, 'octaves' octaves
// of lacunarity / gain), normalised to [0,1] and, when shells > 0, quantised
// into 'shells' nested level sets: value = (#thresholds k/(shells+1) below the
// noise) / shells.
cvr_status cvr_synth_value_noise(void* out, int w, int h, int d, int dtype, int octaves, float lacunarity, float gain,
                                 int shells, uint64_t seed) {
  if (!out || w <= 0 || h <= 0 || d <= 0 || octaves < 1 || octaves > 12 || shells < 0 ||
      (dtype != CVR_U8 && dtype != CVR_U16))
    return CVR_ERR_INVALID_ARG;
  double norm = 0.0, amp = 1.0;
  for (int o = 0; o < octaves; ++o) { norm += amp; amp *= gain; }
  const int side = std::max(w, std::max(h, d));
#pragma omp parallel for schedule(static)
  for (int z = 0; z < d; ++z) {
    for (int y = 0; y < h; ++y) {
      for (int x = 0; x < w; ++x) {
        double v = 0.0, a = 1.0, freq = 4.0;
        for (int o = 0; o < octaves; ++o) {
          double px = (x + 0.5) / side * freq, py = (y + 0.5) / side * freq, pz = (z + 0.5) / side * freq;
          int64_t ix = (int64_t)std::floor(px), iy = (int64_t)std::floor(py), iz = (int64_t)std::floor(pz);
          double fx = px - ix, fy = py - iy, fz = pz - iz;
          fx = fx * fx * (3 - 2 * fx); fy = fy * fy * (3 - 2 * fy); fz = fz * fz * (3 - 2 * fz);
          uint64_t os = seed + 0x9E3779B97F4A7C15ull * (uint64_t)(o + 1);
          double c[8];
          for (int k = 0; k < 8; ++k)
            c[k] = (double)(hash3(os, ix + (k & 1), iy + ((k >> 1) & 1), iz + (k >> 2)) >> 11) *
                   (1.0 / 9007199254740992.0);
          double x0 = c[0] + fx * (c[1] - c[0]), x1 = c[2] + fx * (c[3] - c[2]);
          double x2 = c[4] + fx * (c[5] - c[4]), x3 = c[6] + fx * (c[7] - c[6]);
          double y0 = x0 + fy * (x1 - x0), y1 = x2 + fy * (x3 - x2);
          v += a * (y0 + fz * (y1 - y0));
          a *= gain;
          freq *= lacunarity;
        }
        v /= norm;
        if (shells > 0) {
          int k = 0;
          for (int s = 1; s <= shells; ++s)
            if (v > (double)s / (shells + 1)) ++k;
          v = (double)k / shells;
        }
        store_voxel(out, (size_t)x + (size_t)w * ((size_t)y + (size_t)h * z), dtype, v);
      }
    }
  }
  return CVR_OK;
}

}  // extern "C"
