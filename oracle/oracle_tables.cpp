// oracle_tables.cpp — TEST INFRASTRUCTURE ONLY.
//
// The oracle's own restatement of every host-side table and input the
// renderers consume, so that the oracle (and the CPU reference arm of the
// benchmark) never loads the product library:
//   * the 1D transfer function (TransferFunction1D::BuildLinear / Get /
//     GetExtN / GenerateTexture_1D_RGBt / _RGBA),
//   * the cone-section tables (ConeGaussianSampler),
//   * the ground-truth kernel vectors (RC1PConeLightGroundTruthSteps),
//   * the seeded synthetic volumes of the workloads (this project's own
//     generators: no reference counterpart; the same SplitMix64 stream and
//     lattice hash as the product's generator, checked equal to it on CPU).
// The reference-derived tables are pinned bit for bit against the golden
// vectors that the reference's own C++ produced (tests/test_tables.py).
// Only tests/, the smoke check and the benchmark's CPU legs use this file.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <random>
#include <vector>

#include "../include/cvr.h"

namespace {

// ------------------------------------------------------------ transfer function
// libs/volvis_utils/transferfunction.cpp:8-24: control points store glm::vec4
// colours (single precision) and an integer isovalue.
struct ColourPoint {
  float c[4];
  int iso;
};

// TransferFunction1D::BuildLinear (libs/volvis_utils/transferfunction1d.cpp:319-358):
// a dvec4 per density; colour differences are single-precision vec4
// differences widened to double, k = (x - i0) / (i1 - i0) in double.
// Densities outside [0, max_density] are skipped (the reference writes past
// its table there).
std::vector<double> build_linear(int md, int n_rgb, const double* rgb, int n_alpha, const double* alpha) {
  std::vector<double> t((size_t)(md + 1) * 4, 0.0);
  std::vector<ColourPoint> cr(n_rgb), ca(n_alpha);
  for (int i = 0; i < n_rgb; ++i)
    cr[i] = ColourPoint{{(float)rgb[4 * i], (float)rgb[4 * i + 1], (float)rgb[4 * i + 2], 1.0f}, (int)rgb[4 * i + 3]};
  for (int i = 0; i < n_alpha; ++i) ca[i] = ColourPoint{{0.0f, 0.0f, 0.0f, (float)alpha[2 * i]}, (int)alpha[2 * i + 1]};
  for (int i = 0; i + 1 < n_rgb; ++i) {
    const int i0 = cr[i].iso, i1 = cr[i + 1].iso;
    double diff[3];
    for (int c = 0; c < 3; ++c) diff[c] = (double)(cr[i + 1].c[c] - cr[i].c[c]);
    for (int x = i0; x <= i1; ++x) {
      if (x < 0 || x > md) continue;
      const double k = (double)(x - i0) / (double)(i1 - i0);
      for (int c = 0; c < 3; ++c) t[(size_t)x * 4 + c] = (double)cr[i].c[c] + diff[c] * k;
    }
  }
  for (int i = 0; i + 1 < n_alpha; ++i) {
    const int i0 = ca[i].iso, i1 = ca[i + 1].iso;
    const double diff = (double)(ca[i + 1].c[3] - ca[i].c[3]);
    for (int x = i0; x <= i1; ++x) {
      if (x < 0 || x > md) continue;
      const double k = (double)(x - i0) / (double)(i1 - i0);
      t[(size_t)x * 4 + 3] = (double)ca[i].c[3] + diff * k;
    }
  }
  return t;
}

// libs/volvis_utils/transferfunction.h:74-82: the argument is single
// precision; glm::exp of it is a single-precision exp, glm::log gets a double.
double opacity_to_extinction(float opacity) { return std::log(1.0 / (1.0 - (double)opacity)); }
double extinction_to_opacity(float extinction) { return 1.0 - (double)std::exp(-extinction); }

// TransferFunction1D::Get(value, 1.0).a (transferfunction1d.cpp:132-157):
// zero outside [0, max_density], the last entry within 1e-6 of max_density,
// else the double lerp of the two neighbouring entries, rounded to float.
float tf_get_alpha(const std::vector<double>& t, int md, double value) {
  value = value * (double(md) / 1.0);
  if (value < 0.0f || value > (float)md) return 0.0f;
  if (std::fabs(value - (float)md) < 0.000001) return (float)t[(size_t)md * 4 + 3];
  const int i = (int)value;
  const double u = value - i;
  return (float)((1.0 - u) * t[(size_t)i * 4 + 3] + u * t[(size_t)(i + 1) * 4 + 3]);
}

bool tf_args_ok(int md, int n_rgb, const double* rgb, int n_alpha, const double* alpha) {
  return md >= 1 && md <= (1 << 20) && n_rgb >= 0 && n_alpha >= 0 && (n_rgb == 0 || rgb) && (n_alpha == 0 || alpha);
}

// ------------------------------------------------------------ Rodrigues rotation
// libs/math_utils/utils.cpp:149-156, single-precision glm: v cos + (k x v) sin
// + k (k.v)(1 - cos), then glm::normalize (v * (1 / sqrt(v.v))).
struct V3 {
  float x, y, z;
};
V3 rodrigues(V3 v, float th, V3 k) {
  const float c = std::cos(th), s = std::sin(th);
  const V3 kv{k.y * v.z - k.z * v.y, k.z * v.x - k.x * v.z, k.x * v.y - k.y * v.x};
  const float kd = k.x * v.x + k.y * v.y + k.z * v.z;
  const float omc = 1.0f - c;
  const V3 a{v.x * c, v.y * c, v.z * c};
  const V3 b{kv.x * s, kv.y * s, kv.z * s};
  const V3 r{a.x + b.x + k.x * kd * omc, a.y + b.y + k.y * kd * omc, a.z + b.z + k.z * kd * omc};
  const float inv = 1.0f / std::sqrt(r.x * r.x + r.y * r.y + r.z * r.z);
  return V3{r.x * inv, r.y * inv, r.z * inv};
}

// ------------------------------------------------------------ cone sections
// ConeGaussianSampler (cppvolrend/structured/rc1pdosct/conegaussiansampler.cpp).
// Its members are single precision; the section arithmetic runs in double.
struct Cone {
  float half_angle = 30.0f, initial_step = 3.0f, covered = 100.0f, d_sigma = 1.25f, r_sigma = 2.0f, ui = 1.0f;
  int packing = 2;  // CONEPACKING _1 = 0, _3 = 1, _7 = 2
  struct Sec {
    int n;
    double pos, radius, sigma, d_integral = 0, amplitude = 0, level = 0;
  };
  std::vector<Sec> secs;
  std::vector<double> ipos, idist;  // IntervalsInfo (s_position, s_distance)
  V3 r3[3], r7[7];
  double w7 = 0;

  // conegaussiansampler.h:18-19
  static double div3() { return 1.0 + (2.0 / std::sqrt(3.0)); }
  static double div7() { return 3.010000; }

  // AddGaussianSampleStep / With3 / With7 (conegaussiansampler.cpp:418-498):
  // the first section size (1, 3 or 7 rays) whose radius pos*tan(angle/div)
  // stays within r_sigma * sigma, never going back to fewer rays.
  bool add(double pos, double sg, int* n) {
    const double pi = 3.14159265358979323846;
    if (*n <= 1) {
      *n = 1;
      const double cr = pos * std::tan(half_angle * pi / 180.0);
      if (!(cr > r_sigma * sg)) { secs.push_back(Sec{1, pos, cr, sg}); return true; }
      if (packing <= 0) return false;
    }
    if (*n <= 3) {
      *n = 3;
      const double cr = pos * std::tan((half_angle / div3()) * pi / 180.0);
      if (!(cr > r_sigma * sg)) { secs.push_back(Sec{3, pos, cr, sg}); return true; }
      if (packing <= 1) return false;
    }
    *n = 7;
    const double cr = pos * std::tan((half_angle / div7()) * pi / 180.0);
    if (cr > r_sigma * sg) return false;
    secs.push_back(Sec{7, pos, cr, sg});
    return true;
  }

  // GaussianEval + IntegrateGaussian (conegaussiansampler.cpp:388-414): the
  // midpoint rule over [-r, r] with segments of about 0.05.
  static double gauss(double x, double sig) {
    const double pi = 3.14159265358979323846;
    return (1.0 / (std::sqrt(2.0 * pi) * sig)) * std::exp(-(x * x) / (2.0 * sig * sig));
  }
  static double integrate(double sdev, double r) {
    const double t = (2.0 * r) / 0.05;
    const int nt = (int)std::ceil(t);
    const double seg = (2.0 * r) / double(nt);
    const double s0 = -r + seg * 0.5;
    double S = 0.0;
    for (int i = 0; i < nt; ++i) S += gauss(s0 + seg * double(i), sdev) * seg;
    return S;
  }

  // ComputeConeIntegrationSteps + ComputeAdditionalInfo (conegaussiansampler.cpp:224-386).
  bool build(double min_sg) {
    const double pi = 3.14159265358979323846;
    const V3 zax{0, 0, 1}, yax{0, 1, 0};
    {
      const double adj = half_angle / div3();
      const double t1 = (half_angle - adj) * pi / 180.0;
      r3[0] = rodrigues(zax, (float)t1, yax);
      r3[0] = rodrigues(r3[0], (float)(30.0 * pi / 180.0), zax);
      const double at = 120.0 * pi / 180.0;
      r3[1] = rodrigues(r3[0], (float)at, zax);
      r3[2] = rodrigues(r3[1], (float)at, zax);
    }
    {
      r7[0] = zax;
      const double adj = half_angle / div7();
      const double t1 = (half_angle - adj) * pi / 180.0;
      r7[1] = rodrigues(r7[0], (float)t1, yax);
      const double at = 60.0 * pi / 180.0;
      for (int i = 2; i < 7; ++i) r7[i] = rodrigues(r7[i - 1], (float)at, zax);
    }
    int n = 1;
    double pos = initial_step, sg = min_sg;
    for (int g = 0; !add(pos, sg, &n); ++g) {
      if (g > 256) return false;
      sg *= 2.0;
    }
    while (pos < covered) {
      double si = d_sigma * sg;
      for (int g = 0; !add(pos + si + (d_sigma * sg), sg, &n); ++g) {
        if (g > 256) return false;
        sg *= 2.0;
      }
      si += d_sigma * sg;
      ipos.push_back(pos);
      idist.push_back(si);
      pos += si;
      if (secs.size() > 100000) return false;
    }
    if (secs.empty() || ipos.empty() || secs.size() != ipos.size() + 1) return false;
    w7 = (double)(0.0f * r7[1].x + 0.0f * r7[1].y + 1.0f * r7[1].z);
    ipos.push_back(ipos.back() + idist.back());
    idist.push_back(0.0);
    for (size_t i = 0; i < secs.size(); ++i) {
      Sec& s = secs[i];
      s.d_integral = i == 0 ? s.sigma * std::sqrt(2.0 * pi) * 0.5 : idist[i - 1] * 0.5;
      const double pr = integrate(s.sigma, s.radius);
      const double ac = pi * s.radius * s.radius;
      const double ig = s.sigma * std::sqrt(2.0 * pi);
      s.amplitude = ((pr * pr) * (ig * ig)) / ac;
      s.level = std::log2(s.sigma / min_sg);
    }
    return true;
  }
};

// ------------------------------------------------------------ synthetic inputs
// This project's seeded generators (no reference counterpart): SplitMix64
// (Steele, Lea & Flood 2014) and a lattice hash built on it.
struct SplitMix64 {
  uint64_t s;
  uint64_t next() {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  }
  double unit() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
  double range(double a, double b) { return a + (b - a) * unit(); }
};
uint64_t lattice(uint64_t seed, int64_t x, int64_t y, int64_t z) {
  SplitMix64 m{seed ^ ((uint64_t)x * 0x8CB92BA72F3D8DD7ull) ^ ((uint64_t)y * 0x9E3779B97F4A7C15ull) ^
               ((uint64_t)z * 0xC2B2AE3D27D4EB4Full)};
  m.next();
  return m.next();
}
double lattice_unit(uint64_t seed, int64_t x, int64_t y, int64_t z) {
  return (double)(lattice(seed, x, y, z) >> 11) * (1.0 / 9007199254740992.0);
}
void put(void* out, size_t i, int dtype, double v) {
  v = std::min(1.0, std::max(0.0, v));
  if (dtype == CVR_U8) static_cast<uint8_t*>(out)[i] = (uint8_t)std::lround(v * 255.0);
  else static_cast<uint16_t*>(out)[i] = (uint16_t)std::lround(v * 65535.0);
}

}  // namespace

extern "C" {

int oracle_tf_tables(int md, int n_rgb, const double* rgb, int n_alpha, const double* alpha, int ext_input,
                     float* rgbt, float* rgba) {
  if (!tf_args_ok(md, n_rgb, rgb, n_alpha, alpha)) return -1;
  const std::vector<double> t = build_linear(md, n_rgb, rgb, n_alpha, alpha);
  for (int i = 0; i <= md; ++i) {
    for (int c = 0; c < 3; ++c) {
      if (rgbt) rgbt[4 * i + c] = (float)t[(size_t)i * 4 + c];
      if (rgba) rgba[4 * i + c] = (float)t[(size_t)i * 4 + c];
    }
    const float a = (float)t[(size_t)i * 4 + 3];
    // GenerateTexture_1D_RGBt (transferfunction1d.cpp:89-118): alpha -> extinction
    if (rgbt) rgbt[4 * i + 3] = ext_input ? a : (float)opacity_to_extinction(a);
    // GenerateTexture_1D_RGBA (transferfunction1d.cpp:58-87): extinction -> alpha
    if (rgba) rgba[4 * i + 3] = ext_input ? (float)extinction_to_opacity(a) : a;
  }
  return 0;
}

// GenerateExtinctionSAT3DTex's per-voxel extinction tf->GetExtN(v / max)
// (ebsrenderer.cpp:655, transferfunction1d.cpp:189-197), one per voxel value.
int oracle_tf_ext_per_value(int md, int n_rgb, const double* rgb, int n_alpha, const double* alpha, int ext_input,
                            int dtype, double* out) {
  if (!tf_args_ok(md, n_rgb, rgb, n_alpha, alpha) || !out || (dtype != CVR_U8 && dtype != CVR_U16)) return -1;
  const std::vector<double> t = build_linear(md, n_rgb, rgb, n_alpha, alpha);
  const int n = dtype == CVR_U8 ? 256 : 65536;
  const double mx = dtype == CVR_U8 ? 255.0 : 65535.0;  // StructuredGridVolume::GetNormalizedSample
  for (int v = 0; v < n; ++v) {
    const float a = tf_get_alpha(t, md, (double)v / mx);
    out[v] = ext_input ? (double)a : (double)(float)opacity_to_extinction(a);
  }
  return 0;
}

// The renderer's cone table (GetConeSectionsInfoTex, conegaussiansampler.cpp:179-205,
// plus the axes and weights BindConeOcclusionUniforms passes, dosrcrenderer.cpp:823-990).
int oracle_cone_table(float half_angle, int packing, float covered, float initial_step, float ui_weight,
                      double min_sigma, cvr_cone_table* out) {
  if (!out || packing < 0 || packing > 2 || !(min_sigma > 0.0)) return -1;
  Cone c;
  c.half_angle = std::min(89.5f, std::max(0.5f, half_angle));  // SetConeHalfAngle
  c.packing = packing;
  c.covered = covered > 10.0f ? covered : 10.0f;                 // SetCoveredDistance
  c.initial_step = initial_step > 0.0f ? initial_step : 0.0f;    // SetInitialStep
  c.ui = ui_weight;
  if (!c.build(min_sigma)) return -1;
  const int n = (int)c.secs.size();
  if (n > CVR_MAX_CONE_SECTIONS) return -2;
  std::memset(out, 0, sizeof(*out));
  out->n_sections = n;
  for (int i = 0; i < n; ++i) {
    out->sections[i][0] = (float)c.idist[i];
    out->sections[i][1] = (float)c.secs[i].level;
    out->sections[i][2] = (float)c.secs[i].d_integral;
    out->sections[i][3] = (float)c.secs[i].amplitude;
    out->integration_samples[c.secs[i].n == 1 ? 0 : (c.secs[i].n == 3 ? 1 : 2)] += 1;
  }
  for (int i = 0; i < 3; ++i) { out->axes[i][0] = c.r3[i].x; out->axes[i][1] = c.r3[i].y; out->axes[i][2] = c.r3[i].z; }
  for (int i = 0; i < 7; ++i) {
    out->axes[3 + i][0] = c.r7[i].x; out->axes[3 + i][1] = c.r7[i].y; out->axes[3 + i][2] = c.r7[i].z;
  }
  out->initial_step = c.initial_step;
  out->ray7_adj_weight = (float)c.w7;
  out->ui_weight = c.ui;
  return 0;
}

// RC1PConeLightGroundTruthSteps' kernel vectors (crtgtrenderer.cpp:131-187):
// theta = U * aperture, phi = U * 360 deg from std::default_random_engine and
// uniform_real_distribution<float>, (0,0,1) rotated about y by theta, then
// about z by phi.  seed 1 is the reference's default-constructed engine.
int oracle_gt_vectors(int n_occ, float occ_aperture, int n_sdw, float sdw_aperture, unsigned seed, float* occ,
                      float* sdw) {
  if (n_occ < 0 || n_sdw < 0 || (n_occ && !occ) || (n_sdw && !sdw)) return -1;
  std::default_random_engine gen(seed);
  std::uniform_real_distribution<float> u(0.0, 1.0);
  const float pi = 3.14159265358979323846f;
  const V3 z{0, 0, 1}, y{0, 1, 0};
  auto one = [&](float aperture, float* dst) {
    const float th = u(gen) * (pi * (aperture / 180.f));
    const float ph = u(gen) * (pi * (360.f / 180.f));
    const V3 v = rodrigues(rodrigues(z, th, y), ph, z);
    dst[0] = v.x; dst[1] = v.y; dst[2] = v.z;
  };
  for (int i = 0; i < n_occ; ++i) one(occ_aperture, occ + 3 * i);
  for (int i = 0; i < n_sdw; ++i) one(sdw_aperture, sdw + 3 * i);
  return 0;
}

// n isotropic Gaussian blobs in the unit cube (centres U[0.2,0.8]^3, sigma
// U[0.05,0.15], amplitude U[0.5,1]) at voxel centres, clamped to [0,1], plus
// U[0, noise_max/255] background noise from the lattice hash.
int oracle_synth_blobs(void* out, int w, int h, int d, int dtype, int n_blobs, uint64_t seed, float noise_max) {
  if (!out || w <= 0 || h <= 0 || d <= 0 || n_blobs < 0 || (dtype != CVR_U8 && dtype != CVR_U16)) return -1;
  SplitMix64 rng{seed};
  std::vector<double> b((size_t)n_blobs * 5);
  for (int i = 0; i < n_blobs; ++i) {
    b[5 * i] = rng.range(0.2, 0.8);
    b[5 * i + 1] = rng.range(0.2, 0.8);
    b[5 * i + 2] = rng.range(0.2, 0.8);
    const double s = rng.range(0.05, 0.15);
    b[5 * i + 3] = 1.0 / (2.0 * s * s);
    b[5 * i + 4] = rng.range(0.5, 1.0);
  }
  const uint64_t nseed = seed ^ 0x6A09E667F3BCC909ull;
#pragma omp parallel for schedule(static)
  for (int z = 0; z < d; ++z)
    for (int y = 0; y < h; ++y)
      for (int x = 0; x < w; ++x) {
        const double px = (x + 0.5) / w, py = (y + 0.5) / h, pz = (z + 0.5) / d;
        double v = 0.0;
        for (int i = 0; i < n_blobs; ++i) {
          const double dx = px - b[5 * i], dy = py - b[5 * i + 1], dz = pz - b[5 * i + 2];
          v += b[5 * i + 4] * std::exp(-(dx * dx + dy * dy + dz * dz) * b[5 * i + 3]);
        }
        v = std::min(1.0, std::max(0.0, v));
        if (noise_max > 0.0f) v = std::min(1.0, v + lattice_unit(nseed, x, y, z) * (double)noise_max / 255.0);
        put(out, (size_t)x + (size_t)w * ((size_t)y + (size_t)h * z), dtype, v);
      }
  return 0;
}

// Fractal value noise: per octave a smoothstep-weighted trilinear
// interpolation of lattice values (base frequency 4 cells per longest side,
// then times lacunarity, amplitude times gain), normalised by the amplitude
// sum, optionally quantised into `shells` nested level sets.
int oracle_synth_value_noise(void* out, int w, int h, int d, int dtype, int octaves, float lacunarity, float gain,
                             int shells, uint64_t seed) {
  if (!out || w <= 0 || h <= 0 || d <= 0 || octaves < 1 || octaves > 12 || shells < 0 ||
      (dtype != CVR_U8 && dtype != CVR_U16))
    return -1;
  double norm = 0.0;
  {
    double amp = 1.0;
    for (int o = 0; o < octaves; ++o) { norm += amp; amp *= gain; }
  }
  const int side = std::max(w, std::max(h, d));
  auto smooth = [](double t) { return t * t * (3 - 2 * t); };
#pragma omp parallel for schedule(static)
  for (int z = 0; z < d; ++z)
    for (int y = 0; y < h; ++y)
      for (int x = 0; x < w; ++x) {
        double v = 0.0, amp = 1.0, freq = 4.0;
        for (int o = 0; o < octaves; ++o) {
          const double p[3] = {(x + 0.5) / side * freq, (y + 0.5) / side * freq, (z + 0.5) / side * freq};
          int64_t i[3];
          double f[3];
          for (int k = 0; k < 3; ++k) {
            i[k] = (int64_t)std::floor(p[k]);
            f[k] = smooth(p[k] - i[k]);
          }
          const uint64_t os = seed + 0x9E3779B97F4A7C15ull * (uint64_t)(o + 1);
          auto L = [&](int dx, int dy, int dz) { return lattice_unit(os, i[0] + dx, i[1] + dy, i[2] + dz); };
          const double c000 = L(0, 0, 0), c100 = L(1, 0, 0), c010 = L(0, 1, 0), c110 = L(1, 1, 0);
          const double c001 = L(0, 0, 1), c101 = L(1, 0, 1), c011 = L(0, 1, 1), c111 = L(1, 1, 1);
          const double x0 = c000 + f[0] * (c100 - c000), x1 = c010 + f[0] * (c110 - c010);
          const double x2 = c001 + f[0] * (c101 - c001), x3 = c011 + f[0] * (c111 - c011);
          const double y0 = x0 + f[1] * (x1 - x0), y1 = x2 + f[1] * (x3 - x2);
          v += amp * (y0 + f[2] * (y1 - y0));
          amp *= gain;
          freq *= lacunarity;
        }
        v /= norm;
        if (shells > 0) {
          int k = 0;
          for (int s = 1; s <= shells; ++s)
            if (v > (double)s / (shells + 1)) ++k;
          v = (double)k / shells;
        }
        put(out, (size_t)x + (size_t)w * ((size_t)y + (size_t)h * z), dtype, v);
      }
  return 0;
}

}  // extern "C"
