// cone_sampler.cpp — section tables of the cone-traced directional occlusion.
// The step structure (sections of 1, then 3, then 7 Gaussian rays packed in
// the cone, sigma doubling when the cone radius exceeds r_sigma * sigma) is
// the reference's published algorithm; see the citations per function.
#include "cone_sampler.hpp"

#include <cmath>

namespace cvrhost {

static const double kPi = 3.14159265358979323846;
// D_HEMISPHERE_CONE_DIV_3 / _7 (conegaussiansampler.h:18-19): circle packing ratios.
static const double kDiv3 = 1.0 + (2.0 / std::sqrt(3.0));
static const double kDiv7 = 3.010000;

Vec3f RodriguesRotation(Vec3f v, float theta, Vec3f k) {
  float c = std::cos(theta), s = std::sin(theta);
  Vec3f kxv{k.y * v.z - k.z * v.y, k.z * v.x - k.x * v.z, k.x * v.y - k.y * v.x};
  float kd = k.x * v.x + k.y * v.y + k.z * v.z;
  float omc = 1.0f - c;
  Vec3f r{v.x * c + kxv.x * s + k.x * kd * omc, v.y * c + kxv.y * s + k.y * kd * omc,
          v.z * c + kxv.z * s + k.z * kd * omc};
  float inv = 1.0f / std::sqrt(r.x * r.x + r.y * r.y + r.z * r.z);
  return Vec3f{r.x * inv, r.y * inv, r.z * inv};
}

ConeGaussianSampler::ConeGaussianSampler() {
  // conegaussiansampler.cpp:30-47
  cone_half_angle = 30.0f;
  initial_step = 3.0f;
  max_packing = P7;
  covered_distance = 100.0f;
  d_sigma = 1.25f;
  r_sigma = 2.0f;
  ui_weight = 1.0f;
}

void ConeGaussianSampler::SetConeHalfAngle(float a) {
  cone_half_angle = a < 0.5f ? 0.5f : (a > 89.5f ? 89.5f : a);
}

bool ConeGaussianSampler::ComputeConeIntegrationSteps(double min_sg) {
  sections.clear();
  gaussian_samples_1 = gaussian_samples_3 = gaussian_samples_7 = 0;
  const Vec3f zax{0, 0, 1}, yax{0, 1, 0};
  {
    // 3 rays: tilted by (half_angle - half_angle/div3), 30 deg, then 120 deg steps.
    double adj = cone_half_angle / kDiv3;
    double t1 = (cone_half_angle - adj) * kPi / 180.0;
    ray3_axis[0] = RodriguesRotation(zax, (float)t1, yax);
    ray3_axis[0] = RodriguesRotation(ray3_axis[0], (float)(30.0 * kPi / 180.0), zax);
    double at = 120.0 * kPi / 180.0;
    ray3_axis[1] = RodriguesRotation(ray3_axis[0], (float)at, zax);
    ray3_axis[2] = RodriguesRotation(ray3_axis[1], (float)at, zax);
  }
  {
    // 7 rays: the axis plus six at (half_angle - half_angle/div7), 60 deg steps.
    ray7_axis[0] = zax;
    double adj = cone_half_angle / kDiv7;
    double t1 = (cone_half_angle - adj) * kPi / 180.0;
    ray7_axis[1] = RodriguesRotation(ray7_axis[0], (float)t1, yax);
    double at = 60.0 * kPi / 180.0;
    for (int i = 2; i < 7; ++i) ray7_axis[i] = RodriguesRotation(ray7_axis[i - 1], (float)at, zax);
  }
  intervals.clear();
  int n_g = 1;
  double pos = initial_step;
  double sg = min_sg;
  int guard = 0;
  while (!Add1(pos, sg, &n_g)) {
    sg *= 2.0;
    if (++guard > 256) return false;
  }
  while (pos < covered_distance) {
    double si = d_sigma * sg;
    guard = 0;
    while (!Add1(pos + si + (d_sigma * sg), sg, &n_g)) {
      sg *= 2.0;
      if (++guard > 256) return false;
    }
    si += d_sigma * sg;
    intervals.push_back(Interval{pos, si});
    pos += si;
    if (sections.size() > 100000) return false;
  }
  return ComputeAdditionalInfo(min_sg);
}

// ComputeAdditionalInfo (conegaussiansampler.cpp:318-386).
bool ConeGaussianSampler::ComputeAdditionalInfo(double min_sg) {
  ray3_adj_weight = (double)(ray3_axis[0].z);  // dot((0,0,1), axis) in float
  ray7_adj_weight = (double)(ray7_axis[1].z);
  for (size_t i = 0; i + 1 < sections.size(); ++i)
    if (!(sections[i].number_of_gaussians <= sections[i + 1].number_of_gaussians)) return false;
  if (sections.empty() || intervals.empty() || sections.size() != intervals.size() + 1) return false;
  double last_pos = intervals.back().s_position + intervals.back().s_distance;
  intervals.push_back(Interval{last_pos, 0});
  for (size_t i = 0; i < sections.size(); ++i) {
    Section* s = &sections[i];
    if (s->number_of_gaussians == 1) gaussian_samples_1 += 1;
    else if (s->number_of_gaussians == 3) gaussian_samples_3 += 1;
    else if (s->number_of_gaussians == 7) gaussian_samples_7 += 1;
    double cr = s->cone_radius;
    if (i == 0) s->d_integral = s->sampled_gaussian_sigma * std::sqrt(2.0 * kPi) * 0.5;
    else s->d_integral = intervals[i - 1].s_distance * 0.5;
    double pr = IntegrateGaussian(s->sampled_gaussian_sigma, cr);
    double ac = kPi * cr * cr;
    double ig = s->sampled_gaussian_sigma * std::sqrt(2.0 * kPi);
    s->amplitude = ((pr * pr) * (ig * ig)) / ac;
    s->mip_map_level = std::log2(s->sampled_gaussian_sigma / min_sg);
  }
  return true;
}

double ConeGaussianSampler::GaussianEval(double x, double sig) {
  return (1.0 / (std::sqrt(2.0 * kPi) * sig)) * std::exp(-(x * x) / (2.0 * sig * sig));
}

// Midpoint rule over [-r, r] in segments of about 0.05 (conegaussiansampler.cpp:393-414).
double ConeGaussianSampler::IntegrateGaussian(double sdev, double cone_radius) {
  double t = (2.0 * cone_radius) / 0.05;
  int nt = (int)std::ceil(t);
  double seg = (2.0 * cone_radius) / double(nt);
  double s0 = -cone_radius + seg * 0.5;
  double S = 0.0;
  for (int i = 0; i < nt; ++i) S += GaussianEval(s0 + seg * double(i), sdev) * seg;
  return S;
}

// AddGaussianSampleStep / With3 / With7 (conegaussiansampler.cpp:418-498).
bool ConeGaussianSampler::Add1(double pos, double sg, int* n) {
  if (*n > 1) return Add3(pos, sg, n);
  *n = 1;
  double rad = cone_half_angle * kPi / 180.0;
  double cr = pos * std::tan(rad);
  if (cr > r_sigma * sg) {
    if (max_packing > P1) return Add3(pos, sg, n);
    return false;
  }
  sections.push_back(Section{1, pos, cr, sg});
  return true;
}
bool ConeGaussianSampler::Add3(double pos, double sg, int* n) {
  if (*n > 3) return Add7(pos, sg, n);
  *n = 3;
  double rad = (cone_half_angle / kDiv3) * kPi / 180.0;
  double cr = pos * std::tan(rad);
  if (cr > r_sigma * sg) {
    if (max_packing > P3) return Add7(pos, sg, n);
    return false;
  }
  sections.push_back(Section{3, pos, cr, sg});
  return true;
}
bool ConeGaussianSampler::Add7(double pos, double sg, int* n) {
  *n = 7;
  double rad = (cone_half_angle / kDiv7) * kPi / 180.0;
  double cr = pos * std::tan(rad);
  if (cr > r_sigma * sg) return false;
  sections.push_back(Section{7, pos, cr, sg});
  return true;
}

}  // namespace cvrhost
