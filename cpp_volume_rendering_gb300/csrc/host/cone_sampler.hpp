// cone_sampler.hpp — host mirror of ConeGaussianSampler
// (cppvolrend/structured/rc1pdosct/conegaussiansampler.h:21-163).
#pragma once

#include <vector>

namespace cvrhost {

struct Vec3f { float x = 0, y = 0, z = 0; };

// RodriguesRotation, float version (libs/math_utils/utils.cpp:149-156).
Vec3f RodriguesRotation(Vec3f v, float theta, Vec3f k);

class ConeGaussianSampler {
 public:
  enum Packing { P1 = 0, P3 = 1, P7 = 2 };
  struct Section {
    int number_of_gaussians;
    double distance_from_origin, cone_radius, sampled_gaussian_sigma;
    double d_integral = 0, mip_map_level = 0, amplitude = 0;
  };
  struct Interval { double s_position, s_distance; };

  ConeGaussianSampler();
  void SetConeHalfAngle(float a);     // clamped to [0.5, 89.5]
  void SetInitialStep(float s) { initial_step = s > 0.0f ? s : 0.0f; }
  void SetMaxGaussianPacking(int p) { max_packing = p; }
  void SetCoveredDistance(float d) { covered_distance = d > 10.0f ? d : 10.0f; }  // clamp as reference
  void SetCoveredDistanceUnclamped(float d) { covered_distance = d; }
  void SetUIWeightPercentage(float w) { ui_weight = w; }

  // ComputeConeIntegrationSteps (conegaussiansampler.cpp:212-285); returns false
  // where the reference would exit() on an inconsistent section list.
  bool ComputeConeIntegrationSteps(double min_sg_gaussian);

  float cone_half_angle, initial_step, covered_distance, ui_weight, d_sigma, r_sigma;
  int max_packing;
  int gaussian_samples_1 = 0, gaussian_samples_3 = 0, gaussian_samples_7 = 0;
  Vec3f ray3_axis[3], ray7_axis[7];
  double ray3_adj_weight = 0, ray7_adj_weight = 0;
  std::vector<Section> sections;
  std::vector<Interval> intervals;

 private:
  bool ComputeAdditionalInfo(double min_sg_gaussian);
  double GaussianEval(double x, double sig);
  double IntegrateGaussian(double sdev, double cone_radius);
  bool Add1(double pos, double sg, int* n);
  bool Add3(double pos, double sg, int* n);
  bool Add7(double pos, double sg, int* n);
};

}  // namespace cvrhost
