// tf1d.hpp — host mirror of vis::TransferFunction1D
// (libs/volvis_utils/transferfunction1d.h:33-76, transferfunction.h:14-82).
#pragma once

#include <string>
#include <vector>

namespace vis {

// TransferControlPoint (libs/volvis_utils/transferfunction.cpp:8-24): the
// colour is held in single precision (a glm::vec4 in the reference), which
// matters for the exact table values BuildLinear produces.
struct TransferControlPoint {
  float r = 0.0f, g = 0.0f, b = 0.0f, a = 0.0f;
  int iso = 0;
  static TransferControlPoint RGB(double r, double g, double b, int iso);
  static TransferControlPoint Alpha(double a, int iso);
};

double MaterialOpacityToExtinction(float opacity);   // transferfunction.h:79-82
double ExtinctionToMaterialOpacity(float extinction); // transferfunction.h:74-77

class TransferFunction1D {
 public:
  explicit TransferFunction1D(int max_value = 255);

  void AddRGBControlPoint(const TransferControlPoint& p) { m_rgb.push_back(p); m_built = false; }
  void AddAlphaControlPoint(const TransferControlPoint& p) { m_alpha.push_back(p); m_built = false; }
  void ClearControlPoints() { m_rgb.clear(); m_alpha.clear(); m_built = false; }
  void SetExtinctionCoefficientInput(bool s) { m_extinction_input = s; }
  bool IsExtinctionCoefficientInput() const { return m_extinction_input; }
  int GetMaxDensity() const { return m_max_density; }

  void Build();
  // Get(value, max_data_value) (transferfunction1d.cpp:132-157), single precision result.
  void Get(double value, double max_data_value, float out[4]);
  float GetOpcN(double normalized_value);
  float GetExtN(double normalized_value);

  // GenerateTexture_1D_RGBt / _RGBA contents: (max_density+1) x RGBA float.
  std::vector<float> TableRGBt();
  std::vector<float> TableRGBA();

  std::string name;

 private:
  void BuildLinear();
  std::vector<TransferControlPoint> m_rgb, m_alpha;
  std::vector<double> m_table;  // (max_density+1) x 4, glm::dvec4 in the reference
  int m_max_density;
  bool m_extinction_input = false;
  bool m_built = false;
};

// readtf1d (libs/volvis_utils/reader.cpp:744-814).  Returns nullptr-equivalent
// (false) when the file cannot be opened; never exits.
bool ReadTransferFunction1D(const std::string& path, TransferFunction1D* out, std::string* err);

}  // namespace vis
