// tf1d.cpp — host mirror of vis::TransferFunction1D.  Every expression keeps
// the reference's single/double precision mix so the tables match it bit for
// bit (pinned against the reference's own code in the tests).
#include "tf1d.hpp"

#include <cmath>
#include <fstream>
#include <sstream>

namespace vis {

TransferControlPoint TransferControlPoint::RGB(double r, double g, double b, int iso) {
  TransferControlPoint p;
  p.r = (float)r; p.g = (float)g; p.b = (float)b; p.a = 1.0f; p.iso = iso;
  return p;
}
TransferControlPoint TransferControlPoint::Alpha(double a, int iso) {
  TransferControlPoint p;
  p.a = (float)a; p.iso = iso;
  return p;
}

double MaterialOpacityToExtinction(float opacity) { return std::log(1.0 / (1.0 - (double)opacity)); }
double ExtinctionToMaterialOpacity(float extinction) { return 1.0 - (double)std::exp(-extinction); }

TransferFunction1D::TransferFunction1D(int max_value) : m_max_density(max_value) {}

void TransferFunction1D::Build() {
  m_table.assign((size_t)(m_max_density + 1) * 4, 0.0);  // glm 0.9.5 dvec4() is zero
  BuildLinear();
  m_built = true;
}

// transferfunction1d.cpp:319-358.  The colour differences are formed in
// single precision (glm::vec4 members) and widened, the interpolation runs in
// double.
void TransferFunction1D::BuildLinear() {
  for (int i = 0; i + 1 < (int)m_rgb.size(); ++i) {
    int i0 = m_rgb[i].iso, i1 = m_rgb[i + 1].iso;
    double dr = (double)(m_rgb[i + 1].r - m_rgb[i].r);
    double dg = (double)(m_rgb[i + 1].g - m_rgb[i].g);
    double db = (double)(m_rgb[i + 1].b - m_rgb[i].b);
    for (int x = i0; x <= i1; ++x) {
      if (x < 0 || x > m_max_density) continue;
      double k = (double)(x - i0) / (double)(i1 - i0);
      m_table[(size_t)x * 4 + 0] = (double)m_rgb[i].r + dr * k;
      m_table[(size_t)x * 4 + 1] = (double)m_rgb[i].g + dg * k;
      m_table[(size_t)x * 4 + 2] = (double)m_rgb[i].b + db * k;
    }
  }
  for (int i = 0; i + 1 < (int)m_alpha.size(); ++i) {
    int i0 = m_alpha[i].iso, i1 = m_alpha[i + 1].iso;
    double da = (double)(m_alpha[i + 1].a - m_alpha[i].a);
    for (int x = i0; x <= i1; ++x) {
      if (x < 0 || x > m_max_density) continue;
      double k = (double)(x - i0) / (double)(i1 - i0);
      m_table[(size_t)x * 4 + 3] = (double)m_alpha[i].a + da * k;
    }
  }
}

// transferfunction1d.cpp:132-157.
void TransferFunction1D::Get(double value, double max_data_value, float out[4]) {
  if (!m_built) Build();
  if (max_data_value >= 0) value = value * (double(m_max_density) / max_data_value);
  if (value < 0.0f || value > (float)m_max_density) {
    out[0] = out[1] = out[2] = out[3] = 0.0f;
    return;
  }
  if (std::fabs(value - (float)m_max_density) < 0.000001) {
    for (int c = 0; c < 4; ++c) out[c] = (float)m_table[(size_t)m_max_density * 4 + c];
    return;
  }
  int i = (int)value;
  double t = value - i;
  for (int c = 0; c < 4; ++c)
    out[c] = (float)((1.0 - t) * m_table[(size_t)i * 4 + c] + t * m_table[(size_t)(i + 1) * 4 + c]);
}

float TransferFunction1D::GetOpcN(double normalized_value) {
  float v[4];
  Get(normalized_value, 1.0, v);
  if (m_extinction_input) return (float)ExtinctionToMaterialOpacity(v[3]);
  return v[3];
}

float TransferFunction1D::GetExtN(double normalized_value) {
  float v[4];
  Get(normalized_value, 1.0, v);
  if (!m_extinction_input) return (float)MaterialOpacityToExtinction(v[3]);
  return v[3];
}

// GenerateTexture_1D_RGBt (transferfunction1d.cpp:89-118).
std::vector<float> TransferFunction1D::TableRGBt() {
  if (!m_built) Build();
  std::vector<float> t((size_t)(m_max_density + 1) * 4);
  for (int i = 0; i <= m_max_density; ++i) {
    t[i * 4 + 0] = (float)m_table[i * 4 + 0];
    t[i * 4 + 1] = (float)m_table[i * 4 + 1];
    t[i * 4 + 2] = (float)m_table[i * 4 + 2];
    float v4 = (float)m_table[i * 4 + 3];
    if (!m_extinction_input) v4 = (float)MaterialOpacityToExtinction(v4);
    t[i * 4 + 3] = v4;
  }
  return t;
}

// GenerateTexture_1D_RGBA (transferfunction1d.cpp:58-87).
std::vector<float> TransferFunction1D::TableRGBA() {
  if (!m_built) Build();
  std::vector<float> t((size_t)(m_max_density + 1) * 4);
  for (int i = 0; i <= m_max_density; ++i) {
    t[i * 4 + 0] = (float)m_table[i * 4 + 0];
    t[i * 4 + 1] = (float)m_table[i * 4 + 1];
    t[i * 4 + 2] = (float)m_table[i * 4 + 2];
    float v4 = (float)(double)m_table[i * 4 + 3];
    if (m_extinction_input) v4 = (float)ExtinctionToMaterialOpacity(v4);
    t[i * 4 + 3] = v4;
  }
  return t;
}

// readtf1d (reader.cpp:744-814): interpolation line, type (0/1/2), optional
// max density / extinction flag, RGB points, alpha points.
bool ReadTransferFunction1D(const std::string& path, TransferFunction1D* out, std::string* err) {
  std::ifstream f(path);
  if (!f.is_open()) {
    if (err) *err = "cannot open transfer function file: " + path;
    return false;
  }
  std::string interpolation;
  std::getline(f, interpolation);
  int init = 0;
  if (!(f >> init)) {
    if (err) *err = "malformed .tf1d header: " + path;
    return false;
  }
  int max_density = 255;
  int extuse = 0;
  if (init == 2) {
    f >> max_density >> extuse;
  } else if (init == 1) {
    f >> max_density;
  }
  if (!f || max_density < 1 || max_density > (1 << 20)) {
    if (err) *err = "malformed .tf1d max density: " + path;
    return false;
  }
  *out = TransferFunction1D(max_density);
  out->SetExtinctionCoefficientInput(init == 2 && extuse == 1);
  out->name = path;
  int n_rgb = 0;
  if (!(f >> n_rgb) || n_rgb < 0 || n_rgb > (1 << 20)) {
    if (err) *err = "malformed .tf1d rgb count: " + path;
    return false;
  }
  for (int i = 0; i < n_rgb; ++i) {
    double r, g, b;
    int iso;
    if (!(f >> r >> g >> b >> iso)) {
      if (err) *err = "truncated .tf1d rgb points: " + path;
      return false;
    }
    out->AddRGBControlPoint(TransferControlPoint::RGB(r, g, b, iso));
  }
  int n_a = 0;
  if (!(f >> n_a) || n_a < 0 || n_a > (1 << 20)) {
    if (err) *err = "malformed .tf1d alpha count: " + path;
    return false;
  }
  for (int i = 0; i < n_a; ++i) {
    double a;
    int iso;
    if (!(f >> a >> iso)) {
      if (err) *err = "truncated .tf1d alpha points: " + path;
      return false;
    }
    out->AddAlphaControlPoint(TransferControlPoint::Alpha(a, iso));
  }
  return true;
}

}  // namespace vis
