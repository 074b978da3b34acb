// ref_shim.cpp — TEST INFRASTRUCTURE ONLY.  Compiled by oracle/build_ref.py
// together with the reference's own, unmodified C++ sources (read in place
// from the reference checkout; nothing is copied) into oracle/_ref/.  It
// exposes the reference's CPU table builders through a C interface so the
// oracle and the product's host code can be pinned against them:
//   * vis::SummedAreaTable3D<double>::BuildSAT   (libs/vis_utils/summedareatable.h:218-280)
//   * vis::TransferFunction1D::Get / GetExtN     (libs/volvis_utils/transferfunction1d.cpp:132-197)
//   * ConeGaussianSampler::ComputeConeIntegrationSteps
//                                                (cppvolrend/structured/rc1pdosct/conegaussiansampler.cpp:212-386)
//   * RodriguesRotation                          (libs/math_utils/utils.cpp:149-156)
//   * GenerateGradientTexture / GenerateSobelFeldmanGradientTexture
//                                                (libs/volvis_utils/utils.cpp:146-351)
//   * Pvm (DDSV3::readPVMvolume + PostProcessData) (libs/file_utils/pvm.cpp:23-108,191-309)
//   * the image reconstruction kernels and digital filters (libs/vis_utils/filters/*.hpp,
//     header-only; the CPU twins of shader/renderoutputframe/*.comp)
// The GL texture classes those headers mention are stubbed below; no GL code
// runs.  Private members of ConeGaussianSampler are read through the access
// macro below (the interval list feeds the shader table but has no getter).
#include <cstring>
#include <random>
#include <vector>

#include <glm/gtc/constants.hpp>
#include <vis_utils/summedareatable.h>
#include <volvis_utils/transferfunction1d.h>
#include <math_utils/utils.h>
#include <volvis_utils/structuredgridvolume.h>
#include <volvis_utils/utils.h>
#include <file_utils/pvm.h>
// filters/utils.hpp's Symmetric4Pieces names its base class's buffer 'b'
// unqualified, which GCC's two-phase lookup rejects; a namespace-scope 'b'
// makes the header compile.  Only the kernels' operator() and digital_filter
// are called here, and neither touches the buffer.
namespace vis {
static float b[4];
}
#include <vis_utils/filters/box.hpp>
#include <vis_utils/filters/bspline3.hpp>
#include <vis_utils/filters/catmullrom.hpp>
#include <vis_utils/filters/hat.hpp>
#include <vis_utils/filters/mitchellnetravali.hpp>
#include <vis_utils/filters/omoms3.hpp>
#define private public
#include "structured/rc1pdosct/conegaussiansampler.h"
#undef private

// Stubs for the GL texture wrappers referenced by the reference headers.
namespace gl {
Texture1D::Texture1D(unsigned int) {}
Texture1D::~Texture1D() {}
void Texture1D::GenerateTexture(GLint, GLint, GLint) {}
bool Texture1D::SetData(GLvoid*, GLint, GLenum, GLenum) { return true; }
GLuint Texture1D::GetTextureID() { return 0; }
unsigned int Texture1D::GetLength() { return 0; }
void ExitOnGLError(const char*) {}
Texture2D::Texture2D(unsigned int, unsigned int) {}
void Texture2D::GenerateTexture(GLint, GLint, GLint, GLint) {}
bool Texture2D::SetData(GLvoid*, GLint, GLenum, GLenum) { return true; }
// A 3D texture keeps its size; SetData hands the host array to the capture
// buffer below (the gradient builders upload glm::vec3 RGB float texels).
std::vector<float> g_tex3d_data;
Texture3D::Texture3D(unsigned int w, unsigned int h, unsigned int d) : m_width(w), m_height(h), m_depth(d), m_textureID(0) {}
Texture3D::~Texture3D() {}
void Texture3D::GenerateTexture(GLint, GLint, GLint, GLint, GLint, bool) {}
bool Texture3D::SetData(GLvoid* data, GLint, GLenum format, GLenum type) {
  if (format != GL_RGB || type != GL_FLOAT) return false;
  const float* f = static_cast<const float*>(data);
  g_tex3d_data.assign(f, f + 3 * (size_t)m_width * m_height * m_depth);
  return true;
}
}  // namespace gl

namespace {
vis::TransferFunction1D* make_tf(int max_density, int n_rgb, const double* rgb, int n_alpha, const double* alpha,
                                 int ext_input) {
  vis::TransferFunction1D* tf = new vis::TransferFunction1D(max_density);
  tf->SetExtinctionCoefficientInput(ext_input != 0);
  for (int i = 0; i < n_rgb; ++i)
    tf->AddRGBControlPoint(vis::TransferControlPoint(rgb[4 * i], rgb[4 * i + 1], rgb[4 * i + 2], (int)rgb[4 * i + 3]));
  for (int i = 0; i < n_alpha; ++i) tf->AddAlphaControlPoint(vis::TransferControlPoint(alpha[2 * i], (int)alpha[2 * i + 1]));
  return tf;
}
}  // namespace

namespace {
template <class K>
int kernel_weights(K& kern, const float* x, int n, float* out, int* support) {
  *support = kern.support();
  for (int i = 0; i < n; ++i) out[i] = kern(x[i]);
  return 0;
}
template <class K>
int kernel_digital_filter(K& kern, float* f, int n) {
  std::vector<float> v(f, f + n);
  kern.digital_filter(v);
  for (int i = 0; i < n; ++i) f[i] = v[i];
  return 0;
}
}  // namespace

extern "C" {

// IMAGE_FILTER_KERNEL k: support and weights at n points x[i].
int ref_filter_weights(int k, const float* x, int n, float* out, int* support) {
  switch (k) {
    case 0: { vis::Box q; return kernel_weights(q, x, n, out, support); }
    case 1: { vis::Hat q; return kernel_weights(q, x, n, out, support); }
    case 2: { vis::CatmullRom q; return kernel_weights(q, x, n, out, support); }
    case 3: { vis::MitchellNetravali q; return kernel_weights(q, x, n, out, support); }
    case 4: { vis::CardinalBspline3 q; return kernel_weights(q, x, n, out, support); }
    case 5: { vis::CardinalOMOMS3 q; return kernel_weights(q, x, n, out, support); }
  }
  return -1;
}

// The kernel's digital filter applied to one line in place.
int ref_digital_filter(int k, float* f, int n) {
  switch (k) {
    case 4: { vis::CardinalBspline3 q; return kernel_digital_filter(q, f, n); }
    case 5: { vis::CardinalOMOMS3 q; return kernel_digital_filter(q, f, n); }
  }
  return -1;
}

// SAT of a full (W x H x D) grid given cell values (x fastest).
int ref_sat_build(int w, int h, int d, const double* cells, double* out) {
  vis::SummedAreaTable3D<double> sat(w, h, d);
  for (int z = 0; z < d; ++z)
    for (int y = 0; y < h; ++y)
      for (int x = 0; x < w; ++x) sat.SetValue(cells[(size_t)x + (size_t)w * ((size_t)y + (size_t)h * z)], x, y, z);
  sat.BuildSAT();
  std::memcpy(out, sat.GetData(), sizeof(double) * (size_t)w * h * d);
  return 0;
}

// GenerateTexture_1D_RGBt / _RGBA contents, reconstructed from Get(i) (which
// returns the float-rounded table entry at integer i) and the reference's
// opacity <-> extinction conversions, exactly as those two functions do.
int ref_tf_tables(int max_density, int n_rgb, const double* rgb, int n_alpha, const double* alpha, int ext_input,
                  float* rgbt, float* rgba) {
  vis::TransferFunction1D* tf = make_tf(max_density, n_rgb, rgb, n_alpha, alpha, ext_input);
  for (int i = 0; i <= max_density; ++i) {
    glm::vec4 v = tf->Get((double)i);
    for (int c = 0; c < 3; ++c) { rgbt[4 * i + c] = v[c]; rgba[4 * i + c] = v[c]; }
    float a = v.w;
    rgbt[4 * i + 3] = ext_input ? a : (float)tf->MaterialOpacityToExtinction(a);
    rgba[4 * i + 3] = ext_input ? (float)tf->ExtinctionToMaterialOpacity(a) : a;
  }
  delete tf;
  return 0;
}

// tf->GetExtN(vol->GetNormalizedSample(...)) for every u8 / u16 value.
int ref_tf_ext_per_value(int max_density, int n_rgb, const double* rgb, int n_alpha, const double* alpha,
                         int ext_input, int bytes_per_voxel, double* out) {
  vis::TransferFunction1D* tf = make_tf(max_density, n_rgb, rgb, n_alpha, alpha, ext_input);
  int n = bytes_per_voxel == 1 ? 256 : 65536;
  double denom = bytes_per_voxel == 1 ? (256.0 - 1.0) : (65536.0 - 1.0);
  for (int v = 0; v < n; ++v) out[v] = (double)tf->GetExtN((double)v / denom);
  delete tf;
  return 0;
}

// ConeGaussianSampler tables: sections as (interval distance, mip level,
// d_integral, amplitude) in double, counts, axes, adjacent weight.
int ref_cone_sampler(float half_angle, int packing, float covered, float initial_step, double min_sigma,
                     int max_sections, double* sections, int* counts, float* axes, double* w7) {
  ConeGaussianSampler s;
  s.SetConeHalfAngle(half_angle);
  s.SetMaxGaussianPacking(packing);
  s.covered_distance = covered;  // the setter clamps to >= 10 world units
  s.SetInitialStep(initial_step);
  s.ComputeConeIntegrationSteps(min_sigma);
  int n = (int)s.data_cone_sectionsinfo.size();
  if (n > max_sections) return -1;
  for (int i = 0; i < n; ++i) {
    sections[4 * i + 0] = s.data_cone_intervalsinfo[i].s_distance;
    sections[4 * i + 1] = s.data_cone_sectionsinfo[i].mip_map_level;
    sections[4 * i + 2] = s.data_cone_sectionsinfo[i].d_integral;
    sections[4 * i + 3] = s.data_cone_sectionsinfo[i].amplitude;
  }
  counts[0] = s.gaussian_samples_1; counts[1] = s.gaussian_samples_3; counts[2] = s.gaussian_samples_7;
  for (int i = 0; i < 3; ++i) { axes[3 * i] = s.ray3_axis[i].x; axes[3 * i + 1] = s.ray3_axis[i].y; axes[3 * i + 2] = s.ray3_axis[i].z; }
  for (int i = 0; i < 7; ++i) { axes[9 + 3 * i] = s.ray7_axis[i].x; axes[9 + 3 * i + 1] = s.ray7_axis[i].y; axes[9 + 3 * i + 2] = s.ray7_axis[i].z; }
  *w7 = s.GetRay7AdjacentWeight();
  return n;
}

// The GT kernel-vector loop of crtgtrenderer.cpp:131-187 written against the
// reference's RodriguesRotation (that renderer's Update() itself needs GL).
int ref_gt_vectors(int n_occ, float occ_ap, int n_sdw, float sdw_ap, unsigned seed, float* occ, float* sdw) {
  std::default_random_engine generator(seed);
  std::uniform_real_distribution<float> distribution(0.0, 1.0);
  glm::vec3 gtray(0, 0, 1);
  for (int i = 0; i < n_occ; ++i) {
    float theta = distribution(generator) * (glm::pi<float>() * (occ_ap / 180.f));
    float phi = distribution(generator) * (glm::pi<float>() * (360.f / 180.f));
    glm::vec3 v = RodriguesRotation(gtray, theta, glm::vec3(0, 1, 0));
    v = RodriguesRotation(v, phi, gtray);
    occ[3 * i] = v.x; occ[3 * i + 1] = v.y; occ[3 * i + 2] = v.z;
  }
  for (int i = 0; i < n_sdw; ++i) {
    float theta = distribution(generator) * (glm::pi<float>() * (sdw_ap / 180.f));
    float phi = distribution(generator) * (glm::pi<float>() * (360.f / 180.f));
    glm::vec3 v = RodriguesRotation(gtray, theta, glm::vec3(0, 1, 0));
    v = RodriguesRotation(v, phi, gtray);
    sdw[3 * i] = v.x; sdw[3 * i + 1] = v.y; sdw[3 * i + 2] = v.z;
  }
  return 0;
}

// The reference's gradient texture contents (float RGB per voxel, before
// the OpenGL driver's RGB16F rounding) of a u8 (bytes 1) or u16 (bytes 2) volume.
// model: 0 Sobel-Feldman, 1 finite differences (sample size, filter,
// normalized as given).
int ref_gradient(const void* vox, int w, int h, int d, int bytes, int model, int sample_size, int filter,
                 int normalized, float* out) {
  const size_t n = (size_t)w * h * d;
  vis::StructuredGridVolume vol("shim", w, h, d);
  if (bytes == 1) {
    unsigned char* a = new unsigned char[n];
    std::memcpy(a, vox, n);
    vol.SetArrayData(a, vis::DataStorageSize::_8_BITS);  // the volume frees it
  } else {
    unsigned short* a = new unsigned short[n];
    std::memcpy(a, vox, 2 * n);
    vol.SetArrayData(a, vis::DataStorageSize::_16_BITS);
  }
  gl::g_tex3d_data.clear();
  gl::Texture3D* t = model == 0 ? vis::GenerateSobelFeldmanGradientTexture(&vol)
                                : vis::GenerateGradientTexture(&vol, sample_size, filter, normalized != 0);
  delete t;
  if (gl::g_tex3d_data.size() != 3 * n) return -1;
  std::memcpy(out, gl::g_tex3d_data.data(), sizeof(float) * 3 * n);
  return 0;
}

// The reference's .pvm loader (readpvm's Pvm object): dims, bytes per voxel,
// spacing and the voxels (u8, or u16 as PostProcessData assembles them).
// The reference exits the process on a malformed file: valid files only.
int ref_read_pvm(const char* path, int* dims, int* components, double* scale, void* out, size_t out_bytes) {
  Pvm p(path);
  unsigned int w, h, d;
  p.GetDimensions(&w, &h, &d);
  dims[0] = (int)w; dims[1] = (int)h; dims[2] = (int)d;
  *components = p.GetComponents();
  p.GetScale(&scale[0], &scale[1], &scale[2]);
  const size_t n = (size_t)w * h * d * (size_t)(*components);
  if (!out) return 0;
  if (out_bytes < n || !p.GetData()) return -1;
  std::memcpy(out, p.GetData(), n);
  return 0;
}

}  // extern "C"
