// renderers.hpp — headless mirror of the reference's renderer plugin API.
//
// BaseVolumeRenderer (cppvolrend/volrenderbase.h:25-97) keeps its virtuals
// (GetName, Init, Update, Redraw, Reshape, Clean, FillParameterSpace,
// GetDataTypeSupport, PrepareRender / SetOutdated), its dirty-flag protocol
// and its ownership rules (the manager owns renderers; DataManager and
// RenderingParameters are borrowed).  GetScreenTextureID becomes
// GetOutputDevicePtr + ReadbackRGBA32F; GL errors and exit() become false
// returns with LastError().  Each concrete renderer keeps the reference class
// name and constructor defaults, and calls the C ABI (include/cvr.h) where the
// reference dispatched a GLSL compute shader.
#pragma once

#include <memory>
#include <string>
#include <vector>

#include "../../../include/cvr.h"
#include "cone_sampler.hpp"
#include "tf1d.hpp"
#include "volume.hpp"

namespace vis {

// Camera state consumed by the renderers (CameraData, libs/vis_utils/camera.cpp:17-54).
struct Camera {
  float eye[3] = {0, 0, 512}, center[3] = {0, 0, 0}, up[3] = {0, 1, 0};
  float fovy = 45.0f;
  float aspect = 1.0f;
  cvr_camera ToABI() const;
};

// RenderingParameters (libs/volvis_utils/renderingparameters.cpp:17-32).
class RenderingParameters {
 public:
  RenderingParameters();
  int GetScreenWidth() const { return screen_width; }
  int GetScreenHeight() const { return screen_height; }
  void SetScreenSize(int w, int h) { screen_width = w; screen_height = h; }
  float GetBlinnPhongKambient() const { return ka; }
  float GetBlinnPhongKdiffuse() const { return kd; }
  float GetBlinnPhongKspecular() const { return ks; }
  float GetBlinnPhongNshininess() const { return shininess; }
  void SetPhongParameters(float a, float d, float s, float n) { ka = a; kd = d; ks = s; shininess = n; }
  // GetLightSourceSpecular (renderingparameters.cpp:132-135); (1,1,1) without lights.
  void LightSpecular(float out[3]) const;
  int GetNumberOfLightSources() const { return (int)lights.size(); }
  void CreateNewLightSource(const LightSourceData& l) { lights.push_back(l); }
  LightSourceData* GetCurrentLight() { return lights.empty() ? nullptr : &lights[current_light]; }
  // GetBlinnPhongLightSourceCameraForward returns -z_axis (renderingparameters.cpp:154-157).
  void LightForward(float out[3]) const;
  Camera camera;

 private:
  int screen_width = 768, screen_height = 768;
  float ka = 0.5f, kd = 0.5f, ks = 0.8f, shininess = 30.0f;
  std::vector<LightSourceData> lights;
  int current_light = 0;
};

// DataManager (libs/volvis_utils/datamanager.cpp:69-101) reduced to the
// current volume + transfer function, plus the device context that holds
// their device copies (the "textures").
class DataManager {
 public:
  DataManager();
  ~DataManager();
  bool ReadVolume(const std::string& path, std::string* err);
  bool ReadTransferFunction(const std::string& path, std::string* err);
  void SetVolume(const StructuredGridVolume& v) { volume = v; has_volume = true; uploaded = false; }
  void SetTransferFunction(const TransferFunction1D& t) { tf = t; has_tf = true; uploaded = false; }
  StructuredGridVolume* GetCurrentStructuredVolume() { return has_volume ? &volume : nullptr; }
  TransferFunction1D* GetCurrentTransferFunction() { return has_tf ? &tf : nullptr; }
  // GetCurrentVolumeTexture(): the device context with the volume uploaded
  // (and its gradient, built with the current gradient model).
  cvr_ctx* GetDeviceContext(std::string* err);
  // STRUCTURED_GRADIENT_TYPE (datamanager.h:64-69): CVR_GRADIENT_*; the
  // gradient is (re)built with the next upload (UpdateStructuredGradientTexture).
  void SetCurrentGradient(int model) { gradient_model = model; gradient_built = false; }
  int GetCurrentGradientGenerationTypeID() const { return gradient_model; }
  // GetCurrentGradientTexture() != nullptr
  bool HasGradient() const { return gradient_model != CVR_GRADIENT_NONE; }

 private:
  StructuredGridVolume volume;
  TransferFunction1D tf;
  bool has_volume = false, has_tf = false, uploaded = false;
  int gradient_model = CVR_GRADIENT_NONE;  // curr_gradient_comp_model (datamanager.cpp:27)
  bool gradient_built = false;
  cvr_ctx* ctx = nullptr;
};

}  // namespace vis

// ParameterSpace (cppvolrend/utils/parameterspace.h:170-225): named float ranges.
struct ParameterRangeFloat {
  std::string name;
  float* value;
  float min, max, step;
};
class ParameterSpace {
 public:
  void ClearParameterDimensions() { dims.clear(); }
  void AddParameterDimension(const ParameterRangeFloat& p) { dims.push_back(p); }
  std::vector<ParameterRangeFloat> dims;
  // Number of points of the cartesian sweep.
  long long Size() const;
};

class BaseVolumeRenderer {
 public:
  BaseVolumeRenderer() = default;
  virtual ~BaseVolumeRenderer() = default;

  void SetExternalResources(vis::DataManager* dm, vis::RenderingParameters* rp) {
    m_ext_data_manager = dm;
    m_ext_rendering_parameters = rp;
  }
  virtual const char* GetName() = 0;
  virtual const char* GetAbbreviationName() = 0;
  virtual void Clean() { vr_built = false; }
  virtual bool Init(int width, int height) = 0;
  virtual bool Update(const vis::Camera& camera) = 0;
  virtual bool Redraw();
  virtual void Reshape(int w, int h);
  virtual int GetDataTypeSupport() { return 0; }  // structured grid
  virtual void FillParameterSpace(ParameterSpace& ps) { ps.ClearParameterDimensions(); }
  // The occlusion / shadow check boxes of the illumination renderers' UI
  // (SetImGuiComponents); a no-op for renderers without illumination.
  virtual void SetIllumination(bool occlusion, bool shadow) { (void)occlusion; (void)shadow; }
  // The "Apply Gradient Shading" checkbox of every renderer
  // (m_apply_gradient_shading / m_apply_gradient, default false).
  void SetApplyGradientShading(bool on) { m_apply_gradient_shading = on; SetOutdated(); }
  bool GetApplyGradientShading() const { return m_apply_gradient_shading; }
  // MULTISCALING (volrenderbase.h:28-33, volrenderbase.cpp:101-114): modes 0..3,
  // honoured only by renderers that declare support (the reference: the
  // extinction renderer, ebsrenderer.cpp:51); 2 x 2 factors
  // (MULTISAMPLE_NUMBEROFSAMPLES_W/H); the image kernel of RenderFrameToScreen
  // (IMAGE_FILTER_KERNEL, default K2_HAT).
  bool IsPixelMultiScalingSupported() const { return vr_pixel_multiscaling_support; }
  int GetCurrentMultiScalingMode() const { return IsPixelMultiScalingSupported() ? vr_pixel_multiscaling_mode : 0; }
  void SetCurrentMultiScalingMode(int f) { vr_pixel_multiscaling_mode = f; SetOutdated(); }
  unsigned int GetImageKernelFilter() const { return m_kernel_filter; }
  void SetImageKernelFilter(unsigned int k) { m_kernel_filter = k; SetOutdated(); }

  // volrenderbase.cpp:77-84: Update only when outdated.
  bool PrepareRender(const vis::Camera& camera);
  virtual void SetOutdated() { vr_outdated = true; }
  bool IsOutdated() const { return vr_outdated; }
  bool IsBuilt() const { return vr_built; }

  const float* GetOutputDevicePtr() const { return m_frame; }
  bool ReadbackRGBA32F(float* host_rgba);
  int GetWidth() const { return m_width; }
  int GetHeight() const { return m_height; }
  const cvr_frame_stats& LastStats() const { return m_stats; }
  const std::string& LastError() const { return m_err; }

 protected:
  // The method's cvr_render call (the reference's Dispatch()).
  virtual int Method() const = 0;
  virtual const void* Params(size_t* size) = 0;
  bool Fail(const std::string& msg);
  bool CheckABI(int code, const char* what);
  bool BeginInit(int w, int h, bool need_tf = true);  // common part of Init(): device context + frame

  bool vr_built = false, vr_outdated = true;
  bool m_apply_gradient_shading = false;
  bool vr_pixel_multiscaling_support = false;
  int vr_pixel_multiscaling_mode = 0;
  unsigned int m_kernel_filter = CVR_FILTER_HAT;
  vis::DataManager* m_ext_data_manager = nullptr;
  vis::RenderingParameters* m_ext_rendering_parameters = nullptr;
  cvr_ctx* m_ctx = nullptr;
  float* m_frame = nullptr;
  int m_width = 0, m_height = 0;
  cvr_camera m_cam{};
  cvr_light m_light{};
  cvr_frame_stats m_stats{};
  std::string m_err;
};

// rc1pass: RayCasting1Pass (cppvolrend/structured/rc1pass/rc1prenderer.cpp).
class RayCasting1Pass : public BaseVolumeRenderer {
 public:
  const char* GetName() override { return "1-Pass - Ray Casting"; }
  const char* GetAbbreviationName() override { return "s_1rc"; }
  bool Init(int w, int h) override;
  bool Update(const vis::Camera& camera) override;
  void FillParameterSpace(ParameterSpace& ps) override;
  float m_u_step_size = 0.5f;

 protected:
  int Method() const override { return CVR_METHOD_PLAIN; }
  const void* Params(size_t* size) override;
  cvr_plain_params m_p{};
};

// rc1pisoadapt: RayCasting1PassIsoAdapt (rc1pisoadaptrenderer.cpp:10-200):
// first-hit isosurfaces with adaptive steps; needs no transfer function.
class RayCasting1PassIsoAdapt : public BaseVolumeRenderer {
 public:
  const char* GetName() override { return "1-Pass - Isosurface Raycaster Adaptive"; }
  const char* GetAbbreviationName() override { return "iso"; }
  bool Init(int w, int h) override;
  bool Update(const vis::Camera& camera) override;
  void FillParameterSpace(ParameterSpace& ps) override;
  float m_u_isovalue = 0.5f;
  float m_u_step_size_small = 0.05f;
  float m_u_step_size_large = 1.0f;
  float m_u_step_size_range = 0.1f;
  float m_u_color[4] = {0.66f, 0.6f, 0.05f, 1.0f};

 protected:
  int Method() const override { return CVR_METHOD_ISO; }
  const void* Params(size_t* size) override;
  cvr_iso_params m_p{};
};

// rc1pextbsd: RC1PExtinctionBasedShading (ebsrenderer.cpp:19-260).
class RC1PExtinctionBasedShading : public BaseVolumeRenderer {
 public:
  RC1PExtinctionBasedShading();
  const char* GetName() override { return "1-Pass - Extinction Based Shading"; }
  const char* GetAbbreviationName() override { return "s_1pebs"; }
  bool Init(int w, int h) override;
  bool Update(const vis::Camera& camera) override;
  void FillParameterSpace(ParameterSpace& ps) override;
  void SetIllumination(bool o, bool s) override { apply_ambient_occlusion = o; apply_directional_shadows = s; SetOutdated(); }

  float m_u_step_size = 0.5f;
  bool apply_ambient_occlusion = true;
  int ambient_occlusion_shells = 15;
  float ambient_occlusion_radius = 1.0f;
  std::vector<float> ambient_occlusion_radii;  // non-empty: explicit shell radii (generalisation)
  bool apply_directional_shadows = true;
  float dir_shadow_cone_angle = 1.0f;  // degrees
  float dir_shadow_sample_interval = 2.0f;
  float dir_shadow_initial_step = 2.0f;
  float dir_shadow_user_interface_weight = 1.0f;
  float dir_cone_max_distance = 0.0f;
  int type_of_shadow = 0;  // 0 point, 1 directional

 protected:
  int Method() const override { return CVR_METHOD_EXTINCTION; }
  const void* Params(size_t* size) override;
  cvr_ext_params m_p{};
};

// rc1pdosct: RC1PConeTracingDirOcclusionShading (dosrcrenderer.cpp:29-260).
class RC1PConeTracingDirOcclusionShading : public BaseVolumeRenderer {
 public:
  RC1PConeTracingDirOcclusionShading();
  const char* GetName() override { return "1-Pass - Directional Occlusion Shading using Cone Tracing"; }
  const char* GetAbbreviationName() override { return "s_1pdosct"; }
  bool Init(int w, int h) override;
  bool Update(const vis::Camera& camera) override;
  void SetIllumination(bool o, bool s) override { glsl_apply_occlusion = o; glsl_apply_shadow = s; SetOutdated(); }

  float m_u_step_size = 0.5f;
  bool glsl_apply_occlusion = true, glsl_apply_shadow = false;
  int type_of_shadow = 0;  // 0 point, 1 spot, 2 directional
  cvrhost::ConeGaussianSampler sampler_occlusion, sampler_shadow;
  float base_level_sigma0 = 1.0f;
  int ext_coef_resolution[3] = {128, 128, 128};
  int pyramid_levels = 0;  // 0: full mip chain (reference)

 protected:
  int Method() const override { return CVR_METHOD_CONE_DOS; }
  const void* Params(size_t* size) override;
  bool GenerateConeSamples();
  cvr_dos_params m_p{};
};

// rc1pcrtgt: RC1PConeLightGroundTruthSteps (crtgtrenderer.cpp:23-350), single pass.
class RC1PConeLightGroundTruthSteps : public BaseVolumeRenderer {
 public:
  RC1PConeLightGroundTruthSteps();
  const char* GetName() override { return "1-Pass - Cone Light Ground Truth Steps"; }
  const char* GetAbbreviationName() override { return "s_1pcrtgt"; }
  bool Init(int w, int h) override;
  bool Update(const vis::Camera& camera) override;
  void SetIllumination(bool o, bool s) override { m_apply_occlusion = o; m_apply_shadows = s; SetOutdated(); }

  float m_u_step_size = 0.5f;
  float m_u_light_ray_initial_step = 1.0f, m_u_light_ray_step_size = 0.5f;
  bool m_apply_occlusion = false;
  int m_occ_num_rays_sampled = 1;
  float m_occ_cone_aperture_angle = 90.f, m_occ_cone_distance_eval = 100.0f;
  bool m_apply_shadows = false;
  int m_sdw_num_rays_sampled = 1;
  float m_sdw_cone_aperture_angle = 1.0f, m_sdw_cone_distance_eval = 100.0f;
  int m_shadow_type = 0;  // 0 point, 1 spot, 2 directional
  unsigned int m_seed = 1;
  bool m_light_parameters_outdated = true;

 protected:
  int Method() const override { return CVR_METHOD_GROUND_TRUTH; }
  const void* Params(size_t* size) override;
  cvr_gt_params m_p{};
};

// No reference counterpart: the ground-truth renderer with its light
// integrals replaced by the learned network (CVR_METHOD_SURROGATE), same
// parameters.  Init builds the 6-level pyramid of base n/2 the network's
// inputs are defined on and loads the network from m_weights_path (a
// cvr_mlp_save checkpoint) unless the context already holds one.
class RC1PSurrogateShading : public RC1PConeLightGroundTruthSteps {
 public:
  const char* GetName() override { return "1-Pass - Learned Occlusion Surrogate"; }
  const char* GetAbbreviationName() override { return "s_1psurr"; }
  bool Init(int w, int h) override;
  std::string m_weights_path;

 protected:
  int Method() const override { return CVR_METHOD_SURROGATE; }
};

// Headless RenderingManager (cppvolrend/renderingmanager.cpp:119-319): owns the
// renderers, keeps the data / parameters, and runs the per-frame sequence
// PrepareRender -> Redraw, with readback in place of the on-screen blit.
class RenderingManager {
 public:
  RenderingManager();
  ~RenderingManager();
  void AddVolumeRenderer(BaseVolumeRenderer* r);  // takes ownership
  bool SetCurrentVolumeRenderer(int id);
  bool SetCurrentVolumeRenderer(const std::string& abbreviation);
  BaseVolumeRenderer* GetCurrentVolumeRenderer() { return m_current; }
  int NumberOfRenderers() const { return (int)m_renderers.size(); }
  bool Display();                        // one frame
  bool Readback(std::vector<float>* rgba);
  bool SaveFramePFM(const std::string& path);
  vis::DataManager data;
  vis::RenderingParameters params;
  const std::string& LastError() const { return m_err; }

 private:
  std::vector<std::unique_ptr<BaseVolumeRenderer>> m_renderers;
  BaseVolumeRenderer* m_current = nullptr;
  std::string m_err;
};
