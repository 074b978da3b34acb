// renderers.cpp — the headless renderer plugins and manager (see renderers.hpp).
#include "renderers.hpp"

#include <cmath>
#include <cstdio>
#include <cstring>

namespace vis {

cvr_camera Camera::ToABI() const {
  cvr_camera c{};
  for (int i = 0; i < 3; ++i) {
    c.eye[i] = eye[i];
    c.center[i] = center[i];
    c.up[i] = up[i];
  }
  c.fovy_deg = fovy;
  c.aspect = aspect;
  return c;
}

RenderingParameters::RenderingParameters() {}

void RenderingParameters::LightForward(float out[3]) const {
  if (lights.empty()) {
    out[0] = 0; out[1] = 0; out[2] = -1;
    return;
  }
  for (int i = 0; i < 3; ++i) out[i] = -lights[current_light].z_axis[i];
}

void RenderingParameters::LightSpecular(float out[3]) const {
  for (int i = 0; i < 3; ++i) out[i] = lights.empty() ? 1.0f : lights[current_light].specular[i];
}

DataManager::DataManager() {}
DataManager::~DataManager() {
  if (ctx) cvr_destroy(ctx);
}

bool DataManager::ReadVolume(const std::string& path, std::string* err) {
  StructuredGridVolume v;
  if (!ReadStructuredVolume(path, &v, err)) return false;
  SetVolume(v);
  return true;
}

bool DataManager::ReadTransferFunction(const std::string& path, std::string* err) {
  TransferFunction1D t;
  if (!ReadTransferFunction1D(path, &t, err)) return false;
  SetTransferFunction(t);
  return true;
}

cvr_ctx* DataManager::GetDeviceContext(std::string* err) {
  if (!has_volume) {
    if (err) *err = "no volume loaded";
    return nullptr;
  }
  if (!ctx) {
    if (cvr_create(&ctx, 0) != CVR_OK) {
      if (err) *err = cvr_last_error(nullptr);
      ctx = nullptr;
      return nullptr;
    }
  }
  if (!uploaded) {
    int dt = volume.GetStorage() == DataStorageSize::_16_BITS ? CVR_U16 : CVR_U8;
    if (cvr_set_volume(ctx, volume.GetArrayData(), volume.GetWidth(), volume.GetHeight(), volume.GetDepth(), dt,
                       (float)volume.GetScaleX(), (float)volume.GetScaleY(), (float)volume.GetScaleZ()) != CVR_OK) {
      if (err) *err = cvr_last_error(ctx);
      return nullptr;
    }
    if (has_tf) {
      std::vector<float> rgbt = tf.TableRGBt(), rgba = tf.TableRGBA();
      if (cvr_set_transfer_function(ctx, rgbt.data(), rgba.data(), (int)rgbt.size() / 4) != CVR_OK) {
        if (err) *err = cvr_last_error(ctx);
        return nullptr;
      }
    }
    uploaded = true;
    gradient_built = false;
  }
  if (!gradient_built) {
    // GenerateStructuredGradientTexture (datamanager.cpp:332-352), library defaults
    cvr_gradient_params gp{gradient_model, 1, 0, 1};
    if (cvr_build_gradient(ctx, &gp) != CVR_OK) {
      if (err) *err = cvr_last_error(ctx);
      return nullptr;
    }
    gradient_built = true;
  }
  return ctx;
}

}  // namespace vis

long long ParameterSpace::Size() const {
  long long n = 1;
  for (const auto& d : dims) n *= (long long)std::floor((d.max - d.min) / d.step + 1.5);
  return n;
}

// ------------------------------------------------------------ base
bool BaseVolumeRenderer::Fail(const std::string& msg) {
  m_err = msg;
  return false;
}

bool BaseVolumeRenderer::CheckABI(int code, const char* what) {
  if (code == CVR_OK) return true;
  return Fail(std::string(what) + ": " + (m_ctx ? cvr_last_error(m_ctx) : cvr_last_error(nullptr)));
}

bool BaseVolumeRenderer::BeginInit(int w, int h, bool need_tf) {
  if (IsBuilt()) Clean();
  if (!m_ext_data_manager || !m_ext_data_manager->GetCurrentStructuredVolume())
    return Fail("Init: no volume loaded");  // rc1prenderer.cpp:54
  if (need_tf && !m_ext_data_manager->GetCurrentTransferFunction()) return Fail("Init: no transfer function");
  std::string err;
  m_ctx = m_ext_data_manager->GetDeviceContext(&err);
  if (!m_ctx) return Fail("Init: " + err);
  Reshape(w, h);
  return m_frame != nullptr;
}

void BaseVolumeRenderer::Reshape(int w, int h) {
  m_width = w;
  m_height = h;
  if (m_ctx && cvr_get_frame_buffer(m_ctx, w, h, &m_frame) != CVR_OK) m_frame = nullptr;
  SetOutdated();
}

bool BaseVolumeRenderer::PrepareRender(const vis::Camera& camera) {
  if (IsOutdated()) {
    if (!Update(camera)) return false;
    vr_outdated = false;
  }
  return true;
}

bool BaseVolumeRenderer::Redraw() {
  if (!IsBuilt()) return Fail("Redraw: renderer not built");
  size_t n = 0;
  const void* p = Params(&n);
  // ApplyGradientPhongShading = checkbox && gradient texture, with
  // RenderingParameters' Blinn-Phong terms (rc1prenderer.cpp:112-130)
  cvr_blinn_phong bp{};
  bp.apply = m_apply_gradient_shading && m_ext_data_manager && m_ext_data_manager->HasGradient();
  vis::RenderingParameters dflt;
  vis::RenderingParameters* rp = m_ext_rendering_parameters ? m_ext_rendering_parameters : &dflt;
  bp.ka = rp->GetBlinnPhongKambient();
  bp.kd = rp->GetBlinnPhongKdiffuse();
  bp.ks = rp->GetBlinnPhongKspecular();
  bp.shininess = rp->GetBlinnPhongNshininess();
  rp->LightSpecular(bp.specular);
  if (!CheckABI(cvr_set_blinn_phong(m_ctx, &bp), "Redraw")) return false;
  // Redraw / MultiSampleRedraw / DownScalingRedraw / UpScalingRedraw
  // (renderingmanager.cpp:1196-1218) by the current mode
  if (!CheckABI(cvr_set_multiscaling(m_ctx, GetCurrentMultiScalingMode(), (int)m_kernel_filter, 2, 2), "Redraw"))
    return false;
  return CheckABI(cvr_render(m_ctx, Method(), &m_cam, &m_light, p, n, m_frame, m_width, m_height, nullptr, &m_stats),
                  "Redraw");
}

bool BaseVolumeRenderer::ReadbackRGBA32F(float* host) {
  if (!m_frame || !m_ctx) return Fail("Readback: no frame");
  return CheckABI(cvr_download_frame(m_ctx, m_frame, m_width, m_height, host), "Readback");
}

static void fill_light(vis::RenderingParameters* rp, const vis::Camera& cam, cvr_light* L, int type) {
  std::memset(L, 0, sizeof(*L));
  L->type = type;
  vis::LightSourceData* ld = rp ? rp->GetCurrentLight() : nullptr;
  if (ld) {
    for (int i = 0; i < 3; ++i) {
      L->position[i] = ld->position[i];
      L->forward[i] = -ld->z_axis[i];
      L->up[i] = ld->y_axis[i];
      L->right[i] = ld->x_axis[i];
    }
    L->spot_cos_max = std::cos(3.14159265f * ld->spot_light_angle / 180.f);
  } else {
    // No light source: a headlight with the camera's axes (crtgtrenderer.cpp:220-223;
    // CameraData z = normalize(eye - center), x = normalize(cross(up, z)),
    // y = normalize(cross(z, x)), camera.cpp:48-50).
    auto nrm = [](float* v) {
      float n = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
      for (int i = 0; i < 3; ++i) v[i] /= n;
    };
    auto crs = [](const float* a, const float* b, float* o) {
      o[0] = a[1] * b[2] - a[2] * b[1];
      o[1] = a[2] * b[0] - a[0] * b[2];
      o[2] = a[0] * b[1] - a[1] * b[0];
    };
    float z[3] = {cam.eye[0] - cam.center[0], cam.eye[1] - cam.center[1], cam.eye[2] - cam.center[2]};
    nrm(z);
    float x[3], y[3];
    crs(cam.up, z, x);
    nrm(x);
    crs(z, x, y);
    nrm(y);
    for (int i = 0; i < 3; ++i) {
      L->position[i] = cam.eye[i];
      L->forward[i] = z[i];
      L->up[i] = y[i];
      L->right[i] = x[i];
    }
  }
}

static float default_step(const vis::StructuredGridVolume* v) {
  double sx = v->GetScaleX(), sy = v->GetScaleY(), sz = v->GetScaleZ();
  return float((0.5f / std::sqrt(3.0f)) * std::sqrt(sx * sx + sy * sy + sz * sz));
}

// ------------------------------------------------------------ rc1pass
bool RayCasting1Pass::Init(int w, int h) {
  if (!BeginInit(w, h)) return false;
  m_u_step_size = default_step(m_ext_data_manager->GetCurrentStructuredVolume());  // rc1prenderer.cpp:62-63
  vr_built = true;
  SetOutdated();
  return true;
}
bool RayCasting1Pass::Update(const vis::Camera& camera) {
  m_cam = camera.ToABI();
  fill_light(m_ext_rendering_parameters, camera, &m_light, CVR_LIGHT_POINT);
  m_p.step_size = m_u_step_size;
  return true;
}
void RayCasting1Pass::FillParameterSpace(ParameterSpace& ps) {
  ps.ClearParameterDimensions();
  ps.AddParameterDimension({"StepSize", &m_u_step_size, 0.2f, 2.0f, 0.1f});  // rc1prenderer.cpp:225-229
}
const void* RayCasting1Pass::Params(size_t* size) {
  *size = sizeof(m_p);
  return &m_p;
}

// ------------------------------------------------------------ rc1pisoadapt
bool RayCasting1PassIsoAdapt::Init(int w, int h) {
  if (!BeginInit(w, h, false)) return false;  // the volume alone (rc1pisoadaptrenderer.cpp:58)
  vr_built = true;
  SetOutdated();
  return true;
}
bool RayCasting1PassIsoAdapt::Update(const vis::Camera& camera) {
  m_cam = camera.ToABI();
  fill_light(m_ext_rendering_parameters, camera, &m_light, CVR_LIGHT_POINT);  // LightSourcePosition
  m_p.step_size_small = m_u_step_size_small;
  m_p.step_size_large = m_u_step_size_large;
  m_p.step_size_range = m_u_step_size_range;
  m_p.isovalue = m_u_isovalue;
  for (int i = 0; i < 4; ++i) m_p.color[i] = m_u_color[i];
  return true;
}
void RayCasting1PassIsoAdapt::FillParameterSpace(ParameterSpace& ps) {
  ps.ClearParameterDimensions();  // rc1pisoadaptrenderer.cpp:190-196
  ps.AddParameterDimension({"StepSizeSmall", &m_u_step_size_small, 0.01f, 0.25f, 0.05f});
  ps.AddParameterDimension({"StepSizeLarge", &m_u_step_size_large, 0.25f, 2.0f, 0.25f});
  ps.AddParameterDimension({"StepSizeRange", &m_u_step_size_range, 0.05f, 0.26f, 0.05f});
}
const void* RayCasting1PassIsoAdapt::Params(size_t* size) {
  *size = sizeof(m_p);
  return &m_p;
}

// ------------------------------------------------------------ rc1pextbsd
RC1PExtinctionBasedShading::RC1PExtinctionBasedShading() {
  vr_pixel_multiscaling_support = true;  // ebsrenderer.cpp:51
}

bool RC1PExtinctionBasedShading::Init(int w, int h) {
  if (!BeginInit(w, h)) return false;
  vis::StructuredGridVolume* v = m_ext_data_manager->GetCurrentStructuredVolume();
  vis::TransferFunction1D* tf = m_ext_data_manager->GetCurrentTransferFunction();
  // GenerateExtinctionSAT3DTex: per-voxel GetExtN of the normalised value.
  bool u16 = v->GetStorage() == vis::DataStorageSize::_16_BITS;
  int nv = u16 ? 65536 : 256;
  std::vector<double> ext(nv);
  double denom = u16 ? 65535.0 : 255.0;
  for (int i = 0; i < nv; ++i) ext[i] = (double)tf->GetExtN((double)i / denom);
  if (!CheckABI(cvr_build_sat(m_ctx, ext.data(), nv), "Init: SAT")) return false;
  dir_cone_max_distance = 0.75f * (float)v->GetDiagonal();  // ebsrenderer.cpp:98-105
  m_u_step_size = default_step(v);
  vr_built = true;
  SetOutdated();
  return true;
}

bool RC1PExtinctionBasedShading::Update(const vis::Camera& camera) {
  m_cam = camera.ToABI();
  fill_light(m_ext_rendering_parameters, camera, &m_light, type_of_shadow == 0 ? CVR_LIGHT_POINT : CVR_LIGHT_DIRECTIONAL);
  std::memset(&m_p, 0, sizeof(m_p));
  m_p.step_size = m_u_step_size;
  m_p.apply_occlusion = apply_ambient_occlusion;
  m_p.apply_shadow = apply_directional_shadows;
  if (!ambient_occlusion_radii.empty()) {
    m_p.ao_n_shells = (int)std::min<size_t>(ambient_occlusion_radii.size(), CVR_MAX_AO_SHELLS);
    for (int i = 0; i < m_p.ao_n_shells; ++i) m_p.ao_radii[i] = ambient_occlusion_radii[i];
  } else {
    m_p.ao_n_shells = std::min(ambient_occlusion_shells, CVR_MAX_AO_SHELLS);
    for (int i = 0; i < m_p.ao_n_shells; ++i) m_p.ao_radii[i] = ambient_occlusion_radius * float(i + 1);
  }
  m_p.sdw_cone_angle_rad = (float)(dir_shadow_cone_angle * 3.14159265358979323846 / 180.0);
  m_p.sdw_sample_interval = dir_shadow_sample_interval;
  m_p.sdw_initial_step = dir_shadow_initial_step;
  m_p.sdw_ui_weight = dir_shadow_user_interface_weight;
  m_p.sdw_max_distance = dir_cone_max_distance;
  m_p.shadow_type = type_of_shadow;
  m_p.ka = m_ext_rendering_parameters ? m_ext_rendering_parameters->GetBlinnPhongKambient() : 0.5f;
  m_p.kd = m_ext_rendering_parameters ? m_ext_rendering_parameters->GetBlinnPhongKdiffuse() : 0.5f;
  return true;
}
void RC1PExtinctionBasedShading::FillParameterSpace(ParameterSpace& ps) {
  ps.ClearParameterDimensions();
  ps.AddParameterDimension({"StepSize", &m_u_step_size, 0.2f, 2.0f, 0.1f});
}
const void* RC1PExtinctionBasedShading::Params(size_t* size) {
  *size = sizeof(m_p);
  return &m_p;
}

// ------------------------------------------------------------ rc1pdosct
RC1PConeTracingDirOcclusionShading::RC1PConeTracingDirOcclusionShading() {
  // dosrcrenderer.cpp:47-59
  sampler_occlusion.SetUIWeightPercentage(0.350f);
  sampler_occlusion.SetConeHalfAngle(20.0f);
  sampler_occlusion.SetMaxGaussianPacking(cvrhost::ConeGaussianSampler::P3);
  sampler_shadow.SetUIWeightPercentage(1.0f);
  sampler_shadow.SetConeHalfAngle(0.5f);
  sampler_shadow.SetMaxGaussianPacking(cvrhost::ConeGaussianSampler::P1);
}

static void to_table(const cvrhost::ConeGaussianSampler& s, cvr_cone_table* t) {
  std::memset(t, 0, sizeof(*t));
  t->n_sections = (int)std::min<size_t>(s.sections.size(), CVR_MAX_CONE_SECTIONS);
  for (int i = 0; i < t->n_sections; ++i) {
    t->sections[i][0] = (float)s.intervals[i].s_distance;
    t->sections[i][1] = (float)s.sections[i].mip_map_level;
    t->sections[i][2] = (float)s.sections[i].d_integral;
    t->sections[i][3] = (float)s.sections[i].amplitude;
  }
  t->integration_samples[0] = s.gaussian_samples_1;
  t->integration_samples[1] = s.gaussian_samples_3;
  t->integration_samples[2] = s.gaussian_samples_7;
  for (int i = 0; i < 3; ++i) { t->axes[i][0] = s.ray3_axis[i].x; t->axes[i][1] = s.ray3_axis[i].y; t->axes[i][2] = s.ray3_axis[i].z; }
  for (int i = 0; i < 7; ++i) { t->axes[3 + i][0] = s.ray7_axis[i].x; t->axes[3 + i][1] = s.ray7_axis[i].y; t->axes[3 + i][2] = s.ray7_axis[i].z; }
  t->initial_step = s.initial_step;
  t->ray7_adj_weight = (float)s.ray7_adj_weight;
  t->ui_weight = s.ui_weight;
}

bool RC1PConeTracingDirOcclusionShading::GenerateConeSamples() {
  if (!sampler_occlusion.ComputeConeIntegrationSteps(base_level_sigma0) ||
      !sampler_shadow.ComputeConeIntegrationSteps(base_level_sigma0))
    return Fail("Init: inconsistent cone section tables");
  cvr_cone_table occ, sdw;
  to_table(sampler_occlusion, &occ);
  to_table(sampler_shadow, &sdw);
  return CheckABI(cvr_set_cone_tables(m_ctx, &occ, &sdw), "Init: cone tables");
}

bool RC1PConeTracingDirOcclusionShading::Init(int w, int h) {
  if (!BeginInit(w, h)) return false;
  vis::StructuredGridVolume* v = m_ext_data_manager->GetCurrentStructuredVolume();
  sampler_occlusion.SetCoveredDistance((float)v->GetDiagonal() * 0.50f);  // dosrcrenderer.cpp:112-113
  sampler_shadow.SetCoveredDistance((float)v->GetDiagonal() * 0.75f);
  cvr_pyramid_params pp{};
  for (int i = 0; i < 3; ++i) pp.base_dims[i] = ext_coef_resolution[i];
  pp.sigma0 = base_level_sigma0;
  pp.n_levels = pyramid_levels;
  if (!CheckABI(cvr_build_ext_pyramid(m_ctx, &pp), "Init: extinction pyramid")) return false;
  if (!GenerateConeSamples()) return false;
  m_u_step_size = default_step(v);
  vr_built = true;
  SetOutdated();
  return true;
}

bool RC1PConeTracingDirOcclusionShading::Update(const vis::Camera& camera) {
  m_cam = camera.ToABI();
  fill_light(m_ext_rendering_parameters, camera, &m_light, type_of_shadow);
  m_p.step_size = m_u_step_size;
  m_p.apply_occlusion = glsl_apply_occlusion;
  m_p.apply_shadow = glsl_apply_shadow;
  m_p.shadow_type = type_of_shadow;
  m_p.ka = m_ext_rendering_parameters ? m_ext_rendering_parameters->GetBlinnPhongKambient() : 0.5f;
  m_p.kd = m_ext_rendering_parameters ? m_ext_rendering_parameters->GetBlinnPhongKdiffuse() : 0.5f;
  return true;
}
const void* RC1PConeTracingDirOcclusionShading::Params(size_t* size) {
  *size = sizeof(m_p);
  return &m_p;
}

// ------------------------------------------------------------ rc1pcrtgt
RC1PConeLightGroundTruthSteps::RC1PConeLightGroundTruthSteps() {}

bool RC1PConeLightGroundTruthSteps::Init(int w, int h) {
  if (!BeginInit(w, h)) return false;
  vis::StructuredGridVolume* v = m_ext_data_manager->GetCurrentStructuredVolume();
  m_u_step_size = default_step(v);
  m_occ_cone_distance_eval = (float)v->GetDiagonal() * 0.50f;  // crtgtrenderer.cpp:110-114
  m_sdw_cone_distance_eval = (float)v->GetDiagonal() * 0.75f;
  m_light_parameters_outdated = true;
  vr_built = true;
  SetOutdated();
  return true;
}

bool RC1PConeLightGroundTruthSteps::Update(const vis::Camera& camera) {
  if (m_light_parameters_outdated) {
    std::vector<float> occ(3 * std::max(1, m_occ_num_rays_sampled)), sdw(3 * std::max(1, m_sdw_num_rays_sampled));
    if (!CheckABI(cvr_gt_kernel_vectors(m_occ_num_rays_sampled, m_occ_cone_aperture_angle, m_sdw_num_rays_sampled,
                                        m_sdw_cone_aperture_angle, m_seed, occ.data(), sdw.data()),
                  "Update: kernel vectors"))
      return false;
    if (!CheckABI(cvr_set_gt_kernels(m_ctx, occ.data(), m_occ_num_rays_sampled, sdw.data(), m_sdw_num_rays_sampled),
                  "Update: kernel vectors upload"))
      return false;
    m_light_parameters_outdated = false;
  }
  m_cam = camera.ToABI();
  fill_light(m_ext_rendering_parameters, camera, &m_light, m_shadow_type);
  // crtgtrenderer.cpp:220-234: with a light source the shader's LightCamForward
  // is -GetBlinnPhongLightSourceCameraForward().
  if (m_ext_rendering_parameters && m_ext_rendering_parameters->GetNumberOfLightSources() > 0)
    for (int i = 0; i < 3; ++i) m_light.forward[i] = -m_light.forward[i];
  m_p.step_size = m_u_step_size;
  m_p.light_ray_initial_gap = m_u_light_ray_initial_step;
  m_p.light_ray_step_size = m_u_light_ray_step_size;
  m_p.apply_occlusion = m_apply_occlusion;
  m_p.occ_distance = m_occ_cone_distance_eval;
  m_p.apply_shadow = m_apply_shadows;
  m_p.sdw_distance = m_sdw_cone_distance_eval;
  m_p.shadow_type = m_shadow_type;
  m_p.ka = m_ext_rendering_parameters ? m_ext_rendering_parameters->GetBlinnPhongKambient() : 0.5f;
  m_p.kd = m_ext_rendering_parameters ? m_ext_rendering_parameters->GetBlinnPhongKdiffuse() : 0.5f;
  return true;
}
const void* RC1PConeLightGroundTruthSteps::Params(size_t* size) {
  *size = sizeof(m_p);
  return &m_p;
}

bool RC1PSurrogateShading::Init(int w, int h) {
  if (!RC1PConeLightGroundTruthSteps::Init(w, h)) return false;
  vr_built = false;
  vis::StructuredGridVolume* v = m_ext_data_manager->GetCurrentStructuredVolume();
  cvr_pyramid_params pp{};
  pp.base_dims[0] = std::max(1, v->GetWidth() / 2);
  pp.base_dims[1] = std::max(1, v->GetHeight() / 2);
  pp.base_dims[2] = std::max(1, v->GetDepth() / 2);
  pp.sigma0 = 1.0f;
  pp.n_levels = CVR_SURROGATE_LEVELS;
  if (!CheckABI(cvr_build_ext_pyramid(m_ctx, &pp), "Init: extinction pyramid")) return false;
  if (!m_weights_path.empty()) {
    if (!CheckABI(cvr_mlp_load(m_ctx, m_weights_path.c_str()), "Init: network checkpoint")) return false;
  } else {
    float probe = 0.0f;
    if (cvr_mlp_get_params(m_ctx, &probe, 1) == CVR_ERR_NOT_READY)
      return Fail("Init: no network (set m_weights_path to a cvr_mlp_save checkpoint)");
  }
  vr_built = true;
  SetOutdated();
  return true;
}

// ------------------------------------------------------------ manager
RenderingManager::RenderingManager() {}
RenderingManager::~RenderingManager() { m_renderers.clear(); }

void RenderingManager::AddVolumeRenderer(BaseVolumeRenderer* r) {
  r->SetExternalResources(&data, &params);
  m_renderers.emplace_back(r);
}

bool RenderingManager::SetCurrentVolumeRenderer(int id) {
  if (id < 0 || id >= (int)m_renderers.size()) {
    m_err = "renderer index out of range";
    return false;
  }
  if (m_current) m_current->Clean();
  m_current = m_renderers[id].get();
  // UpdateDataAndResetCurrentVRMode -> Init(w, h) (renderingmanager.cpp:404, 521-540)
  if (!m_current->Init(params.GetScreenWidth(), params.GetScreenHeight())) {
    m_err = m_current->LastError();
    return false;
  }
  return true;
}

bool RenderingManager::SetCurrentVolumeRenderer(const std::string& abbr) {
  for (size_t i = 0; i < m_renderers.size(); ++i)
    if (abbr == m_renderers[i]->GetAbbreviationName()) return SetCurrentVolumeRenderer((int)i);
  m_err = "no renderer named " + abbr;
  return false;
}

bool RenderingManager::Display() {
  if (!m_current) {
    m_err = "no current renderer";
    return false;
  }
  if (!m_current->PrepareRender(params.camera) || !m_current->Redraw()) {
    m_err = m_current->LastError();
    return false;
  }
  return true;
}

bool RenderingManager::Readback(std::vector<float>* rgba) {
  if (!m_current) return false;
  rgba->resize((size_t)m_current->GetWidth() * m_current->GetHeight() * 4);
  if (!m_current->ReadbackRGBA32F(rgba->data())) {
    m_err = m_current->LastError();
    return false;
  }
  return true;
}

// Portable float map: the headless stand-in for SaveScreenshot (renderingmanager.cpp:409-419).
bool RenderingManager::SaveFramePFM(const std::string& path) {
  std::vector<float> px;
  if (!Readback(&px)) return false;
  FILE* f = std::fopen(path.c_str(), "wb");
  if (!f) {
    m_err = "cannot write " + path;
    return false;
  }
  int w = m_current->GetWidth(), h = m_current->GetHeight();
  std::fprintf(f, "PF\n%d %d\n-1.0\n", w, h);
  std::vector<float> rgb((size_t)w * 3);
  for (int y = 0; y < h; ++y) {  // PFM rows are bottom-to-top, like the frame
    for (int x = 0; x < w; ++x)
      for (int c = 0; c < 3; ++c) rgb[(size_t)x * 3 + c] = px[((size_t)y * w + x) * 4 + c];
    std::fwrite(rgb.data(), sizeof(float), rgb.size(), f);
  }
  std::fclose(f);
  return true;
}
