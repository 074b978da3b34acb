// cvr_headless — headless counterpart of the reference application's main()
// (cppvolrend/main.cpp:49-79) and RenderingManager frame loop: registers the
// renderer plugins, loads a volume and a transfer function (and optionally a
// camera-state list and a light-source list), selects a renderer by its
// abbreviation, renders frames and writes the last one as a .pfm image.
//
//   cvr_headless --volume V.raw|.syn|.pvm|.nrrd|.nhrd|.dat --tf T.tf1d --renderer s_1pebs
//                [--width 768 --height 768] [--frames 1]
//                [--cameras LIST --camera-index i] [--lights LIST --light-index i]
//                [--eye x y z] [--fovy deg] [--occlusion 0|1] [--shadow 0|1]
//                [--gradient sobel|fd|cs|none] [--gradient-shading 0|1]
//                [--multiscaling 0..3 (s_1pebs)] [--image-filter 0..5]
//                [--out frame.pfm]
// Exit code 0 on success, 1 on a usage error, 2 on a data error, 3 on a
// rendering error; messages go to stderr.
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>

#include "../host/renderers.hpp"

static int usage() {
  std::fprintf(stderr,
               "usage: cvr_headless --volume FILE --tf FILE --renderer ABBR [--width W --height H] [--frames N]\n"
               "       [--cameras FILE --camera-index I] [--lights FILE --light-index I] [--eye X Y Z]\n"
               "       [--fovy DEG] [--occlusion 0|1] [--shadow 0|1] [--weights FILE] [--out FILE.pfm]\n"
               "       [--gradient sobel|fd|cs|none] [--gradient-shading 0|1]\n"
               "       [--multiscaling 0..3 (s_1pebs)] [--image-filter 0..5]\n"
               "renderers: s_1rc s_1pebs s_1pdosct s_1pcrtgt iso s_1psurr (needs --weights)\n");
  return 1;
}

int main(int argc, char** argv) {
  std::string vol, tf, rend, out, cams, lights, weights;
  int w = 768, h = 768, frames = 1, cam_i = 0, light_i = 0;
  bool have_eye = false;
  int occlusion = -1, shadow = -1, gradient = CVR_GRADIENT_NONE, gradient_shading = 0;
  int multiscaling = 0, image_filter = CVR_FILTER_HAT;
  float eye[3] = {0, 0, 0}, fovy = 45.0f;
  for (int i = 1; i < argc; ++i) {
    std::string a = argv[i];
    auto next = [&](void) -> const char* { return i + 1 < argc ? argv[++i] : nullptr; };
    const char* v = nullptr;
    if (a == "--volume" && (v = next())) vol = v;
    else if (a == "--tf" && (v = next())) tf = v;
    else if (a == "--renderer" && (v = next())) rend = v;
    else if (a == "--out" && (v = next())) out = v;
    else if (a == "--weights" && (v = next())) weights = v;
    else if (a == "--width" && (v = next())) w = std::atoi(v);
    else if (a == "--height" && (v = next())) h = std::atoi(v);
    else if (a == "--frames" && (v = next())) frames = std::atoi(v);
    else if (a == "--cameras" && (v = next())) cams = v;
    else if (a == "--camera-index" && (v = next())) cam_i = std::atoi(v);
    else if (a == "--lights" && (v = next())) lights = v;
    else if (a == "--light-index" && (v = next())) light_i = std::atoi(v);
    else if (a == "--fovy" && (v = next())) fovy = (float)std::atof(v);
    else if (a == "--occlusion" && (v = next())) occlusion = std::atoi(v);
    else if (a == "--shadow" && (v = next())) shadow = std::atoi(v);
    else if (a == "--gradient-shading" && (v = next())) gradient_shading = std::atoi(v);
    else if (a == "--multiscaling" && (v = next())) multiscaling = std::atoi(v);
    else if (a == "--image-filter" && (v = next())) image_filter = std::atoi(v);
    else if (a == "--gradient" && (v = next())) {
      // DataManager's gradient models (datamanager.h:64-69)
      std::string g = v;
      if (g == "sobel") gradient = CVR_GRADIENT_SOBEL_FELDMAN;
      else if (g == "fd") gradient = CVR_GRADIENT_FINITE_DIFFERENCES;
      else if (g == "cs") gradient = CVR_GRADIENT_COMPUTE_SOBEL;
      else if (g == "none") gradient = CVR_GRADIENT_NONE;
      else return usage();
    }
    else if (a == "--eye" && i + 3 < argc) {
      for (int k = 0; k < 3; ++k) eye[k] = (float)std::atof(argv[++i]);
      have_eye = true;
    } else
      return usage();
  }
  if (vol.empty() || tf.empty() || rend.empty() || w <= 0 || h <= 0 || frames <= 0 || multiscaling < 0 ||
      multiscaling > 3 || image_filter < 0 || image_filter > 5)
    return usage();

  RenderingManager mgr;
  // main.cpp:57-68: the renderers available to the manager.
  // (in its order; the null, VCT and slice-based renderers are not built)
  mgr.AddVolumeRenderer(new RayCasting1Pass());
  mgr.AddVolumeRenderer(new RayCasting1PassIsoAdapt());
  mgr.AddVolumeRenderer(new RC1PConeLightGroundTruthSteps());
  mgr.AddVolumeRenderer(new RC1PConeTracingDirOcclusionShading());
  mgr.AddVolumeRenderer(new RC1PExtinctionBasedShading());
  RC1PSurrogateShading* surr = new RC1PSurrogateShading();  // no reference counterpart
  surr->m_weights_path = weights;
  mgr.AddVolumeRenderer(surr);

  std::string err;
  if (!mgr.data.ReadVolume(vol, &err) || !mgr.data.ReadTransferFunction(tf, &err)) {
    std::fprintf(stderr, "cvr_headless: %s\n", err.c_str());
    return 2;
  }
  mgr.data.SetCurrentGradient(gradient);
  mgr.params.SetScreenSize(w, h);
  vis::Camera& cam = mgr.params.camera;
  cam.fovy = fovy;
  cam.aspect = (float)w / (float)h;
  vis::StructuredGridVolume* v = mgr.data.GetCurrentStructuredVolume();
  // CameraBehaviour default: eye at +z, distance 2 x the largest side.
  float side = (float)std::max(v->GetWidth() * v->GetScaleX(),
                               std::max(v->GetHeight() * v->GetScaleY(), v->GetDepth() * v->GetScaleZ()));
  cam.eye[0] = 0; cam.eye[1] = 0; cam.eye[2] = 2.0f * side;
  if (!cams.empty()) {
    std::vector<vis::CameraState> states;
    if (!vis::ReadCameraStates(cams, &states, &err) || cam_i < 0 || cam_i >= (int)states.size()) {
      std::fprintf(stderr, "cvr_headless: camera states: %s\n", err.empty() ? "index out of range" : err.c_str());
      return 2;
    }
    for (int k = 0; k < 3; ++k) {
      cam.eye[k] = states[cam_i].eye[k];
      cam.center[k] = states[cam_i].center[k];
      cam.up[k] = states[cam_i].up[k];
    }
  }
  if (have_eye)
    for (int k = 0; k < 3; ++k) cam.eye[k] = eye[k];
  if (!lights.empty()) {
    std::vector<vis::LightSourceList> lists;
    if (!vis::ReadLightSourceLists(lights, &lists, &err) || light_i < 0 || light_i >= (int)lists.size()) {
      std::fprintf(stderr, "cvr_headless: light lists: %s\n", err.empty() ? "index out of range" : err.c_str());
      return 2;
    }
    for (const auto& l : lists[light_i].lights) mgr.params.CreateNewLightSource(l);
  }
  if (!mgr.SetCurrentVolumeRenderer(rend)) {
    std::fprintf(stderr, "cvr_headless: %s\n", mgr.LastError().c_str());
    return 3;
  }
  if (occlusion >= 0 || shadow >= 0) {
    // Defaults of the renderer stay where a switch is not given.
    BaseVolumeRenderer* r = mgr.GetCurrentVolumeRenderer();
    r->SetIllumination(occlusion != 0, shadow != 0);
  }
  mgr.GetCurrentVolumeRenderer()->SetApplyGradientShading(gradient_shading != 0);
  mgr.GetCurrentVolumeRenderer()->SetCurrentMultiScalingMode(multiscaling);
  mgr.GetCurrentVolumeRenderer()->SetImageKernelFilter((unsigned)image_filter);
  auto t0 = std::chrono::steady_clock::now();
  for (int f = 0; f < frames; ++f) {
    if (!mgr.Display()) {
      std::fprintf(stderr, "cvr_headless: %s\n", mgr.LastError().c_str());
      return 3;
    }
  }
  std::vector<float> px;
  if (!mgr.Readback(&px)) {
    std::fprintf(stderr, "cvr_headless: %s\n", mgr.LastError().c_str());
    return 3;
  }
  double s = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  const cvr_frame_stats& st = mgr.GetCurrentVolumeRenderer()->LastStats();
  std::printf("renderer=%s frames=%d %dx%d samples=%llu shaded=%llu aux=%llu kernel_ms=%.3f wall_s=%.3f\n",
              mgr.GetCurrentVolumeRenderer()->GetAbbreviationName(), frames, w, h,
              (unsigned long long)st.samples, (unsigned long long)st.shaded_samples,
              (unsigned long long)st.aux_fetches, st.kernel_ms, s);
  if (!out.empty() && !mgr.SaveFramePFM(out)) {
    std::fprintf(stderr, "cvr_headless: %s\n", mgr.LastError().c_str());
    return 3;
  }
  return 0;
}
