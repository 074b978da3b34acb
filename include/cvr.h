/*
 * cvr.h — C ABI of the GB300-native structured volume ray caster (libcvr.so).
 *
 * This is the device boundary that replaces the reference's GLSL compute
 * dispatch.  In the reference every renderer plugin reaches the GPU through
 *   BaseVolumeRenderer::Redraw()            (cppvolrend/volrenderbase.h:49)
 *     -> gl::ComputeShader::Dispatch()      (libs/gl_utils/computeshader.cpp:120-126)
 *       -> glDispatchCompute of a *.comp shader, 8x8 work groups
 * with all state passed as uniforms / textures in Init() and Update()
 * (e.g. RayCasting1Pass::Init/Update, cppvolrend/structured/rc1pass/rc1prenderer.cpp:50-138).
 * Here the same state is uploaded once through cvr_set_* calls (the Init()
 * half) and each frame is one cvr_render call (the Update()+Redraw() half).
 *
 * Conventions
 *  - Every entry point returns cvr_status: 0 on success, a negative code on
 *    failure.  Nothing in the library calls exit(); the reference's
 *    gl::ExitOnGLError / loader exit() paths become error codes.
 *  - Handles are opaque.  The library owns every device buffer it allocates;
 *    the caller owns host buffers and any device output buffer it passes in.
 *  - A context is bound to one CUDA device and one CUDA stream.  Rendering is
 *    asynchronous on that stream unless a call says otherwise.  Contexts are
 *    thread-compatible, not thread-safe: one context per host thread.
 *  - Images are RGBA32F, row 0 = bottom row (OpenGL image convention used by
 *    imageStore in the reference shaders); pixels whose ray misses the volume
 *    are (0,0,0,0) as after RenderFrameToScreen::ClearTexture.
 *  - World space: the volume occupies the axis-aligned box
 *    [-S/2, S/2] with S = dims * spacing (ray_bbox_intersection.comp:34-52).
 */
#ifndef CVR_H
#define CVR_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CVR_ABI_VERSION 1

typedef int cvr_status;

enum cvr_status_codes {
  CVR_OK = 0,
  CVR_ERR_INVALID_ARG = -1,  /* bad pointer, size or enum value */
  CVR_ERR_NO_VOLUME = -2,    /* Init() returns false without a volume (rc1prenderer.cpp:54) */
  CVR_ERR_NOT_READY = -3,    /* a table the method needs (SAT, pyramid, cone or kernel tables) is missing */
  CVR_ERR_CUDA = -4,         /* CUDA runtime / launch error; see cvr_last_error() */
  CVR_ERR_OUT_OF_MEMORY = -5,
  CVR_ERR_IO = -6,           /* file could not be opened / was short (rawloader.cpp:16-35) */
  CVR_ERR_FORMAT = -7,       /* file content malformed */
  CVR_ERR_TIMEOUT = -8,      /* a bounded device-side wait gave up */
  CVR_ERR_UNSUPPORTED = -9
};

typedef enum cvr_dtype {
  CVR_U8 = 1,   /* DataStorageSize::_8_BITS,  normalised by 255   (structuredgridvolume.cpp:121-151) */
  CVR_U16 = 2   /* DataStorageSize::_16_BITS, normalised by 65535 */
} cvr_dtype;

typedef enum cvr_method {
  CVR_METHOD_PLAIN = 0,       /* rc1pass    : ray_marching_1p.comp */
  CVR_METHOD_EXTINCTION = 1,  /* rc1pextbsd : ebs_ray_bbox_marching.comp */
  CVR_METHOD_CONE_DOS = 2,    /* rc1pdosct  : ray_bbox_marching.comp */
  CVR_METHOD_GROUND_TRUTH = 3, /* rc1pcrtgt  : gt_ray_marching.comp (single pass) */
  CVR_METHOD_SURROGATE = 4,    /* no reference counterpart: rc1pcrtgt with the light integrals
                                  replaced by the learned network (see the surrogate section) */
  CVR_METHOD_ISO = 5           /* rc1pisoadapt: ray_marching_1p_iso_adapt.comp (first-hit isosurfaces) */
} cvr_method;

typedef struct cvr_ctx cvr_ctx;

/* Camera state: vis::CameraData (libs/vis_utils/camera.cpp:17-54) reduced to
 * what the shaders consume: eye, LookAt = glm::lookAt(eye, center, up)
 * (camera.cpp:281-284), tan(fovy/2) and aspect ratio. */
typedef struct cvr_camera {
  float eye[3];
  float center[3];
  float up[3];
  float fovy_deg;  /* reference default 45 */
  float aspect;    /* <= 0: use image width / height (Camera::UpdateAspectRatio) */
} cvr_camera;

typedef enum cvr_light_type {
  CVR_LIGHT_POINT = 0,
  CVR_LIGHT_SPOT = 1,
  CVR_LIGHT_DIRECTIONAL = 2
} cvr_light_type;

/* Light state: vis::LightSourceData (libs/volvis_utils/lightsourcelist.h:17-50).
 * forward/up/right are the light camera vectors as the renderer's shader
 * receives them (LightCamForward / LightCamUp / LightCamRight uniforms). */
typedef struct cvr_light {
  int type;            /* cvr_light_type */
  float position[3];   /* WorldLightingPos / LightSourcePosition */
  float forward[3];    /* LightCamForward: for directional lights the direction towards the light */
  float up[3];         /* LightCamUp */
  float right[3];      /* LightCamRight */
  float spot_cos_max;  /* SpotLightMaxAngle uniform (a cosine), spot lights only */
} cvr_light;

/* ---- per-method parameters (the renderers' uniforms) ------------------- */

/* RayCasting1Pass (rc1prenderer.cpp:72-138, ray_marching_1p.comp:85-178). */
typedef struct cvr_plain_params {
  float step_size;  /* StepSize, world units; Init default 0.5*|spacing|/sqrt(3) (rc1prenderer.cpp:63) */
} cvr_plain_params;

/* RC1PExtinctionBasedShading (ebsrenderer.cpp:19-247, ebs_ray_bbox_marching.comp). */
#define CVR_MAX_AO_SHELLS 32
typedef struct cvr_ext_params {
  float step_size;
  int apply_occlusion;           /* ApplyOcclusion */
  int apply_shadow;              /* ApplyShadow */
  int ao_n_shells;               /* AmbOccShells (reference default 15) */
  float ao_radii[CVR_MAX_AO_SHELLS]; /* shell radius i in voxels; reference: AmbOccRadius*(i+1) */
  float sdw_cone_angle_rad;      /* DirSdwConeAngle (default 1 degree) */
  float sdw_sample_interval;     /* DirSdwSampleInterval, voxels (default 2) */
  float sdw_initial_step;        /* DirSdwInitialStep, voxels (default 2) */
  float sdw_ui_weight;           /* DirSdwUserInterfaceWeight (default 1) */
  float sdw_max_distance;        /* DirSdwConeMaxDistance, world (default 0.75*diagonal) */
  int shadow_type;               /* TypeOfShadow: 0 point light (position), 1 directional (forward) */
  float ka, kd;                  /* Kambient, Kdiffuse (RenderingParameters defaults 0.5, 0.5) */
} cvr_ext_params;

/* RC1PConeTracingDirOcclusionShading (dosrcrenderer.cpp:134-247, ray_bbox_marching.comp). */
typedef struct cvr_dos_params {
  float step_size;
  int apply_occlusion;  /* default true */
  int apply_shadow;     /* default false (dosrcrenderer.cpp:53) */
  int shadow_type;      /* TypeOfShadow: 0 point, 1 spot, 2 directional */
  float ka, kd;
} cvr_dos_params;

/* RC1PConeLightGroundTruthSteps (crtgtrenderer.cpp:23-260, gt_ray_marching.comp). */
typedef struct cvr_gt_params {
  float step_size;
  float light_ray_initial_gap;  /* LightRayInitialGap (default 1) */
  float light_ray_step_size;    /* LightRayStepSize (default 0.5) */
  int apply_occlusion;          /* ApplyConeOcclusion */
  float occ_distance;           /* OccConeDistanceEvaluation (default 0.5*diagonal) */
  int apply_shadow;             /* ApplyConeShadow */
  float sdw_distance;           /* SdwConeDistanceEvaluation (default 0.75*diagonal) */
  int shadow_type;              /* SdwShadowType: 0 point, 1 spot, 2 directional */
  float ka, kd;
} cvr_gt_params;

/* RayCasting1PassIsoAdapt (rc1pisoadaptrenderer.cpp:10-19): adaptive steps
 * along the ray, small within step_size_range of the isovalue (normalised
 * density), large elsewhere; each crossing of the isovalue between two
 * samples is refined linearly and composited with the constant colour
 * (premultiplied), stopping at opacity 0.99.  Gradient shading is
 * ShadeBlinnPhong with cvr_set_blinn_phong's ka, kd, ks, shininess. */
typedef struct cvr_iso_params {
  float step_size_small;  /* StepSizeSmall, world units (default 0.05) */
  float step_size_large;  /* StepSizeLarge (default 1.0) */
  float step_size_range;  /* StepSizeRange (default 0.1) */
  float isovalue;         /* Isovalue, normalised density (default 0.5) */
  float color[4];         /* Color (default 0.66, 0.6, 0.05, 1) */
} cvr_iso_params;

/* Cone section table of one ConeGaussianSampler
 * (cppvolrend/structured/rc1pdosct/conegaussiansampler.cpp:179-205, 212-386).
 * sections[i] = (interval distance, mip level, d_integral, amplitude). */
#define CVR_MAX_CONE_SECTIONS 512
typedef struct cvr_cone_table {
  int n_sections;
  float sections[CVR_MAX_CONE_SECTIONS][4];
  int integration_samples[3];   /* gaussian_samples_1 / _3 / _7 */
  float axes[10][3];            /* ray3_axis[0..2], ray7_axis[0..6] */
  float initial_step;           /* OccInitialStep / SdwInitialStep */
  float ray7_adj_weight;        /* OccRay7AdjWeight / SdwRay7AdjWeight */
  float ui_weight;              /* OccUIWeight / SdwUIWeight */
} cvr_cone_table;

/* Extinction pyramid parameters (ExtinctionCoefficientVolume,
 * cppvolrend/structured/rc1pdosct/extcoefvolumegenerator.cpp:20-408). */
typedef struct cvr_pyramid_params {
  int base_dims[3];   /* custom base resolution (reference default 128^3) */
  float sigma0;       /* S0, world units (reference default 1) */
  int n_levels;       /* 0 = until a level would have size 0 (reference behaviour) */
} cvr_pyramid_params;

typedef struct cvr_frame_stats {
  uint64_t samples;         /* executed primary-ray steps (volume fetches) */
  uint64_t shaded_samples;  /* steps with extinction > 0 that went through ShadeSample */
  uint64_t aux_fetches;     /* secondary lookups: SAT box queries (extinction), pyramid
                               taps (cone; the surrogate: 67 per shaded sample),
                               light-ray volume samples (ground truth) */
  float kernel_ms;          /* device time of the render kernel (CUDA events) */
} cvr_frame_stats;

/* ---- context ------------------------------------------------------------ */
cvr_status cvr_create(cvr_ctx** out, int device);
void cvr_destroy(cvr_ctx* ctx);
/* Last error message of this context (or of the last failed cvr_create when ctx == NULL). */
const char* cvr_last_error(const cvr_ctx* ctx);
int cvr_abi_version(void);
/* Blocks until all work queued on the context stream has finished. */
cvr_status cvr_sync(cvr_ctx* ctx);
/* The CUDA stream (cudaStream_t) the context launches on. */
void* cvr_stream(cvr_ctx* ctx);

/* ---- Init() state ------------------------------------------------------- */
/* Volume upload; replaces DataManager::GenerateStructuredVolumeTexture +
 * vis::GenerateRTexture (libs/volvis_utils/utils.cpp:20-56).  Voxels stay
 * u8/u16 on the device (x fastest: x + W*y + W*H*z). */
cvr_status cvr_set_volume(cvr_ctx* ctx, const void* host_voxels, int w, int h, int d,
                          int dtype, float sx, float sy, float sz);
/* Same, from device memory already resident on this context's device. */
cvr_status cvr_set_volume_device(cvr_ctx* ctx, const void* dev_voxels, int w, int h, int d,
                                 int dtype, float sx, float sy, float sz);

/* Resident volumes (no reference counterpart: the reference's DataManager
 * holds one volume).  A context keeps up to CVR_MAX_VOLUMES volumes, each
 * with its own SAT, pyramid and texture copies; cvr_select_volume makes slot
 * s current, and the volume calls above, cvr_build_sat, cvr_build_ext_pyramid
 * and cvr_render act on the current slot.  Slot 0 is current at creation.
 * The transfer function, cone tables, GT kernel vectors and the network are
 * shared by all slots.  Batches (cvr_batch_create) name slots per job. */
#define CVR_MAX_VOLUMES 16
cvr_status cvr_select_volume(cvr_ctx* ctx, int slot);
int cvr_current_volume(cvr_ctx* ctx);

/* Transfer function tables (TransferFunction1D::GenerateTexture_1D_RGBt and
 * GenerateTexture_1D_RGBA, transferfunction1d.cpp:58-118): n entries of RGBA.
 * rgbt alpha = extinction; rgba alpha = opacity (may be NULL: derived as 1-exp(-t)). */
cvr_status cvr_set_transfer_function(cvr_ctx* ctx, const float* rgbt, const float* rgba, int n);

/* Extinction SAT (GenerateExtinctionSAT3DTex, ebsrenderer.cpp:624-723).
 * ext_per_value[v] = extinction of voxel value v (TransferFunction1D::GetExtN of
 * the normalised value), n_values = 256 (u8) or 65536 (u16).  The SAT is
 * (W+2)(H+2)(D+2), zero border, built on the device by exact int64
 * fixed-point prefix sums.  The call validates the table and uploads its
 * fixed-point values; the int64 table itself is built on the context's stream
 * by the first call that reads it (a frame the compact 32-bit table does not
 * serve, a batch, cvr_download_sat) or by cvr_prepare_sat.  Frames served by
 * the compact table never wait for it. */
cvr_status cvr_build_sat(cvr_ctx* ctx, const double* ext_per_value, int n_values);
/* Enqueues the build of a pending int64 SAT now (no-op when none is pending). */
cvr_status cvr_prepare_sat(cvr_ctx* ctx);
/* Fixed-point scale of the SAT: entry = round(sum * 2^frac_bits). */
cvr_status cvr_get_sat_info(cvr_ctx* ctx, int dims[3], int* frac_bits);
/* Copies the SAT to host memory (dims[0]*dims[1]*dims[2] int64). Synchronous. */
cvr_status cvr_download_sat(cvr_ctx* ctx, int64_t* host_out);

/* Gaussian extinction mip pyramid (gen_extcoefvol_anysize*.comp + backtotau.comp);
 * all levels together hold fewer than 2^31 values (CVR_ERR_INVALID_ARG otherwise). */
cvr_status cvr_build_ext_pyramid(cvr_ctx* ctx, const cvr_pyramid_params* params);
/* Level count and per-level dims (level_dims is [max_levels][3]). */
cvr_status cvr_get_pyramid_info(cvr_ctx* ctx, int* n_levels, int (*level_dims)[3], int max_levels);
/* Copies one level (float32, x fastest) to host memory. Synchronous. */
cvr_status cvr_download_pyramid_level(cvr_ctx* ctx, int level, float* host_out);

/* Cone tables of the occlusion and shadow samplers (BindConeOcclusionUniforms /
 * BindConeShadowUniforms, dosrcrenderer.cpp:823-990). */
cvr_status cvr_set_cone_tables(cvr_ctx* ctx, const cvr_cone_table* occlusion, const cvr_cone_table* shadow);

/* Ground-truth kernel vectors (TexOccRaysSampledVectors / TexSdwRaysSampledVectors,
 * crtgtrenderer.cpp:131-187): n x 3 floats, in the (right, up, dir) frame. */
cvr_status cvr_set_gt_kernels(cvr_ctx* ctx, const float* occ_vectors, int n_occ,
                              const float* sdw_vectors, int n_sdw);

/* ---- Update() + Redraw() ---------------------------------------------- */
/* Renders one w x h RGBA32F frame into out_rgba_dev (device memory, 16*w*h bytes).
 * params points to the method's cvr_*_params struct, params_size = sizeof it.
 * sample_counts_dev (nullable) receives the per-pixel primary step count.
 * stats (nullable): when given, the call synchronises and fills it. */
cvr_status cvr_render(cvr_ctx* ctx, int method, const cvr_camera* camera, const cvr_light* light,
                      const void* params, size_t params_size, float* out_rgba_dev, int w, int h,
                      uint32_t* sample_counts_dev, cvr_frame_stats* stats);
/* Same as cvr_render but the image lands in host memory (synchronous): the
 * RenderFrameToScreen readback path (renderingmanager.cpp:638-639). */
cvr_status cvr_render_host(cvr_ctx* ctx, int method, const cvr_camera* camera, const cvr_light* light,
                           const void* params, size_t params_size, float* out_rgba_host, int w, int h,
                           cvr_frame_stats* stats);

/* Library-owned device frame buffer of at least w*h RGBA32F pixels (the
 * headless counterpart of GetScreenTextureID, volrenderbase.h:73-75).  The
 * pointer stays valid until the next call with a larger size or cvr_destroy. */
cvr_status cvr_get_frame_buffer(cvr_ctx* ctx, int w, int h, float** dev_out);
/* Copies w*h RGBA32F pixels of a device frame (e.g. the frame buffer above)
 * to host memory; synchronous (the glGetTexImage readback of the reference). */
cvr_status cvr_download_frame(cvr_ctx* ctx, const float* dev_frame, int w, int h, float* host_out);

/* Launch configuration of the marchers (no reference counterpart: the
 * reference always dispatches 8x8 work groups, computeshader.h:37).  A CTA is
 * 2, 4 or 8 warps, each covering an 8x4 pixel block, arranged as
 * (tile_w/8) x (tile_h/4) warps: tiles 8x8, 16x8, 32x4, 8x16, 32x8 or 16x16.
 * variant selects the register budget of the kernel (0: compiler's choice,
 * 1: <= 128, 2: <= 80, 3: <= 96 registers per thread; 3 only for the
 * extinction marchers, the others treat it as 0); for CVR_METHOD_SURROGATE,
 * whose persistent launch ignores the tile, it selects the CTAs per SM (0: 4,
 * 1 and 3: as many as fit, 2: 3), the rest of the SM's shared memory serving
 * as cache.  Results do not depend on the choice. */
cvr_status cvr_set_tuning(cvr_ctx* ctx, int tile_w, int tile_h, int variant);
cvr_status cvr_get_tuning(cvr_ctx* ctx, int* tile_w, int* tile_h, int* variant);
/* Storage of the volume the marchers read: 0 = the plain x-fastest array,
 * else bricks of edge^3 voxels (edge 4, 8, 16 or 32; bricks x-fastest, voxels
 * x-fastest inside a brick), a copy made on the first frame after the volume
 * or the size changed.  Results do not depend on it. */
cvr_status cvr_set_brick_size(cvr_ctx* ctx, int edge);
int cvr_get_brick_size(cvr_ctx* ctx);
/* Volume layout of the marchers' FP32 samples (no reference counterpart):
 * CVR_LAYOUT_QUADS keeps copies of the volume and of the extinction pyramid
 * where each cell holds the 2 x 2 values of its x-y neighbourhood (4 x the
 * volume's bytes, 16 bytes per pyramid value), so a trilinear sample is two
 * loads instead of eight; results are bit-identical to the plain layout.
 * It takes precedence over bricks; the autotuner tries it with them. */
/* Warp shape of the marchers' pixel tiles (no reference counterpart): 4, 8
 * (default) or 16 pixels per warp row (warps of 4x8, 8x4 or 16x2 pixels),
 * used where the tile holds whole warps of that shape (8x4 otherwise); same
 * images.  The autotuner tries 4 and 16 at its best tile. */
cvr_status cvr_set_warp_shape(cvr_ctx* ctx, int warp_w);
int cvr_get_warp_shape(cvr_ctx* ctx);
/* Persistent ray refill (no reference counterpart; default off): the plain,
 * extinction, cone and ground-truth marchers run as persistent CTAs of 128
 * threads whose lanes each advance their own ray to its next shaded sample,
 * shade together, and take the next ray of the frame (8x4-pixel tiles in a
 * spiral around the projected volume centre) when theirs ends; a warp leaves
 * when a ballot finds no lane with a ray.  Same images; the tile shape does
 * not apply.  The autotuner tries it at every register variant. */
cvr_status cvr_set_ray_refill(cvr_ctx* ctx, int enable);
int cvr_get_ray_refill(const cvr_ctx* ctx);
/* Shared-memory brick staging for CVR_METHOD_PLAIN (no reference counterpart;
 * default off): 16x8-pixel tiles marched slab by slab along the ray, each
 * slab's voxel box loaded into shared memory once and sampled from there.
 * Plain volume layout, FP32 samples and transfer functions of at most 512
 * entries only (otherwise ignored); same images.  The autotuner tries it for
 * the plain method. */
cvr_status cvr_set_brick_staging(cvr_ctx* ctx, int enable);
int cvr_get_brick_staging(const cvr_ctx* ctx);
#define CVR_LAYOUT_PLAIN 0
#define CVR_LAYOUT_QUADS 1
cvr_status cvr_set_volume_layout(cvr_ctx* ctx, int layout);
int cvr_get_volume_layout(cvr_ctx* ctx);
/* Compact SAT (no reference counterpart; default on): frames of
 * CVR_METHOD_EXTINCTION whose box queries all span a bounded region (the
 * ambient-occlusion boxes and, for directional shadows, the per-frame cone
 * boxes) read a 32-bit copy of the SAT: prefix sums of round(sigma * 2^F32)
 * modulo 2^32, F32 chosen per frame so that every sub-box sum stays below
 * 2^31 and its wrapped differences are exact, stored as x-y quads (the four
 * taps of a plane in one load).  Frames where that would resolve the largest
 * extinction in fewer than 2^15 steps (very large boxes), point-light cones
 * too wide to bound (lean + angle >= 90 degrees) and the light cache keep the
 * int64 table; batches build their own.  0 disables it. */
cvr_status cvr_set_compact_sat(cvr_ctx* ctx, int enable);
int cvr_get_compact_sat(cvr_ctx* ctx);
/* Walk tables (no reference counterpart; default on): a frame on the compact
 * SAT whose directional-shadow boxes all have integer widths (the sample
 * interval along the walk axis, ceil-rounded cross-sections) reads a second
 * table for its shadow queries: the compact sums differenced along the walk
 * axis by the interval, 32 bytes per cell (8 x the volume's cells x 4 bytes),
 * built on the first frame that needs it and kept until the SAT, the walk
 * axis or the interval changes.  A shadow box is then four 32-byte loads
 * instead of sixteen 16-byte ones; same images.  0 disables it. */
cvr_status cvr_set_walk_tables(cvr_ctx* ctx, int enable);
int cvr_get_walk_tables(const cvr_ctx* ctx);

/* Object-space light cache (PreIlluminationStructuredVolume,
 * cppvolrend/utils/preillumination.h:15-47; reference default 32^3, off):
 * when on, CVR_METHOD_EXTINCTION and CVR_METHOD_CONE_DOS evaluate occlusion
 * and shadow once per frame at the centres of a w x h x d grid
 * (lightcachecomputation.comp of rc1pextbsd / rc1pdosct) and shade every
 * sample from a trilinear lookup of it (obj_ray_marching.comp, which, like
 * the reference, composites nothing when both terms are off).  0,0,0 = off.
 * The cache is stored as FP32 pairs (the reference: RG16F). */
cvr_status cvr_set_light_cache(cvr_ctx* ctx, int w, int h, int d);
/* The last frame's cache: (occlusion, shadow) per cell, x fastest; synchronous. */
cvr_status cvr_download_light_cache(cvr_ctx* ctx, float* host_out, size_t n_floats);
/* Autotuner: renders the given frame with every tile shape x register variant
 * (reps timed frames each, CUDA events, L2 flushed before each), then the
 * 4x8 and 16x2 warp shapes, every brick size and the quad layout at the best
 * of those, then the persistent ray-refill marcher at every register variant
 * (plain, extinction, cone, ground truth) and, for the plain method, brick
 * staging; keeps the fastest configuration on the context and reports it
 * (cvr_get_warp_shape, cvr_get_brick_size, cvr_get_volume_layout,
 * cvr_get_ray_refill and cvr_get_brick_staging report the rest).  best_ms may
 * be NULL. */
cvr_status cvr_autotune(cvr_ctx* ctx, int method, const cvr_camera* camera, const cvr_light* light,
                        const void* params, size_t params_size, int w, int h, int reps,
                        int* best_tile_w, int* best_tile_h, int* best_variant, float* best_ms);

/* Sampling of secondary lookups (no reference counterpart; the reference's GL
 * texture() fetches are hardware-filtered, the FP32 hand-written trilinear is
 * this project's exact form).  CVR_SAMPLING_TEX_FEATURES: the surrogate
 * network's inputs (the pyramid taps) go
 * through the texture unit (trilinear filtering with 8-bit interpolation
 * weights, |input error| below 3e-2) instead of the FP32 trilinear; the
 * default, since the network's inputs dominate a surrogate frame; the
 * pyramid is read as FP16 there, as the reference stores it).
 * CVR_SAMPLING_TEX_VOLUME: the primary volume samples of every marcher (and
 * the ground truth's light rays) through the texture unit; images within
 * 1/255 of the FP32 path.  A network is best used with the flags it was
 * trained with. */
#define CVR_SAMPLING_TEX_FEATURES 1
#define CVR_SAMPLING_TEX_VOLUME 2
/* CVR_SAMPLING_TEX_PYRAMID: the cone method's pyramid taps through the
 * texture unit from FP16 level textures (the reference's R16F pyramid and
 * GL_LINEAR_MIPMAP_LINEAR filtering, with 8-bit interpolation weights). */
#define CVR_SAMPLING_TEX_PYRAMID 4
cvr_status cvr_set_sampling(cvr_ctx* ctx, int flags);
int cvr_get_sampling(cvr_ctx* ctx);

/* ---- pixel multiscaling --------------------------------------------------------
 * BaseVolumeRenderer::MULTISCALING (cppvolrend/volrenderbase.h:28-33) with
 * RenderFrameToScreen's post-passes (libs/vis_utils/renderoutputframe.cpp:
 * 265-539, and the shader/renderoutputframe compute shaders), run on the device after the
 * marcher: MULTISAMPLE renders factor_w x factor_h times the output size and
 * takes a bilinear lookup per output pixel; DOWNSCALE renders at that size
 * and filters down with the kernel; UPSCALE renders at the output size divided
 * by the factors (integer division) and filters up.  The cardinal B-spline
 * and OMOMS kernels add their recursive digital filter (rows then columns) on
 * the output (down) or on the generated frame (up).  The reference's factors
 * are 2 x 2 (MULTISAMPLE_NUMBEROFSAMPLES_W/H, cppvolrend/defines.h:16-17) and
 * its kernel K2_HAT (renderoutputframe.cpp:34).  Applies to cvr_render /
 * cvr_render_host of every method (the per-pixel step counts are then not
 * available); not to batches. */
#define CVR_MULTISCALE_SINGLE 0       /* SINGLE_RAY_PER_PIXEL (default) */
#define CVR_MULTISCALE_MULTISAMPLE 1  /* MULTIPLE_RAYS_PER_PIXEL */
#define CVR_MULTISCALE_DOWNSCALE 2    /* DOWN_SCALING_RENDER */
#define CVR_MULTISCALE_UPSCALE 3      /* UP_SCALING_RENDER */
/* IMAGE_FILTER_KERNEL (libs/vis_utils/filters/utils.hpp:8-15) */
#define CVR_FILTER_BOX 0
#define CVR_FILTER_HAT 1
#define CVR_FILTER_CATMULL_ROM 2
#define CVR_FILTER_MITCHELL_NETRAVALI 3
#define CVR_FILTER_CARDINAL_BSPLINE3 4
#define CVR_FILTER_CARDINAL_OMOMS3 5
cvr_status cvr_set_multiscaling(cvr_ctx* ctx, int mode, int kernel, int factor_w, int factor_h);
cvr_status cvr_get_multiscaling(cvr_ctx* ctx, int* mode, int* kernel, int* factor_w, int* factor_h);
/* The post-pass alone: src (sw x sh RGBA32F, device; not modified) to dst
 * (w x h, device) with mode MULTISAMPLE / DOWNSCALE / UPSCALE and a kernel. */
cvr_status cvr_rescale_frame(cvr_ctx* ctx, int mode, int kernel, const float* src_dev, int sw, int sh,
                             float* dst_dev, int w, int h);

/* ---- gradient Blinn-Phong shading -------------------------------------------
 * Gradient models: DataManager::STRUCTURED_GRADIENT_TYPE
 * (libs/volvis_utils/datamanager.h:64-69, default NONE_GRADIENT). */
#define CVR_GRADIENT_SOBEL_FELDMAN 0       /* GenerateSobelFeldmanGradientTexture (libs/volvis_utils/utils.cpp:287-351) */
#define CVR_GRADIENT_FINITE_DIFFERENCES 1  /* GenerateGradientTexture (utils.cpp:146-284) */
#define CVR_GRADIENT_COMPUTE_SOBEL 2       /* GenerateGradientWithComputeShader (datamanager.cpp:623-700) */
#define CVR_GRADIENT_NONE 3
typedef struct cvr_gradient_params {
  int model;          /* CVR_GRADIENT_* */
  int sample_size;    /* gradient_sample_size, finite differences only (default 1) */
  int filter_nxnxn;   /* filter_nxnxn, finite differences only (default 0) */
  int normalized;     /* normalized_gradient, finite differences only (default 1) */
} cvr_gradient_params;
/* Builds the current volume's per-voxel gradient on the device (stored as
 * FP16 x, y, z like the reference's RGB16F texture) and keeps the model: a
 * later cvr_set_volume into this slot rebuilds it on the next shaded frame, as
 * DataManager regenerates it with each volume (datamanager.cpp:326-327).
 * params NULL or model CVR_GRADIENT_NONE drops it. */
cvr_status cvr_build_gradient(cvr_ctx* ctx, const cvr_gradient_params* params);
/* The gradient as 3 floats per voxel (x fastest); synchronous. */
cvr_status cvr_download_gradient(cvr_ctx* ctx, float* host_xyz, size_t n_floats);
/* Device builder of the 3x3x3 stencils (Sobel-Feldman, compute Sobel and
 * finite differences of sample size 1; no reference counterpart, all give the
 * same values): AUTO streams the volume's planes through the tensor memory
 * accelerator when the row pitch (width x voxel bytes) is a multiple of 16
 * bytes and falls back to TILED (plain loads into a shared-memory ring)
 * otherwise; GENERIC is one thread per voxel straight from global memory
 * (always used for finite differences of sample size > 1).
 * cvr_get_gradient_kernel reports the builder the last build ran
 * (CVR_GRADIENT_KERNEL_TMA, _TILED or _GENERIC; -1 before any build). */
#define CVR_GRADIENT_KERNEL_AUTO 0
#define CVR_GRADIENT_KERNEL_TILED 1
#define CVR_GRADIENT_KERNEL_GENERIC 2
#define CVR_GRADIENT_KERNEL_TMA 3
cvr_status cvr_set_gradient_kernel(cvr_ctx* ctx, int kernel);
int cvr_get_gradient_kernel(cvr_ctx* ctx);
/* RenderingParameters' Blinn-Phong terms (renderingparameters.cpp:23-26,
 * lightsourcelist.cpp:24) and the renderers' "Apply Gradient Shading" switch
 * (m_apply_gradient_shading, default off).  When apply is set and the volume
 * has a gradient, every method shades with the gradient branch of its
 * ShadeSample: plain ShadeBlinnPhong (ray_marching_1p.comp:48-81, with ka,
 * kd here), extinction and the light cache (ebs_ray_bbox_marching.comp:524-546,
 * obj_ray_marching.comp:111-129), cone (ray_bbox_marching.comp:630-648),
 * ground truth and surrogate (gt_ray_marching.comp:277-295, specular colour
 * 1).  The light position is cvr_light.position (a light is then required). */
typedef struct cvr_blinn_phong {
  int apply;           /* default 0 */
  float ka, kd;        /* BlinnPhongKa / Kd (0.5, 0.5): the plain renderer's; the others use their params' */
  float ks;            /* BlinnPhongKs / Kspecular (0.8) */
  float shininess;     /* BlinnPhongShininess / Nshininess (30) */
  float specular[3];   /* light source specular colour, Ispecular (1, 1, 1) */
} cvr_blinn_phong;
cvr_status cvr_set_blinn_phong(cvr_ctx* ctx, const cvr_blinn_phong* bp);
cvr_status cvr_get_blinn_phong(cvr_ctx* ctx, cvr_blinn_phong* out);

/* ---- batched rendering ------------------------------------------------------
 * No reference counterpart (the reference renders one view per Redraw()).
 * A batch is a fixed list of frames over the resident volumes, views and
 * lights, rendered by persistent launches (CVR_METHOD_EXTINCTION: one over
 * all its jobs; CVR_METHOD_SURROGATE: one per 32 jobs, their descriptors the
 * launch's parameters; other methods are rejected) whose CTAs take ray tiles
 * of their jobs from one work counter per launch, longest jobs first.  The
 * launches, with the resets of their counters, are captured in one CUDA
 * graph at creation; cvr_batch_run replays it.  Every image equals the image
 * of the same job rendered alone by cvr_render with the context's tuning at
 * creation.  Jobs keep pointers to their output buffers; the volumes, tables
 * and network they use must not change while the batch exists (re-create it). */
typedef struct cvr_job {
  int volume;           /* volume slot */
  int method;           /* CVR_METHOD_EXTINCTION or CVR_METHOD_SURROGATE */
  const void* params;   /* cvr_ext_params or cvr_gt_params, copied at creation */
  size_t params_size;
  cvr_camera camera;
  cvr_light light;
  int width, height;
  float* out_rgba_dev;  /* device frame of 16 * width * height bytes */
} cvr_job;

typedef struct cvr_batch cvr_batch;
cvr_status cvr_batch_create(cvr_ctx* ctx, const cvr_job* jobs, int n_jobs, cvr_batch** out);
/* One replay of the batch's graph on the context stream (asynchronous). */
cvr_status cvr_batch_run(cvr_batch* batch);
/* Step counts of job j from the last run (synchronises). */
cvr_status cvr_batch_job_stats(cvr_batch* batch, int job, cvr_frame_stats* out);
void cvr_batch_destroy(cvr_batch* batch);

/* ---- device timing on the context stream --------------------------------- */
cvr_status cvr_timer_start(cvr_ctx* ctx);
/* Records the stop event, synchronises and returns elapsed milliseconds. */
cvr_status cvr_timer_stop(cvr_ctx* ctx, float* ms);
/* Writes a device buffer larger than L2 (flushes the L2 cache) on the stream. */
cvr_status cvr_flush_l2(cvr_ctx* ctx);
/* Measured L1 hit bandwidth (GB/s, whole GPU) of coalesced 16-byte
 * non-coherent loads, the load instruction of the marchers' quad gathers: the
 * denominator of their roofline (their tables are cache-resident).  No
 * reference counterpart (the reference reports no roofline).  Synchronises. */
cvr_status cvr_measure_l1_bandwidth(cvr_ctx* ctx, float* gbs);

/* ---- learned occlusion / shadow surrogate ---------------------------------
 * No reference counterpart: a small MLP that stands in for the ray-traced
 * ground-truth integrator (RC1PConeLightGroundTruthSteps).  48 inputs ->
 * 64 -> 64 -> 2 outputs (ambient occlusion, shadow), ReLU hidden layers, BF16
 * operands with FP32 accumulation on the tensor cores.  Parameter vector
 * (FP32, CVR_MLP_PARAMS floats): W1[64][48], b1[64], W2[64][64], b2[64],
 * W3[2][64], b3[2] with W[out][in]. */
#define CVR_MLP_INPUTS 48
#define CVR_MLP_HIDDEN 64
#define CVR_MLP_OUTPUTS 2
#define CVR_MLP_PARAMS 7426

/* He-uniform weights from a seed, zero biases, fresh Adam state. */
cvr_status cvr_mlp_init(cvr_ctx* ctx, uint64_t seed);
cvr_status cvr_mlp_set_params(cvr_ctx* ctx, const float* params, int n);
cvr_status cvr_mlp_get_params(cvr_ctx* ctx, float* params, int n);
/* Batch inference of n points (host buffers: x n*48, y n*2). Synchronous. */
cvr_status cvr_mlp_forward(cvr_ctx* ctx, const float* x, int n, float* y);
/* Gradient of L = 1/(2n) sum (y - t)^2 over n points w.r.t. every parameter,
 * without updating them (grad: CVR_MLP_PARAMS floats).  Synchronous. */
cvr_status cvr_mlp_gradients(cvr_ctx* ctx, const float* x, const float* t, int n, float* grad, float* loss);
/* The same gradient from device buffers without allocating any memory (no
 * counterpart in the reference).  x_dev: n*48 floats, t_dev: n*2, grad_dev:
 * CVR_MLP_PARAMS floats, loss_dev: 1 float (nullable); all device memory of
 * the context's device.  Asynchronous on the context stream.  For callers that
 * must not allocate device memory inside their loop (memory held by another
 * allocator, or loops where an allocation's synchronisation would stall).
 * The scratch is one fixed array per device of about 1.9 MB shared by every
 * context on that device, so calls that overlap in time (other threads or
 * streams) race on it.  The first call on a device sets the scratch up (its
 * address, an index list written by a kernel) and synchronises the context
 * stream, so make that first call before any stream capture begins; the
 * set-up is per process and is not redone after cudaDeviceReset.  n above
 * CVR_MLP_NOALLOC_MAX_POINTS is an invalid argument.  The call returns before
 * its kernels run, so a tensor-core wait that gives up inside them (the
 * kernels' bounded mbarrier waits) cannot show in its return value: it is
 * reported by the next cvr_mlp_check (or the next synchronous network call)
 * on the context, which reads and clears the flag. */
#define CVR_MLP_NOALLOC_MAX_POINTS 8192
cvr_status cvr_mlp_gradients_noalloc(cvr_ctx* ctx, const float* x_dev, const float* t_dev, int n, float* grad_dev,
                                     float* loss_dev);
/* Synchronises the context stream and reports (then clears) a tensor-core
 * wait that gave up in an asynchronous network call: CVR_ERR_TIMEOUT, else
 * CVR_OK.  Allocates nothing. */
cvr_status cvr_mlp_check(cvr_ctx* ctx);
/* Training set from host memory (features n*48, targets n*2); n = 0 clears it. */
cvr_status cvr_mlp_set_training_data(cvr_ctx* ctx, const float* x, const float* t, int n);
cvr_status cvr_mlp_get_training_data(cvr_ctx* ctx, float* x, float* t, int n);
int cvr_mlp_training_size(cvr_ctx* ctx);
/* Adam over the training set: epochs x ceil(n/batch) steps (batch a multiple
 * of 128); each epoch is one replay of a captured CUDA graph.
 * loss_per_epoch (nullable) receives the mean batch loss of every epoch. */
cvr_status cvr_mlp_train(cvr_ctx* ctx, int epochs, int batch, float lr, uint64_t seed, float* loss_per_epoch);
/* Checkpoint: parameters, Adam moments and step in a versioned binary file
 * ("CVRMLP01", u32 version 1, u32 CVR_MLP_PARAMS, params, m, v as FP32, i32 step). */
cvr_status cvr_mlp_save(cvr_ctx* ctx, const char* path);
cvr_status cvr_mlp_load(cvr_ctx* ctx, const char* path);

/* ---- surrogate shading ----------------------------------------------------
 * CVR_METHOD_SURROGATE renders the image of RC1PConeLightGroundTruthSteps
 * (method params: cvr_gt_params; step_size, apply_occlusion, apply_shadow,
 * shadow_type, ka, kd are used, the light-ray fields describe the integrator
 * the network was trained against) with the per-sample occlusion and shadow
 * integrals replaced by the network, evaluated on the tensor cores inside the
 * marcher.  It needs a network (cvr_mlp_init / _set_params / _load / _train)
 * and an extinction pyramid with at least CVR_SURROGATE_LEVELS levels whose
 * base is half the volume resolution (the configuration the features are
 * defined on).
 *
 * Network inputs at a shading point (texture-space position p, primary ray
 * direction dir), in the frame n = -dir, r = normalize(dir x (0,1,0)),
 * u = normalize(-dir x r) of the ground-truth occlusion kernel:
 *   x[7l+k], l = 0..5, k = 0..6: 1 - exp(-sigma_l(p + o_k) d_l), with
 *     d_l = 2^(l+1) voxels, sigma_l pyramid level l (0 outside the volume),
 *     L the direction towards the light and offsets o_0 = 0, o_3 = n d_l,
 *     o_4 = 3 n d_l; k = 5 and 6 take the mean extinction of the taps at
 *     +-r d_l and +-u d_l; and the light taps k = 1,
 *     2: the segments [2 d_l - 4, 3 d_l - 4] and [3 d_l - 4, 4 d_l - 4]
 *     (voxels) of the light ray p + L s (the twelve partition [0, 252]),
 *     clipped to t_end = min(box exit, sdw_distance):
 *     1 - exp(-sigma_l(midpoint) * clipped length), 0 when empty; and
 *     x[35]: the same over the rest of the ray, the eight level-5 segments
 *     [(4+j) d_5 - 4, (5+j) d_5 - 4], j < 8 (252 ... 764 voxels), summed;
 *   x[42..44] = L in (r, u, n); x[45..47] = gradient of pyramid level 0
 *     (central differences at +-1 voxel, times the voxel length) in (r, u, n).
 * Outputs: (ambient occlusion, shadow) as the ground-truth integrator defines
 * them (gt_ray_marching.comp:109-252), clamped to [0, 1] when shading. */
#define CVR_SURROGATE_LEVELS 6

/* Shading points of one frame: every shaded sample of the primary rays (the
 * samples that reach ShadeSample) is kept with probability rate and appended
 * to the context's point list (position in texture space [0, S], primary ray
 * direction), which holds at most max_points.  n_added (nullable) receives
 * the number appended. */
cvr_status cvr_surrogate_collect(cvr_ctx* ctx, const cvr_camera* camera, int w, int h, float step_size,
                                 float rate, uint64_t seed, int max_points, int* n_added);
cvr_status cvr_surrogate_clear_points(cvr_ctx* ctx);
int cvr_surrogate_point_count(cvr_ctx* ctx);
/* Point list from / to host memory: n x 6 floats (px, py, pz, dx, dy, dz). */
cvr_status cvr_surrogate_set_points(cvr_ctx* ctx, const float* points, int n);
cvr_status cvr_surrogate_get_points(cvr_ctx* ctx, float* points, int n);
/* Network inputs (n x 48) and ground-truth targets (n x 2: occlusion and
 * shadow of the GT integrator with the context's kernel vectors, whatever the
 * apply flags say) of the n points of the list.  x_host / t_host (nullable)
 * receive them; append_training != 0 appends them to the network's training
 * set on the device. */
cvr_status cvr_surrogate_label(cvr_ctx* ctx, const cvr_light* light, const cvr_gt_params* params,
                               int append_training, float* x_host, float* t_host, int n);
/* Error against the ground-truth integrator over the point list.
 * out[0], out[1]: RMSE of the network's (occlusion, shadow) as used in shading;
 * out[2], out[3]: RMSE of the cone method (cvr_dos_params; needs cone tables)
 * when cone != NULL, else 0; out[4]: points; out[5], out[6]: mean GT
 * occlusion and shadow; out[7]: largest absolute occlusion error of the network. */
cvr_status cvr_surrogate_evaluate(cvr_ctx* ctx, const cvr_light* light, const cvr_gt_params* params,
                                  const cvr_dos_params* cone, double out[8]);

/* ---- host-side helpers (no GPU needed) ------------------------------------ */
/* TransferFunction1D::BuildLinear over control points (transferfunction1d.cpp:319-358)
 * followed by GenerateTexture_1D_RGBt / _RGBA; tables hold max_density+1 entries. */
cvr_status cvr_tf_build_linear(int max_density, int n_rgb, const double* rgb_points /* r,g,b,iso */,
                               int n_alpha, const double* alpha_points /* a,iso */,
                               int extinction_input, float* rgbt_out, float* rgba_out);
/* TransferFunction1D::GetExtN for every voxel value of a dtype (the SAT input). */
cvr_status cvr_tf_ext_per_value(int max_density, int n_rgb, const double* rgb_points,
                                int n_alpha, const double* alpha_points, int extinction_input,
                                int dtype, double* out /* 256 or 65536 */);
/* .tf1d reader (readtf1d, libs/volvis_utils/reader.cpp:744-814): returns control points. */
cvr_status cvr_read_tf1d(const char* path, int* max_density, int* extinction_input,
                         int* n_rgb, double* rgb_points, int max_rgb,
                         int* n_alpha, double* alpha_points, int max_alpha);
/* Volume file header: dims, dtype and voxel spacing, by extension as
 * VolumeReader::ReadStructuredVolume (reader.cpp:28-58): .raw (name convention
 * "name.<bytes>.<W>x<H>x<D>.raw", reader.cpp:162-225), .syn (reader.cpp:283-371),
 * .pvm / .pvmold (V^3 PVM, plain or DDS-compressed, readpvm reader.cpp:100-160),
 * .nrrd / .nhrd (detached header, reader.cpp:373-496), .dat (reader.cpp:498-628).
 * CVR_ERR_IO: missing or short file; CVR_ERR_FORMAT: malformed;
 * CVR_ERR_UNSUPPORTED: other extensions. */
cvr_status cvr_read_volume_info(const char* path, int dims[3], int* dtype, float spacing[3]);
/* Reads the voxels into host_out (W*H*D*bytes). */
cvr_status cvr_read_volume(const char* path, void* host_out, size_t out_bytes);
/* ConeGaussianSampler::ComputeConeIntegrationSteps (conegaussiansampler.cpp:212-386). */
cvr_status cvr_cone_sampler_build(float cone_half_angle_deg, int max_packing /* 0:1, 1:3, 2:7 */,
                                  float covered_distance, float initial_step, float ui_weight,
                                  double min_sigma, cvr_cone_table* out);
/* GT kernel vectors (crtgtrenderer.cpp:131-187): one std::default_random_engine
 * (libstdc++ minstd_rand0, seeded with 'seed'; the reference uses the default
 * seed 1) draws the n_occ occlusion vectors and then the n_sdw shadow vectors. */
cvr_status cvr_gt_kernel_vectors(int n_occ, float occ_aperture_deg, int n_sdw, float sdw_aperture_deg,
                                 unsigned int seed, float* occ_xyz, float* sdw_xyz);

/* Page-locked host memory for asynchronous copies (cudaHostAlloc / cudaFreeHost). */
cvr_status cvr_host_alloc_pinned(size_t bytes, void** out);
void cvr_host_free_pinned(void* p);

/* Seeded synthetic volumes used by the benchmark configurations. */
cvr_status cvr_synth_blobs(void* host_out, int w, int h, int d, int dtype, int n_blobs,
                           uint64_t seed, float noise_max);
cvr_status cvr_synth_value_noise(void* host_out, int w, int h, int d, int dtype, int octaves,
                                 float lacunarity, float gain, int shells, uint64_t seed);

#ifdef __cplusplus
}
#endif

#endif /* CVR_H */
