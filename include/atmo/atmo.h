/*
 * atmo.h -- C ABI of the GB300-native atmosphere LUT precomputation.
 *
 * Drop-in boundary for the precomputation path of
 * ebruneton/precomputed_atmospheric_scattering:
 *
 *   reference (C++ / OpenGL)                          this ABI
 *   -----------------------------------------------  ------------------------------
 *   DensityProfileLayer        atmosphere/model.h:165-178   atmo_density_layer
 *   Model::Model(19 params)    atmosphere/model.h:182-281   atmo_model_create
 *   Model::~Model              atmosphere/model.cc:801-811  atmo_model_destroy
 *   Model::Init(orders)        atmosphere/model.h:285       atmo_model_init
 *   Model::shader()            atmosphere/model.h:287       atmo_model_shader_source
 *   Model::SetProgramUniforms  atmosphere/model.h:289-294   atmo_model_get_lut (device
 *                                                          buffers; GL binding is
 *                                                          unavailable on this machine)
 *   Model::ConvertSpectrumToLinearSrgb  model.h:301-304    atmo_convert_spectrum_to_linear_srgb
 *   kLambdaR/G/B               atmosphere/model.h:306-308   ATMO_LAMBDA_R/G/B
 *   texture sizes              atmosphere/constants.h:47-61 atmo_lut_shape
 *   glGetTexImage read-back    atmosphere/demo/webgl/precompute.cc:63-72
 *                                                          atmo_model_read_lut
 *   shader API (GLSL)          atmosphere/model.cc:221-281, functions.glsl:1633-1896
 *     GetSolarRadiance/Luminance                          atmo_solar_radiance
 *     GetSkyRadiance/Luminance                            atmo_sky_radiance
 *     GetSkyRadiance/LuminanceToPoint                     atmo_sky_radiance_to_point
 *     GetSunAndSkyIrradiance/Illuminance                  atmo_sun_and_sky_irradiance
 *     (a demo-style pinhole view of all three)            atmo_shade_view
 *
 * All entry points return an atmo_status.  Plain C types only: device
 * pointers are exported as integers/void*, streams as opaque pointers that
 * are CUDA cudaStream_t values (NULL = the legacy default stream).
 *
 * Threading: one model / batch / server object per host thread, or an
 * external lock; work is ordered on the stream given to each call.
 */
#ifndef ATMO_ATMO_H_
#define ATMO_ATMO_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ATMO_ABI_VERSION 3

#define ATMO_LAMBDA_R 680.0
#define ATMO_LAMBDA_G 550.0
#define ATMO_LAMBDA_B 440.0

typedef struct CUstream_st* atmo_stream;

typedef enum {
  ATMO_OK = 0,
  ATMO_INVALID_ARG = 1,   /* NULL pointer, bad size, NaN or inconsistent parameter */
  ATMO_OOM = 2,           /* device or host allocation failed */
  ATMO_CUDA_ERROR = 3,    /* a CUDA runtime call failed; see atmo_last_error() */
  ATMO_TIMEOUT = 4,       /* a bounded wait ran out */
  ATMO_BUDGET = 5,        /* the request does not fit the device-memory budget */
  ATMO_UNAVAILABLE = 6,   /* feature not available here (e.g. OpenGL interop) */
  ATMO_NOT_READY = 7,     /* LUTs requested before Init */
  ATMO_CANCELLED = 8      /* a serving request cancelled by atmo_server_cancel */
} atmo_status;

/* atmosphere/model.h:165-178: density = exp_term*exp(exp_scale*h)
   + linear_term*h + constant_term, clamped to [0,1]; h and width in m,
   exp_scale and linear_term in 1/m. */
typedef struct {
  double width, exp_term, exp_scale, linear_term, constant_term;
} atmo_density_layer;

/* The 19 constructor parameters of atmosphere/model.h:182-281.  Spectral
   arrays have num_wavelengths entries, sampled at `wavelengths` (nm, sorted). */
typedef struct {
  const double* wavelengths;
  unsigned num_wavelengths;
  const double* solar_irradiance;              /* W/m^2/nm */
  double sun_angular_radius;                   /* rad */
  double bottom_radius;                        /* m */
  double top_radius;                           /* m */
  const atmo_density_layer* rayleigh_density;  /* 1 or 2 layers, bottom first */
  unsigned num_rayleigh_layers;
  const double* rayleigh_scattering;           /* 1/m */
  const atmo_density_layer* mie_density;
  unsigned num_mie_layers;
  const double* mie_scattering;                /* 1/m */
  const double* mie_extinction;                /* 1/m */
  double mie_phase_function_g;
  const atmo_density_layer* absorption_density;
  unsigned num_absorption_layers;
  const double* absorption_extinction;         /* 1/m */
  const double* ground_albedo;
  double max_sun_zenith_angle;                 /* rad */
  double length_unit_in_meters;
  unsigned num_precomputed_wavelengths;        /* <= 3: radiance; > 3: luminance */
  int combine_scattering_textures;
  int half_precision;
} atmo_model_params;

/* LUT sizes (atmosphere/constants.h:47-61) as run-time values.  A NULL shape
   selects the reference's defaults: 256x64, NU 8 x MU_S 32 x MU 128 x R 32,
   64x16.  scattering_mu must be even and every size >= 2. */
typedef struct {
  int transmittance_width, transmittance_height;
  int scattering_r, scattering_mu, scattering_mu_s, scattering_nu;
  int irradiance_width, irradiance_height;
} atmo_lut_shape;

/* One precomputation group's atmosphere (atmosphere/definitions.glsl:205-255)
   at 3 wavelengths, already in length units: what the reference bakes into
   its GLSL header (atmosphere/model.cc:716-744). */
typedef struct {
  atmo_density_layer layers[2];
} atmo_density_profile;

typedef struct {
  double solar_irradiance[3];
  double sun_angular_radius;
  double bottom_radius;
  double top_radius;
  atmo_density_profile rayleigh_density;
  double rayleigh_scattering[3];
  atmo_density_profile mie_density;
  double mie_scattering[3];
  double mie_extinction[3];
  double mie_phase_function_g;
  atmo_density_profile absorption_density;
  double absorption_extinction[3];
  double ground_albedo[3];
  double mu_s_min;
} atmo_atmosphere;

typedef enum {
  ATMO_LUT_TRANSMITTANCE = 0,   /* 2D W_T x H_T, float32 RGBA */
  ATMO_LUT_SCATTERING = 1,      /* 3D (NU*MU_S) x MU x R, float32 or float16 RGBA */
  ATMO_LUT_SINGLE_MIE = 2,      /* same layout; only when not combined */
  ATMO_LUT_IRRADIANCE = 3       /* 2D W_I x H_I, float32 RGBA */
} atmo_lut_kind;

typedef enum { ATMO_DTYPE_F32 = 0, ATMO_DTYPE_F16 = 1 } atmo_dtype;

typedef struct {
  void* device_ptr;        /* RGBA texels, x fastest, then y, then z */
  int width, height, depth;
  atmo_dtype dtype;
  size_t bytes;
} atmo_lut_view;

/* Kernel implementation used by Init: the plain per-texel kernels (the
   reference's per-fragment structure) or the restructured fast kernels. */
typedef enum { ATMO_PATH_FAST = 0, ATMO_PATH_PLAIN = 1 } atmo_path;

typedef struct atmo_model atmo_model;
typedef struct atmo_batch atmo_batch;
typedef struct atmo_lut_set atmo_lut_set;
typedef struct atmo_server atmo_server;

/* ---- library --------------------------------------------------------------- */
int atmo_abi_version(void);
/* Message of the last failing call on this host thread (never NULL). */
const char* atmo_last_error(void);
/* Waits for the work enqueued on `stream` (cudaStreamSynchronize). */
atmo_status atmo_synchronize(atmo_stream stream);

/* ---- Model (atmosphere/model.h) ------------------------------------------- */
/* Validates and converts the parameters like atmosphere/model.cc:613-745.
   Device memory is allocated by the first atmo_model_init, LUT request or
   atmo_model_load_luts, on the CUDA device current then.  shape may be NULL
   (the reference's sizes). */
atmo_status atmo_model_create(const atmo_model_params* params, const atmo_lut_shape* shape,
                              atmo_model** out);
atmo_status atmo_model_destroy(atmo_model* model);
/* Precomputes the LUTs (atmosphere/model.cc:866-975), ordered on `stream`;
   returns after the work is enqueued.  num_scattering_orders >= 1. */
atmo_status atmo_model_init(atmo_model* model, unsigned num_scattering_orders,
                            atmo_stream stream);
atmo_status atmo_model_set_path(atmo_model* model, atmo_path path);
/* exact != 0: compute with the parameters as given instead of the 6-decimal
   values the reference prints into its GLSL header (model.cc:636-666).
   Takes effect at the next atmo_model_init. */
atmo_status atmo_model_set_exact_parameters(atmo_model* model, int exact);
/* Device buffers of the final LUTs (valid until atmo_model_destroy). */
atmo_status atmo_model_get_lut(const atmo_model* model, atmo_lut_kind kind,
                               atmo_lut_view* view);
/* Copies a LUT to host memory (glGetTexImage equivalent): always float32
   RGBA, `bytes` must equal width*height*depth*16.  Synchronous. */
atmo_status atmo_model_read_lut(const atmo_model* model, atmo_lut_kind kind, float* host_dst,
                                size_t bytes);
/* The 3-wavelength atmosphere the model computes with for `lambdas` (nm),
   including the std::to_string rounding of atmosphere/model.cc:636-666 unless
   the model was created with exact parameters. */
atmo_status atmo_model_atmosphere_at(const atmo_model* model, const double lambdas[3],
                                     atmo_atmosphere* out);
/* GLSL source of the reference's shader() for this model (the header of
   atmosphere/model.cc:691-744 followed by the API shader of :221-281); the
   reference's functions.glsl text is not bundled, a marker stands in for it.
   Writes at most `capacity` bytes (NUL-terminated); *needed gets the size. */
atmo_status atmo_model_shader_source(const atmo_model* model, char* dst, size_t capacity,
                                     size_t* needed);
/* SKY_ and SUN_SPECTRAL_RADIANCE_TO_LUMINANCE (atmosphere/model.cc:663-686). */
atmo_status atmo_model_luminance_factors(const atmo_model* model, double sky[3],
                                         double sun[3]);
/* OpenGL texture binding (atmosphere/model.cc:984-1011): the box has no
   graphics stack; always returns ATMO_UNAVAILABLE. */
atmo_status atmo_model_set_program_uniforms(const atmo_model* model, unsigned program,
                                            unsigned transmittance_unit,
                                            unsigned scattering_unit,
                                            unsigned irradiance_unit,
                                            unsigned single_mie_unit);

/* atmosphere/model.cc:1020-1040 (host computation). */
atmo_status atmo_convert_spectrum_to_linear_srgb(const double* wavelengths,
                                                 const double* spectrum, unsigned n,
                                                 double* r, double* g, double* b);

/* ---- one precomputation group over caller-owned device buffers ------------- */
/* The Model::Precompute step (atmosphere/model.cc:1048-1215) for one
   3-wavelength atmosphere: writes transmittance, scattering (and single_mie
   when !combined) and irradiance, all float32 RGBA device buffers in the
   layouts above.  lum is the row-major luminance_from_radiance matrix
   (NULL = identity); blend accumulates like the reference's second and later
   wavelength groups.  Allocates its temporaries with cudaMallocAsync. */
atmo_status atmo_precompute(const atmo_atmosphere* atmosphere, const atmo_lut_shape* shape,
                            unsigned num_scattering_orders, const float lum[9], int blend,
                            int combined, atmo_path path, float* transmittance,
                            float* scattering, float* single_mie, float* irradiance,
                            atmo_stream stream);

/* The same precomputation without any device-memory allocation, for callers
   that cannot allocate: plugins of applications that own and pre-reserve all
   device memory (an engine's texture budget, a framework's caching
   allocator) and latency-bound code that must avoid cudaMalloc's implicit
   synchronisation.  No counterpart in the reference (its Init allocates GL
   textures).  The temporaries live in a fixed 64 MiB device array that every
   GPU loading this library holds until exit; shapes needing more (the
   reference's default shape needs ~49 MiB) return ATMO_BUDGET.  All calls
   share that array: calls whose GPU work overlaps race, so serialise them.
   The array's memory is taken when the library's device code for this entry
   point loads: with CUDA's default lazy loading, at the first call on each
   device (make that call, or set CUDA_MODULE_LOADING=EAGER, before reserving
   all device memory; otherwise it fails with ATMO_OOM).  The first call in
   each CUDA context looks up the array's device address and should come
   before any stream capture.  The launch descriptors travel as kernel
   parameters: a call copies nothing from host memory.  Path: ATMO_PATH_FAST. */
atmo_status atmo_precompute_noalloc(const atmo_atmosphere* atmosphere,
                                    const atmo_lut_shape* shape,
                                    unsigned num_scattering_orders, const float lum[9],
                                    int blend, int combined, float* transmittance,
                                    float* scattering, float* single_mie, float* irradiance,
                                    atmo_stream stream);

/* ---- one pass of the order loop over caller-owned LUTs --------------------- */
/* The draws of Model::Precompute's order loop (atmosphere/model.cc:1137-1211),
   one at a time, on float32 RGBA device LUTs the caller fills: an inspection
   and test hook for the per-pass kernels, e.g. with the uniform radiance,
   uniform irradiance and unit transmittance under which
   atmosphere/reference/functions_test.cc:1130-1344 states closed forms.
     ATMO_PASS_SCATTERING_DENSITY   ComputeScatteringDensityTexture
       (functions.glsl:1348-1367) of order `order` >= 2: reads
       delta_rayleigh and delta_mie (single scattering, order 2) or
       delta_rayleigh (delta multiple scattering, order > 2) and
       delta_irradiance; writes delta_density.
     ATMO_PASS_INDIRECT_IRRADIANCE  ComputeIndirectIrradianceTexture
       (:1573-1586) from the scattering of order `order` >= 1 (1: delta_rayleigh
       and delta_mie with their phase functions; > 1: delta_rayleigh); writes
       delta_irradiance and adds it to irradiance.
     ATMO_PASS_MULTIPLE_SCATTERING  ComputeMultipleScatteringTexture
       (:1369-1383) of order `order` >= 2: reads delta_density; writes
       delta_rayleigh (delta multiple scattering) and adds it / the Rayleigh
       phase function to scattering (combined layout).
   The set-up tables and ground transmittances come from `atmosphere`, the
   shape and `transmittance`.  Allocates its tables with cudaMallocAsync;
   returns after the pass completed. */
typedef enum {
  ATMO_PASS_SCATTERING_DENSITY = 4,
  ATMO_PASS_INDIRECT_IRRADIANCE = 5,
  ATMO_PASS_MULTIPLE_SCATTERING = 6
} atmo_pass_kind;
typedef struct {
  const float* transmittance;   /* W_T x H_T */
  float* delta_rayleigh;        /* scattering-LUT layout */
  float* delta_mie;             /* scattering-LUT layout (order-2 density, order-1 indirect) */
  float* delta_irradiance;      /* W_I x H_I */
  float* delta_density;         /* scattering-LUT layout */
  float* scattering;            /* scattering-LUT layout (multiple scattering adds to it) */
  float* irradiance;            /* W_I x H_I (indirect irradiance adds to it) */
} atmo_pass_buffers;
atmo_status atmo_run_pass(const atmo_atmosphere* atmosphere, const atmo_lut_shape* shape,
                          atmo_pass_kind pass, unsigned order, atmo_path path,
                          const atmo_pass_buffers* buffers, atmo_stream stream);

/* ---- batched precomputation (many atmospheres, uneven shapes/orders) ------- */
/* Creates a batch of n independent atmospheres, each with its own shape and
   scattering-order count; allocates every instance's LUTs and temporaries. */
atmo_status atmo_batch_create(const atmo_atmosphere* atmospheres, const atmo_lut_shape* shapes,
                              const unsigned* num_scattering_orders, unsigned n,
                              int combined, atmo_batch** out);
atmo_status atmo_batch_destroy(atmo_batch* batch);
/* Replaces the parameters of instance i (same shape and order count). */
atmo_status atmo_batch_set_atmosphere(atmo_batch* batch, unsigned i,
                                      const atmo_atmosphere* atmosphere);
/* Runs every instance's full precomputation; the pass sequence is captured
   in a CUDA graph on first use and replayed afterwards. */
atmo_status atmo_batch_run(atmo_batch* batch, atmo_stream stream);
atmo_status atmo_batch_get_lut(const atmo_batch* batch, unsigned i, atmo_lut_kind kind,
                               atmo_lut_view* view);
atmo_status atmo_batch_read_lut(const atmo_batch* batch, unsigned i, atmo_lut_kind kind,
                                float* host_dst, size_t bytes);
/* Copies a LUT of instance i (float32 RGBA, `bytes` = the view's bytes) to
   `dst` (device or host memory; pinned host memory makes it asynchronous),
   ordered on `stream` (make it wait for the run first, e.g. with an event). */
atmo_status atmo_batch_copy_lut(const atmo_batch* batch, unsigned i, atmo_lut_kind kind,
                                void* dst, size_t bytes, atmo_stream stream);
/* Number of kernels one atmo_batch_run launches (for launch accounting). */
atmo_status atmo_batch_kernel_count(const atmo_batch* batch, unsigned* count);
/* Runs the batch once without a graph and times every kernel with CUDA
   events on `stream`: ms[i], pass[i] (0 tables, 1 transmittance, 2 direct
   irradiance, 3 single scattering, 4 scattering density, 5 indirect
   irradiance, 6 multiple scattering, 7 FP16 conversion) and order[i] for
   i < *count (at most `capacity` entries).  Synchronous. */
atmo_status atmo_batch_time_passes(atmo_batch* batch, atmo_stream stream, unsigned capacity,
                                   float* ms, int* pass, int* order, unsigned* count);

/* ---- render-time queries ---------------------------------------------------- */
/* The shader API of atmosphere/model.cc:221-281 (functions.glsl:1705-1896),
   evaluated by CUDA kernels on a resident LUT set instead of in a GLSL
   shader.  A LUT set is the ATMOSPHERE constant plus the textures of one
   precomputation: a model's after atmo_model_init (the atmosphere at
   kLambdaR/G/B with the header's 6-decimal rounding; valid until the model is
   destroyed, refreshed by each Init) or instance i of a batch after
   atmo_batch_run (refreshed by each run).
   Query arrays are DEVICE arrays of n float triples in length units, the
   planet centre at the origin; directions are unit vectors.  sun_direction
   holds one direction for every query (sun_stride 0) or one per query
   (sun_stride 3); shadow_length may be NULL (0 for every query).
   luminance != 0 selects the luminance API (GetSkyLuminance ...: results
   times SKY_/SUN_SPECTRAL_RADIANCE_TO_LUMINANCE); luminance == 0 the radiance
   API, which the reference enables only for <= 3 precomputed wavelengths.
   Batch instances have no spectrum, hence no luminance API.
   The scattering texture is read in float32 also for half-precision models. */
atmo_status atmo_model_lut_set(const atmo_model* model, const atmo_lut_set** out);
atmo_status atmo_batch_lut_set(const atmo_batch* batch, unsigned i, const atmo_lut_set** out);
/* radiance[n][3], transmittance[n][3] (may be NULL). */
atmo_status atmo_sky_radiance(const atmo_lut_set* set, const float* camera, const float* view_ray,
                              const float* shadow_length, const float* sun_direction,
                              int sun_stride, unsigned n, int luminance, float* radiance,
                              float* transmittance, atmo_stream stream);
atmo_status atmo_sky_radiance_to_point(const atmo_lut_set* set, const float* camera,
                                       const float* point, const float* shadow_length,
                                       const float* sun_direction, int sun_stride, unsigned n,
                                       int luminance, float* radiance, float* transmittance,
                                       atmo_stream stream);
/* sun_irradiance[n][3] (the return value of GetSunAndSkyIrradiance),
   sky_irradiance[n][3] (may be NULL). */
atmo_status atmo_sun_and_sky_irradiance(const atmo_lut_set* set, const float* point,
                                        const float* normal, const float* sun_direction,
                                        int sun_stride, unsigned n, int luminance,
                                        float* sun_irradiance, float* sky_irradiance,
                                        atmo_stream stream);
/* Copies a LUT of the set to host memory (float32 RGBA; bytes = texels x 16;
   the scattering LUT is read in float32).  Synchronous. */
atmo_status atmo_lut_set_read(const atmo_lut_set* set, atmo_lut_kind kind, float* host_dst,
                              size_t bytes);
/* GetSolarRadiance / GetSolarLuminance (host). */
atmo_status atmo_solar_radiance(const atmo_lut_set* set, int luminance, double out[3]);
/* A pinhole view: pixel (i, j) of width x height (row j from the top) looks
   along normalize(forward + ((2i+1)/width - 1) tan(fov_y/2) width/height right
   + (1 - (2j+1)/height) tan(fov_y/2) up). */
typedef struct {
  float camera[3];
  float right[3], up[3], forward[3];
  float fov_y;                 /* radians */
  int width, height;
  float sun_direction[3];
  float albedo[3];             /* of the shaded points */
} atmo_pinhole_view;
/* One shading request over a pinhole view (device arrays, row-major pixels):
   sky_rgba[pixel] = GetSkyRadiance(camera, view ray) (alpha: the green
   transmittance); shaded_rgba[pixel] = GetSkyRadianceToPoint(camera, p) +
   transmittance x albedo / pi x (sun + sky irradiance of GetSunAndSkyIrradiance
   at p with normal -view ray), p = camera + depth[pixel] x view ray.  The
   radiance to p is integrated along the view ray itself (the query form takes
   the direction of p - camera). */
atmo_status atmo_shade_view(const atmo_lut_set* set, const atmo_pinhole_view* view,
                            const float* depth, int luminance, float* sky_rgba,
                            float* shaded_rgba, atmo_stream stream);
/* ---- LUT files -------------------------------------------------------------- */
/* Writes the LUTs the way the reference's precompute tool does
   (atmosphere/demo/webgl/precompute.cc:63-106, read by demo.js:364-377): raw
   little-endian float32 RGBA texels, x fastest, in transmittance.dat,
   scattering.dat, irradiance.dat and, for a model, the shader source in
   atmosphere_shader.txt; also single_mie_scattering.dat when the textures are
   not combined and optical_depth.dat (this library's -ln T LUT, used for
   ratios of transmittances below FP32's normal range).  `directory` must
   exist.  Synchronous. */
atmo_status atmo_model_save_luts(const atmo_model* model, const char* directory);
atmo_status atmo_batch_save_luts(const atmo_batch* batch, unsigned i, const char* directory);
/* Loads LUT files into a model as if atmo_model_init had computed them (a
   cache or checkpoint: render-time queries work without a rebuild).  Sizes
   must match the model's LUT shape; without optical_depth.dat (files of the
   reference's tool) -ln T stands in for it.  Synchronous. */
atmo_status atmo_model_load_luts(atmo_model* model, const char* directory);
/* ---- serving ------------------------------------------------------------------ */
/* A request loop over resident LUT sets (no counterpart in the reference,
   whose Model is one synchronous precomputation): rebuild requests are
   admitted while their final LUTs and temporaries fit hbm_budget_bytes,
   evicting idle ready sets least recently used first, and are batched at
   pass granularity with the rebuilds already running (uneven LUT shapes and
   order counts in one launch); shading requests (atmo_shade_view on a ready
   set) run on their own streams beside the rebuilds.  A result is the same
   alone and in any mix.  Sets are 3-wavelength radiance sets (FP32).  All
   calls are thread-safe; waits are bounded by their timeout. */
typedef struct {
  size_t hbm_budget_bytes;           /* 0: 120 GiB */
  unsigned max_rebuilds_in_flight;   /* admitted, not yet built (0: 64; <= 4096) */
  unsigned shade_streams;            /* 0: 4 */
  int combined;                      /* combine_scattering_textures of every set */
  unsigned admit_window_us;          /* batching window: a queued rebuild waits up to this
                                        long for others to be admitted with it (0: none) */
  size_t pool_max_bytes;             /* cap of the private memory pool the sets come from
                                        (0: the device's default); a rebuild admitted under
                                        the budget that the pool cannot serve fails with
                                        ATMO_OOM */
  unsigned max_shades_in_flight;     /* shading kernels enqueued and not complete at once
                                        (0: no cap); a cap keeps SMs free for the rebuild
                                        rounds at the cost of queueing shading on the host */
} atmo_server_config;
typedef struct {
  int state;             /* 0 queued, 1 running, 2 done, 3 failed (or cancelled) */
  atmo_status status;    /* of a failed request (ATMO_BUDGET, ATMO_OOM, ATMO_CANCELLED ...) */
  double queue_ms;       /* submission to admission (rebuild: budget, instance rows, batching
                            window) or to launch (shading); -1 before */
  double latency_ms;     /* submission to completion on the GPU (-1 before) */
  uint64_t set_id;       /* the LUT set (a rebuild's own ticket) */
  double launch_ms;      /* submission to the enqueue of its first kernel (-1 before) */
  double device_ms;      /* GPU time (CUDA events) of the launches it took part in: the
                            rounds of a rebuild (shared with the rebuilds batched with it),
                            the kernel of a shading request; summed as they retire */
  unsigned rounds;       /* those launches retired so far */
} atmo_ticket_info;
typedef struct {
  size_t used_bytes, budget_bytes;
  unsigned resident_sets, building, pending;
  unsigned long long evictions, rounds, kernels, shades_launched;
} atmo_server_stats;
atmo_status atmo_server_create(const atmo_server_config* config, atmo_server** out);
/* Waits for the work in flight, then frees every set. */
atmo_status atmo_server_destroy(atmo_server* server);
/* A rebuild of `atmosphere` (shape may be NULL); the ticket doubles as the
   LUT set's id. */
atmo_status atmo_server_submit_rebuild(atmo_server* server, const atmo_atmosphere* atmosphere,
                                       const atmo_lut_shape* shape, unsigned num_scattering_orders,
                                       uint64_t* ticket);
/* A shading request on set `set_id` (it runs once the set is built); depth,
   sky_rgba and shaded_rgba are device buffers (atmo_shade_view) that the
   caller keeps alive until the ticket completes. */
atmo_status atmo_server_submit_shade(atmo_server* server, uint64_t set_id,
                                     const atmo_pinhole_view* view, const float* depth,
                                     float* sky_rgba, float* shaded_rgba, uint64_t* ticket);
atmo_status atmo_server_poll(atmo_server* server, uint64_t ticket, atmo_ticket_info* info);
/* ATMO_OK when done (for a rebuild: its set is ready), the request's status
   when it failed, ATMO_TIMEOUT after timeout_ms. */
atmo_status atmo_server_wait(atmo_server* server, uint64_t ticket, unsigned timeout_ms,
                             atmo_ticket_info* info);
/* Cancels a request that has not completed.  A queued rebuild or shading
   request is dropped; a rebuild already being built gets no further pass and
   its memory returns to the budget (the blocks are freed behind the passes
   already enqueued).  The ticket then reports state 3 with ATMO_CANCELLED;
   shading requests waiting on a cancelled set fail with ATMO_NOT_READY.  A
   launched shading request, or a rebuild whose last pass is enqueued, cannot
   be cancelled (ATMO_INVALID_ARG). */
atmo_status atmo_server_cancel(atmo_server* server, uint64_t ticket);
/* Forgets a completed shading ticket (rebuild tickets go with their set). */
atmo_status atmo_server_release_ticket(atmo_server* server, uint64_t ticket);
/* The render-time query interface of a ready set (marks it used). */
atmo_status atmo_server_lut_set(atmo_server* server, uint64_t set_id, const atmo_lut_set** out);
/* Frees a ready, idle set now. */
atmo_status atmo_server_evict(atmo_server* server, uint64_t set_id);
atmo_status atmo_server_get_stats(atmo_server* server, atmo_server_stats* out);
/* ---- autotuner --------------------------------------------------------------- */
/* Block shape of the row-restructured single- and multiple-scattering kernels
   for one LUT shape: scattering-LUT rows per block and ray samples per
   shared-memory line stage (0, 0: the built-in choice).  A tuning changes
   only how work is grouped: every LUT is bit-identical under every tuning. */
typedef struct {
  int multiple_rows, multiple_group;
  int single_rows, single_group;
  float multiple_ms, single_ms;   /* atmo_autotune: best time per instance of each kernel */
} atmo_tuning;
/* Times every launchable block shape on this GPU for `shape` (a batch of
   `instances` copies of `atmosphere`, 0: 4) and registers the fastest for
   every model, batch and server instance of that shape created afterwards
   in this process.  Synchronous. */
atmo_status atmo_autotune(const atmo_atmosphere* atmosphere, const atmo_lut_shape* shape,
                          unsigned instances, atmo_tuning* out);
/* Registers a tuning for `shape` (checked for launchability); NULL restores
   the built-in choice.  Host only. */
atmo_status atmo_set_tuning(const atmo_lut_shape* shape, const atmo_tuning* tuning);
atmo_status atmo_get_tuning(const atmo_lut_shape* shape, atmo_tuning* out);
/* ---- diagnostics ----------------------------------------------------------- */
/* Measures this GPU's FP32 FMA throughput (TFLOP/s, 2 FLOP per FMA) with a
   short dependent-chain kernel over every SM: the denominator of the
   precomputation kernels' FP32 roofline.  Synchronous, ~10 ms. */
atmo_status atmo_measure_fp32_peak(double* tflops);
/* Device-side access checks.  The reference checks its L0 functions with
   asserts in its C++ Debug build and compiles them out of the shaders
   (atmosphere/model.cc:698); here the checked build of this library
   (libatmo_gb300_checked.so, compiled with -DATMO_DEVICE_CHECKS) tests the
   indices the kernels compute -- shared-memory table lookups, line-build rows
   and taps, staged texels, the texels of every LUT lookup -- against the
   buffers they read, records the first failure and reads element 0 instead.
   Reads (after a device synchronisation) and, with `reset`, clears the
   record: *compiled = 1 in the checked build, 0 in the ordinary one (whose
   record is always 0); *first_failure = 0 when every check passed, else the
   failing site (top 8 bits: 1 shared-memory lookup, 2 LUT texel, 3 staged
   texel, 4 line-build row, 5 line tap, 6 output texel, 255 self-test) and the
   failing index (low 56 bits). */
atmo_status atmo_device_checks(int reset, int* compiled, unsigned long long* first_failure);
/* Launches one check that fails by construction (index 5 of 3, no memory
   access) on `stream`: in the checked build the record then holds site 255,
   index 5.  Tests the recording path without an invalid access. */
atmo_status atmo_device_checks_selftest(atmo_stream stream);

#ifdef __cplusplus
}
#endif

#endif /* ATMO_ATMO_H_ */
