/*
 * CPU oracle for the atmosphere LUT precomputation -- TEST INFRASTRUCTURE ONLY.
 *
 * This header declares a double-precision CPU restatement of the reference's
 * precomputation path (ebruneton/precomputed_atmospheric_scattering):
 *   atmosphere/functions.glsl:113-1601   (physics functions, precompute part)
 *   atmosphere/functions.glsl:1633-1896  (render-time lookups)
 *   atmosphere/model.cc:521-595, 866-1215 (spectral set-up, Init, Precompute)
 *   atmosphere/reference/model.cc:73-245 (CPU pass driver)
 *
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may load
 * this library, and only to check results or as the timed CPU baseline.  The
 * product (libatmo_gb300.so) never links or calls it.
 *
 * Textures cross this interface as double RGBA arrays, x fastest, then y,
 * then z (the glGetTexImage order of atmosphere/demo/webgl/precompute.cc:63-72).
 * Spectra are 3-wavelength vectors (one precomputation group).
 */
#ifndef ATMO_ORACLE_H_
#define ATMO_ORACLE_H_

#ifdef __cplusplus
extern "C" {
#endif

/* atmosphere/definitions.glsl:185-191 */
typedef struct {
  double width, exp_term, exp_scale, linear_term, constant_term;
} oracle_layer;

/* atmosphere/definitions.glsl:197-199 */
typedef struct {
  oracle_layer layers[2];
} oracle_profile;

/* atmosphere/definitions.glsl:205-255, at 3 wavelengths, in length units. */
typedef struct {
  double solar_irradiance[3];
  double sun_angular_radius;
  double bottom_radius;
  double top_radius;
  oracle_profile rayleigh_density;
  double rayleigh_scattering[3];
  oracle_profile mie_density;
  double mie_scattering[3];
  double mie_extinction[3];
  double mie_phase_function_g;
  oracle_profile absorption_density;
  double absorption_extinction[3];
  double ground_albedo[3];
  double mu_s_min;
} oracle_atmosphere;

/* atmosphere/constants.h:47-61, as run-time values. */
typedef struct {
  int transmittance_width, transmittance_height;
  int scattering_r, scattering_mu, scattering_mu_s, scattering_nu;
  int irradiance_width, irradiance_height;
} oracle_shape;

/* ---- point functions (functions.glsl), for known-answer tests ---------- */
double oracle_distance_to_top(const oracle_atmosphere* a, double r, double mu);
double oracle_distance_to_bottom(const oracle_atmosphere* a, double r, double mu);
int oracle_ray_intersects_ground(const oracle_atmosphere* a, double r, double mu);
double oracle_distance_to_nearest(const oracle_atmosphere* a, double r, double mu,
                                  int ground);
double oracle_profile_density(const oracle_profile* p, double altitude);
double oracle_optical_length(const oracle_atmosphere* a, const oracle_profile* p,
                             double r, double mu);
void oracle_transmittance_to_top(const oracle_atmosphere* a, double r, double mu,
                                 double out[3]);
double oracle_tex_coord_from_unit_range(double x, int n);
double oracle_unit_range_from_tex_coord(double u, int n);
void oracle_transmittance_uv_from_rmu(const oracle_atmosphere* a, const oracle_shape* s,
                                      double r, double mu, double uv[2]);
void oracle_rmu_from_transmittance_uv(const oracle_atmosphere* a, const oracle_shape* s,
                                      double u, double v, double* r, double* mu);
void oracle_lookup_transmittance_to_top(const oracle_atmosphere* a, const oracle_shape* s,
                                        const double* T, double r, double mu, double out[3]);
void oracle_lookup_transmittance(const oracle_atmosphere* a, const oracle_shape* s,
                                 const double* T, double r, double mu, double d,
                                 int ground, double out[3]);
void oracle_lookup_transmittance_to_sun(const oracle_atmosphere* a, const oracle_shape* s,
                                        const double* T, double r, double mu_s,
                                        double out[3]);
void oracle_single_scattering_integrand(const oracle_atmosphere* a, const oracle_shape* s,
                                        const double* T, double r, double mu, double mu_s,
                                        double nu, double d, int ground,
                                        double rayleigh[3], double mie[3]);
void oracle_single_scattering(const oracle_atmosphere* a, const oracle_shape* s,
                              const double* T, double r, double mu, double mu_s,
                              double nu, int ground, double rayleigh[3], double mie[3]);
double oracle_rayleigh_phase(double nu);
double oracle_mie_phase(double g, double nu);
void oracle_scattering_uvwz(const oracle_atmosphere* a, const oracle_shape* s, double r,
                            double mu, double mu_s, double nu, int ground, double uvwz[4]);
void oracle_rmumusnu_from_uvwz(const oracle_atmosphere* a, const oracle_shape* s,
                               const double uvwz[4], double out[4], int* ground);
void oracle_rmumusnu_from_frag_coord(const oracle_atmosphere* a, const oracle_shape* s,
                                     const double frag[3], double out[4], int* ground);
/* GetScattering (functions.glsl:958-976) on an RGBA 3D texture. */
void oracle_lookup_scattering(const oracle_atmosphere* a, const oracle_shape* s,
                              const double* S, double r, double mu, double mu_s,
                              double nu, int ground, double out[3]);
/* The texel indices (after CLAMP_TO_EDGE) and weights that the two trilinear
   lookups of GetScattering read: 16 taps. */
void oracle_scattering_taps(const oracle_atmosphere* a, const oracle_shape* s, double r,
                            double mu, double mu_s, double nu, int ground, int idx[16],
                            double w[16]);
void oracle_scattering_density(const oracle_atmosphere* a, const oracle_shape* s,
                               const double* T, const double* SR, const double* SM,
                               const double* SMulti, const double* I, double r,
                               double mu, double mu_s, double nu, int order,
                               double out[3]);
void oracle_multiple_scattering(const oracle_atmosphere* a, const oracle_shape* s,
                                const double* T, const double* J, double r, double mu,
                                double mu_s, double nu, int ground, double out[3]);
void oracle_direct_irradiance(const oracle_atmosphere* a, const oracle_shape* s,
                              const double* T, double r, double mu_s, double out[3]);
void oracle_indirect_irradiance(const oracle_atmosphere* a, const oracle_shape* s,
                                const double* SR, const double* SM, const double* SMulti,
                                double r, double mu_s, int order, double out[3]);
void oracle_irradiance_uv_from_rmus(const oracle_atmosphere* a, const oracle_shape* s,
                                    double r, double mu_s, double uv[2]);
void oracle_rmus_from_irradiance_uv(const oracle_atmosphere* a, const oracle_shape* s,
                                    double u, double v, double* r, double* mu_s);
void oracle_lookup_irradiance(const oracle_atmosphere* a, const oracle_shape* s,
                              const double* I, double r, double mu_s, double out[3]);

/* ---- per-texel pass evaluation (the *Texture functions) ----------------- */
/* kind: 0 transmittance, 1 direct irradiance, 2 single scattering (out RGB =
   Rayleigh, out2 RGB = Mie), 3 scattering density, 4 indirect irradiance,
   5 multiple scattering (out = delta, out2[0] = nu).  idx are flat texel
   indices of the pass's target texture; outputs are RGBA per index. */
void oracle_eval_texels(int kind, const oracle_atmosphere* a, const oracle_shape* s,
                        const double* T, const double* SR, const double* SM,
                        const double* SMulti, const double* I, const double* J,
                        int order, int n, const long long* idx, double* out,
                        double* out2, int threads);

/* ---- the pass driver ----------------------------------------------------- */
/* One Model::Precompute group (atmosphere/model.cc:1048-1215):
   lum: 3x3 row-major luminance_from_radiance, blend as in the reference.
   combined != 0: scattering alpha = (lum * mie).r (model.cc:151-155);
   single_mie may be NULL when combined.
   Outputs are RGBA double arrays; with blend they accumulate. */
int oracle_precompute(const oracle_atmosphere* a, const oracle_shape* s,
                      unsigned num_scattering_orders, const double lum[9], int blend,
                      int combined, int threads, double* transmittance,
                      double* scattering, double* single_mie, double* irradiance);

/* Timing sample for the CPU baseline: runs the same passes but evaluates the
   scattering-density and multiple-scattering passes only on every
   `stride`-th texel.  Fills seconds[6] with per-pass wall times (transmittance,
   direct irradiance, single scattering, density, indirect, multiple).  */
int oracle_time_precompute_sample(const oracle_atmosphere* a, const oracle_shape* s,
                                  unsigned num_scattering_orders, int stride,
                                  int threads, double seconds[6]);
/* The same with by_rows != 0: the threads take whole texture rows
   (transmittance, irradiance) and r-slices (scattering) as work items, the
   partition of the reference's CPU driver (atmosphere/reference/model.cc:
   140-237), instead of blocks of 64 texels. */
int oracle_time_precompute_partitioned(const oracle_atmosphere* a, const oracle_shape* s,
                                       unsigned num_scattering_orders, int stride,
                                       int threads, int by_rows, double seconds[6]);

/* ---- spectral set-up and render-time functions --------------------------- */
/* atmosphere/model.cc:535-552 */
double oracle_interpolate(const double* wavelengths, const double* values, int n,
                          double wavelength);
/* atmosphere/model.cc:521-533 */
double oracle_cie_table_value(double wavelength, int column);
/* atmosphere/model.cc:562-595 */
void oracle_radiance_to_luminance_factors(const double* wavelengths,
                                          const double* solar, int n,
                                          double lambda_power, double k[3]);
/* atmosphere/model.cc:1020-1040 */
void oracle_convert_spectrum_to_linear_srgb(const double* wavelengths,
                                            const double* spectrum, int n,
                                            double rgb[3]);

/* functions.glsl:1705-1769 / 1787-1863 / 1878-1896; combined selects the
   COMBINED_SCATTERING_TEXTURES branches.  S and M are RGBA 3D textures (M is
   ignored when combined). */
void oracle_sky_radiance(const oracle_atmosphere* a, const oracle_shape* s,
                         const double* T, const double* S, const double* M,
                         int combined, const double camera[3], const double view[3],
                         double shadow_length, const double sun[3], double out[3],
                         double transmittance[3]);
void oracle_sky_radiance_to_point(const oracle_atmosphere* a, const oracle_shape* s,
                                  const double* T, const double* S, const double* M,
                                  int combined, const double camera[3],
                                  const double point[3], double shadow_length,
                                  const double sun[3], double out[3],
                                  double transmittance[3]);
void oracle_sun_and_sky_irradiance(const oracle_atmosphere* a, const oracle_shape* s,
                                   const double* T, const double* I,
                                   const double point[3], const double normal[3],
                                   const double sun[3], double sun_irr[3],
                                   double sky_irr[3]);

#ifdef __cplusplus
}
#endif

#endif  /* ATMO_ORACLE_H_ */
