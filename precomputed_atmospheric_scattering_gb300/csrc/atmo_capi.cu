// atmo_capi.cu -- the C ABI of include/atmo/atmo.h over the launch programs.
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <algorithm>
#include <cstring>
#include <fstream>
#include <memory>
#include <string>
#include <vector>

#include "../../include/atmo/atmo.h"
#include "atmo_check.cuh"
#include "atmo_consts.h"
#include "atmo_kernels.h"
#include "atmo_program.h"
#include "atmo_render.h"

namespace atmo {
const char* LastError();
}

using namespace atmo;

namespace {

constexpr double kMaxLuminousEfficacy = 683.0;   // atmosphere/constants.h:64
constexpr double kLambdaMin = 360.0, kLambdaMax = 830.0;

// CIE 1931 2-degree colour matching functions (atmosphere/constants.h:69-165).
const double kCie[95][4] = {
#include "cie_1931_2deg.inc"
};
// XYZ to linear sRGB (atmosphere/constants.h:169-173).
const double kXyzToSrgb[9] = {3.2406, -1.5372, -0.4986, -0.9689, 1.8758,
                              0.0415, 0.0557,  -0.2040, 1.0570};

atmo_status Fail(atmo_status s, const std::string& msg) {
  SetError(msg);
  return s;
}

// atmosphere/model.cc:521-533
double CieValue(double wavelength, int column) {
  if (wavelength <= kLambdaMin || wavelength >= kLambdaMax) return 0.0;
  double u = (wavelength - kLambdaMin) / 5.0;
  int row = (int)std::floor(u);
  if (row < 0 || row + 1 >= 95) return 0.0;
  u -= row;
  return kCie[row][column] * (1.0 - u) + kCie[row + 1][column] * u;
}

// atmosphere/model.cc:535-552
double Interpolate(const std::vector<double>& wl, const std::vector<double>& f, double w) {
  if (w < wl[0]) return f[0];
  for (size_t i = 0; i + 1 < wl.size(); ++i) {
    if (w < wl[i + 1]) {
      double u = (w - wl[i]) / (wl[i + 1] - wl[i]);
      return f[i] * (1.0 - u) + f[i + 1] * u;
    }
  }
  return f.back();
}

// atmosphere/model.cc:562-595
void RadianceToLuminanceFactors(const std::vector<double>& wl, const std::vector<double>& solar,
                                double lambda_power, double k[3]) {
  k[0] = k[1] = k[2] = 0.0;
  const double lr = ATMO_LAMBDA_R, lg = ATMO_LAMBDA_G, lb = ATMO_LAMBDA_B;
  double sr = Interpolate(wl, solar, lr), sg = Interpolate(wl, solar, lg),
         sb = Interpolate(wl, solar, lb);
  for (int lambda = (int)kLambdaMin; lambda < (int)kLambdaMax; ++lambda) {
    double x = CieValue(lambda, 1), y = CieValue(lambda, 2), z = CieValue(lambda, 3);
    const double* m = kXyzToSrgb;
    double r_bar = m[0] * x + m[1] * y + m[2] * z;
    double g_bar = m[3] * x + m[4] * y + m[5] * z;
    double b_bar = m[6] * x + m[7] * y + m[8] * z;
    double irr = Interpolate(wl, solar, lambda);
    k[0] += r_bar * irr / sr * std::pow(lambda / lr, lambda_power);
    k[1] += g_bar * irr / sg * std::pow(lambda / lg, lambda_power);
    k[2] += b_bar * irr / sb * std::pow(lambda / lb, lambda_power);
  }
  for (int i = 0; i < 3; ++i) k[i] *= kMaxLuminousEfficacy;
}

// std::to_string(double) prints "%f": the reference bakes every parameter into
// its GLSL header with 6 decimals (atmosphere/model.cc:636-666, :718-734).
double Round6(double x) {
  char buf[512];
  std::snprintf(buf, sizeof(buf), "%f", x);
  return std::strtod(buf, nullptr);
}
std::string Str6(double x) {
  char buf[512];
  std::snprintf(buf, sizeof(buf), "%f", x);
  return buf;
}

bool Finite(const double* v, unsigned n) {
  for (unsigned i = 0; i < n; ++i)
    if (!std::isfinite(v[i])) return false;
  return true;
}

struct Group {
  double lambdas[3];
  float lum[9];
  bool blend;
};

}  // namespace

struct atmo_model {
  std::unique_ptr<atmo_lut_set> lut_set;
  std::vector<double> wavelengths, solar, rayleigh, mie_sca, mie_ext, absorption, albedo;
  std::vector<atmo_density_layer> ray_layers, mie_layers, abs_layers;   // 2 each
  double sun_angular_radius = 0, bottom = 0, top = 0, g = 0, max_sun_zenith = 0, unit = 1;
  unsigned num_precomputed_wavelengths = 3;
  bool combined = true, half = false, exact = false;
  atmo_lut_shape shape{};
  atmo_path path = ATMO_PATH_FAST;
  int device = 0;
  Storage storage;
  std::unique_ptr<Program> program;
  unsigned program_orders = 0;
  atmo_path program_path = ATMO_PATH_FAST;
  bool program_exact = false;
  bool initialized = false;
  double sky_k[3] = {0, 0, 0}, sun_k[3] = {0, 0, 0};

  // atmosphere/model.cc:627-666 and :716-744 at `lambdas`.
  atmo_atmosphere AtmosphereAt(const double lambdas[3]) const {
    auto R = [&](double x) { return exact ? x : Round6(x); };
    atmo_atmosphere a;
    std::memset(&a, 0, sizeof(a));
    for (int i = 0; i < 3; ++i) {
      a.solar_irradiance[i] = R(Interpolate(wavelengths, solar, lambdas[i]));
      a.rayleigh_scattering[i] = R(Interpolate(wavelengths, rayleigh, lambdas[i]) * unit);
      a.mie_scattering[i] = R(Interpolate(wavelengths, mie_sca, lambdas[i]) * unit);
      a.mie_extinction[i] = R(Interpolate(wavelengths, mie_ext, lambdas[i]) * unit);
      a.absorption_extinction[i] = R(Interpolate(wavelengths, absorption, lambdas[i]) * unit);
      a.ground_albedo[i] = R(Interpolate(wavelengths, albedo, lambdas[i]));
    }
    a.sun_angular_radius = R(sun_angular_radius);
    a.bottom_radius = R(bottom / unit);
    a.top_radius = R(top / unit);
    auto prof = [&](const std::vector<atmo_density_layer>& ls, atmo_density_profile* p) {
      for (int i = 0; i < 2; ++i) {
        p->layers[i].width = R(ls[i].width / unit);
        p->layers[i].exp_term = R(ls[i].exp_term);
        p->layers[i].exp_scale = R(ls[i].exp_scale * unit);
        p->layers[i].linear_term = R(ls[i].linear_term * unit);
        p->layers[i].constant_term = R(ls[i].constant_term);
      }
    };
    prof(ray_layers, &a.rayleigh_density);
    prof(mie_layers, &a.mie_density);
    prof(abs_layers, &a.absorption_density);
    a.mie_phase_function_g = R(g);
    a.mu_s_min = R(std::cos(max_sun_zenith));
    return a;
  }

  // The wavelength groups of atmosphere/model.cc:905-948.
  std::vector<Group> Groups() const {
    std::vector<Group> gs;
    if (num_precomputed_wavelengths <= 3) {
      Group g0{{ATMO_LAMBDA_R, ATMO_LAMBDA_G, ATMO_LAMBDA_B},
               {1, 0, 0, 0, 1, 0, 0, 0, 1},
               false};
      gs.push_back(g0);
      return gs;
    }
    int n = (int)(num_precomputed_wavelengths + 2) / 3;
    double dlambda = (kLambdaMax - kLambdaMin) / (3 * n);
    for (int i = 0; i < n; ++i) {
      Group gr;
      for (int k = 0; k < 3; ++k) gr.lambdas[k] = kLambdaMin + (3 * i + 0.5 + k) * dlambda;
      auto coeff = [&](double lambda, int component) {
        double x = CieValue(lambda, 1), y = CieValue(lambda, 2), z = CieValue(lambda, 3);
        return (float)((kXyzToSrgb[component * 3] * x + kXyzToSrgb[component * 3 + 1] * y +
                        kXyzToSrgb[component * 3 + 2] * z) *
                       dlambda);
      };
      for (int row = 0; row < 3; ++row)
        for (int col = 0; col < 3; ++col) gr.lum[row * 3 + col] = coeff(gr.lambdas[col], row);
      gr.blend = i > 0;
      gs.push_back(gr);
    }
    return gs;
  }

  Instance SlotFor(const double lambdas[3], const float* lum, bool blend) const {
    Instance in;
    std::memset(&in, 0, sizeof(in));
    atmo_atmosphere a = AtmosphereAt(lambdas);
    in.c = MakeConsts(a, lum);
    in.s = storage.s;
    in.tab = storage.tab;
    in.T = storage.T;
    in.Tau = storage.Tau;
    in.I = storage.I;
    in.dI = storage.dI;
    in.dI2 = storage.dI2;
    in.dR = storage.dR;
    in.dM = storage.dM;
    in.dJ = storage.dJ;
    in.S = storage.S;
    in.M = storage.M;
    in.S_half = storage.S_half;
    in.M_half = storage.M_half;
    in.combined = combined ? 1 : 0;
    in.blend = blend ? 1 : 0;
    return in;
  }
};

struct atmo_batch {
  std::vector<Storage> storages;
  std::unique_ptr<Program> program;
  bool combined = true;
  bool ran = false;
  std::vector<atmo_lut_set> lut_sets;   // per instance, filled by the first run
};



extern "C" {

int atmo_abi_version(void) { return ATMO_ABI_VERSION; }
const char* atmo_last_error(void) { return atmo::LastError(); }

atmo_status atmo_synchronize(atmo_stream stream) {
  ATMO_CUDA_TRY(cudaStreamSynchronize(reinterpret_cast<cudaStream_t>(stream)));
  return ATMO_OK;
}

atmo_status atmo_model_create(const atmo_model_params* p, const atmo_lut_shape* shape,
                              atmo_model** out) {
  if (!p || !out) return Fail(ATMO_INVALID_ARG, "NULL argument");
  *out = nullptr;
  const unsigned n = p->num_wavelengths;
  if (n == 0 || !p->wavelengths || !p->solar_irradiance || !p->rayleigh_scattering ||
      !p->mie_scattering || !p->mie_extinction || !p->absorption_extinction ||
      !p->ground_albedo)
    return Fail(ATMO_INVALID_ARG, "missing spectral array");
  if (!Finite(p->wavelengths, n) || !Finite(p->solar_irradiance, n) ||
      !Finite(p->rayleigh_scattering, n) || !Finite(p->mie_scattering, n) ||
      !Finite(p->mie_extinction, n) || !Finite(p->absorption_extinction, n) ||
      !Finite(p->ground_albedo, n))
    return Fail(ATMO_INVALID_ARG, "non-finite spectral value");
  for (unsigned i = 0; i + 1 < n; ++i)
    if (!(p->wavelengths[i] < p->wavelengths[i + 1]))
      return Fail(ATMO_INVALID_ARG, "wavelengths must be sorted in increasing order");
  if (p->num_rayleigh_layers > 2 || p->num_mie_layers > 2 || p->num_absorption_layers > 2)
    return Fail(ATMO_INVALID_ARG, "at most 2 density layers per profile");
  if ((p->num_rayleigh_layers && !p->rayleigh_density) ||
      (p->num_mie_layers && !p->mie_density) ||
      (p->num_absorption_layers && !p->absorption_density))
    return Fail(ATMO_INVALID_ARG, "missing density layers");
  if (!(p->length_unit_in_meters > 0.0) || !std::isfinite(p->length_unit_in_meters))
    return Fail(ATMO_INVALID_ARG, "length_unit_in_meters must be > 0");
  if (!std::isfinite(p->max_sun_zenith_angle))
    return Fail(ATMO_INVALID_ARG, "non-finite max_sun_zenith_angle");
  atmo_lut_shape s = shape ? *shape : DefaultShape();
  std::string why;
  if (!ValidShape(s, &why)) return Fail(ATMO_INVALID_ARG, why);

  std::unique_ptr<atmo_model> m(new atmo_model());
  m->wavelengths.assign(p->wavelengths, p->wavelengths + n);
  m->solar.assign(p->solar_irradiance, p->solar_irradiance + n);
  m->rayleigh.assign(p->rayleigh_scattering, p->rayleigh_scattering + n);
  m->mie_sca.assign(p->mie_scattering, p->mie_scattering + n);
  m->mie_ext.assign(p->mie_extinction, p->mie_extinction + n);
  m->absorption.assign(p->absorption_extinction, p->absorption_extinction + n);
  m->albedo.assign(p->ground_albedo, p->ground_albedo + n);
  // Profiles are padded with zero layers at the front (model.cc:676-690).
  auto pad = [](const atmo_density_layer* l, unsigned k) {
    std::vector<atmo_density_layer> v(l, l + k);
    while (v.size() < 2) v.insert(v.begin(), atmo_density_layer{0, 0, 0, 0, 0});
    return v;
  };
  m->ray_layers = pad(p->rayleigh_density, p->num_rayleigh_layers);
  m->mie_layers = pad(p->mie_density, p->num_mie_layers);
  m->abs_layers = pad(p->absorption_density, p->num_absorption_layers);
  m->sun_angular_radius = p->sun_angular_radius;
  m->bottom = p->bottom_radius;
  m->top = p->top_radius;
  m->g = p->mie_phase_function_g;
  m->max_sun_zenith = p->max_sun_zenith_angle;
  m->unit = p->length_unit_in_meters;
  m->num_precomputed_wavelengths = p->num_precomputed_wavelengths;
  m->combined = p->combine_scattering_textures != 0;
  m->half = p->half_precision != 0;
  m->shape = s;
  // Validate the converted parameters of every group.
  for (const Group& gr : m->Groups()) {
    atmo_atmosphere a = m->AtmosphereAt(gr.lambdas);
    if (!ValidAtmosphere(a, &why)) return Fail(ATMO_INVALID_ARG, why);
  }
  // atmosphere/model.cc:663-686
  if (m->num_precomputed_wavelengths > 3) {
    m->sky_k[0] = m->sky_k[1] = m->sky_k[2] = kMaxLuminousEfficacy;
  } else {
    RadianceToLuminanceFactors(m->wavelengths, m->solar, -3.0, m->sky_k);
  }
  RadianceToLuminanceFactors(m->wavelengths, m->solar, 0.0, m->sun_k);
  // Device storage is allocated by the first Init or LUT request, on the
  // device current at that time.
  *out = m.release();
  return ATMO_OK;
}

static atmo_status EnsureStorage(atmo_model* m) {
  if (!m->storage.owned.empty()) return ATMO_OK;
  ATMO_CUDA_TRY(cudaGetDevice(&m->device));
  return m->storage.Allocate(ToShape(m->shape), m->combined, m->half);
}

atmo_status atmo_model_destroy(atmo_model* m) {
  if (!m) return ATMO_OK;
  m->program.reset();
  m->storage.Free();
  delete m;
  return ATMO_OK;
}

atmo_status atmo_model_set_path(atmo_model* m, atmo_path path) {
  if (!m || (path != ATMO_PATH_FAST && path != ATMO_PATH_PLAIN))
    return Fail(ATMO_INVALID_ARG, "bad model or path");
  m->path = path;
  return ATMO_OK;
}

atmo_status atmo_model_set_exact_parameters(atmo_model* m, int exact) {
  if (!m) return Fail(ATMO_INVALID_ARG, "NULL model");
  m->exact = exact != 0;
  return ATMO_OK;
}

// The shader's ATMOSPHERE constant and luminance factors (model.cc:691-744)
// over the model's LUTs.
static void BuildModelLutSet(atmo_model* m) {
  const double l[3] = {ATMO_LAMBDA_R, ATMO_LAMBDA_G, ATMO_LAMBDA_B};
  if (!m->lut_set) m->lut_set.reset(new atmo_lut_set());
  atmo_lut_set* set = m->lut_set.get();
  const atmo_atmosphere a = m->AtmosphereAt(l);
  Instance in = m->SlotFor(l, nullptr, false);
  set->luts = LutsOf(in);
  for (int i = 0; i < 3; ++i) {
    set->luts.sky_k[i] = (float)(m->exact ? m->sky_k[i] : Round6(m->sky_k[i]));
    set->luts.sun_k[i] = (float)(m->exact ? m->sun_k[i] : Round6(m->sun_k[i]));
    set->solar[i] = a.solar_irradiance[i];
  }
  set->sun_angular_radius = a.sun_angular_radius;
  set->radiance_api = m->num_precomputed_wavelengths <= 3;
}

atmo_status atmo_model_init(atmo_model* m, unsigned num_scattering_orders, atmo_stream stream) {
  if (!m) return Fail(ATMO_INVALID_ARG, "NULL model");
  if (num_scattering_orders < 1 || num_scattering_orders > 64)
    return Fail(ATMO_INVALID_ARG, "num_scattering_orders must be in [1, 64]");
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  atmo_status as = EnsureStorage(m);
  if (as != ATMO_OK) return as;
  if (!m->program || m->program_orders != num_scattering_orders || m->program_path != m->path ||
      m->program_exact != m->exact) {
    std::unique_ptr<Program> prog(new Program());
    prog->path = m->path;
    std::vector<Group> groups = m->Groups();
    for (const Group& gr : groups) {
      prog->slots.push_back(m->SlotFor(gr.lambdas, gr.lum, gr.blend));
      prog->orders.push_back(num_scattering_orders);
    }
    for (size_t i = 0; i < groups.size(); ++i) prog->AddStage({(int)i});
    if (m->num_precomputed_wavelengths > 3) {
      // Transmittance at kLambdaR/G/B after the groups (model.cc:949-963).
      const double l[3] = {ATMO_LAMBDA_R, ATMO_LAMBDA_G, ATMO_LAMBDA_B};
      prog->slots.push_back(m->SlotFor(l, nullptr, false));
      prog->orders.push_back(1);
      prog->AddStage({(int)groups.size()}, true);
    }
    if (m->half) prog->AddToHalf({0});
    m->program = std::move(prog);
    m->program_orders = num_scattering_orders;
    m->program_path = m->path;
    m->program_exact = m->exact;
  }
  atmo_status s = m->program->Run(st, /*use_graph=*/true);
  if (s != ATMO_OK) return s;
  m->initialized = true;
  BuildModelLutSet(m);
  return ATMO_OK;
}

static atmo_status ViewOf(const Storage& sto, atmo_lut_kind kind, atmo_lut_view* v) {
  const Shape& s = sto.s;
  std::memset(v, 0, sizeof(*v));
  switch (kind) {
    case ATMO_LUT_TRANSMITTANCE:
      *v = atmo_lut_view{sto.T, s.tw, s.th, 1, ATMO_DTYPE_F32, (size_t)s.t_texels() * 16};
      return ATMO_OK;
    case ATMO_LUT_IRRADIANCE:
      *v = atmo_lut_view{sto.I, s.iw, s.ih, 1, ATMO_DTYPE_F32, (size_t)s.i_texels() * 16};
      return ATMO_OK;
    case ATMO_LUT_SCATTERING:
      if (sto.half)
        *v = atmo_lut_view{sto.S_half, s.sw(), s.smu, s.sr, ATMO_DTYPE_F16,
                           (size_t)s.s_texels() * 8};
      else
        *v = atmo_lut_view{sto.S, s.sw(), s.smu, s.sr, ATMO_DTYPE_F32,
                           (size_t)s.s_texels() * 16};
      return ATMO_OK;
    case ATMO_LUT_SINGLE_MIE:
      if (sto.combined)
        return Fail(ATMO_INVALID_ARG, "no single-Mie texture with combined scattering textures");
      if (sto.half)
        *v = atmo_lut_view{sto.M_half, s.sw(), s.smu, s.sr, ATMO_DTYPE_F16,
                           (size_t)s.s_texels() * 8};
      else
        *v = atmo_lut_view{sto.M, s.sw(), s.smu, s.sr, ATMO_DTYPE_F32,
                           (size_t)s.s_texels() * 16};
      return ATMO_OK;
  }
  return Fail(ATMO_INVALID_ARG, "unknown LUT kind");
}

static atmo_status ReadView(const atmo_lut_view& v, float* dst, size_t bytes) {
  size_t texels = (size_t)v.width * v.height * v.depth;
  if (!dst || bytes != texels * 16)
    return Fail(ATMO_INVALID_ARG, "host buffer must hold width*height*depth float RGBA texels");
  if (v.dtype == ATMO_DTYPE_F32) {
    ATMO_CUDA_TRY(cudaMemcpy(dst, v.device_ptr, bytes, cudaMemcpyDeviceToHost));
    return ATMO_OK;
  }
  std::vector<__half> h(texels * 4);
  ATMO_CUDA_TRY(cudaMemcpy(h.data(), v.device_ptr, texels * 8, cudaMemcpyDeviceToHost));
  for (size_t i = 0; i < texels * 4; ++i) dst[i] = __half2float(h[i]);
  return ATMO_OK;
}

atmo_status atmo_model_get_lut(const atmo_model* m, atmo_lut_kind kind, atmo_lut_view* view) {
  if (!m || !view) return Fail(ATMO_INVALID_ARG, "NULL argument");
  atmo_status as = EnsureStorage(const_cast<atmo_model*>(m));
  if (as != ATMO_OK) return as;
  return ViewOf(m->storage, kind, view);
}

atmo_status atmo_model_read_lut(const atmo_model* m, atmo_lut_kind kind, float* dst,
                                size_t bytes) {
  if (!m) return Fail(ATMO_INVALID_ARG, "NULL model");
  if (!m->initialized) return Fail(ATMO_NOT_READY, "Init has not been called");
  atmo_lut_view v;
  atmo_status s = ViewOf(m->storage, kind, &v);
  if (s != ATMO_OK) return s;
  return ReadView(v, dst, bytes);
}

atmo_status atmo_model_atmosphere_at(const atmo_model* m, const double lambdas[3],
                                     atmo_atmosphere* out) {
  if (!m || !lambdas || !out) return Fail(ATMO_INVALID_ARG, "NULL argument");
  *out = m->AtmosphereAt(lambdas);
  return ATMO_OK;
}

atmo_status atmo_model_luminance_factors(const atmo_model* m, double sky[3], double sun[3]) {
  if (!m) return Fail(ATMO_INVALID_ARG, "NULL model");
  for (int i = 0; i < 3; ++i) {
    if (sky) sky[i] = m->sky_k[i];
    if (sun) sun[i] = m->sun_k[i];
  }
  return ATMO_OK;
}

atmo_status atmo_model_shader_source(const atmo_model* m, char* dst, size_t capacity,
                                     size_t* needed) {
  if (!m) return Fail(ATMO_INVALID_ARG, "NULL model");
  // The generated header of atmosphere/model.cc:691-744 for kLambdaR/G/B.
  const double l[3] = {ATMO_LAMBDA_R, ATMO_LAMBDA_G, ATMO_LAMBDA_B};
  bool exact_saved = m->exact;
  const_cast<atmo_model*>(m)->exact = true;   // literals are printed from exact values
  atmo_atmosphere a = m->AtmosphereAt(l);
  const_cast<atmo_model*>(m)->exact = exact_saved;
  auto v3 = [](const double* v) {
    return "vec3(" + Str6(v[0]) + "," + Str6(v[1]) + "," + Str6(v[2]) + ")";
  };
  auto layer = [](const atmo_density_layer& x) {
    return "DensityProfileLayer(" + Str6(x.width) + "," + Str6(x.exp_term) + "," +
           Str6(x.exp_scale) + "," + Str6(x.linear_term) + "," + Str6(x.constant_term) + ")";
  };
  auto prof = [&](const atmo_density_profile& p) {
    return "DensityProfile(DensityProfileLayer[2](" + layer(p.layers[0]) + "," +
           layer(p.layers[1]) + "))";
  };
  const atmo_lut_shape& s = m->shape;
  std::string src;
  src += "#version 330\n#define IN(x) const in x\n#define OUT(x) out x\n";
  src += "#define TEMPLATE(x)\n#define TEMPLATE_ARGUMENT(x)\n#define assert(x)\n";
  src += "const int TRANSMITTANCE_TEXTURE_WIDTH = " + std::to_string(s.transmittance_width) + ";\n";
  src += "const int TRANSMITTANCE_TEXTURE_HEIGHT = " + std::to_string(s.transmittance_height) + ";\n";
  src += "const int SCATTERING_TEXTURE_R_SIZE = " + std::to_string(s.scattering_r) + ";\n";
  src += "const int SCATTERING_TEXTURE_MU_SIZE = " + std::to_string(s.scattering_mu) + ";\n";
  src += "const int SCATTERING_TEXTURE_MU_S_SIZE = " + std::to_string(s.scattering_mu_s) + ";\n";
  src += "const int SCATTERING_TEXTURE_NU_SIZE = " + std::to_string(s.scattering_nu) + ";\n";
  src += "const int IRRADIANCE_TEXTURE_WIDTH = " + std::to_string(s.irradiance_width) + ";\n";
  src += "const int IRRADIANCE_TEXTURE_HEIGHT = " + std::to_string(s.irradiance_height) + ";\n";
  if (m->combined) src += "#define COMBINED_SCATTERING_TEXTURES\n";
  src += "// <atmosphere/definitions.glsl of the reference goes here>\n";
  src += "const AtmosphereParameters ATMOSPHERE = AtmosphereParameters(\n";
  src += v3(a.solar_irradiance) + ",\n" + Str6(a.sun_angular_radius) + ",\n" +
         Str6(a.bottom_radius) + ",\n" + Str6(a.top_radius) + ",\n" + prof(a.rayleigh_density) +
         ",\n" + v3(a.rayleigh_scattering) + ",\n" + prof(a.mie_density) + ",\n" +
         v3(a.mie_scattering) + ",\n" + v3(a.mie_extinction) + ",\n" +
         Str6(a.mie_phase_function_g) + ",\n" + prof(a.absorption_density) + ",\n" +
         v3(a.absorption_extinction) + ",\n" + v3(a.ground_albedo) + ",\n" +
         Str6(a.mu_s_min) + ");\n";
  src += "const vec3 SKY_SPECTRAL_RADIANCE_TO_LUMINANCE = vec3(" + Str6(m->sky_k[0]) + "," +
         Str6(m->sky_k[1]) + "," + Str6(m->sky_k[2]) + ");\n";
  src += "const vec3 SUN_SPECTRAL_RADIANCE_TO_LUMINANCE = vec3(" + Str6(m->sun_k[0]) + "," +
         Str6(m->sun_k[1]) + "," + Str6(m->sun_k[2]) + ");\n";
  src += "// <atmosphere/functions.glsl of the reference goes here>\n";
  if (m->num_precomputed_wavelengths <= 3) src += "#define RADIANCE_API_ENABLED\n";
  // API entry points of atmosphere/model.h:51-89 over the LUT samplers.
  src +=
      "uniform sampler2D transmittance_texture;\n"
      "uniform sampler3D scattering_texture;\n"
      "uniform sampler3D single_mie_scattering_texture;\n"
      "uniform sampler2D irradiance_texture;\n"
      "#ifdef RADIANCE_API_ENABLED\n"
      "RadianceSpectrum GetSolarRadiance() {\n"
      "  float a = ATMOSPHERE.sun_angular_radius;\n"
      "  return ATMOSPHERE.solar_irradiance / (PI * a * a);\n"
      "}\n"
      "RadianceSpectrum GetSkyRadiance(Position camera, Direction view_ray,\n"
      "    Length shadow_length, Direction sun_direction,\n"
      "    out DimensionlessSpectrum transmittance) {\n"
      "  return GetSkyRadiance(ATMOSPHERE, transmittance_texture, scattering_texture,\n"
      "      single_mie_scattering_texture, camera, view_ray, shadow_length,\n"
      "      sun_direction, transmittance);\n"
      "}\n"
      "RadianceSpectrum GetSkyRadianceToPoint(Position camera, Position point,\n"
      "    Length shadow_length, Direction sun_direction,\n"
      "    out DimensionlessSpectrum transmittance) {\n"
      "  return GetSkyRadianceToPoint(ATMOSPHERE, transmittance_texture,\n"
      "      scattering_texture, single_mie_scattering_texture, camera, point,\n"
      "      shadow_length, sun_direction, transmittance);\n"
      "}\n"
      "IrradianceSpectrum GetSunAndSkyIrradiance(Position p, Direction normal,\n"
      "    Direction sun_direction, out IrradianceSpectrum sky_irradiance) {\n"
      "  return GetSunAndSkyIrradiance(ATMOSPHERE, transmittance_texture,\n"
      "      irradiance_texture, p, normal, sun_direction, sky_irradiance);\n"
      "}\n"
      "#endif\n"
      "Luminance3 GetSolarLuminance() {\n"
      "  float a = ATMOSPHERE.sun_angular_radius;\n"
      "  return ATMOSPHERE.solar_irradiance / (PI * a * a) *\n"
      "      SUN_SPECTRAL_RADIANCE_TO_LUMINANCE;\n"
      "}\n"
      "Luminance3 GetSkyLuminance(Position camera, Direction view_ray,\n"
      "    Length shadow_length, Direction sun_direction,\n"
      "    out DimensionlessSpectrum transmittance) {\n"
      "  return GetSkyRadiance(ATMOSPHERE, transmittance_texture, scattering_texture,\n"
      "      single_mie_scattering_texture, camera, view_ray, shadow_length,\n"
      "      sun_direction, transmittance) * SKY_SPECTRAL_RADIANCE_TO_LUMINANCE;\n"
      "}\n"
      "Luminance3 GetSkyLuminanceToPoint(Position camera, Position point,\n"
      "    Length shadow_length, Direction sun_direction,\n"
      "    out DimensionlessSpectrum transmittance) {\n"
      "  return GetSkyRadianceToPoint(ATMOSPHERE, transmittance_texture,\n"
      "      scattering_texture, single_mie_scattering_texture, camera, point,\n"
      "      shadow_length, sun_direction, transmittance) *\n"
      "      SKY_SPECTRAL_RADIANCE_TO_LUMINANCE;\n"
      "}\n"
      "Illuminance3 GetSunAndSkyIlluminance(Position p, Direction normal,\n"
      "    Direction sun_direction, out IrradianceSpectrum sky_irradiance) {\n"
      "  IrradianceSpectrum sun_irradiance = GetSunAndSkyIrradiance(ATMOSPHERE,\n"
      "      transmittance_texture, irradiance_texture, p, normal, sun_direction,\n"
      "      sky_irradiance);\n"
      "  sky_irradiance *= SKY_SPECTRAL_RADIANCE_TO_LUMINANCE;\n"
      "  return sun_irradiance * SUN_SPECTRAL_RADIANCE_TO_LUMINANCE;\n"
      "}\n";
  if (needed) *needed = src.size() + 1;
  if (dst && capacity > 0) {
    size_t k = src.size() < capacity - 1 ? src.size() : capacity - 1;
    std::memcpy(dst, src.data(), k);
    dst[k] = '\0';
  }
  return ATMO_OK;
}

atmo_status atmo_model_set_program_uniforms(const atmo_model* m, unsigned, unsigned, unsigned,
                                            unsigned, unsigned) {
  if (!m) return Fail(ATMO_INVALID_ARG, "NULL model");
  return Fail(ATMO_UNAVAILABLE,
              "OpenGL texture binding is unavailable: this library has no graphics stack; use "
              "atmo_model_get_lut device buffers");
}

atmo_status atmo_convert_spectrum_to_linear_srgb(const double* wavelengths,
                                                 const double* spectrum, unsigned n, double* r,
                                                 double* g, double* b) {
  // atmosphere/model.cc:1020-1040
  if (!wavelengths || !spectrum || n == 0 || !r || !g || !b)
    return Fail(ATMO_INVALID_ARG, "NULL argument");
  std::vector<double> wl(wavelengths, wavelengths + n), sp(spectrum, spectrum + n);
  double x = 0.0, y = 0.0, z = 0.0;
  for (int lambda = (int)kLambdaMin; lambda < (int)kLambdaMax; ++lambda) {
    double v = Interpolate(wl, sp, lambda);
    x += CieValue(lambda, 1) * v;
    y += CieValue(lambda, 2) * v;
    z += CieValue(lambda, 3) * v;
  }
  const double* m = kXyzToSrgb;
  *r = kMaxLuminousEfficacy * (m[0] * x + m[1] * y + m[2] * z);
  *g = kMaxLuminousEfficacy * (m[3] * x + m[4] * y + m[5] * z);
  *b = kMaxLuminousEfficacy * (m[6] * x + m[7] * y + m[8] * z);
  return ATMO_OK;
}

atmo_status atmo_precompute(const atmo_atmosphere* atmosphere, const atmo_lut_shape* shape,
                            unsigned num_scattering_orders, const float lum[9], int blend,
                            int combined, atmo_path path, float* transmittance,
                            float* scattering, float* single_mie, float* irradiance,
                            atmo_stream stream) {
  if (!atmosphere || !transmittance || !scattering || !irradiance)
    return Fail(ATMO_INVALID_ARG, "NULL argument");
  if (!combined && !single_mie)
    return Fail(ATMO_INVALID_ARG, "single_mie is required when combined == 0");
  if (num_scattering_orders < 1 || num_scattering_orders > 64)
    return Fail(ATMO_INVALID_ARG, "num_scattering_orders must be in [1, 64]");
  atmo_lut_shape ls = shape ? *shape : DefaultShape();
  std::string why;
  if (!ValidShape(ls, &why) || !ValidAtmosphere(*atmosphere, &why))
    return Fail(ATMO_INVALID_ARG, why);
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  const Shape s = ToShape(ls);
  const size_t nI = (size_t)s.i_texels(), nS = (size_t)s.s_texels();
  Instance in;
  std::memset(&in, 0, sizeof(in));
  in.c = MakeConsts(*atmosphere, lum);
  in.s = s;
  in.T = reinterpret_cast<float4*>(transmittance);
  in.S = reinterpret_cast<float4*>(scattering);
  in.M = combined ? nullptr : reinterpret_cast<float4*>(single_mie);
  in.I = reinterpret_cast<float4*>(irradiance);
  in.combined = combined ? 1 : 0;
  in.blend = blend ? 1 : 0;
  // Temporaries, stream ordered.
  const size_t nT = (size_t)s.t_texels();
  const size_t bytes[9] = {nI * 16, nS * 16, nS * 16, nS * 16,
                           (size_t)s.sr * s.smu * sizeof(TexelRow),
                           (size_t)s.smus * sizeof(TexelCol),
                           (size_t)s.sr * kDensityThetaSamples * sizeof(DensityRow),
                           (size_t)s.ih * sizeof(IrrRow) + (size_t)s.iw * sizeof(float),
                           nT * 16};
  void* tmp[9] = {nullptr};
  for (int i = 0; i < 9; ++i) {
    cudaError_t e = cudaMallocAsync(&tmp[i], bytes[i], st);
    if (e != cudaSuccess) {
      for (int j = 0; j < i; ++j) cudaFreeAsync(tmp[j], st);
      return CudaFail(e, "cudaMallocAsync");
    }
  }
  in.dI = (float4*)tmp[0];
  in.dR = (float4*)tmp[1];
  in.dM = (float4*)tmp[2];
  in.dJ = (float4*)tmp[3];
  in.tab.rows = (TexelRow*)tmp[4];
  in.tab.cols = (TexelCol*)tmp[5];
  in.tab.drows = (DensityRow*)tmp[6];
  in.tab.irows = (IrrRow*)tmp[7];
  in.tab.mus_i = (float*)((char*)tmp[7] + (size_t)s.ih * sizeof(IrrRow));
  in.Tau = (float4*)tmp[8];
  atmo_status result;
  {
    Program prog;
    prog.path = path;
    prog.slots.push_back(in);
    prog.orders.push_back(num_scattering_orders);
    prog.AddStage({0});
    result = prog.Run(st, /*use_graph=*/false);
    // The program's work lists are freed when it goes out of scope: wait for
    // the launches that read them.
    cudaError_t e = cudaStreamSynchronize(st);
    if (result == ATMO_OK && e != cudaSuccess) result = CudaFail(e, "precompute");
  }
  for (int i = 0; i < 9; ++i) cudaFreeAsync(tmp[i], st);
  return result;
}

atmo_status atmo_batch_create(const atmo_atmosphere* atmospheres, const atmo_lut_shape* shapes,
                              const unsigned* num_scattering_orders, unsigned n, int combined,
                              atmo_batch** out) {
  if (!atmospheres || !num_scattering_orders || !out || n == 0)
    return Fail(ATMO_INVALID_ARG, "NULL argument or empty batch");
  *out = nullptr;
  std::string why;
  for (unsigned i = 0; i < n; ++i) {
    atmo_lut_shape ls = shapes ? shapes[i] : DefaultShape();
    if (!ValidShape(ls, &why) || !ValidAtmosphere(atmospheres[i], &why))
      return Fail(ATMO_INVALID_ARG, "instance " + std::to_string(i) + ": " + why);
    if (num_scattering_orders[i] < 1 || num_scattering_orders[i] > 64)
      return Fail(ATMO_INVALID_ARG, "num_scattering_orders must be in [1, 64]");
  }
  std::unique_ptr<atmo_batch> b(new atmo_batch());
  b->combined = combined != 0;
  b->storages.resize(n);
  std::unique_ptr<Program> prog(new Program());
  prog->path = ATMO_PATH_FAST;
  std::vector<int> members;
  for (unsigned i = 0; i < n; ++i) {
    atmo_lut_shape ls = shapes ? shapes[i] : DefaultShape();
    atmo_status st = b->storages[i].Allocate(ToShape(ls), b->combined, false);
    if (st != ATMO_OK) {
      for (auto& s : b->storages) s.Free();
      return st;
    }
    const Storage& sto = b->storages[i];
    Instance in;
    std::memset(&in, 0, sizeof(in));
    in.c = MakeConsts(atmospheres[i], nullptr);
    in.s = sto.s;
    in.tab = sto.tab;
    in.T = sto.T;
    in.Tau = sto.Tau;
    in.I = sto.I;
    in.dI = sto.dI;
    in.dI2 = sto.dI2;
    in.dR = sto.dR;
    in.dM = sto.dM;
    in.dJ = sto.dJ;
    in.S = sto.S;
    in.M = sto.M;
    in.combined = b->combined ? 1 : 0;
    in.blend = 0;
    prog->slots.push_back(in);
    prog->orders.push_back(num_scattering_orders[i]);
    members.push_back((int)i);
  }
  prog->AddStage(members);
  b->program = std::move(prog);
  *out = b.release();
  return ATMO_OK;
}

atmo_status atmo_batch_destroy(atmo_batch* b) {
  if (!b) return ATMO_OK;
  b->program.reset();
  for (auto& s : b->storages) s.Free();
  delete b;
  return ATMO_OK;
}

atmo_status atmo_batch_set_atmosphere(atmo_batch* b, unsigned i, const atmo_atmosphere* a) {
  if (!b || !a || i >= b->storages.size()) return Fail(ATMO_INVALID_ARG, "bad argument");
  std::string why;
  if (!ValidAtmosphere(*a, &why)) return Fail(ATMO_INVALID_ARG, why);
  b->program->slots[i].c = MakeConsts(*a, nullptr);
  return ATMO_OK;
}

static void RefreshBatchSets(atmo_batch* b) {
  b->lut_sets.resize(b->storages.size());
  for (size_t i = 0; i < b->storages.size(); ++i) {
    atmo_lut_set& set = b->lut_sets[i];
    set.luts = LutsOf(b->program->slots[i]);
    set.luminance_api = false;
    set.radiance_api = true;
    const Consts& c = b->program->slots[i].c;
    set.solar[0] = c.solar.x;
    set.solar[1] = c.solar.y;
    set.solar[2] = c.solar.z;
    set.sun_angular_radius = c.alpha_s;
  }
}

atmo_status atmo_batch_run(atmo_batch* b, atmo_stream stream) {
  if (!b) return Fail(ATMO_INVALID_ARG, "NULL batch");
  atmo_status s = b->program->Run(reinterpret_cast<cudaStream_t>(stream), /*use_graph=*/true);
  if (s != ATMO_OK) return s;
  b->ran = true;
  RefreshBatchSets(b);
  return ATMO_OK;
}

atmo_status atmo_batch_get_lut(const atmo_batch* b, unsigned i, atmo_lut_kind kind,
                               atmo_lut_view* view) {
  if (!b || !view || i >= b->storages.size()) return Fail(ATMO_INVALID_ARG, "bad argument");
  return ViewOf(b->storages[i], kind, view);
}

atmo_status atmo_batch_read_lut(const atmo_batch* b, unsigned i, atmo_lut_kind kind,
                                float* dst, size_t bytes) {
  if (!b || i >= b->storages.size()) return Fail(ATMO_INVALID_ARG, "bad argument");
  if (!b->ran) return Fail(ATMO_NOT_READY, "atmo_batch_run has not been called");
  atmo_lut_view v;
  atmo_status s = ViewOf(b->storages[i], kind, &v);
  if (s != ATMO_OK) return s;
  return ReadView(v, dst, bytes);
}

atmo_status atmo_batch_copy_lut(const atmo_batch* b, unsigned i, atmo_lut_kind kind, void* dst,
                                size_t bytes, atmo_stream stream) {
  if (!b || !dst || i >= b->storages.size()) return Fail(ATMO_INVALID_ARG, "bad argument");
  atmo_lut_view v;
  atmo_status s = ViewOf(b->storages[i], kind, &v);
  if (s != ATMO_OK) return s;
  if (bytes != v.bytes) return Fail(ATMO_INVALID_ARG, "destination size mismatch");
  ATMO_CUDA_TRY(cudaMemcpyAsync(dst, v.device_ptr, bytes, cudaMemcpyDefault,
                                reinterpret_cast<cudaStream_t>(stream)));
  return ATMO_OK;
}

atmo_status atmo_batch_kernel_count(const atmo_batch* b, unsigned* count) {
  if (!b || !count) return Fail(ATMO_INVALID_ARG, "NULL argument");
  *count = (unsigned)b->program->KernelCount();
  return ATMO_OK;
}

atmo_status atmo_batch_time_passes(atmo_batch* b, atmo_stream stream, unsigned capacity,
                                   float* ms, int* pass, int* order, unsigned* count) {
  if (!b || !count) return Fail(ATMO_INVALID_ARG, "NULL argument");
  std::vector<float> t;
  atmo_status s = b->program->TimeSteps(reinterpret_cast<cudaStream_t>(stream), &t);
  if (s != ATMO_OK) return s;
  b->ran = true;
  RefreshBatchSets(b);
  const auto& steps = b->program->steps();
  *count = (unsigned)steps.size();
  for (size_t i = 0; i < steps.size() && i < capacity; ++i) {
    if (ms) ms[i] = t[i];
    if (pass) pass[i] = (int)steps[i].pass;
    if (order) order[i] = steps[i].order;
  }
  return ATMO_OK;
}

atmo_status atmo_measure_fp32_peak(double* tflops) {
  if (!tflops) return Fail(ATMO_INVALID_ARG, "NULL argument");
  ATMO_CUDA_TRY(MeasureFp32Peak(tflops));
  return ATMO_OK;
}

atmo_status atmo_device_checks(int reset, int* compiled, unsigned long long* first_failure) {
  if (!compiled || !first_failure) return Fail(ATMO_INVALID_ARG, "NULL argument");
  *compiled = kDeviceChecks ? 1 : 0;
  *first_failure = 0;
  if (!kDeviceChecks) return ATMO_OK;
  ATMO_CUDA_TRY(cudaDeviceSynchronize());
  // One word per translation unit with kernels; the first nonzero one.
  unsigned long long (*const words[4])(bool) = {CheckWordKernels, CheckWordRays,
                                                CheckWordFast, CheckWordRender};
  for (auto word : words) {
    const unsigned long long w = word(reset != 0);
    if (w == ~0ull) return Fail(ATMO_CUDA_ERROR, "reading a device check word");
    if (*first_failure == 0) *first_failure = w;
  }
  return ATMO_OK;
}

atmo_status atmo_device_checks_selftest(atmo_stream stream) {
  ATMO_CUDA_TRY(LaunchCheckSelfTest(reinterpret_cast<cudaStream_t>(stream)));
  return ATMO_OK;
}


// ---- render-time queries ----------------------------------------------------
atmo_status atmo_model_lut_set(const atmo_model* m, const atmo_lut_set** out) {
  if (!m || !out) return Fail(ATMO_INVALID_ARG, "NULL argument");
  if (!m->initialized || !m->lut_set) return Fail(ATMO_NOT_READY, "Init has not been called");
  *out = m->lut_set.get();
  return ATMO_OK;
}

atmo_status atmo_batch_lut_set(const atmo_batch* b, unsigned i, const atmo_lut_set** out) {
  if (!b || !out || i >= b->storages.size()) return Fail(ATMO_INVALID_ARG, "bad argument");
  if (!b->ran || b->lut_sets.size() != b->storages.size())
    return Fail(ATMO_NOT_READY, "atmo_batch_run has not been called");
  *out = &b->lut_sets[i];
  return ATMO_OK;
}

static atmo_status CheckApi(const atmo_lut_set* set, int luminance) {
  if (!set) return Fail(ATMO_INVALID_ARG, "NULL LUT set");
  if (luminance && !set->luminance_api)
    return Fail(ATMO_INVALID_ARG,
                "no radiance-to-luminance factors for this LUT set (batch instances carry "
                "3-wavelength atmospheres without a spectrum)");
  if (!luminance && !set->radiance_api)
    return Fail(ATMO_INVALID_ARG,
                "the radiance API is not enabled with more than 3 precomputed wavelengths "
                "(model.cc RADIANCE_API_ENABLED); use luminance = 1");
  return ATMO_OK;
}

static atmo_status RunQuery(Query kind, const atmo_lut_set* set, const float* a, const float* b,
                            const float* shadow, const float* sun, int sun_stride, unsigned n,
                            int luminance, float* out0, float* out1, atmo_stream stream) {
  atmo_status cs = CheckApi(set, luminance);
  if (cs != ATMO_OK) return cs;
  if (n == 0) return ATMO_OK;
  if (!a || !b || !sun || !out0 || (sun_stride != 0 && sun_stride != 3))
    return Fail(ATMO_INVALID_ARG, "NULL array or sun_stride not 0 or 3");
  QueryArrays x;
  x.a = a;
  x.b = b;
  x.shadow = shadow;
  x.sun = sun;
  x.sun_stride = sun_stride;
  x.n = n;
  x.luminance = luminance ? 1 : 0;
  x.out0 = out0;
  x.out1 = out1;
  cudaError_t e = LaunchQuery(kind, set->luts, x, reinterpret_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return CudaFail(e, "query kernel launch");
  return ATMO_OK;
}

atmo_status atmo_sky_radiance(const atmo_lut_set* set, const float* camera, const float* view_ray,
                              const float* shadow_length, const float* sun_direction,
                              int sun_stride, unsigned n, int luminance, float* radiance,
                              float* transmittance, atmo_stream stream) {
  return RunQuery(Query::kSkyRadiance, set, camera, view_ray, shadow_length, sun_direction,
                  sun_stride, n, luminance, radiance, transmittance, stream);
}

atmo_status atmo_sky_radiance_to_point(const atmo_lut_set* set, const float* camera,
                                       const float* point, const float* shadow_length,
                                       const float* sun_direction, int sun_stride, unsigned n,
                                       int luminance, float* radiance, float* transmittance,
                                       atmo_stream stream) {
  return RunQuery(Query::kSkyRadianceToPoint, set, camera, point, shadow_length, sun_direction,
                  sun_stride, n, luminance, radiance, transmittance, stream);
}

atmo_status atmo_sun_and_sky_irradiance(const atmo_lut_set* set, const float* point,
                                        const float* normal, const float* sun_direction,
                                        int sun_stride, unsigned n, int luminance,
                                        float* sun_irradiance, float* sky_irradiance,
                                        atmo_stream stream) {
  return RunQuery(Query::kSunAndSkyIrradiance, set, point, normal, nullptr, sun_direction,
                  sun_stride, n, luminance, sun_irradiance, sky_irradiance, stream);
}

atmo_status atmo_solar_radiance(const atmo_lut_set* set, int luminance, double out[3]) {
  atmo_status cs = CheckApi(set, luminance);
  if (cs != ATMO_OK) return cs;
  if (!out) return Fail(ATMO_INVALID_ARG, "NULL argument");
  // model.cc:226-229 and :251-255; PI as in the reference's definitions.
  const double a = set->sun_angular_radius;
  for (int i = 0; i < 3; ++i) {
    out[i] = set->solar[i] / (kPiD * a * a);
    if (luminance) out[i] *= set->luts.sun_k[i];
  }
  return ATMO_OK;
}

atmo_status atmo_shade_view(const atmo_lut_set* set, const atmo_pinhole_view* view,
                            const float* depth, int luminance, float* sky_rgba,
                            float* shaded_rgba, atmo_stream stream) {
  atmo_status cs = CheckApi(set, luminance);
  if (cs != ATMO_OK) return cs;
  if (!view || !depth || !sky_rgba || !shaded_rgba)
    return Fail(ATMO_INVALID_ARG, "NULL argument");
  if (view->width <= 0 || view->height <= 0 || !(view->fov_y > 0.0f && view->fov_y < 3.1f))
    return Fail(ATMO_INVALID_ARG, "bad view size or field of view");
  PinholeView v;
  for (int i = 0; i < 3; ++i) {
    v.camera[i] = view->camera[i];
    v.right[i] = view->right[i];
    v.up[i] = view->up[i];
    v.forward[i] = view->forward[i];
    v.sun[i] = view->sun_direction[i];
    v.albedo[i] = view->albedo[i];
  }
  v.tan_half_fov_y = std::tan(0.5f * view->fov_y);
  v.width = view->width;
  v.height = view->height;
  v.depth = depth;
  v.luminance = luminance ? 1 : 0;
  v.sky = reinterpret_cast<float4*>(sky_rgba);
  v.shaded = reinterpret_cast<float4*>(shaded_rgba);
  cudaError_t e = LaunchShadeView(set->luts, v, reinterpret_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return CudaFail(e, "shading kernel launch");
  return ATMO_OK;
}

// ---- LUT files (atmosphere/demo/webgl/precompute.cc:63-106) ------------------
static std::string JoinPath(const char* dir, const char* name) {
  std::string d(dir);
  if (!d.empty() && d.back() != '/') d += '/';
  return d + name;
}

static atmo_status WriteFile(const std::string& path, const void* data, size_t bytes) {
  std::ofstream out(path, std::ofstream::out | std::ofstream::binary);
  if (!out) return Fail(ATMO_INVALID_ARG, "cannot open " + path + " for writing");
  out.write(static_cast<const char*>(data), (std::streamsize)bytes);
  if (!out) return Fail(ATMO_INVALID_ARG, "cannot write " + path);
  return ATMO_OK;
}

// Reads exactly `bytes` bytes; *present = false when the file does not exist.
static atmo_status ReadFile(const std::string& path, size_t bytes, std::vector<float>* out,
                            bool* present) {
  std::ifstream in(path, std::ifstream::in | std::ifstream::binary);
  if (present) *present = (bool)in;
  if (!in) {
    if (present) return ATMO_OK;
    return Fail(ATMO_INVALID_ARG, "cannot open " + path);
  }
  in.seekg(0, std::ios::end);
  const std::streamoff size = in.tellg();
  if (size < 0 || (size_t)size != bytes)
    return Fail(ATMO_INVALID_ARG, path + " has " + std::to_string((long long)size) +
                                      " bytes, the LUT shape needs " + std::to_string(bytes));
  in.seekg(0, std::ios::beg);
  out->resize(bytes / sizeof(float));
  in.read(reinterpret_cast<char*>(out->data()), (std::streamsize)bytes);
  if (!in) return Fail(ATMO_INVALID_ARG, "cannot read " + path);
  return ATMO_OK;
}

static atmo_status SaveStorage(const Storage& sto, const char* dir, const std::string* shader) {
  if (!dir) return Fail(ATMO_INVALID_ARG, "NULL directory");
  struct Item {
    atmo_lut_kind kind;
    const char* name;
  };
  std::vector<Item> items = {{ATMO_LUT_TRANSMITTANCE, "transmittance.dat"},
                             {ATMO_LUT_SCATTERING, "scattering.dat"},
                             {ATMO_LUT_IRRADIANCE, "irradiance.dat"}};
  if (!sto.combined) items.push_back({ATMO_LUT_SINGLE_MIE, "single_mie_scattering.dat"});
  std::vector<float> host;
  for (const Item& it : items) {
    atmo_lut_view v;
    atmo_status s = ViewOf(sto, it.kind, &v);
    if (s != ATMO_OK) return s;
    host.resize((size_t)v.width * v.height * v.depth * 4);
    if ((s = ReadView(v, host.data(), host.size() * sizeof(float))) != ATMO_OK) return s;
    if ((s = WriteFile(JoinPath(dir, it.name), host.data(), host.size() * sizeof(float))) !=
        ATMO_OK)
      return s;
  }
  // This library's optical-depth LUT, so that a reload keeps the ratios of
  // transmittances below FP32's normal range.
  host.resize((size_t)sto.s.t_texels() * 4);
  ATMO_CUDA_TRY(
      cudaMemcpy(host.data(), sto.Tau, host.size() * sizeof(float), cudaMemcpyDeviceToHost));
  atmo_status s = WriteFile(JoinPath(dir, "optical_depth.dat"), host.data(),
                            host.size() * sizeof(float));
  if (s != ATMO_OK) return s;
  if (shader) s = WriteFile(JoinPath(dir, "atmosphere_shader.txt"), shader->data(), shader->size());
  return s;
}

static atmo_status LoadStorage(Storage& sto, const char* dir) {
  if (!dir) return Fail(ATMO_INVALID_ARG, "NULL directory");
  const Shape& sh = sto.s;
  const size_t t_bytes = (size_t)sh.t_texels() * 16, s_bytes = (size_t)sh.s_texels() * 16,
               i_bytes = (size_t)sh.i_texels() * 16;
  std::vector<float> T, S, M, I, Tau;
  atmo_status s;
  // Every file is read and checked before any device buffer changes.
  if ((s = ReadFile(JoinPath(dir, "transmittance.dat"), t_bytes, &T, nullptr)) != ATMO_OK)
    return s;
  if ((s = ReadFile(JoinPath(dir, "scattering.dat"), s_bytes, &S, nullptr)) != ATMO_OK) return s;
  if ((s = ReadFile(JoinPath(dir, "irradiance.dat"), i_bytes, &I, nullptr)) != ATMO_OK) return s;
  if (!sto.combined &&
      (s = ReadFile(JoinPath(dir, "single_mie_scattering.dat"), s_bytes, &M, nullptr)) != ATMO_OK)
    return s;
  bool have_tau = false;
  if ((s = ReadFile(JoinPath(dir, "optical_depth.dat"), t_bytes, &Tau, &have_tau)) != ATMO_OK)
    return s;
  if (!have_tau) {
    // Files of the reference's tool: the optical depth from T itself.
    Tau.resize(T.size());
    for (size_t i = 0; i < T.size(); ++i)
      Tau[i] = (i % 4 == 3) ? 0.0f : -std::log(std::fmax(T[i], 1.17549435e-38f));
  }
  ATMO_CUDA_TRY(cudaMemcpy(sto.T, T.data(), t_bytes, cudaMemcpyHostToDevice));
  ATMO_CUDA_TRY(cudaMemcpy(sto.Tau, Tau.data(), t_bytes, cudaMemcpyHostToDevice));
  ATMO_CUDA_TRY(cudaMemcpy(sto.S, S.data(), s_bytes, cudaMemcpyHostToDevice));
  ATMO_CUDA_TRY(cudaMemcpy(sto.I, I.data(), i_bytes, cudaMemcpyHostToDevice));
  if (!sto.combined) ATMO_CUDA_TRY(cudaMemcpy(sto.M, M.data(), s_bytes, cudaMemcpyHostToDevice));
  if (sto.half) {
    cudaError_t e = LaunchToHalf(sto.S, sto.S_half, sh.s_texels(), nullptr);
    if (e == cudaSuccess && !sto.combined) e = LaunchToHalf(sto.M, sto.M_half, sh.s_texels(), nullptr);
    if (e != cudaSuccess) return CudaFail(e, "FP16 conversion");
  }
  ATMO_CUDA_TRY(cudaDeviceSynchronize());
  return ATMO_OK;
}

atmo_status atmo_model_save_luts(const atmo_model* m, const char* directory) {
  if (!m) return Fail(ATMO_INVALID_ARG, "NULL model");
  if (!m->initialized) return Fail(ATMO_NOT_READY, "Init has not been called");
  size_t need = 0;
  atmo_status s = atmo_model_shader_source(m, nullptr, 0, &need);
  if (s != ATMO_OK) return s;
  std::string shader(need, '\0');
  if ((s = atmo_model_shader_source(m, &shader[0], need, &need)) != ATMO_OK) return s;
  shader.resize(need > 0 ? need - 1 : 0);
  return SaveStorage(m->storage, directory, &shader);
}

atmo_status atmo_model_load_luts(atmo_model* m, const char* directory) {
  if (!m) return Fail(ATMO_INVALID_ARG, "NULL model");
  // Size checks first: they need no device.
  const Shape sh = ToShape(m->shape);
  const size_t t_bytes = (size_t)sh.t_texels() * 16, s_bytes = (size_t)sh.s_texels() * 16,
               i_bytes = (size_t)sh.i_texels() * 16;
  std::vector<float> probe;
  atmo_status s;
  if ((s = ReadFile(JoinPath(directory ? directory : "", "transmittance.dat"), t_bytes, &probe,
                    nullptr)) != ATMO_OK ||
      (s = ReadFile(JoinPath(directory ? directory : "", "irradiance.dat"), i_bytes, &probe,
                    nullptr)) != ATMO_OK)
    return s;
  (void)s_bytes;
  if ((s = EnsureStorage(m)) != ATMO_OK) return s;
  if ((s = LoadStorage(m->storage, directory)) != ATMO_OK) return s;
  m->initialized = true;
  BuildModelLutSet(m);
  return ATMO_OK;
}

atmo_status atmo_batch_save_luts(const atmo_batch* b, unsigned i, const char* directory) {
  if (!b || i >= b->storages.size()) return Fail(ATMO_INVALID_ARG, "bad argument");
  if (!b->ran) return Fail(ATMO_NOT_READY, "atmo_batch_run has not been called");
  return SaveStorage(b->storages[i], directory, nullptr);
}

atmo_status atmo_lut_set_read(const atmo_lut_set* set, atmo_lut_kind kind, float* host_dst,
                              size_t bytes) {
  if (!set || !host_dst) return Fail(ATMO_INVALID_ARG, "NULL argument");
  const Shape& sh = set->luts.s;
  const float4* src = nullptr;
  size_t texels = 0;
  switch (kind) {
    case ATMO_LUT_TRANSMITTANCE: src = set->luts.T; texels = sh.t_texels(); break;
    case ATMO_LUT_SCATTERING: src = set->luts.S; texels = (size_t)sh.s_texels(); break;
    case ATMO_LUT_SINGLE_MIE: src = set->luts.M; texels = (size_t)sh.s_texels(); break;
    case ATMO_LUT_IRRADIANCE: src = set->luts.I; texels = sh.i_texels(); break;
    default: return Fail(ATMO_INVALID_ARG, "unknown LUT kind");
  }
  if (!src) return Fail(ATMO_INVALID_ARG, "no single-Mie texture with combined scattering textures");
  if (bytes != texels * 16) return Fail(ATMO_INVALID_ARG, "host buffer size mismatch");
  ATMO_CUDA_TRY(cudaMemcpy(host_dst, src, bytes, cudaMemcpyDeviceToHost));
  return ATMO_OK;
}

// ---- autotuner ---------------------------------------------------------------
atmo_status atmo_set_tuning(const atmo_lut_shape* shape, const atmo_tuning* tuning) {
  atmo_lut_shape ls = shape ? *shape : DefaultShape();
  std::string why;
  if (!ValidShape(ls, &why)) return Fail(ATMO_INVALID_ARG, why);
  if (!tuning) {
    SetTuning(ls, nullptr);
    return ATMO_OK;
  }
  SetTuning(ls, nullptr);
  const Shape s = ToShape(ls);
  const bool m_default = tuning->multiple_rows == 0 && tuning->multiple_group == 0;
  const bool s_default = tuning->single_rows == 0 && tuning->single_group == 0;
  if ((!m_default && !FastTuningValid(s, false, tuning->multiple_rows, tuning->multiple_group)) ||
      (!s_default && !FastTuningValid(s, true, tuning->single_rows, tuning->single_group)))
    return Fail(ATMO_INVALID_ARG,
                "block shape not launchable for this LUT shape (rows 1-4 with rows x NU x "
                "MU_S <= 256, samples per stage 1-8, shared memory <= 48 KB)");
  const int t[4] = {tuning->multiple_rows, tuning->multiple_group, tuning->single_rows,
                    tuning->single_group};
  SetTuning(ls, t);
  return ATMO_OK;
}

atmo_status atmo_get_tuning(const atmo_lut_shape* shape, atmo_tuning* out) {
  if (!out) return Fail(ATMO_INVALID_ARG, "NULL argument");
  atmo_lut_shape ls = shape ? *shape : DefaultShape();
  std::string why;
  if (!ValidShape(ls, &why)) return Fail(ATMO_INVALID_ARG, why);
  const Shape s = ToShape(ls);
  out->multiple_rows = s.tune[0];
  out->multiple_group = s.tune[1];
  out->single_rows = s.tune[2];
  out->single_group = s.tune[3];
  return ATMO_OK;
}

atmo_status atmo_autotune(const atmo_atmosphere* atmosphere, const atmo_lut_shape* shape,
                          unsigned instances, atmo_tuning* out) {
  if (!atmosphere || !out) return Fail(ATMO_INVALID_ARG, "NULL argument");
  atmo_lut_shape ls = shape ? *shape : DefaultShape();
  std::string why;
  if (!ValidShape(ls, &why) || !ValidAtmosphere(*atmosphere, &why))
    return Fail(ATMO_INVALID_ARG, why);
  const unsigned n = instances ? instances : 4;
  if (n > 64) return Fail(ATMO_INVALID_ARG, "instances must be <= 64");
  SetTuning(ls, nullptr);
  const Shape base = ToShape(ls);
  std::vector<Storage> storages(n);
  for (unsigned i = 0; i < n; ++i) {
    atmo_status st = storages[i].Allocate(base, true, false);
    if (st != ATMO_OK) {
      for (auto& x : storages) x.Free();
      return st;
    }
  }
  struct Trial {
    int rows, group;
    float single_ms, multiple_ms;
  };
  std::vector<Trial> trials;
  const int rows_c[3] = {1, 2, 4}, group_c[6] = {1, 2, 3, 4, 6, 8};
  for (int r : rows_c) {
    for (int g : group_c) {
      const bool ms_ok = FastTuningValid(base, false, r, g);
      const bool ss_ok = FastTuningValid(base, true, r, g);
      if (!ms_ok && !ss_ok) continue;
      Shape s = base;
      s.tune[0] = ms_ok ? r : 0;
      s.tune[1] = ms_ok ? g : 0;
      s.tune[2] = ss_ok ? r : 0;
      s.tune[3] = ss_ok ? g : 0;
      Program prog;
      prog.path = ATMO_PATH_FAST;
      std::vector<int> members;
      for (unsigned i = 0; i < n; ++i) {
        const Storage& sto = storages[i];
        Instance in;
        std::memset(&in, 0, sizeof(in));
        in.c = MakeConsts(*atmosphere, nullptr);
        in.s = s;
        in.tab = sto.tab;
        in.T = sto.T;
        in.Tau = sto.Tau;
        in.I = sto.I;
        in.dI = sto.dI;
        in.dI2 = sto.dI2;
        in.dR = sto.dR;
        in.dM = sto.dM;
        in.dJ = sto.dJ;
        in.S = sto.S;
        in.combined = 1;
        prog.slots.push_back(in);
        prog.orders.push_back(2);
        members.push_back((int)i);
      }
      prog.AddStage(members);
      Trial t{r, g, 1e30f, 1e30f};
      for (int rep = 0; rep < 3; ++rep) {
        std::vector<float> ms;
        atmo_status st = prog.TimeSteps(nullptr, &ms);
        if (st != ATMO_OK) {
          for (auto& x : storages) x.Free();
          return st;
        }
        float single = 0.0f, multiple = 0.0f;
        for (size_t i = 0; i < prog.steps().size(); ++i) {
          if (prog.steps()[i].pass == Pass::kSingle) single += ms[i];
          if (prog.steps()[i].pass == Pass::kMultiple) multiple += ms[i];
        }
        if (ss_ok) t.single_ms = std::min(t.single_ms, single);
        if (ms_ok) t.multiple_ms = std::min(t.multiple_ms, multiple);
      }
      trials.push_back(t);
    }
  }
  for (auto& x : storages) x.Free();
  atmo_tuning best{0, 0, 0, 0, 0.0f, 0.0f};
  float best_s = 1e30f, best_m = 1e30f;
  for (const Trial& t : trials) {
    if (t.multiple_ms < best_m) {
      best_m = t.multiple_ms;
      best.multiple_rows = t.rows;
      best.multiple_group = t.group;
    }
    if (t.single_ms < best_s) {
      best_s = t.single_ms;
      best.single_rows = t.rows;
      best.single_group = t.group;
    }
  }
  best.multiple_ms = best_m / (float)n;
  best.single_ms = best_s / (float)n;
  const int tv[4] = {best.multiple_rows, best.multiple_group, best.single_rows, best.single_group};
  SetTuning(ls, tv);
  *out = best;
  return ATMO_OK;
}
}  // extern "C"
