// atmo_pass_api.cu -- atmo_run_pass: one pass of the order loop of
// Model::Precompute (atmosphere/model.cc:1137-1211) over caller-owned device
// LUTs.  The scattering density, indirect irradiance and multiple scattering
// kernels then run on inputs the caller chooses, e.g. the uniform radiance,
// uniform irradiance and unit transmittance under which
// atmosphere/reference/functions_test.cc:1130-1344 states closed forms.
//
// The pass reads the instance's set-up tables (per-texel r, mu, mu_s, nu in
// FP64-derived form, k_tables) and the ground transmittance of every density
// quadrature row (computed by the direct-irradiance pass from the
// transmittance LUT), and the optical depth -ln T beside the transmittance
// LUT.  This entry point derives all three from the caller's transmittance,
// writing the direct-irradiance pass's own outputs into private temporaries,
// then runs the requested pass with the caller's buffers in the instance
// record.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <string>

#include "../../include/atmo/atmo.h"
#include "atmo_consts.h"
#include "atmo_kernels.h"
#include "atmo_program.h"

namespace atmo {
namespace {

// -ln T per channel (alpha 0), with T clamped to FP32's smallest normal as
// the LUT-file loader does.
__global__ void k_optical_depth(const float4* __restrict__ T, float4* __restrict__ tau, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float4 t = T[i];
  const float lo = 1.17549435e-38f;
  tau[i] = make_float4(-logf(fmaxf(t.x, lo)), -logf(fmaxf(t.y, lo)), -logf(fmaxf(t.z, lo)), 0.0f);
}

}  // namespace
}  // namespace atmo

using namespace atmo;

extern "C" atmo_status atmo_run_pass(const atmo_atmosphere* atmosphere,
                                     const atmo_lut_shape* shape, atmo_pass_kind pass,
                                     unsigned order, atmo_path path,
                                     const atmo_pass_buffers* b, atmo_stream stream) {
  if (!atmosphere || !b || !b->transmittance) {
    SetError("NULL argument");
    return ATMO_INVALID_ARG;
  }
  if (path != ATMO_PATH_FAST && path != ATMO_PATH_PLAIN) {
    SetError("unknown path");
    return ATMO_INVALID_ARG;
  }
  Pass p;
  bool ok = order >= 1 && order <= 64;
  switch (pass) {
    case ATMO_PASS_SCATTERING_DENSITY:
      p = Pass::kDensity;
      ok = ok && order >= 2 && b->delta_rayleigh && b->delta_irradiance && b->delta_density &&
           (order > 2 || b->delta_mie);
      break;
    case ATMO_PASS_INDIRECT_IRRADIANCE:
      p = Pass::kIndirect;
      ok = ok && b->delta_rayleigh && b->delta_irradiance && b->irradiance &&
           (order > 1 || b->delta_mie);
      break;
    case ATMO_PASS_MULTIPLE_SCATTERING:
      p = Pass::kMultiple;
      ok = ok && order >= 2 && b->delta_rayleigh && b->delta_density && b->scattering;
      break;
    default:
      SetError("unknown pass");
      return ATMO_INVALID_ARG;
  }
  if (!ok) {
    SetError("atmo_run_pass: order out of range or a buffer the pass reads or writes is NULL");
    return ATMO_INVALID_ARG;
  }
  atmo_lut_shape ls = shape ? *shape : DefaultShape();
  std::string why;
  if (!ValidShape(ls, &why) || !ValidAtmosphere(*atmosphere, &why)) {
    SetError(why);
    return ATMO_INVALID_ARG;
  }
  const Shape s = ToShape(ls);
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);

  // Instance records: [0] for the set-up passes, [1] for the requested pass;
  // then three work lists {inst = k; start = 0, tiles}.
  Instance in[2];
  std::memset(in, 0, sizeof(in));
  in[0].c = MakeConsts(*atmosphere, nullptr);
  in[0].s = s;
  in[0].combined = 1;
  const size_t nT = (size_t)s.t_texels(), nI = (size_t)s.i_texels();
  const size_t bytes[7] = {nT * 16,
                           nI * 16,
                           nI * 16,
                           (size_t)s.sr * s.smu * sizeof(TexelRow),
                           (size_t)s.smus * sizeof(TexelCol),
                           (size_t)s.sr * kDensityThetaSamples * sizeof(DensityRow),
                           (size_t)s.ih * sizeof(IrrRow) + (size_t)s.iw * sizeof(float)};
  const size_t desc_bytes = sizeof(in) + 9 * sizeof(int);
  void* tmp[8] = {nullptr};
  for (int i = 0; i < 8; ++i) {
    cudaError_t e = cudaMallocAsync(&tmp[i], i < 7 ? bytes[i] : desc_bytes, st);
    if (e != cudaSuccess) {
      for (int j = 0; j < i; ++j) cudaFreeAsync(tmp[j], st);
      return CudaFail(e, "cudaMallocAsync");
    }
  }
  in[0].T = const_cast<float4*>(reinterpret_cast<const float4*>(b->transmittance));
  in[0].Tau = (float4*)tmp[0];
  in[0].dI = (float4*)tmp[1];   // the direct pass's outputs stay private
  in[0].I = (float4*)tmp[2];
  in[0].tab.rows = (TexelRow*)tmp[3];
  in[0].tab.cols = (TexelCol*)tmp[4];
  in[0].tab.drows = (DensityRow*)tmp[5];
  in[0].tab.irows = (IrrRow*)tmp[6];
  in[0].tab.mus_i = (float*)((char*)tmp[6] + (size_t)s.ih * sizeof(IrrRow));
  in[1] = in[0];
  in[1].dR = reinterpret_cast<float4*>(b->delta_rayleigh);
  in[1].dM = reinterpret_cast<float4*>(b->delta_mie);
  in[1].dI = reinterpret_cast<float4*>(b->delta_irradiance);
  in[1].dJ = reinterpret_cast<float4*>(b->delta_density);
  in[1].S = reinterpret_cast<float4*>(b->scattering);
  in[1].I = reinterpret_cast<float4*>(b->irradiance);

  const atmo_path pp = PassPath(p, s, path);
  const int step_order = (int)order;
  const int tiles[3] = {Tiles(Pass::kTables, s, path), Tiles(Pass::kDirect, s, path),
                        Tiles(p, s, pp)};
  struct {
    Instance in[2];
    int wl[9];
  } desc;
  desc.in[0] = in[0];
  desc.in[1] = in[1];
  const int owner[3] = {0, 0, 1};
  for (int i = 0; i < 3; ++i) {
    desc.wl[3 * i] = owner[i];
    desc.wl[3 * i + 1] = 0;
    desc.wl[3 * i + 2] = tiles[i];
  }
  Instance* d_in = (Instance*)tmp[7];
  const int* d_wl = reinterpret_cast<const int*>((char*)tmp[7] + sizeof(desc.in));
  auto wl_of = [&](int i) {
    WorkList wl;
    wl.inst = d_wl + 3 * i;
    wl.start = d_wl + 3 * i + 1;
    wl.count = 1;
    return wl;
  };
  atmo_status result = ATMO_OK;
  cudaError_t e = cudaMemcpyAsync(d_in, &desc, desc_bytes, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) {
    k_optical_depth<<<(int)((nT + 255) / 256), 256, 0, st>>>(in[0].T, in[0].Tau, (int)nT);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = LaunchPass(Pass::kTables, 0, 0, d_in, wl_of(0), tiles[0], path, st);
  if (e == cudaSuccess) e = LaunchPass(Pass::kDirect, 0, 0, d_in, wl_of(1), tiles[1], path, st);
  if (e == cudaSuccess)
    e = LaunchPass(p, step_order, SharedBytes(p, s, in[1].c, step_order, pp), d_in, wl_of(2),
                   tiles[2], pp, st);
  if (e != cudaSuccess) result = CudaFail(e, "atmo_run_pass launch");
  // The host copy of the descriptors lives on this stack frame.
  const cudaError_t se = cudaStreamSynchronize(st);
  if (result == ATMO_OK && se != cudaSuccess) result = CudaFail(se, "atmo_run_pass");
  for (int i = 0; i < 8; ++i) cudaFreeAsync(tmp[i], st);
  return result;
}
