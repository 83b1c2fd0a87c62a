// atmo_rays.cu -- sm_103a kernels that march along the scattering texels'
// rays: single scattering, the plain per-texel scattering density and
// multiple scattering (atmosphere/model.cc:142-208 shaders).  Built with the
// approximate (<= 2 ulp) FP32 division and square root: the samples move
// continuously along each ray, and the ray's end points are exact by
// construction (the remaining distance is carried separately).
#include "atmo_kernels.h"
#include "atmo_passes.cuh"

namespace atmo {

__global__ void __launch_bounds__(kTexelThreads)
k_single_scattering(const Instance* __restrict__ insts, WorkList wl) {
  int local;
  const Instance& in = insts[FindEntry(wl, blockIdx.x, &local)];
  long long texel = (long long)local * kTexelThreads + threadIdx.x;
  if (texel >= in.s.s_texels()) return;
  F3 ray, mie;
  SingleScatteringTexel(in, texel, &ray, &mie);
  StoreSingleScattering(in, texel, ray, mie);
}

__global__ void __launch_bounds__(kTexelThreads)
k_density_plain(const Instance* __restrict__ insts, WorkList wl, int order) {
  int local;
  const Instance& in = insts[FindEntry(wl, blockIdx.x, &local)];
  long long texel = (long long)local * kTexelThreads + threadIdx.x;
  if (texel >= in.s.s_texels()) return;
  in.dJ[texel] = to4(ScatteringDensityTexel(in, texel, order), 1.0f);
}

__global__ void __launch_bounds__(kTexelThreads)
k_multiple_plain(const Instance* __restrict__ insts, WorkList wl) {
  int local;
  const Instance& in = insts[FindEntry(wl, blockIdx.x, &local)];
  long long texel = (long long)local * kTexelThreads + threadIdx.x;
  if (texel >= in.s.s_texels()) return;
  float nu;
  F3 dm = MultipleScatteringTexel(in, texel, &nu);
  in.dR[texel] = to4(dm, 1.0f);   // delta multiple aliases delta Rayleigh
  F3 add = MatVec(in.c.lum, dm) * (1.0f / RayleighPhase(in.c, nu));
  float4 o = in.S[texel];
  in.S[texel] = make_float4(o.x + add.x, o.y + add.y, o.z + add.z, o.w);
}

// ---------------------------------------------------------------------------
// Host-side launchers.
// ---------------------------------------------------------------------------
cudaError_t LaunchSingleScattering(const Instance* insts, WorkList wl, int tiles,
                                   cudaStream_t st) {
  k_single_scattering<<<tiles, kTexelThreads, 0, st>>>(insts, wl);
  return cudaGetLastError();
}
cudaError_t LaunchDensityPlain(const Instance* insts, WorkList wl, int tiles, int order,
                               cudaStream_t st) {
  k_density_plain<<<tiles, kTexelThreads, 0, st>>>(insts, wl, order);
  return cudaGetLastError();
}
cudaError_t LaunchMultiplePlain(const Instance* insts, WorkList wl, int tiles,
                                cudaStream_t st) {
  k_multiple_plain<<<tiles, kTexelThreads, 0, st>>>(insts, wl);
  return cudaGetLastError();
}

ATMO_CHECK_WORD_ACCESSOR(CheckWordRays)

}  // namespace atmo
