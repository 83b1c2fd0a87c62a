// atmo_kernels.cu -- sm_103a kernels of the transmittance and irradiance
// passes: one launch per pass of atmosphere/model.cc:1048-1215 covering every
// instance of a work list (a single model is a work list of one).  IEEE
// division and square root: their lookups start from LUT rows and columns of
// the set-up tables and must land on texel centres and LUT edges exactly.
#include "atmo_kernels.h"
#include "atmo_passes.cuh"

namespace atmo {

// Transmittance: kTransmittanceLanes lanes per texel split the 501 samples of
// each optical length; the partial Kahan sums are reduced with shuffles.
__global__ void __launch_bounds__(kTransmittanceThreads)
k_transmittance(const Instance* __restrict__ insts, WorkList wl) {
  int local;
  const Instance& in = insts[FindEntry(wl, blockIdx.x, &local)];
  const int lane = threadIdx.x % kTransmittanceLanes;
  const int texel = local * kTransmittanceTexelsPerTile + threadIdx.x / kTransmittanceLanes;
  const bool valid = texel < in.s.t_texels();
  float sums[3] = {0.0f, 0.0f, 0.0f};
  TransmittanceRay ray{0.0f, 0.0f, 0.0f};
  if (valid) {
    ray = TransmittanceTexelRay(in.c, in.s, texel);
    OpticalLengthPartial(in.c, ray, lane, kTransmittanceLanes, sums);
  }
#pragma unroll
  for (int off = kTransmittanceLanes / 2; off > 0; off >>= 1) {
    sums[0] += __shfl_xor_sync(0xffffffffu, sums[0], off, kTransmittanceLanes);
    sums[1] += __shfl_xor_sync(0xffffffffu, sums[1], off, kTransmittanceLanes);
    sums[2] += __shfl_xor_sync(0xffffffffu, sums[2], off, kTransmittanceLanes);
  }
  if (valid && lane == 0) {
    F3 tau = OpticalDepth(in.c, ray, sums);
    in.T[texel] = to4(exp3(f3(0.0f) - tau), 1.0f);
    in.Tau[texel] = to4(tau, 0.0f);
  }
}

// Direct irradiance texels, then the ground transmittance of every density
// quadrature row (both read only the transmittance LUT).
__global__ void __launch_bounds__(kTexelThreads)
k_direct_irradiance(const Instance* __restrict__ insts, WorkList wl) {
  int local;
  const Instance& in = insts[FindEntry(wl, blockIdx.x, &local)];
  int e = local * kTexelThreads + threadIdx.x;
  const int n_i = in.s.i_texels();
  if (e < n_i) {
    in.dI[e] = to4(DirectIrradianceTexel(in, e), 1.0f);
    if (!in.blend) in.I[e] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    return;
  }
  e -= n_i;
  if (e < in.s.sr * kDensityThetaSamples) in.tab.drows[e].t_ground = GroundRowTransmittance(in, e);
}

// Indirect irradiance: one warp per texel, lanes over the 64 phi samples.
__global__ void __launch_bounds__(kIndirectThreads)
k_indirect_irradiance(const Instance* __restrict__ insts, WorkList wl, int order) {
  int local;
  const Instance& in = insts[FindEntry(wl, blockIdx.x, &local)];
  const int lane = threadIdx.x & 31;
  const int texel = local * kIndirectTexelsPerTile + threadIdx.x / 32;
  const bool valid = texel < in.s.i_texels();
  F3 acc = valid ? IndirectIrradiancePartial(in, texel, order, lane, 32) : f3(0.0f);
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    acc.x += __shfl_xor_sync(0xffffffffu, acc.x, off);
    acc.y += __shfl_xor_sync(0xffffffffu, acc.y, off);
    acc.z += __shfl_xor_sync(0xffffffffu, acc.z, off);
  }
  if (valid && lane == 0) {
    in.dI[texel] = to4(acc, 1.0f);
    F3 add = MatVec(in.c.lum, acc);
    float4 o = in.I[texel];
    in.I[texel] = make_float4(o.x + add.x, o.y + add.y, o.z + add.z, o.w);
  }
}

// ---------------------------------------------------------------------------
// Host-side launchers.
// ---------------------------------------------------------------------------
cudaError_t LaunchTransmittance(const Instance* insts, WorkList wl, int tiles, cudaStream_t st) {
  k_transmittance<<<tiles, kTransmittanceThreads, 0, st>>>(insts, wl);
  return cudaGetLastError();
}
cudaError_t LaunchDirectIrradiance(const Instance* insts, WorkList wl, int tiles,
                                   cudaStream_t st) {
  k_direct_irradiance<<<tiles, kTexelThreads, 0, st>>>(insts, wl);
  return cudaGetLastError();
}
cudaError_t LaunchIndirectIrradiance(const Instance* insts, WorkList wl, int tiles, int order,
                                     cudaStream_t st) {
  k_indirect_irradiance<<<tiles, kIndirectThreads, 0, st>>>(insts, wl, order);
  return cudaGetLastError();
}
}  // namespace atmo
