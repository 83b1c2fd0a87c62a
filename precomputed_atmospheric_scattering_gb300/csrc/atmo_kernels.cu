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

// Indirect irradiance, staged.  Every lookup of an irradiance texel is made
// at the texel's own r and mu_s, and on theta row t at mu = cos(theta_t):
// only nu varies with phi.  The warp of a texel therefore stages, per theta
// row, the trilinear (mu_s, mu, r) part of the 4D lookup at each nu node
// (n = 0..NU; node NU is the clamped edge the lerp reaches at nu = 1), and
// each direction's lookup becomes a lerp between two staged nodes: 16 (NU +
// 1) eight-tap fetches per texel instead of 1024 sixteen-tap ones.  The
// arithmetic is that of Scattering4 with the nu lerp applied to the node sums.
constexpr int kIndirectWarps = kIndirectThreads / 32;
__host__ __device__ inline int IndirectStagedSmem(const Shape& s, int order) {
  return kIndirectWarps * kIndirectThetaSamples * (s.snu + 1) * (order == 1 ? 2 : 1) * 16;
}
int IndirectSmem(const Shape& s, int order) {
  const int b = IndirectStagedSmem(s, order);
  return b <= 48 * 1024 ? b : 0;
}

// The trilinear (x within the node's block, y, z) part of Scattering4 for the
// nu node whose block starts at column base.
__device__ F3 ScatteringNode(const float4* __restrict__ tex, const Shape& s, int base, float xl,
                             float y, float z) {
  const int W = s.sw(), Hh = s.smu, D = s.sr;
  const float fy = floorf(y), fz = floorf(z), fx = floorf(xl);
  const float b = y - fy, c = z - fz, a = xl - fx;
  const int j0 = ClampIdx((int)fy, Hh), j1 = ClampIdx((int)fy + 1, Hh);
  const int k0 = ClampIdx((int)fz, D), k1 = ClampIdx((int)fz + 1, D);
  const int i0 = ClampIdx(base + (int)fx, W), i1 = ClampIdx(base + (int)fx + 1, W);
  const int rows[4] = {(k0 * Hh + j0) * W, (k0 * Hh + j1) * W, (k1 * Hh + j0) * W,
                       (k1 * Hh + j1) * W};
  const float wr[4] = {(1.0f - b) * (1.0f - c), b * (1.0f - c), (1.0f - b) * c, b * c};
  F3 acc = f3(0.0f);
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const float4 t0 = __ldg(ATMO_CHECKED_PTR(kCheckLutTexel, tex, rows[q], i0, W * Hh * D));
    const float4 t1 = __ldg(ATMO_CHECKED_PTR(kCheckLutTexel, tex, rows[q], i1, W * Hh * D));
    const float w0 = (1.0f - a) * wr[q], w1 = a * wr[q];
    acc.x += t0.x * w0 + t1.x * w1;
    acc.y += t0.y * w0 + t1.y * w1;
    acc.z += t0.z * w0 + t1.z * w1;
  }
  return acc;
}

// The lane's part (phi samples lane, lane + 32) of a texel's integral, from
// the nodes staged in V (the warp's region; order 1: Rayleigh then Mie).
__device__ F3 IndirectStagedPartial(const Instance& in, int texel, int order, int lane,
                                    float4* V) {
  const Consts& c = in.c;
  const Shape& s = in.s;
  const int i = texel % s.iw, j = texel / s.iw;
  const IrrRow ir = in.tab.irows[j];
  const float mu_s = in.tab.mus_i[i];
  const float sin_s = sqrtf(fmaxf((1.0f - mu_s) * (1.0f + mu_s), 0.0f));
  RadialPoint p;
  p.rho = ir.rho;
  p.r = ir.r;
  p.h = ir.h;
  const float u_r = TexCoord(s, kMapSR, ir.rho / c.H);
  const float u_mu_s = UMuSFromMuS(c, s, mu_s);
  const int NU = s.snu, N1 = NU + 1, nodes = kIndirectThetaSamples * N1;
  const float xl = fmaf(u_mu_s, float(s.smus), -0.5f), z = u_r * float(s.sr) - 0.5f;
  for (int e = lane; e < nodes; e += 32) {
    const int t = e / N1, n = e - t * N1;
    const float2 th = c_indirect_theta[t];
    const float y = UMuFromRMu(c, s, p, ir.r * th.x, false) * float(s.smu) - 0.5f;
    V[e] = to4(ScatteringNode(in.dR, s, n * s.smus, xl, y, z), 0.0f);
    if (order == 1) V[nodes + e] = to4(ScatteringNode(in.dM, s, n * s.smus, xl, y, z), 0.0f);
  }
  __syncwarp();
  const float dtdp = (kPiF / 32.0f) * (kPiF / 32.0f);
  F3 acc = f3(0.0f);
  for (int t = 0; t < kIndirectThetaSamples; ++t) {
    const float2 th = c_indirect_theta[t];
    const float4* row = V + t * N1;
    F3 row_sum = f3(0.0f);
    for (int m = lane; m < kIndirectPhiSamples; m += 32) {
      const float2 ph = c_indirect_phi[m];
      const float nu = fmaf(ph.x * th.y, sin_s, th.x * mu_s);
      const float tex_coord_x = (nu + 1.0f) * 0.5f * float(NU - 1);
      const float tex_x = floorf(tex_coord_x);
      const float l1 = tex_coord_x - tex_x, l0 = 1.0f - l1;
      const int n0 = min(max((int)tex_x, 0), NU - 1);
      const float4 r0 = row[n0], r1 = row[n0 + 1];
      F3 radiance{r0.x * l0 + r1.x * l1, r0.y * l0 + r1.y * l1, r0.z * l0 + r1.z * l1};
      if (order == 1) {
        const float4 m0 = row[nodes + n0], m1 = row[nodes + n0 + 1];
        const F3 mie{m0.x * l0 + m1.x * l1, m0.y * l0 + m1.y * l1, m0.z * l0 + m1.z * l1};
        radiance = radiance * RayleighPhase(c, nu) + mie * MiePhase(c, nu);
      }
      row_sum += radiance;
    }
    acc = fma3(row_sum, th.x * dtdp * th.y, acc);
  }
  return acc;
}

// Indirect irradiance: one warp per texel, lanes over the 64 phi samples;
// staged when the launch's shared memory (smem_bytes) holds the instance's
// nodes, else each lookup is a full Scattering4.
__global__ void __launch_bounds__(kIndirectThreads)
k_indirect_irradiance(const Instance* __restrict__ insts, WorkList wl, int order,
                      int smem_bytes) {
  extern __shared__ float4 ind_smem[];
  int local;
  const Instance& in = insts[FindEntry(wl, blockIdx.x, &local)];
  const int lane = threadIdx.x & 31, warp = threadIdx.x / 32;
  const int texel = local * kIndirectTexelsPerTile + warp;
  const bool valid = texel < in.s.i_texels();
  const int need = IndirectStagedSmem(in.s, order);
  float4* V = ind_smem + warp * (need / kIndirectWarps / 16);
  F3 acc = !valid ? f3(0.0f)
           : need <= smem_bytes ? IndirectStagedPartial(in, texel, order, lane, V)
                                : IndirectIrradiancePartial(in, texel, order, lane, 32);
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    acc.x += __shfl_xor_sync(0xffffffffu, acc.x, off);
    acc.y += __shfl_xor_sync(0xffffffffu, acc.y, off);
    acc.z += __shfl_xor_sync(0xffffffffu, acc.z, off);
  }
  if (valid && lane == 0) {
    DeltaIrradiance(in, order)[texel] = to4(acc, 1.0f);
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
                                     int smem_bytes, cudaStream_t st) {
  // smem_bytes: the largest IndirectSmem of the work list's instances (0: none staged).
  k_indirect_irradiance<<<tiles, kIndirectThreads, (size_t)smem_bytes, st>>>(insts, wl, order,
                                                                           smem_bytes);
  return cudaGetLastError();
}

// A check that fails by construction (index 5 of 3), with no memory access:
// the checked build records it, the ordinary build compiles it to nothing.
__global__ void k_check_selftest(int i, int n) {
  if (blockIdx.x == 0 && threadIdx.x == 0) (void)ATMO_CHECKED_INDEX(kCheckSelfTest, i, n);
}
cudaError_t LaunchCheckSelfTest(cudaStream_t st) {
  k_check_selftest<<<1, 32, 0, st>>>(5, 3);
  return cudaGetLastError();
}

ATMO_CHECK_WORD_ACCESSOR(CheckWordKernels)

}  // namespace atmo
