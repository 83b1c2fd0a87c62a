// atmo_fast.cu -- fast-path kernels: the slab-restructured scattering density
// (the dominant pass, functions.glsl:1163-1260) and the FP16 output conversion.
//
// Scattering density, restructured.  For a texel at r-slice k and mu_s column
// c, every incoming-radiance lookup of ComputeScatteringDensity is made at the
// texel's own r and mu_s, whose texture coordinates land on the centres of
// slice k and column c (the texel mapping and the lookup mapping are inverse
// to each other), while mu = cos(theta_l) takes one of 16 values shared by
// all texels of the slice and only nu varies with the direction.  A block
// therefore owns the slab (k, c) -- the NU x MU texels with that r and mu_s --
// and stages in shared memory, per theta row l and nu node n, the previous
// order's radiance bilinearly interpolated in mu: L[l][n].  The quadrilinear
// lookup of a direction reduces to a lerp between L[l][n0] and L[l][n0 + 1].
// The ground term reads the bottom row of the irradiance LUT (the ground
// point is at r = Rb, on row 0's centre), also staged in shared memory.
#include <cuda_fp16.h>

#include "atmo_kernels.h"
#include "atmo_passes.cuh"

namespace atmo {

constexpr int kDensityFastThreads = 256;

int DensityFastTiles(const Shape& s) { return s.sr * s.smus; }

// Shared memory of one block, bytes: per staged species a [16][NU] float4
// table (L.x, L.y, L.z, D.x) and a [16][NU] float2 table (D.y, D.z), where
// D = L[n + 1] - L[n] is the slope towards the next nu node; then the bottom
// row of the irradiance LUT; then a float temporary per table entry.
int DensityFastSmem(const Shape& s, int order) {
  const int species = order == 2 ? 2 : 1;
  return species * kDensityThetaSamples * s.snu *
             (int)(sizeof(float4) + sizeof(float2) + sizeof(float)) +
         s.iw * (int)sizeof(float4);
}

// The staged radiance at nu1 of theta row l: L[n0] + w D[n0].
__device__ __forceinline__ F3 NuLerp(const float4* __restrict__ P, const float2* __restrict__ Q,
                                     float nu1, float half_nu, float top, int nmax) {
  const float u = clampf(fmaf(nu1, half_nu, half_nu), 0.0f, top);
  const int n0 = min((int)u, nmax);
  const float w = u - float(n0);
  const float4 p = P[n0];
  const float2 q = Q[n0];
  return F3{fmaf(w, p.w, p.x), fmaf(w, q.x, p.y), fmaf(w, q.y, p.z)};
}

template <bool kOrder2>
__global__ void __launch_bounds__(kDensityFastThreads)
k_density_fast(const Instance* __restrict__ insts, WorkList wl) {
  extern __shared__ float4 smem[];
  int local;
  const Instance& in = insts[FindEntry(wl, blockIdx.x, &local)];
  const Shape s = in.s;
  const int NU = s.snu, W = s.sw();
  const int k = local / s.smus, col = local % s.smus;
  const int rows_nu = kDensityThetaSamples * NU;
  float4* PR = smem;                                          // Rayleigh / multiple
  float2* QR = reinterpret_cast<float2*>(PR + rows_nu);
  float4* PM = reinterpret_cast<float4*>(QR + rows_nu);        // Mie (order 2)
  float2* QM = reinterpret_cast<float2*>(PM + rows_nu);
  float4* IR = kOrder2 ? reinterpret_cast<float4*>(QM + rows_nu) : PM;   // [iw]
  const DensityRow* drows = in.tab.drows + k * kDensityThetaSamples;

  // Stage the previous order, bilinear in mu, at column (n * MU_S + col) of
  // slice k: first the values, then (after a barrier) the slopes.
  for (int e = threadIdx.x; e < rows_nu; e += blockDim.x) {
    const int l = e / NU, n = e % NU;
    const float Y = drows[l].u_mu * float(s.smu) - 0.5f;
    const float fy = floorf(Y);
    const float wy = Y - fy;
    const int y0 = ClampIdx((int)fy, s.smu), y1 = ClampIdx((int)fy + 1, s.smu);
    const int base = k * s.smu * W + n * s.smus + col;
    const float4 a = __ldg(in.dR + base + y0 * W);
    const float4 b = __ldg(in.dR + base + y1 * W);
    PR[e] = make_float4(fmaf(wy, b.x - a.x, a.x), fmaf(wy, b.y - a.y, a.y),
                        fmaf(wy, b.z - a.z, a.z), 0.0f);
    if (kOrder2) {
      const float4 p = __ldg(in.dM + base + y0 * W);
      const float4 q = __ldg(in.dM + base + y1 * W);
      PM[e] = make_float4(fmaf(wy, q.x - p.x, p.x), fmaf(wy, q.y - p.y, p.y),
                          fmaf(wy, q.z - p.z, p.z), 0.0f);
    }
  }
  for (int e = threadIdx.x; e < s.iw; e += blockDim.x) IR[e] = __ldg(in.dI + e);
  __syncthreads();
  // Slopes towards the next node (0 at the last node): y, z into Q, x into a
  // temporary, then x into P.w once every value has been read.
  float* TX = reinterpret_cast<float*>(IR + s.iw);                 // [species][rows_nu]
  for (int e = threadIdx.x; e < rows_nu; e += blockDim.x) {
    const bool last = (e % NU) == NU - 1;
    const float4 v = PR[e], nx = last ? v : PR[e + 1];
    QR[e] = make_float2(nx.y - v.y, nx.z - v.z);
    TX[e] = nx.x - v.x;
    if (kOrder2) {
      const float4 vm = PM[e], nm = last ? vm : PM[e + 1];
      QM[e] = make_float2(nm.y - vm.y, nm.z - vm.z);
      TX[rows_nu + e] = nm.x - vm.x;
    }
  }
  __syncthreads();
  for (int e = threadIdx.x; e < rows_nu; e += blockDim.x) {
    PR[e].w = TX[e];
    if (kOrder2) PM[e].w = TX[rows_nu + e];
  }
  __syncthreads();

  const Consts& c = in.c;
  const float m2g = c.m2g, g2p1 = c.g2p1, ray_k = c.ray_k, mie_k = c.mie_k;
  const TexelCol cc = in.tab.cols[col];
  const float half_nu = 0.5f * float(NU - 1);
  const float top = float(NU - 1);
  const int nmax = NU - 2;
  const float iw1 = float(s.iw - 1);
  const int imax = s.iw - 2;
  const float inv_rb = 1.0f / c.Rb;
  const float dtdp = (kPiF / 16.0f) * (kPiF / 16.0f);
  const int texels = NU * s.smu;
  for (int t = threadIdx.x; t < texels; t += blockDim.x) {
    const int j = t % s.smu, n = t / s.smu;
    const TexelRow row = in.tab.rows[k * s.smu + j];
    const TexelAngles ang = MakeAngles(s, row, cc, n);
    const float rmu_s = row.r * ang.mu_s;
    F3 sum_r = f3(0.0f), sum_m = f3(0.0f);   // sums of L (1 + nu2^2) and L P_M(nu2) / mie_k
    for (int l = 0; l < kDensityThetaSamples; ++l) {
      const DensityRow dr = drows[l];
      const float A = ang.mu_s * dr.cos_t, B = ang.mu * dr.cos_t;
      const float sxs = ang.sx * dr.sin_t, sys = ang.sy * dr.sin_t;
      const float oxs = ang.omega_x * dr.sin_t;
      const float4* Pr = PR + l * NU;
      const float2* Qr = QR + l * NU;
      const float4* Pm = PM + l * NU;
      const float2* Qm = QM + l * NU;
      const F3 tg = f3(dr.t_ground);
      const bool ground = dr.ground != 0;
      F3 row_r = f3(0.0f), row_m = f3(0.0f);
      // phi and 2 pi - phi share cos(phi), hence nu2 and the phase functions
      // of the outgoing direction; nu1 differs by the sign of sy sin(phi).
#pragma unroll 2
      for (int m = 0; m < kDensityPhiSamples / 2; ++m) {
        const float2 cs = c_density_phi[m];
        const float base = fmaf(sxs, cs.x, A);
        const float dl = sys * cs.y;
        const float nu2 = fmaf(oxs, cs.x, B);
        F3 Ls = f3(0.0f);
#pragma unroll
        for (int side = 0; side < 2; ++side) {
          const float nu1 = side == 0 ? base + dl : base - dl;
          F3 L = NuLerp(Pr, Qr, nu1, half_nu, top, nmax);
          if (kOrder2) {
            // Single scattering with its phase functions at nu1 (:998-1004).
            const F3 M = NuLerp(Pm, Qm, nu1, half_nu, top, nmax);
            const float q1 = fmaf(nu1, nu1, 1.0f);
            const float r1 = rsqrtf(fmaf(m2g, nu1, g2p1));
            L = L * (ray_k * q1) + M * (mie_k * q1 * (r1 * r1 * r1));
          }
          if (ground) {
            // Ground bounce: the ground point is at radius Rb, so the cosine
            // of its normal with the sun is (r mu_s + dist nu1) / Rb; the
            // irradiance lookup at r = Rb reads row 0 of the LUT.
            const float mu_g = fmaf(dr.dist_ground, nu1, rmu_s) * inv_rb;
            const float X = clampf(fmaf(mu_g, 0.5f, 0.5f), 0.0f, 1.0f) * iw1;
            const int i0 = min((int)X, imax);
            const float wi = X - float(i0);
            const float4 e0 = IR[i0], e1 = IR[i0 + 1];
            L = fma3(tg, F3{fmaf(wi, e1.x - e0.x, e0.x), fmaf(wi, e1.y - e0.y, e0.y),
                            fmaf(wi, e1.z - e0.z, e0.z)}, L);
          }
          Ls += L;
        }
        // Phase functions at nu2 (functions.glsl:739-747, :1245-1254).
        const float q = fmaf(nu2, nu2, 1.0f);
        const float rs = rsqrtf(fmaf(m2g, nu2, g2p1));
        row_r = fma3(Ls, q, row_r);
        row_m = fma3(Ls, q * (rs * rs * rs), row_m);
      }
      const float dw = dtdp * dr.sin_t;
      sum_r = fma3(row_r, dw, sum_r);
      sum_m = fma3(row_m, dw, sum_m);
    }
    const F3 a_r = c.rayleigh * (ProfileDensity(c.prof_r, row.h) * ray_k);
    const F3 a_m = c.mie_sca * (ProfileDensity(c.prof_m, row.h) * mie_k);
    const F3 J = a_r * sum_r + a_m * sum_m;
    const int texel = (k * s.smu + j) * W + n * s.smus + col;
    in.dJ[texel] = to4(J, 1.0f);
  }
}

cudaError_t LaunchDensityFast(const Instance* insts, WorkList wl, int tiles, int order,
                              int smem_bytes, cudaStream_t st) {
  // smem_bytes: the largest DensityFastSmem of the work list's instances.
  const size_t bytes = (size_t)smem_bytes;
  if (order == 2) {
    k_density_fast<true><<<tiles, kDensityFastThreads, bytes, st>>>(insts, wl);
  } else {
    k_density_fast<false><<<tiles, kDensityFastThreads, bytes, st>>>(insts, wl);
  }
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Multiple scattering, restructured (functions.glsl:1268-1308).
//
// Every quantity of a quadrature sample but mu_s depends only on the texel's
// row (r-slice k, mu-row j): the sample's r and mu, hence the (y, z) position
// of its 4D lookup, and the transmittance from the texel to the sample.  A
// block owns whole rows; it computes their samples once (RaySample), then,
// per sample, interpolates the density LUT in (mu, r) at the sample into a
// line of W = NU x MU_S columns in shared memory.  A texel's lookup reduces to
// its own mu_s mapping and a bilinear (mu_s, nu) interpolation of 4 columns
// of that line.  Lines are built G samples at a time, double-buffered, so a
// stage needs one barrier.
// ---------------------------------------------------------------------------
constexpr int kMultipleFastThreads = 256;
constexpr int kMultipleFastMaxCols = 4;   // texel columns per thread (W <= 1024)
constexpr int kRaySamples = kMultipleScatteringSamples + 1;

struct __align__(16) RaySample {
  int r00, r01, r10, r11;    // element offsets of the LUT rows (k0 j0, k0 j1, k1 j0, k1 j1)
  float w00, w01, w10, w11;  // their bilinear weights in (mu, r)
  float tx, ty, tz;          // transmittance texel -> sample x dx x trapezoid weight
  float d;                   // distance from the texel's point along its ray
  float inv_r;               // 1 / r at the sample
  float pad[3];
};

struct MultipleFastDims {
  int rows;    // LUT rows per block
  int group;   // samples per line stage
};
__host__ __device__ inline MultipleFastDims MultipleDims(const Shape& s) {
  const int W = s.sw();
  int rows = kMultipleFastThreads / W;
  rows = rows < 1 ? 1 : (rows > 4 ? 4 : rows);
  // Two line buffers of group x rows x W float4 within 32 KB.
  int group = 32768 / (2 * 16 * rows * W);
  group = group < 1 ? 1 : (group > 4 ? 4 : group);
  return MultipleFastDims{rows, group};
}
bool MultipleFastFits(const Shape& s) {
  return s.sw() <= kMultipleFastThreads * kMultipleFastMaxCols;
}
int MultipleFastTiles(const Shape& s) {
  const int rows = MultipleDims(s).rows;
  return (s.sr * s.smu + rows - 1) / rows;
}
int MultipleFastSmem(const Shape& s) {
  const MultipleFastDims d = MultipleDims(s);
  return d.rows * kRaySamples * (int)sizeof(RaySample) + 2 * d.group * d.rows * s.sw() * 16;
}

// Sample i of the ray of LUT row `rowi` (the per-sample part of
// MultipleScatteringTexel that does not depend on mu_s or nu).
__device__ RaySample MakeRaySample(const Instance& in, int rowi, int i) {
  const Consts& c = in.c;
  const Shape& s = in.s;
  const TexelRow row = in.tab.rows[rowi];
  const bool ground = row.ground != 0;
  const float dx = row.d / float(kMultipleScatteringSamples);
  const float d = float(i) * dx;
  const float e = float(kMultipleScatteringSamples - i) * dx;
  const RadialPoint p = PointFromRho2(c, RayRho2(row, d, e));
  const float u_mu = UMuFromDistance(c, s, p, e, ground);
  const float u_r = TexCoord(s, kMapSR, p.rho / c.H);
  const TStart start = MakeTStart(c, s, in.T, in.Tau, row.rho, row.r,
                                  ground ? -row.rmu : row.rmu, row.delta);
  const F3 t = SegmentTransmittance(c, s, in.T, in.Tau, row.rmu, row.delta, p, d, ground, start);
  const float w = (i == 0 || i == kMultipleScatteringSamples) ? 0.5f : 1.0f;
  const float Y = u_mu * float(s.smu) - 0.5f, Z = u_r * float(s.sr) - 0.5f;
  const float fy = floorf(Y), fz = floorf(Z);
  const float b = Y - fy, cz = Z - fz;
  const int j0 = ClampIdx((int)fy, s.smu), j1 = ClampIdx((int)fy + 1, s.smu);
  const int k0 = ClampIdx((int)fz, s.sr), k1 = ClampIdx((int)fz + 1, s.sr);
  const int W = s.sw();
  RaySample rs;
  rs.r00 = (k0 * s.smu + j0) * W;
  rs.r01 = (k0 * s.smu + j1) * W;
  rs.r10 = (k1 * s.smu + j0) * W;
  rs.r11 = (k1 * s.smu + j1) * W;
  rs.w00 = (1.0f - b) * (1.0f - cz);
  rs.w01 = b * (1.0f - cz);
  rs.w10 = (1.0f - b) * cz;
  rs.w11 = b * cz;
  const float dw = dx * w;
  rs.tx = t.x * dw;
  rs.ty = t.y * dw;
  rs.tz = t.z * dw;
  rs.d = d;
  rs.inv_r = 1.0f / p.r;
  rs.pad[0] = rs.pad[1] = rs.pad[2] = 0.0f;
  return rs;
}

template <int kCols>
__device__ __forceinline__ void MultipleFastBlock(const Instance& in, int local, float4* smem) {
  const Shape s = in.s;
  const Consts& c = in.c;
  const MultipleFastDims dims = MultipleDims(s);
  const int W = s.sw(), R = dims.rows, G = dims.group;
  const int rows_total = s.sr * s.smu;
  const int row0 = local * R;
  RaySample* samp = reinterpret_cast<RaySample*>(smem);                 // [R][kRaySamples]
  float4* line = smem + R * kRaySamples * (int)(sizeof(RaySample) / 16);   // [2][G][R][W]

  for (int e = threadIdx.x; e < R * kRaySamples; e += kMultipleFastThreads) {
    const int rr = e / kRaySamples, i = e - rr * kRaySamples;
    if (row0 + rr < rows_total) samp[e] = MakeRaySample(in, row0 + rr, i);
  }

  // This thread's row within the tile and its texel columns x_t + 256 m.
  const int rr = kCols == 1 ? (int)threadIdx.x / W : 0;
  const int x_t = kCols == 1 ? (int)threadIdx.x - rr * W : (int)threadIdx.x;
  const int rowi = row0 + rr;
  const bool active = rr < R && rowi < rows_total;
  const float smus_f = float(s.smus);
  const int nmax = W - 1;
  float rmu_s[kCols], nu[kCols], xb[kCols], lnu[kCols];
  F3 acc[kCols];
  if (active) {
    const TexelRow row = in.tab.rows[rowi];
#pragma unroll
    for (int m = 0; m < kCols; ++m) {
      const int x = min(x_t + m * kMultipleFastThreads, nmax);
      const int n = x / s.smus, col = x - n * s.smus;
      const TexelAngles ang = MakeAngles(s, row, in.tab.cols[col], n);
      rmu_s[m] = row.r * ang.mu_s;
      nu[m] = ang.nu;
      const float tex_coord_x = (ang.nu + 1.0f) * 0.5f * float(s.snu - 1);
      const float tex_x = floorf(tex_coord_x);
      lnu[m] = tex_coord_x - tex_x;
      xb[m] = tex_x * smus_f - 0.5f;
      acc[m] = f3(0.0f);
    }
  }
  __syncthreads();

  const int line_stride = G * R * W;
  const int stages = (kRaySamples + G - 1) / G;
  for (int stage = 0; stage < stages; ++stage) {
    float4* buf = line + (stage & 1) * line_stride;
    const int first = stage * G;
    const int count = min(G, kRaySamples - first);
    if (active) {
      for (int g = 0; g < count; ++g) {
        const RaySample& sm = samp[rr * kRaySamples + first + g];
        float4* out = buf + (g * R + rr) * W;
#pragma unroll
        for (int m = 0; m < kCols; ++m) {
          const int x = x_t + m * kMultipleFastThreads;
          if (kCols > 1 && x >= W) break;
          const float4 a = __ldg(in.dJ + sm.r00 + x), b = __ldg(in.dJ + sm.r01 + x);
          const float4 p = __ldg(in.dJ + sm.r10 + x), q = __ldg(in.dJ + sm.r11 + x);
          out[x] = make_float4(
              fmaf(q.x, sm.w11, fmaf(p.x, sm.w10, fmaf(b.x, sm.w01, a.x * sm.w00))),
              fmaf(q.y, sm.w11, fmaf(p.y, sm.w10, fmaf(b.y, sm.w01, a.y * sm.w00))),
              fmaf(q.z, sm.w11, fmaf(p.z, sm.w10, fmaf(b.z, sm.w01, a.z * sm.w00))), 0.0f);
        }
      }
    }
    __syncthreads();
    if (active) {
      for (int g = 0; g < count; ++g) {
        const RaySample& sm = samp[rr * kRaySamples + first + g];
        const float4* L = buf + (g * R + rr) * W;
#pragma unroll
        for (int m = 0; m < kCols; ++m) {
          if (kCols > 1 && x_t + m * kMultipleFastThreads >= W) break;
          const float mu_s_i = clampf(fmaf(sm.d, nu[m], rmu_s[m]) * sm.inv_r, -1.0f, 1.0f);
          const float x0 = fmaf(UMuSFromMuS(c, s, mu_s_i), smus_f, xb[m]);
          const float fx = floorf(x0);
          const float a = x0 - fx;
          const int i0 = (int)fx;
          const int c0 = min(max(i0, 0), nmax), c1 = min(max(i0 + 1, 0), nmax);
          const int c2 = min(max(i0 + s.smus, 0), nmax), c3 = min(max(i0 + s.smus + 1, 0), nmax);
          const float l1 = lnu[m], l0 = 1.0f - l1;
          const float v0 = (1.0f - a) * l0, v1 = a * l0, v2 = (1.0f - a) * l1, v3 = a * l1;
          const float4 t0 = L[c0], t1 = L[c1], t2 = L[c2], t3 = L[c3];
          const F3 S{fmaf(t3.x, v3, fmaf(t2.x, v2, fmaf(t1.x, v1, t0.x * v0))),
                     fmaf(t3.y, v3, fmaf(t2.y, v2, fmaf(t1.y, v1, t0.y * v0))),
                     fmaf(t3.z, v3, fmaf(t2.z, v2, fmaf(t1.z, v1, t0.z * v0)))};
          acc[m] = fma3(S, F3{sm.tx, sm.ty, sm.tz}, acc[m]);
        }
      }
    }
  }

  if (!active) return;
#pragma unroll
  for (int m = 0; m < kCols; ++m) {
    const int x = x_t + m * kMultipleFastThreads;
    if (kCols > 1 && x >= W) break;
    const int texel = rowi * W + x;
    in.dR[texel] = to4(acc[m], 1.0f);   // delta multiple aliases delta Rayleigh
    const F3 add = MatVec(c.lum, acc[m]) * (1.0f / RayleighPhase(c, nu[m]));
    const float4 o = in.S[texel];
    in.S[texel] = make_float4(o.x + add.x, o.y + add.y, o.z + add.z, o.w);
  }
}

__global__ void __launch_bounds__(kMultipleFastThreads)
k_multiple_fast(const Instance* __restrict__ insts, WorkList wl) {
  extern __shared__ float4 smem[];
  int local;
  const Instance& in = insts[FindEntry(wl, blockIdx.x, &local)];
  if (in.s.sw() <= kMultipleFastThreads) {
    MultipleFastBlock<1>(in, local, smem);
  } else {
    MultipleFastBlock<kMultipleFastMaxCols>(in, local, smem);
  }
}

cudaError_t LaunchMultipleFast(const Instance* insts, WorkList wl, int tiles, int smem_bytes,
                               cudaStream_t st) {
  // smem_bytes: the largest MultipleFastSmem of the work list's instances.
  k_multiple_fast<<<tiles, kMultipleFastThreads, (size_t)smem_bytes, st>>>(insts, wl);
  return cudaGetLastError();
}

__global__ void k_to_half(const float4* __restrict__ src, __half2* __restrict__ dst, long long n) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float4 v = src[i];
  dst[2 * i] = __floats2half2_rn(v.x, v.y);
  dst[2 * i + 1] = __floats2half2_rn(v.z, v.w);
}

cudaError_t LaunchToHalf(const float4* src, void* dst, long long n, cudaStream_t st) {
  int blocks = (int)((n + 255) / 256);
  k_to_half<<<blocks, 256, 0, st>>>(src, reinterpret_cast<__half2*>(dst), n);
  return cudaGetLastError();
}

// FP32 FMA throughput probe: 8 independent FMA chains per thread.
__global__ void k_fma_probe(float* out, int iters, float a, float b) {
  float x[8];
#pragma unroll
  for (int i = 0; i < 8; ++i) x[i] = threadIdx.x * 1e-3f + i;
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int i = 0; i < 8; ++i) x[i] = fmaf(x[i], a, b);
  }
  float s = 0.0f;
#pragma unroll
  for (int i = 0; i < 8; ++i) s += x[i];
  if (s == 1234.5f) out[blockIdx.x] = s;   // keeps the chains live
}

cudaError_t MeasureFp32Peak(double* tflops) {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  float* out = nullptr;
  cudaError_t e = cudaMalloc(&out, sizeof(float) * sms * 8);
  if (e != cudaSuccess) return e;
  const int blocks = sms * 8, threads = 256, iters = 4096;
  cudaEvent_t t0, t1;
  cudaEventCreate(&t0);
  cudaEventCreate(&t1);
  k_fma_probe<<<blocks, threads>>>(out, iters, 0.999f, 1e-3f);   // warm-up
  cudaEventRecord(t0);
  const int reps = 5;
  for (int r = 0; r < reps; ++r) k_fma_probe<<<blocks, threads>>>(out, iters, 0.999f, 1e-3f);
  cudaEventRecord(t1);
  e = cudaEventSynchronize(t1);
  float ms = 0.0f;
  cudaEventElapsedTime(&ms, t0, t1);
  cudaEventDestroy(t0);
  cudaEventDestroy(t1);
  cudaFree(out);
  double flops = 2.0 * 8.0 * iters * (double)blocks * threads * reps;
  *tflops = flops / (ms * 1e-3) / 1e12;
  return e == cudaSuccess ? cudaGetLastError() : e;
}

}  // namespace atmo
