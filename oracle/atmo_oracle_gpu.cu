/*
 * FP64 GPU oracle -- TEST INFRASTRUCTURE ONLY.
 *
 * The CPU oracle's texel evaluators (atmo_oracle.cc, compiled here as host +
 * device code, FP64, no FMA contraction) run one CUDA thread per texel, in
 * the pass order and with the blending of the CPU oracle's Precompute
 * (atmosphere/model.cc:1048-1215).  It exists so that LUT shapes too large
 * for the CPU oracle (the high-resolution configuration: 16.7 M scattering
 * texels, 8 orders) can be checked texel by texel; tests pin it to the CPU
 * oracle first.  Used only by tests/.
 */
#include "atmo_oracle.cc"

#include <cuda_runtime.h>

namespace {

struct Lum {
  double m[9];
};

constexpr int kThreads = 128;
inline unsigned Blocks(long long n) { return (unsigned)((n + kThreads - 1) / kThreads); }

__global__ void KTransmittance(Atm a, Tex2 T, double* out, long long n) {
  const long long i = (long long)blockIdx.x * kThreads + threadIdx.x;
  if (i >= n) return;
  const Tex3 none{1, 1, 1, nullptr};
  EvalTexel(0, a, T, none, none, none, Tex2{}, none, 0, i, out + 4 * i, nullptr);
}

__global__ void KDirect(Atm a, Tex2 T, double* dI, double* I, int blend, long long n) {
  const long long i = (long long)blockIdx.x * kThreads + threadIdx.x;
  if (i >= n) return;
  const Tex3 none{1, 1, 1, nullptr};
  EvalTexel(1, a, T, none, none, none, Tex2{}, none, 0, i, dI + 4 * i, nullptr);
  if (!blend) Store(I + 4 * i, Spec(0.0), 0.0);
}

__global__ void KSingle(Atm a, Tex2 T, double* dR, double* dM, double* S, double* M, Lum lum,
                        int blend, int combined, long long n) {
  const long long i = (long long)blockIdx.x * kThreads + threadIdx.x;
  if (i >= n) return;
  const Tex3 none{1, 1, 1, nullptr};
  EvalTexel(2, a, T, none, none, none, Tex2{}, none, 0, i, dR + 4 * i, dM + 4 * i);
  const Spec lray = MatVec(lum.m, Spec::From(dR + 4 * i));
  const Spec lmie = MatVec(lum.m, Spec::From(dM + 4 * i));
  double* s = S + 4 * i;
  const double alpha = combined ? lmie[0] : 0.0;
  if (blend) {
    Store(s, Spec::From(s) + lray, s[3] + alpha);
  } else {
    Store(s, lray, alpha);
  }
  if (M) {
    double* m = M + 4 * i;
    if (blend) {
      Store(m, Spec::From(m) + lmie, 0.0);
    } else {
      Store(m, lmie, 0.0);
    }
  }
}

__global__ void KDensity(Atm a, Tex2 T, Tex3 DR, Tex3 DM, Tex3 multi, Tex2 DI, int order,
                         double* dJ, long long n) {
  const long long i = (long long)blockIdx.x * kThreads + threadIdx.x;
  if (i >= n) return;
  const Tex3 none{1, 1, 1, nullptr};
  EvalTexel(3, a, T, DR, DM, multi, DI, none, order, i, dJ + 4 * i, nullptr);
}

__global__ void KIndirect(Atm a, Tex2 T, Tex3 DR, Tex3 DM, Tex3 multi, Tex2 DI, int order,
                          double* newI, long long n) {
  const long long i = (long long)blockIdx.x * kThreads + threadIdx.x;
  if (i >= n) return;
  const Tex3 none{1, 1, 1, nullptr};
  EvalTexel(4, a, T, DR, DM, multi, DI, none, order, i, newI + 4 * i, nullptr);
}

__global__ void KAccumulateIrradiance(const double* dI, double* I, Lum lum, long long n) {
  const long long i = (long long)blockIdx.x * kThreads + threadIdx.x;
  if (i >= n) return;
  const Spec add = MatVec(lum.m, Spec::From(dI + 4 * i));
  double* p = I + 4 * i;
  Store(p, Spec::From(p) + add, p[3]);
}

__global__ void KMultiple(Atm a, Tex2 T, Tex2 DI, Tex3 DJ, double* dMulti, double* S, Lum lum,
                          long long n) {
  const long long i = (long long)blockIdx.x * kThreads + threadIdx.x;
  if (i >= n) return;
  const Tex3 none{1, 1, 1, nullptr};
  double nu;
  EvalTexel(5, a, T, none, none, none, DI, DJ, 0, i, dMulti + 4 * i, &nu);
  const Spec add =
      MatVec(lum.m, Spec::From(dMulti + 4 * i)) * (1.0 / RayleighPhaseFunction(nu));
  double* s = S + 4 * i;
  Store(s, Spec::From(s) + add, s[3]);
}

}  // namespace

extern "C" {

// The CPU oracle's oracle_precompute on the GPU (same arguments, host
// arrays; S, M and I are read first when blending).  0 on success, -1 on a
// CUDA error.
int oracle_gpu_precompute(const oracle_atmosphere* atm, const oracle_shape* shp,
                          unsigned num_scattering_orders, const double lum_in[9], int blend,
                          int combined, double* transmittance, double* scattering,
                          double* single_mie, double* irradiance) {
  const Atm a = ToAtm(atm, shp);
  Lum lum;
  for (int k = 0; k < 9; ++k) lum.m[k] = lum_in[k];
  const long long nT = (long long)a.T_W * a.T_H, nI = (long long)a.I_W * a.I_H;
  const long long nS = (long long)a.S_NU * a.S_MU_S * a.S_MU * a.S_R;
  double *T = nullptr, *S = nullptr, *M = nullptr, *I = nullptr, *dI = nullptr,
         *newI = nullptr, *dR = nullptr, *dM = nullptr, *dJ = nullptr, *dMulti = nullptr;
  bool ok = true;
  auto alloc = [&](double** p, long long n) {
    if (ok && cudaMalloc(p, 4 * n * sizeof(double)) != cudaSuccess) ok = false;
  };
  alloc(&T, nT);
  alloc(&S, nS);
  if (single_mie) alloc(&M, nS);
  alloc(&I, nI);
  alloc(&dI, nI);
  alloc(&newI, nI);
  alloc(&dR, nS);
  alloc(&dM, nS);
  alloc(&dJ, nS);
  alloc(&dMulti, nS);
  auto h2d = [&](double* d, const double* h, long long n) {
    if (ok && cudaMemcpy(d, h, 4 * n * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess)
      ok = false;
  };
  if (blend) {
    h2d(S, scattering, nS);
    if (M) h2d(M, single_mie, nS);
    h2d(I, irradiance, nI);
  }
  if (ok) {
    const Tex2 Tt = MakeT(a, T);
    Tex2 DI = MakeI(a, dI);
    const Tex3 DR = MakeS(a, dR), DM = MakeS(a, dM), DJ = MakeS(a, dJ), DMulti = MakeS(a, dMulti);
    KTransmittance<<<Blocks(nT), kThreads>>>(a, Tt, T, nT);
    KDirect<<<Blocks(nI), kThreads>>>(a, Tt, dI, I, blend, nI);
    KSingle<<<Blocks(nS), kThreads>>>(a, Tt, dR, dM, S, M, lum, blend, combined, nS);
    for (unsigned order = 2; order <= num_scattering_orders; ++order) {
      // delta multiple scattering aliases delta Rayleigh in the reference
      // (model.cc:897); order 2 reads the single-scattering tables.
      const Tex3 multi_in = order == 2 ? DR : DMulti;
      KDensity<<<Blocks(nS), kThreads>>>(a, Tt, DR, DM, multi_in, DI, (int)order, dJ, nS);
      KIndirect<<<Blocks(nI), kThreads>>>(a, Tt, DR, DM, multi_in, DI, (int)order - 1, newI,
                                          nI);
      std::swap(dI, newI);
      DI = MakeI(a, dI);
      KAccumulateIrradiance<<<Blocks(nI), kThreads>>>(dI, I, lum, nI);
      KMultiple<<<Blocks(nS), kThreads>>>(a, Tt, DI, DJ, dMulti, S, lum, nS);
    }
    if (cudaGetLastError() != cudaSuccess || cudaDeviceSynchronize() != cudaSuccess) ok = false;
  }
  auto d2h = [&](double* h, const double* d, long long n) {
    if (ok && cudaMemcpy(h, d, 4 * n * sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess)
      ok = false;
  };
  d2h(transmittance, T, nT);
  d2h(scattering, S, nS);
  if (single_mie) d2h(single_mie, M, nS);
  d2h(irradiance, I, nI);
  for (double* p : {T, S, M, I, dI, newI, dR, dM, dJ, dMulti})
    if (p) cudaFree(p);
  return ok ? 0 : -1;
}

}  // extern "C"
