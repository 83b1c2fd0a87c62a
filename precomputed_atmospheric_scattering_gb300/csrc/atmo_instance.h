// atmo_instance.h -- one atmosphere instance as the kernels see it, and the
// work lists that let a single launch cover many instances (batched rebuilds
// of uneven LUT shapes and order counts).
#ifndef ATMO_INSTANCE_H_
#define ATMO_INSTANCE_H_

#include "atmo_device.cuh"

namespace atmo {

// Device buffers of one instance.  All LUTs are float4 RGBA, x fastest, in the
// reference's texture layouts (atmosphere/model.cc:747-766, :872-897).
struct Instance {
  Consts c;
  Shape s;
  Tables tab;
  float4* T;        // transmittance, W_T x H_T
  float4* Tau;      // optical depth -ln(T) of the same texels (internal)
  float4* I;        // irradiance accumulator, W_I x H_I
  float4* dI;       // delta irradiance
  float4* dI2;      // second delta irradiance (odd indirect orders), or nullptr: dI only
  float4* dR;       // delta Rayleigh; also delta multiple scattering (model.cc:897)
  float4* dM;       // delta Mie
  float4* dJ;       // delta scattering density
  float4* S;        // scattering accumulator (RGB + single-Mie red in alpha if combined)
  float4* M;        // single-Mie accumulator, nullptr when combined
  void* S_half;     // half-precision scattering output (half_precision only)
  void* M_half;     // half-precision single-Mie output (half_precision, not combined)
  int combined;     // combine_scattering_textures
  int blend;        // accumulate into I / S / M (wavelength groups after the first)
};

// The delta irradiance of indirect order k (0: the direct pass).  With two
// buffers the indirect pass of order k + 1 writes the other one while the
// density pass of order k + 2 reads this one, so the two can run at once.
ATMO_HD float4* DeltaIrradiance(const Instance& in, int k) {
  return (k & 1) && in.dI2 ? in.dI2 : in.dI;
}

// A launch covers `count` instances; instance inst[q] owns the tiles
// [start[q], start[q+1]).  Both arrays live in device memory.
struct WorkList {
  const int* inst;
  const int* start;
  int count;
};

#ifdef __CUDACC__
// Finds the work-list entry holding `tile` (binary search over start[]).
__device__ __forceinline__ int FindEntry(const WorkList& wl, int tile, int* local) {
  int lo = 0, hi = wl.count - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (__ldg(wl.start + mid) <= tile) lo = mid; else hi = mid - 1;
  }
  *local = tile - __ldg(wl.start + lo);
  return __ldg(wl.inst + lo);
}
#endif

// Threads per block and texels per tile of each kernel (host and device).
constexpr int kTransmittanceLanes = 16;                 // lanes per texel
constexpr int kTransmittanceThreads = 256;
constexpr int kTransmittanceTexelsPerTile = kTransmittanceThreads / kTransmittanceLanes;
constexpr int kTexelThreads = 128;                      // per-texel kernels
constexpr int kIndirectThreads = 128;                   // one warp per texel
constexpr int kIndirectTexelsPerTile = kIndirectThreads / 32;
constexpr int kTableThreads = 128;

}  // namespace atmo

#endif  // ATMO_INSTANCE_H_
