// atmo_kernels.h -- launchers of the precomputation kernels (host side).
#ifndef ATMO_KERNELS_H_
#define ATMO_KERNELS_H_

#include <cuda_runtime.h>

#include "atmo_instance.h"

namespace atmo {

int TableTiles(const Shape& s);
cudaError_t LaunchTables(const Instance* insts, WorkList wl, int tiles, cudaStream_t st);
cudaError_t LaunchTransmittance(const Instance* insts, WorkList wl, int tiles, cudaStream_t st);
cudaError_t LaunchDirectIrradiance(const Instance* insts, WorkList wl, int tiles,
                                   cudaStream_t st);
cudaError_t LaunchSingleScattering(const Instance* insts, WorkList wl, int tiles,
                                   cudaStream_t st);
cudaError_t LaunchDensityPlain(const Instance* insts, WorkList wl, int tiles, int order,
                               cudaStream_t st);
// smem_bytes: IndirectSmem of the launch (0 on the plain path).
int IndirectSmem(const Shape& s, int order);
cudaError_t LaunchIndirectIrradiance(const Instance* insts, WorkList wl, int tiles, int order,
                                     int smem_bytes, cudaStream_t st);
cudaError_t LaunchMultiplePlain(const Instance* insts, WorkList wl, int tiles,
                                cudaStream_t st);
// Fast path (atmo_fast.cu).
int DensityFastTiles(const Shape& s);
int DensityFastSmem(const Shape& s, const Consts& c, int order);
cudaError_t PrepareDensityFast();
bool DensityFastFits(const Shape& s);
cudaError_t LaunchDensityFast(const Instance* insts, WorkList wl, int tiles, int order,
                              int smem_bytes, cudaStream_t st);
// The row-restructured single-scattering kernel needs W = NU x MU_S <= 1024
// and its transmittance lines within 48 KB of shared memory.
bool SingleFastFits(const Shape& s);
int SingleFastTiles(const Shape& s);
int SingleFastSmem(const Shape& s);
cudaError_t LaunchSingleFast(const Instance* insts, WorkList wl, int tiles, int smem_bytes,
                             cudaStream_t st);
// A (rows per block, samples per line stage) tuning of the single (single =
// true) or multiple scattering kernel that can run for shape s.
bool FastTuningValid(const Shape& s, bool single, int rows, int group);
// The row-restructured multiple-scattering kernel needs W = NU x MU_S <= 1024.
bool MultipleFastFits(const Shape& s);
int MultipleFastTiles(const Shape& s);
int MultipleFastSmem(const Shape& s);
cudaError_t LaunchMultipleFast(const Instance* insts, WorkList wl, int tiles, int smem_bytes,
                               cudaStream_t st);
// Final conversion of the scattering accumulators to half precision.
cudaError_t LaunchToHalf(const float4* src, void* dst, long long n, cudaStream_t st);
cudaError_t MeasureFp32Peak(double* tflops);
// One check that fails by construction, recorded by the checked build only.
cudaError_t LaunchCheckSelfTest(cudaStream_t st);

}  // namespace atmo

#endif  // ATMO_KERNELS_H_
