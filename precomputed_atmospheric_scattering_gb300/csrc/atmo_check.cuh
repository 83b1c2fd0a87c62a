// atmo_check.cuh -- device-side access checks of the checked build.
//
// compute-sanitizer does not run here, so the library has a checked build
// instead: compiled with -DATMO_DEVICE_CHECKS (libatmo_gb300_checked.so, made
// by nvcc_build.build(checked=True)), the accesses whose index comes from
// arithmetic rather than a loop bound test it against the buffer they read:
// the shared-memory table lookups of the density kernels (against the block's
// dynamic shared memory), the delta-density and transmittance rows of the
// line builds and the line taps of single and multiple scattering, the
// previous-order texels staged by the density kernels, and the texels of the
// bilinear, transmittance and 4D scattering lookups shared by all kernels.  A failing
// test records (site, index) in its translation unit's check word -- the
// first failure wins -- and the access reads element 0 instead, so that a
// checked run never reads outside a buffer.  atmo_device_checks() returns the
// words.  In the ordinary build the tests compile to nothing.
#ifndef ATMO_CHECK_CUH_
#define ATMO_CHECK_CUH_

namespace atmo {

// Where a check failed (the top 8 bits of a check word).
enum CheckSite : unsigned {
  kCheckSharedLookup = 1,   // density table lookup outside the dynamic shared memory
  kCheckLutTexel = 2,       // texel of a LUT lookup (transmittance, optical depth,
                            // irradiance, scattering and the delta LUTs)
  kCheckDensityStage = 3,   // previous-order texel staged by the density kernel
  kCheckLineLoad = 4,       // delta-density or transmittance row of a line build
  kCheckLineTap = 5,        // line entry tapped by a texel
  kCheckOutput = 6,         // output texel of a multiple-scattering row
  kCheckSelfTest = 255,     // atmo_device_checks_selftest
};

#ifdef ATMO_DEVICE_CHECKS
constexpr bool kDeviceChecks = true;
#else
constexpr bool kDeviceChecks = false;
#endif

// The check words of the translation units with device code (host side:
// reads the word and, with reset, clears it; 0 in the ordinary build).
unsigned long long CheckWordKernels(bool reset);
unsigned long long CheckWordRays(bool reset);
unsigned long long CheckWordFast(bool reset);
unsigned long long CheckWordRender(bool reset);

}  // namespace atmo

#if defined(__CUDACC__) && defined(ATMO_DEVICE_CHECKS)
namespace atmo {
// This translation unit's word: site << 56 | the failing index (56 bits).
static __device__ unsigned long long g_check_word;
}  // namespace atmo
// The word's host accessor, defined once in each translation unit.
#define ATMO_CHECK_WORD_ACCESSOR(name)                                                 \
  unsigned long long name(bool reset) {                                               \
    unsigned long long w = 0;                                                         \
    if (cudaMemcpyFromSymbol(&w, g_check_word, sizeof w) != cudaSuccess) return ~0ull; \
    if (reset) {                                                                      \
      const unsigned long long z = 0;                                                 \
      cudaMemcpyToSymbol(g_check_word, &z, sizeof z);                                 \
    }                                                                                 \
    return w;                                                                         \
  }
#else
#define ATMO_CHECK_WORD_ACCESSOR(name) \
  unsigned long long name(bool) { return 0; }
#endif

#if defined(__CUDA_ARCH__) && defined(ATMO_DEVICE_CHECKS)
namespace atmo {
__device__ __forceinline__ long long CheckedIndex(unsigned site, long long i, long long n) {
  if (i >= 0 && i < n) return i;
  atomicCAS(&g_check_word, 0ull,
            ((unsigned long long)site << 56) | ((unsigned long long)i & 0x00FFFFFFFFFFFFFFull));
  return 0;
}
}  // namespace atmo
// i when 0 <= i < n; otherwise 0, after recording (site, i).
#define ATMO_CHECKED_INDEX(site, i, n) \
  ::atmo::CheckedIndex((site), (long long)(i), (long long)(n))
// &base[row + col], checked against n elements.
#define ATMO_CHECKED_PTR(site, base, row, col, n) \
  ((base) + ::atmo::CheckedIndex((site), (long long)(row) + (col), (long long)(n)))
#else
#define ATMO_CHECKED_INDEX(site, i, n) (i)
#define ATMO_CHECKED_PTR(site, base, row, col, n) ((base) + (row) + (col))
#endif

#endif  // ATMO_CHECK_CUH_
