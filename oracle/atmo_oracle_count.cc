/*
 * FLOP-counting build of the CPU oracle -- TEST INFRASTRUCTURE ONLY.
 *
 * Compiles atmo_oracle.cc unchanged with its scalar type `double` replaced by
 * oc::Real, a double that tallies every arithmetic operation it takes part
 * in, by pass and by kind.  Running the oracle's precomputation through this
 * library therefore counts the operations of the reference algorithm as the
 * oracle restates it (atmosphere/functions.glsl:113-1601 in the pass order of
 * atmosphere/model.cc:1048-1215), and gives the same LUTs as the plain build.
 *
 * Kinds: add (and subtract), mul, div, sqrt, exp, pow, sin, cos, floor, fmod
 * and cmp (comparisons, min, max).  A FLOP is an add or a mul; a fused
 * multiply-add of a GPU build counts as its mul and its add.  Buckets: the six
 * texel passes (transmittance, direct irradiance, single scattering,
 * scattering density, indirect irradiance, multiple scattering) with the
 * luminance products and blending that follow each, and one for the host
 * set-up.  Texture filtering (GL LINEAR, done by the texture unit in the
 * reference's shaders) is counted apart from the shader arithmetic.
 *
 * Used only by tests/ (tests/golden/make_flops.py freezes the counts).
 */
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <mutex>
#include <thread>
#include <vector>

namespace oc {

enum Op { kAdd, kMul, kDiv, kSqrt, kExp, kPow, kSin, kCos, kFloor, kFmod, kCmp, kNumOps };
constexpr int kNumBuckets = 7;   // passes 0..5, host set-up
constexpr int kHost = 6;

struct Counts {
  uint64_t n[kNumBuckets][2][kNumOps];   // [bucket][filter][op]
  uint64_t calls[kNumBuckets];           // texel evaluations per pass
};

std::mutex g_mutex;
Counts g_total;

// Per-thread tallies, merged into g_total when the thread ends (or, for the
// calling thread, when the counts are read).
struct Local {
  Counts c;
  int bucket = kHost;
  int filter = 0;
  Local() { std::memset(&c, 0, sizeof(c)); }
  void Merge() {
    std::lock_guard<std::mutex> lock(g_mutex);
    for (int b = 0; b < kNumBuckets; ++b) {
      for (int f = 0; f < 2; ++f)
        for (int o = 0; o < kNumOps; ++o) g_total.n[b][f][o] += c.n[b][f][o];
      g_total.calls[b] += c.calls[b];
    }
    std::memset(&c, 0, sizeof(c));
  }
  ~Local() { Merge(); }
};
thread_local Local tl;

inline void Tally(Op op) { ++tl.c.n[tl.bucket][tl.filter][op]; }

// The counting scalar: same size and layout as a double.
struct Real {
  double v;
  Real() = default;
  constexpr Real(double x) : v(x) {}
  explicit operator double() const { return v; }
  explicit operator int() const { return (int)v; }
  explicit operator long long() const { return (long long)v; }
  explicit operator unsigned() const { return (unsigned)v; }
  Real& operator+=(Real b) { Tally(kAdd); v += b.v; return *this; }
  Real& operator-=(Real b) { Tally(kAdd); v -= b.v; return *this; }
  Real& operator*=(Real b) { Tally(kMul); v *= b.v; return *this; }
  Real& operator/=(Real b) { Tally(kDiv); v /= b.v; return *this; }
};
static_assert(sizeof(Real) == sizeof(double), "Real must alias double arrays");

inline Real operator-(Real a) { return Real(-a.v); }   // a sign flip, not counted
inline Real operator+(Real a) { return a; }
#define OC_BINARY(OP, KIND)                                                     \
  inline Real operator OP(Real a, Real b) { Tally(KIND); return Real(a.v OP b.v); } \
  inline Real operator OP(Real a, double b) { Tally(KIND); return Real(a.v OP b); } \
  inline Real operator OP(double a, Real b) { Tally(KIND); return Real(a OP b.v); }
OC_BINARY(+, kAdd)
OC_BINARY(-, kAdd)
OC_BINARY(*, kMul)
OC_BINARY(/, kDiv)
#undef OC_BINARY
#define OC_COMPARE(OP)                                                          \
  inline bool operator OP(Real a, Real b) { Tally(kCmp); return a.v OP b.v; }   \
  inline bool operator OP(Real a, double b) { Tally(kCmp); return a.v OP b; }   \
  inline bool operator OP(double a, Real b) { Tally(kCmp); return a OP b.v; }
OC_COMPARE(<)
OC_COMPARE(<=)
OC_COMPARE(>)
OC_COMPARE(>=)
OC_COMPARE(==)
OC_COMPARE(!=)
#undef OC_COMPARE

// Scope of a texture lookup: its arithmetic is filtering.
struct FilterScope {
  int saved;
  FilterScope() : saved(tl.filter) { tl.filter = 1; }
  ~FilterScope() { tl.filter = saved; }
};
inline void SetPass(int kind) {
  tl.bucket = (kind >= 0 && kind < kHost) ? kind : kHost;
  if (kind >= 0 && kind < kHost) ++tl.c.calls[kind];
}

}  // namespace oc

// The oracle's math layer over oc::Real (the plain build's is in
// atmo_oracle.cc), in the same anonymous namespace as the oracle's code.
namespace {
namespace om {
inline oc::Real sqrt(oc::Real x) { oc::Tally(oc::kSqrt); return oc::Real(::sqrt(x.v)); }
inline oc::Real exp(oc::Real x) { oc::Tally(oc::kExp); return oc::Real(::exp(x.v)); }
inline oc::Real floor(oc::Real x) { oc::Tally(oc::kFloor); return oc::Real(::floor(x.v)); }
inline oc::Real fmod(oc::Real x, oc::Real y) {
  oc::Tally(oc::kFmod);
  return oc::Real(::fmod(x.v, y.v));
}
inline oc::Real pow(oc::Real x, oc::Real y) { oc::Tally(oc::kPow); return oc::Real(::pow(x.v, y.v)); }
inline oc::Real sin(oc::Real x) { oc::Tally(oc::kSin); return oc::Real(::sin(x.v)); }
inline oc::Real cos(oc::Real x) { oc::Tally(oc::kCos); return oc::Real(::cos(x.v)); }
// min / max with the std:: semantics: integers untallied, reals as a compare.
template <class T>
inline T min(T a, T b) { return b < a ? b : a; }
template <class T>
inline T max(T a, T b) { return a < b ? b : a; }
inline oc::Real min(oc::Real a, oc::Real b) { return b < a ? b : a; }
inline oc::Real max(oc::Real a, oc::Real b) { return a < b ? b : a; }
inline oc::Real min(oc::Real a, double b) { return min(a, oc::Real(b)); }
inline oc::Real max(oc::Real a, double b) { return max(a, oc::Real(b)); }
inline oc::Real min(double a, oc::Real b) { return min(oc::Real(a), b); }
inline oc::Real max(double a, oc::Real b) { return max(oc::Real(a), b); }
}  // namespace om
}  // namespace

#define ORACLE_COUNTING 1
#define ORACLE_COUNT_PASS(kind) oc::SetPass(kind)
#define ORACLE_COUNT_FILTER() oc::FilterScope oc_filter_scope_
#define double oc::Real
#include "atmo_oracle.cc"
#undef double

extern "C" {

// Zeroes the tallies (the calling thread's and the merged ones).
void oracle_count_reset(void) {
  oc::tl.Merge();
  std::lock_guard<std::mutex> lock(oc::g_mutex);
  std::memset(&oc::g_total, 0, sizeof(oc::g_total));
  oc::tl.bucket = oc::kHost;
  oc::tl.filter = 0;
}

// Sizes of the tally array: buckets, filter scopes, kinds.
void oracle_count_dims(int dims[3]) {
  dims[0] = oc::kNumBuckets;
  dims[1] = 2;
  dims[2] = oc::kNumOps;
}

// Copies the tallies: counts[bucket][filter][kind] and the texel evaluations
// per pass, calls[bucket] (the worker threads of a finished precomputation
// have merged theirs already).
void oracle_count_read(unsigned long long* counts, unsigned long long* calls) {
  oc::tl.Merge();
  std::lock_guard<std::mutex> lock(oc::g_mutex);
  int q = 0;
  for (int b = 0; b < oc::kNumBuckets; ++b) {
    for (int f = 0; f < 2; ++f)
      for (int o = 0; o < oc::kNumOps; ++o) counts[q++] = oc::g_total.n[b][f][o];
    calls[b] = oc::g_total.calls[b];
  }
}

}  // extern "C"
