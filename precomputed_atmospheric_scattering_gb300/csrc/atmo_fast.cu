// atmo_fast.cu -- fast-path kernels: the slab-restructured scattering density
// (the dominant pass, functions.glsl:1163-1260), the row-restructured single
// and multiple scattering (:650-730, :1285-1330; described where they start
// below), the FP16 output conversion and the FP32 FMA throughput probe.
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

#include <algorithm>
#include <atomic>
#include <cmath>
#include <type_traits>

#include "atmo_kernels.h"
#include "atmo_passes.cuh"

namespace atmo {

constexpr int kDensityFastThreads = 256;

int DensityFastTiles(const Shape& s) { return s.sr * s.smus; }

// Piecewise-linear functions staged in shared memory.  A row of N node
// values L[0..N-1] (node coordinate v in [0, N - 1]) is stored as N + 1
// entries, each the line a + b s of one interval in the unit coordinate
// s = (v + 0.5) / N: entry 0 is L[0] (v < 0), entry N is L[N - 1] (v >
// N - 1), entry e in between the segment [e - 1, e] (b = the slope times N).
// A lookup takes s from a saturating FMA, which clamps it to [0, 1] and maps
// a NaN to 0, then the entry from a second FMA: s N + 1.5 x 2^23, rounded to
// nearest, leaves round(v + 0.5), in [0, N], in the sum's low mantissa bits
// (a v on a node may take either neighbouring entry; both give the node's
// value).  The sum's bit pattern, times the entry size, plus a row offset
// that cancels the constant's exponent bits (mod 2^32), is the entry's
// shared-memory address: no index can leave the row, and the value is one
// FMA per channel.  The intercept's cancellation costs at most ~n ulp of the
// node values (n < 128).
constexpr float kRoundMagic = 12582912.0f;
constexpr uint32_t kRoundMagicBits = 0x4B400000u;

// One entry: a.xyz, b.x | b.y, b.z, -, - at order 2; above order 2 (packed)
// a.xy, b.xy | a.z, b.z, -, -, the x, y channels as aligned register pairs
// for the packed FP32x2 FMA.
constexpr int kNodeBytes = 32;
// One order-2 entry, the Rayleigh and the Mie lines in 48 bytes:
// aR.xyz, bR.x | bR.yz, aM.xy | aM.z, bM.xyz.  The 48-byte stride also puts
// the 8 entries of a 16-bank span on disjoint banks.
constexpr int kPairBytes = 48;

// Three channels as a register pair (x, y) and a scalar (z) for the packed
// FP32x2 instructions (per component the same IEEE operations as fmaf and
// fadd, so the sums are bit-identical to the scalar ones).  Above order 2 the
// density kernel is bound by instruction issue, and the packed FMAs and adds
// of its lookups and sums save ~3% of its time.  At order 2 they do not pay:
// its code stays scalar.
struct P3 {
  float2 xy;
  float z;
};
__device__ __forceinline__ float2 Dup(float a) { return make_float2(a, a); }
__device__ __forceinline__ P3 ToP3(F3 a) { return P3{make_float2(a.x, a.y), a.z}; }
__device__ __forceinline__ F3 ToF3(P3 a) { return F3{a.xy.x, a.xy.y, a.z}; }
__device__ __forceinline__ F3 ToF3(F3 a) { return a; }
__device__ __forceinline__ P3 Fma(P3 a, P3 b, P3 c) {
  return P3{__ffma2_rn(a.xy, b.xy, c.xy), fmaf(a.z, b.z, c.z)};
}
__device__ __forceinline__ P3 Add(P3 a, P3 b) { return P3{__fadd2_rn(a.xy, b.xy), a.z + b.z}; }

// Approximate reciprocal square root, square root and division that flush
// subnormal operands to zero (the PTX .approx.ftz forms).  The non-flushing
// forms that rsqrtf, sqrtf under --prec-sqrt=false and __fdividef compile to
// add a range check and a rescaling of subnormal operands to every call.
// Every operand given to these below is zero, a normal number or negative
// (where both forms return NaN); on normal operands of the ranges used here
// the two forms agree bit for bit (16.7 M operands per range compared on a
// GB300).  Single and multiple scattering take 4.5% and 3.8% less time; their
// LUTs are not bit-identical to the non-flushing build's (the code around the
// calls is scheduled and contracted differently) and meet the same bounds.
__device__ __forceinline__ float RsqrtFtz(float x) {
  float y;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float SqrtFtz(float x) {
  float y;
  asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float DivFtz(float a, float b) {
  float y;
  asm("div.approx.ftz.f32 %0, %1, %2;" : "=f"(y) : "f"(a), "f"(b));
  return y;
}

// a b + c clamped to [0, 1], NaN to 0 (one FMA with the .sat modifier).
__device__ __forceinline__ float FmaSat(float a, float b, float c) {
  float d;
  asm("fma.rn.sat.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
  return d;
}

#ifdef ATMO_DEVICE_CHECKS
// The checked build's test of a table lookup: the `bytes` at shared address
// a lie within the block's dynamic shared memory, else the lookup reads its
// first bytes.
extern __shared__ float4 atmo_fast_dynamic_smem[];
__device__ __forceinline__ uint32_t CheckedShared(uint32_t a, int bytes) {
  const uint32_t base = (uint32_t)__cvta_generic_to_shared(atmo_fast_dynamic_smem);
  uint32_t size;
  asm("mov.u32 %0, %%dynamic_smem_size;" : "=r"(size));
  return base + (uint32_t)ATMO_CHECKED_INDEX(kCheckSharedLookup, a - base,
                                             (long long)size - bytes + 1);
}
#endif

template <int kOffset>
__device__ __forceinline__ float4 LoadShared4(uint32_t addr) {
#ifdef ATMO_DEVICE_CHECKS
  addr = CheckedShared(addr + kOffset, 16) - kOffset;
#endif
  float4 v;
  asm volatile("ld.shared.v4.f32 {%0, %1, %2, %3}, [%4+%5];"
               : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
               : "r"(addr), "n"(kOffset));
  return v;
}
template <int kOffset>
__device__ __forceinline__ float2 LoadShared2(uint32_t addr) {
#ifdef ATMO_DEVICE_CHECKS
  addr = CheckedShared(addr + kOffset, 8) - kOffset;
#endif
  float2 v;
  asm volatile("ld.shared.v2.f32 {%0, %1}, [%2+%3];" : "=f"(v.x), "=f"(v.y) : "r"(addr), "n"(kOffset));
  return v;
}
// The line a + b s of entry e (0 <= e <= N) of a row of N node values v[].
__device__ __forceinline__ void EntryLine(const float4* v, int e, int N, F3* a, F3* b) {
  if (e == 0 || e == N) {
    const float4 p = v[e == 0 ? 0 : N - 1];
    *a = F3{p.x, p.y, p.z};
    *b = f3(0.0f);
    return;
  }
  const float4 p = v[e - 1], q = v[e];
  const F3 d{q.x - p.x, q.y - p.y, q.z - p.z};
  const float c = 0.5f - float(e);   // -(n + 0.5) for the segment n = e - 1
  *a = fma3(d, c, F3{p.x, p.y, p.z});
  *b = d * float(N);
}
template <bool kPacked>
__device__ __forceinline__ void StoreLine(float4* entry, F3 a, F3 b) {
  if (kPacked) {
    entry[0] = make_float4(a.x, a.y, b.x, b.y);
    entry[1] = make_float4(a.z, b.z, 0.0f, 0.0f);
  } else {
    entry[0] = make_float4(a.x, a.y, a.z, b.x);
    entry[1] = make_float4(b.y, b.z, 0.0f, 0.0f);
  }
}
// Entry e (0 <= e <= N) of a row of N node values v[0..N-1].
template <bool kPacked>
__device__ __forceinline__ void StoreEntry(float4* entry, const float4* v, int e, int N) {
  F3 a, b;
  EntryLine(v, e, N, &a, &b);
  StoreLine<kPacked>(entry, a, b);
}
// Entry e of a row of N Rayleigh values r[] and Mie values m[] (order 2).
__device__ __forceinline__ void StorePairEntry(float4* entry, const float4* r, const float4* m,
                                               int e, int N) {
  float4 a[2], b[2];
  StoreEntry<false>(a, r, e, N);
  StoreEntry<false>(b, m, e, N);
  entry[0] = a[0];
  entry[1] = make_float4(a[1].x, a[1].y, b[0].x, b[0].y);
  entry[2] = make_float4(b[0].z, b[0].w, b[1].x, b[1].y);
}
// The staged function at the unit coordinate s, t = fmaf(s, N, kRoundMagic),
// of the table whose entries (kStride bytes apart, the function's at byte
// kOffset) start at row_adj + kRoundMagicBits kStride.
template <int kStride, int kOffset>
__device__ __forceinline__ F3 EvalNodes(float s, float t, uint32_t row_adj) {
  const uint32_t a = (uint32_t)__float_as_int(t) * (uint32_t)kStride + row_adj;
  const float4 p = LoadShared4<kOffset>(a);
  const float2 q = LoadShared2<kOffset + 16>(a);
  return F3{fmaf(s, p.w, p.x), fmaf(s, q.x, p.y), fmaf(s, q.y, p.z)};
}
// The line of the packed entry at shared address a, at s.
__device__ __forceinline__ P3 PackedLine(float s, uint32_t a) {
  const float4 p = LoadShared4<0>(a);
  const float2 q = LoadShared2<16>(a);
  return P3{__ffma2_rn(Dup(s), make_float2(p.z, p.w), make_float2(p.x, p.y)), fmaf(s, q.y, q.x)};
}
// EvalNodes for a packed table of kNodeBytes entries.
__device__ __forceinline__ P3 EvalNodesPacked(float s, float t, uint32_t row_adj) {
  return PackedLine(s, (uint32_t)__float_as_int(t) * (uint32_t)kNodeBytes + row_adj);
}
// Both lines of an order-2 entry (kPairBytes apart).
__device__ __forceinline__ void EvalPair(float s, float t, uint32_t row_adj, F3* ray, F3* mie) {
  const uint32_t a = (uint32_t)__float_as_int(t) * (uint32_t)kPairBytes + row_adj;
  const float4 p = LoadShared4<0>(a), q = LoadShared4<16>(a), r = LoadShared4<32>(a);
  *ray = F3{fmaf(s, p.w, p.x), fmaf(s, q.x, p.y), fmaf(s, q.y, p.z)};
  *mie = F3{fmaf(s, r.y, q.z), fmaf(s, r.z, q.w), fmaf(s, r.w, r.x)};
}
__host__ __device__ constexpr uint32_t RowAdjust(uint32_t base, int stride) {
  return base - kRoundMagicBits * (uint32_t)stride;
}

// Ground rows above order 2.  On a theta row whose directions hit the ground
// the incoming radiance is the sky line (entry i, in s) plus tg times the
// irradiance line (entry j, in the ground coordinate x = gs s + go), and on
// each (i, j) pair their sum is one line in s.  A merged table of (NU + 1) x J
// entries per row (J = the ground entries the row can reach) turns the ground
// lookup into a second index: x and its entry come from the same saturating
// and rounding FMAs as the separate lookup, monotone in s, so the entries
// reached lie between those of s = 0 and s = 1 and no index leaves the table.
// Rows are merged in theta order while their tables fit the budget; the
// others keep the separate lookups.
struct MergeRow {
  float gs, go;       // x = gs s + go (the same values build and read the table)
  uint32_t adj;       // address adjustment of the row's table
  uint32_t jstride;   // J x kNodeBytes; 0 when the row is not merged
};
// Above order 2 a block is limited to 2 per SM by its registers, so its
// shared memory may grow to ~99 KB (opted in above the default 48 KB) at no
// cost in occupancy.
constexpr int kDensityMaxSmem = 99 * 1024;

// Shared memory of one block, bytes, without the merged tables: [16][NU + 1]
// entries (the previous order interpolated in mu at the slab's r and mu_s;
// at order 2 a Rayleigh and a Mie line each), the bottom row of the
// irradiance LUT as [IW + 1] entries, a float4 staging value per node, and
// above order 2 the merge rows' descriptors and the merged entry count.
__host__ __device__ inline int DensityBaseSmem(const Shape& s, int order) {
  const int species = order == 2 ? 2 : 1;
  const int nodes = kDensityThetaSamples * s.snu;
  const int entries = kDensityThetaSamples * (s.snu + 1);
  return entries * (order == 2 ? kPairBytes : kNodeBytes) + (s.iw + 1) * kNodeBytes +
         (species * nodes + s.iw) * 16 +
         (order == 2 ? 0 : kDensityThetaSamples * (int)(sizeof(MergeRow) + sizeof(int4)) + 16);
}
// The merged tables a block of the instance may need above order 2, bytes:
// the largest r-slice's sum over its ground rows of (NU + 1) J entries, with
// J bounded from the ray's distance to the ground (the FP64 geometry of the
// set-up tables at the slice's r and cos(theta_l), plus a margin for the
// rounding of both ends).  Only a budget: rows that do not fit it keep the
// separate sky and ground lookups.
int DensityMergeNeed(const Shape& s, const Consts& c) {
  const double Rb = c.dRb, H = c.dH, pi = 3.14159265358979323846;
  const double k1 = double(s.snu - 1) / (2.0 * s.snu), kg = double(s.iw - 1) / (2.0 * s.iw);
  int worst = 0;
  for (int k = 0; k < s.sr; ++k) {
    const double rho = H * k / double(s.sr > 1 ? s.sr - 1 : 1);
    const double r = std::sqrt(rho * rho + Rb * Rb);
    int entries = 0;
    for (int l = 0; l < kDensityThetaSamples; ++l) {
      const double mu = std::cos((l + 0.5) * pi / kDensityThetaSamples);
      const double disc = r * r * (mu * mu - 1.0) + Rb * Rb;
      if (mu >= 0.0 || disc < 0.0) continue;
      const double gs = kg * (-r * mu - std::sqrt(disc)) / (Rb * k1);
      const int J = std::min((int)std::floor(gs * s.iw) + 3, s.iw + 1);
      entries += (s.snu + 1) * J;
    }
    worst = std::max(worst, entries);
  }
  return worst * kNodeBytes;
}
int DensityFastSmem(const Shape& s, const Consts& c, int order) {
  const int base = DensityBaseSmem(s, order);
  if (order == 2) return base;
  const int room = kDensityMaxSmem - base;
  const int merge = std::min(DensityMergeNeed(s, c), room > 0 ? room : 0);
  return base + merge / kNodeBytes * kNodeBytes;
}


// Shapes whose order-2 tables (the larger) fit the default 48 KB per block;
// the others take the plain density kernel.
bool DensityFastFits(const Shape& s) { return DensityBaseSmem(s, 2) <= 48 * 1024; }

// Texels of one mu row that a thread integrates together: they share the
// outgoing direction's phase functions (4 at every order: at order 2, 128
// registers and 2 blocks per SM beat 2 texels at 80 registers and 3 blocks
// by ~3%).
template <bool kOrder2>
__host__ __device__ constexpr int DensityTexelsPerTask() { return 4; }

// The outgoing direction's phase functions and the scattering coefficients
// fold into one weight per channel and direction, shared by the task's 4
// texels (one mu row: one altitude), so a texel keeps one sum.
template <bool kOrder2>
struct DensityTask {
  static constexpr int kN = DensityTexelsPerTask<kOrder2>();
  using V = std::conditional_t<kOrder2, F3, P3>;   // packed above order 2
  float sx[kN], sy[kN];   // the sun's x, y
  V sum[kN];              // sums of L (a_R P_R(nu2) + a_M P_M(nu2)) dw
};

// The 32 phi samples of theta row l for the texels of one task.  Everything
// is in the unit coordinate s = 1/2 + k1 nu1 (k1 = (NU - 1) / (2 NU)) of the
// staged rows: A is s's part 1/2 + k1 mu_s cos(theta_l), hs = k1 sin(theta_l)
// scales the direction's cos(phi), sin(phi), so a side's coordinate is one
// FMA with the sun's sx or sy and the ground lookup's coordinate another
// (g_scale, g_off map s to the irradiance row's unit coordinate); order 2
// recovers nu1 = (s - 1/2) / k1 for its phase functions.  war, wam: the
// scattering coefficients at the texel times the phase constants and dw.
// kMerged (ground rows above order 2): the row's merged table (MergeRow)
// replaces the sky and ground lookups.
template <bool kOrder2, bool kGround, bool kMerged = false>
__device__ __forceinline__ void DensityThetaRow(DensityTask<kOrder2>& task,
                                                const Consts& c, float A, float hs, float B,
                                                float oxs, F3 war, F3 wam, float fnu,
                                                float inv_k1, uint32_t row_adj, F3 tg,
                                                float g_scale, float g_off, float fiw,
                                                uint32_t ir_adj, uint32_t jstride = 0,
                                                uint32_t madj = 0) {
  static_assert(!kMerged || (kGround && !kOrder2), "merged tables: ground rows above order 2");
  using V = typename DensityTask<kOrder2>::V;
  constexpr int kDensityTexelsPerTask = DensityTexelsPerTask<kOrder2>();
  const float m2g = c.m2g, g2p1 = c.g2p1;
  // phi and 2 pi - phi share cos(phi), hence nu2 and the phase functions of
  // the outgoing direction; nu1 differs by the sign of sy sin(phi).  Unrolled
  // 4 times above order 2, not at order 2 (measured: -1.7% and -1.2%
  // against 2; with the packed arithmetic, 2 and 8 are 2% and 5% slower
  // than 4 above order 2).
#pragma unroll(kOrder2 ? 1 : 4)
  for (int m = 0; m < kDensityPhiSamples / 2; ++m) {
    const float2 cs = c_density_phi[m];
    // Phase functions at nu2 (functions.glsl:739-747, :1245-1254), folded
    // with the scattering coefficients into one weight per channel.
    const float nu2 = fmaf(oxs, cs.x, B);
    const float q2 = fmaf(nu2, nu2, 1.0f);
    // 1 + g^2 - 2 g nu2 >= (1 - g)^2: zero or normal for |g| < 1.
    const float rs = RsqrtFtz(fmaf(m2g, nu2, g2p1));
    const F3 wf = fma3(wam, q2 * (rs * rs * rs), war * q2);
    const P3 w = ToP3(wf);
    const float hc = cs.x * hs, hn = cs.y * hs;
#pragma unroll
    for (int q = 0; q < kDensityTexelsPerTask; ++q) {
      // The unit coordinate of nu1: bu +- sy sin(theta) sin(phi) / 2.
      const float bu = fmaf(task.sx[q], hc, A);
      // Ls is seeded with the first side's radiance (an explicit 0 + x
      // would cost an add per channel: IEEE keeps it).
      V Ls;
#pragma unroll
      for (int side = 0; side < 2; ++side) {
        const float u = FmaSat(side == 0 ? hn : -hn, task.sy[q], bu);
        const float t = fmaf(u, fnu, kRoundMagic);
        if constexpr (kMerged) {
          // Entry (i, j) of the merged table: one line in s for sky + ground.
          const float x = FmaSat(u, g_scale, g_off);
          const uint32_t a = (uint32_t)__float_as_int(t) * jstride +
                             (uint32_t)__float_as_int(fmaf(x, fiw, kRoundMagic)) *
                                 (uint32_t)kNodeBytes +
                             madj;
          const P3 L = PackedLine(u, a);
          Ls = side == 0 ? L : Add(Ls, L);
          continue;
        }
        if constexpr (kOrder2) {
          F3 L, M;
          EvalPair(u, t, row_adj, &L, &M);
          // Single scattering with its phase functions at nu1 (:998-1004):
          // (1 + nu1^2) (R 3/(16 pi) + M k_M / (1 + g^2 - 2 g nu1)^(3/2)),
          // with the constant factors staged into the tables.
          const float nu1 = fmaf(u, inv_k1, -0.5f * inv_k1);
          const float r1 = RsqrtFtz(fmaf(m2g, nu1, g2p1));
          const F3 L1 = fma3(M, r1 * r1 * r1, L);
          const float q1 = fmaf(nu1, nu1, 1.0f);
          Ls = side == 0 ? L1 * q1 : fma3(L1, q1, Ls);
        } else {
          const P3 L = EvalNodesPacked(u, t, row_adj);
          Ls = side == 0 ? L : Add(Ls, L);
        }
        if (kGround) {
          // Ground bounce: the ground point is at radius Rb, so the cosine
          // of its normal with the sun is (r mu_s + dist nu1) / Rb; the
          // irradiance lookup at r = Rb reads row 0 of the LUT.
          const float x = FmaSat(u, g_scale, g_off);
          const float xt = fmaf(x, fiw, kRoundMagic);
          if constexpr (kOrder2) {
            Ls = fma3(tg, EvalNodes<kNodeBytes, 0>(x, xt, ir_adj), Ls);
          } else {
            Ls = Fma(ToP3(tg), EvalNodesPacked(x, xt, ir_adj), Ls);
          }
        }
      }
      if constexpr (kOrder2) {
        task.sum[q] = fma3(Ls, wf, task.sum[q]);
      } else {
        task.sum[q] = Fma(Ls, w, task.sum[q]);
      }
    }
  }
}

template <bool kOrder2>
__global__ void __launch_bounds__(kDensityFastThreads)
k_density_fast(const Instance* __restrict__ insts, WorkList wl, int order, int smem_bytes) {
  extern __shared__ float4 smem[];
  constexpr int kSpecies = kOrder2 ? 2 : 1;
  constexpr int kStride = kOrder2 ? kPairBytes : kNodeBytes;
  constexpr int kDensityTexelsPerTask = DensityTexelsPerTask<kOrder2>();
  int local;
  const Instance& in = insts[FindEntry(wl, blockIdx.x, &local)];
  const Shape s = in.s;
  const int NU = s.snu, W = s.sw();
  const int k = local / s.smus, col = local % s.smus;
  const int nodes = kDensityThetaSamples * NU;
  const int row_entries = NU + 1;
  float4* E = smem;                                            // [16][NU + 1] entries
  float4* G = E + kDensityThetaSamples * row_entries * (kStride / 16);
  float4* V = G + (s.iw + 1) * (kNodeBytes / 16);              // [species][16][NU], [IW] values
  // Above order 2: the merge rows, their table layout (offset, J, j0, size in
  // entries; size 0 when not merged) and the merged tables.
  MergeRow* meta = reinterpret_cast<MergeRow*>(V + kSpecies * nodes + s.iw);
  int4* build = reinterpret_cast<int4*>(meta + kDensityThetaSamples);
  int& merged_entries = *reinterpret_cast<int*>(build + kDensityThetaSamples);
  float4* X = reinterpret_cast<float4*>(build + kDensityThetaSamples + 1);
  const DensityRow* drows = in.tab.drows + k * kDensityThetaSamples;
  const Consts& c = in.c;
  const TexelCol cc = in.tab.cols[col];
  const float fnu = float(NU), fiw = float(s.iw);
  // s = 1/2 + k1 nu1 on the sky rows, 1/2 + kg mu_g on the irradiance row.
  const float k1 = float(NU - 1) / (2.0f * fnu), kg = float(s.iw - 1) / (2.0f * fiw);
  const float inv_k1 = 1.0f / k1, inv_rb = 1.0f / c.Rb;

  // Node values: the previous order (Rayleigh or multiple, then Mie at order
  // 2) at column n MU_S + col of slice k, bilinear in mu; then the irradiance.
  const int staged = kSpecies * nodes + s.iw;
  for (int e = threadIdx.x; e < staged; e += blockDim.x) {
    float4 v;
    if (e < kSpecies * nodes) {
      const int sp = e / nodes, ne = e - sp * nodes;
      const int l = ne / NU, n = ne - l * NU;
      const float Y = drows[l].u_mu * float(s.smu) - 0.5f;
      const float fy = floorf(Y);
      const float wy = Y - fy;
      const int y0 = ClampIdx((int)fy, s.smu), y1 = ClampIdx((int)fy + 1, s.smu);
      const float4* src =
          (kOrder2 && sp == 1 ? in.dM : in.dR) + k * s.smu * W + n * s.smus + col;
#ifdef ATMO_DEVICE_CHECKS
      const long long o = src - (kOrder2 && sp == 1 ? in.dM : in.dR), nS = s.s_texels();
      const float4 a = __ldg(src - o + ATMO_CHECKED_INDEX(kCheckDensityStage, o + y0 * W, nS));
      const float4 b = __ldg(src - o + ATMO_CHECKED_INDEX(kCheckDensityStage, o + y1 * W, nS));
#else
      const float4 a = __ldg(src + y0 * W), b = __ldg(src + y1 * W);
#endif
      // At order 2 the single-scattering tables carry their phase constants.
      const float scale = kOrder2 ? (sp == 1 ? in.c.mie_k : in.c.ray_k) : 1.0f;
      v = make_float4(fmaf(wy, b.x - a.x, a.x) * scale, fmaf(wy, b.y - a.y, a.y) * scale,
                      fmaf(wy, b.z - a.z, a.z) * scale, 0.0f);
    } else {
      v = __ldg(DeltaIrradiance(in, order - 2) + (e - kSpecies * nodes));
    }
    V[e] = v;
  }
  if (!kOrder2 && threadIdx.x < kDensityThetaSamples) {
    // Row l's ground coordinate and the ground entries j0..j1 it can reach.
    const int l = threadIdx.x;
    const DensityRow dr = drows[l];
    MergeRow mr{0.0f, 0.0f, 0u, 0u};
    int4 b = make_int4(0, 0, 0, 0);
    if (dr.ground) {
      // The ground point's mu_g = (r mu_s + dist nu1) / Rb: its irradiance
      // coordinate 1/2 + kg mu_g is w0 + kg dist (s - 1/2) / (k1 Rb).
      const float w0 = fmaf(in.tab.rows[k * s.smu].r * cc.mu_s * inv_rb, kg, 0.5f);
      mr.gs = kg * dr.dist_ground * inv_rb * inv_k1;
      mr.go = fmaf(-0.5f, mr.gs, w0);
      const int j0 = __float_as_int(fmaf(FmaSat(0.0f, mr.gs, mr.go), fiw, kRoundMagic)) -
                     (int)kRoundMagicBits;
      const int j1 = __float_as_int(fmaf(FmaSat(1.0f, mr.gs, mr.go), fiw, kRoundMagic)) -
                     (int)kRoundMagicBits;
      if (j1 >= j0) b = make_int4(0, j1 - j0 + 1, j0, (NU + 1) * (j1 - j0 + 1));
    }
    meta[l] = mr;
    build[l] = b;
  }
  __syncthreads();
  if (!kOrder2 && threadIdx.x == 0) {
    // Table offsets, rows in theta order while they fit the budget.
    // The budget: the launch's shared memory beyond this instance's tables.
    const int budget = max(smem_bytes - DensityBaseSmem(s, 3), 0) / kNodeBytes;
    const uint32_t xbase = (uint32_t)__cvta_generic_to_shared(X);
    int off = 0;
    for (int l = 0; l < kDensityThetaSamples; ++l) {
      int4 b = build[l];
      if (b.w > 0 && off + b.w <= budget) {
        b.x = off;
        const uint32_t js = (uint32_t)(b.y * kNodeBytes);
        meta[l].jstride = js;
        // Entry (i, j) at X + off + i J + (j - j0), addressed from the two
        // rounding sums (magic + i, magic + j).
        meta[l].adj = xbase + (uint32_t)(off * kNodeBytes) - kRoundMagicBits * js -
                      (kRoundMagicBits + (uint32_t)b.z) * (uint32_t)kNodeBytes;
        off += b.w;
      } else {
        b.w = 0;
      }
      build[l] = b;
    }
    merged_entries = off;
  }
  __syncthreads();
  const int sky_entries = kDensityThetaSamples * row_entries;
  const int base_entries = sky_entries + s.iw + 1;
  const int total_entries = base_entries + (kOrder2 ? 0 : merged_entries);
  for (int e = threadIdx.x; e < total_entries; e += blockDim.x) {
    if (e < sky_entries) {
      const int l = e / row_entries, i = e - l * row_entries;
      if (kOrder2) {
        StorePairEntry(E + e * (kPairBytes / 16), V + l * NU, V + nodes + l * NU, i, NU);
      } else {
        StoreEntry<true>(E + e * (kNodeBytes / 16), V + l * NU, i, NU);
      }
    } else if (e < base_entries) {
      const int i = e - sky_entries;
      StoreEntry<!kOrder2>(G + i * (kNodeBytes / 16), V + kSpecies * nodes, i, s.iw);
    } else if (!kOrder2) {
      // Merged entry (i, j) of row l: sky line + tg (ground line at gs s + go).
      const int m = e - base_entries;
      int l = 0;
      while (l < kDensityThetaSamples - 1 && !(build[l].w > 0 && m < build[l].x + build[l].w)) ++l;
      const int4 b = build[l];
      const int idx = m - b.x, i = idx / b.y, j = b.z + (idx - i * b.y);
      F3 sa, sb, ga, gb;
      EntryLine(V + l * NU, i, NU, &sa, &sb);
      EntryLine(V + nodes, j, s.iw, &ga, &gb);
      const F3 tg = f3(drows[l].t_ground);
      const MergeRow mr = meta[l];
      StoreLine<true>(X + m * (kNodeBytes / 16), fma3(tg, fma3(gb, mr.go, ga), sa),
                fma3(tg, gb * mr.gs, sb));
    }
  }
  __syncthreads();

  const float dtdp = (kPiF / 16.0f) * (kPiF / 16.0f);
  const uint32_t e_base = (uint32_t)__cvta_generic_to_shared(E);
  const uint32_t ir_adj = RowAdjust((uint32_t)__cvta_generic_to_shared(G), kNodeBytes);
  const int per_row = (NU + kDensityTexelsPerTask - 1) / kDensityTexelsPerTask;
  const int tasks = s.smu * per_row;
  for (int ti = threadIdx.x; ti < tasks; ti += blockDim.x) {
    const int j = ti % s.smu, n0 = (ti / s.smu) * kDensityTexelsPerTask;
    const TexelRow row = in.tab.rows[k * s.smu + j];
    DensityTask<kOrder2> task;
#pragma unroll
    for (int q = 0; q < kDensityTexelsPerTask; ++q) {
      const TexelAngles ang = MakeAngles(s, row, cc, min(n0 + q, NU - 1));
      task.sx[q] = ang.sx;
      task.sy[q] = ang.sy;
      task.sum[q] = typename DensityTask<kOrder2>::V{};
    }
    // The scattering coefficients at the texel, with the phase constants.
    const F3 a_r = c.rayleigh * (ProfileDensity(c.prof_r, row.h) * c.ray_k);
    const F3 a_m = c.mie_sca * (ProfileDensity(c.prof_m, row.h) * c.mie_k);
    // Order 2: the ground point's mu_g = (r mu_s + dist nu1) / Rb; its
    // irradiance coordinate 1/2 + kg mu_g is w0 + kg dist nu1 / Rb.
    const float w0 = fmaf(row.r * cc.mu_s * inv_rb, kg, 0.5f);
    for (int l = 0; l < kDensityThetaSamples; ++l) {
      const DensityRow dr = drows[l];
      const float B = row.mu * dr.cos_t;
      const float oxs = row.omega_x * dr.sin_t;
      const float dw = dtdp * dr.sin_t;
      // In the unit coordinate of nu1 (see DensityThetaRow).
      const float A = fmaf(cc.mu_s * dr.cos_t, k1, 0.5f);
      const float hs = k1 * dr.sin_t;
      const uint32_t row_adj =
          RowAdjust(e_base + (uint32_t)(l * row_entries * kStride), kStride);
      if (dr.ground) {
        if constexpr (kOrder2) {
          // The ground point's irradiance coordinate from s = 1/2 + k1 nu1:
          // w0 + kg dist (s - 1/2) / (k1 Rb).
          const float gs = kg * dr.dist_ground * inv_rb * inv_k1;
          const float go = fmaf(-0.5f, gs, w0);
          DensityThetaRow<kOrder2, true>(task, c, A, hs, B, oxs, a_r * dw, a_m * dw, fnu,
                                         inv_k1, row_adj, f3(dr.t_ground), gs, go, fiw, ir_adj);
        } else {
          const MergeRow mr = meta[l];
          if (mr.jstride != 0) {
            DensityThetaRow<kOrder2, true, true>(task, c, A, hs, B, oxs, a_r * dw, a_m * dw,
                                                 fnu, inv_k1, row_adj, f3(0.0f), mr.gs, mr.go,
                                                 fiw, ir_adj, mr.jstride, mr.adj);
          } else {
            DensityThetaRow<kOrder2, true>(task, c, A, hs, B, oxs, a_r * dw, a_m * dw, fnu,
                                           inv_k1, row_adj, f3(dr.t_ground), mr.gs, mr.go, fiw,
                                           ir_adj);
          }
        }
      } else {
        DensityThetaRow<kOrder2, false>(task, c, A, hs, B, oxs, a_r * dw, a_m * dw, fnu, inv_k1,
                                        row_adj, f3(0.0f), 0.0f, 0.0f, fiw, ir_adj);
      }
    }
#pragma unroll
    for (int q = 0; q < kDensityTexelsPerTask; ++q) {
      if (n0 + q < NU) {
        const F3 J = ToF3(task.sum[q]);
        in.dJ[(k * s.smu + j) * W + (n0 + q) * s.smus + col] = to4(J, 1.0f);
      }
    }
  }
}

// Lets k_density_fast<false> take kDensityMaxSmem (once per device; every
// later call is a lock-free check).  Called before a CUDA graph capture and
// by the launcher.
cudaError_t PrepareDensityFast() {
  static std::atomic<unsigned long long> done{0};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  const unsigned long long bit = 1ull << (dev & 63);
  if (done.load(std::memory_order_acquire) & bit) return cudaSuccess;
  e = cudaFuncSetAttribute(k_density_fast<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           kDensityMaxSmem);
  if (e == cudaSuccess) done.fetch_or(bit, std::memory_order_acq_rel);
  return e;
}

cudaError_t LaunchDensityFast(const Instance* insts, WorkList wl, int tiles, int order,
                              int smem_bytes, cudaStream_t st) {
  // smem_bytes: the largest DensityFastSmem of the work list's instances.
  const size_t bytes = (size_t)smem_bytes;
  if (order == 2) {
    k_density_fast<true><<<tiles, kDensityFastThreads, bytes, st>>>(insts, wl, order, smem_bytes);
  } else {
    if (smem_bytes > 48 * 1024) {
      const cudaError_t e = PrepareDensityFast();
      if (e != cudaSuccess) return e;
    }
    k_density_fast<false><<<tiles, kDensityFastThreads, bytes, st>>>(insts, wl, order,
                                                                      smem_bytes);
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
// Rows per block and samples per line stage: the tuned values of the shape,
// else as many rows (up to 4) as fill 256 threads and two line buffers of
// group x rows x W float4 within 32 KB.
__host__ __device__ inline MultipleFastDims MultipleDims(const Shape& s) {
  const int W = s.sw();
  int rows = kMultipleFastThreads / W;
  rows = rows < 1 ? 1 : (rows > 4 ? 4 : rows);
  if (s.tune[0] > 0) rows = s.tune[0];
  int group = 32768 / (2 * 16 * rows * W);
  group = group < 1 ? 1 : (group > 4 ? 4 : group);
  if (s.tune[1] > 0) group = s.tune[1];
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

// The LUT row that logical row i of the multiple-scattering blocks takes.
__device__ __forceinline__ int RowAt(const Tables& tab, int i) {
  return tab.row_order ? __ldg(tab.row_order + i) : i;
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

// UMuSFromMuS with the mapping's constant divisions replaced by products
// (inv_range = 1 / (d_max - d_min), inv_A = 1 / A) and the others approximate
// (<= 2 ulp): for samples along a ray, whose mu_s is not a texel's own.
__device__ __forceinline__ float UMuSFromMuSAlongRay(const Consts& c, const Shape& s, float mu_s,
                                                     float inv_range, float inv_A) {
  const float H2 = c.H * c.H;
  const float rmus = c.Rb * mu_s;
  // H^2 + (Rb mu_s)^2 >= H^2 and rmus + sq >= H > 0: normal.  The last
  // quotient's numerator is zero or in [ulp(1), 1], its denominator in
  // [1, 2].
  const float sq = SqrtFtz(fmaf(rmus, rmus, H2));
  const float d = rmus > 0.0f ? DivFtz(H2, rmus + sq) : sq - rmus;
  const float a = (d - (c.Rt - c.Rb)) * inv_range;
  return TexCoord(s, kMapSMUS, DivFtz(fmaxf(fmaf(-a, inv_A, 1.0f), 0.0f), 1.0f + a));
}

// The element at offset + x of a LUT row of a line build.
#define ATMO_LINE_PTR(base, offset, x, n) ATMO_CHECKED_PTR(kCheckLineLoad, base, offset, x, n)

// A read-only global load predicated on p: v keeps its value when p is 0.
// The predicate keeps the line build free of branches, so a sample's loads
// still issue as early as the unconditional ones.
__device__ __forceinline__ void LoadIf(float4& v, const float4* ptr, int p) {
  asm("{\n\t.reg .pred q;\n\tsetp.ne.s32 q, %5, 0;\n\t"
      "@q ld.global.nc.v4.f32 {%0, %1, %2, %3}, [%4];\n\t}"
      : "+f"(v.x), "+f"(v.y), "+f"(v.z), "+f"(v.w)
      : "l"(ptr), "r"(p));
}

template <int kCols>
__device__ __forceinline__ void MultipleFastBlock(const Instance& in, int local, float4* smem) {
  const Shape s = in.s;
  const Consts& c = in.c;
  const MultipleFastDims dims = MultipleDims(s);
  const int W = s.sw(), R = dims.rows, G = dims.group;
  const int rows_total = s.sr * s.smu;
  [[maybe_unused]] const long long nS = s.s_texels();   // checked build
  const int row0 = local * R;
  RaySample* samp = reinterpret_cast<RaySample*>(smem);                 // [R][kRaySamples]
  float4* line = smem + R * kRaySamples * (int)(sizeof(RaySample) / 16);   // [2][G][R][W]

  for (int e = threadIdx.x; e < R * kRaySamples; e += kMultipleFastThreads) {
    const int rr = e / kRaySamples, i = e - rr * kRaySamples;
    if (row0 + rr < rows_total) samp[e] = MakeRaySample(in, RowAt(in.tab, row0 + rr), i);
  }

  // This thread's row within the tile and its texel columns x_t + 256 m.
  const int rr = kCols == 1 ? (int)threadIdx.x / W : 0;
  const int x_t = kCols == 1 ? (int)threadIdx.x - rr * W : (int)threadIdx.x;
  const bool active = rr < R && row0 + rr < rows_total;
  const int rowi = active ? RowAt(in.tab, row0 + rr) : 0;
  const float smus_f = float(s.smus);
  const int nmax = W - 1;
  const float inv_range = 1.0f / (c.H - (c.Rt - c.Rb));
  const float inv_A = 1.0f / c.mus_A;
  float rmu_s[kCols], nu[kCols], lnu[kCols];
  int xb[kCols];
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
      // A texel whose nu is not clamped sits on its own nu node n: the
      // reference's FP64 coordinate (nu + 1) / 2 (NU - 1) is n to ~1e-16, so
      // the neighbouring node's weight is taken as 0 and its taps skipped.
      const float tex_coord_x = (ang.nu + 1.0f) * 0.5f * float(s.snu - 1);
      const float tex_x = ang.on_node ? float(n) : floorf(tex_coord_x);
      lnu[m] = ang.on_node ? 0.0f : tex_coord_x - tex_x;
      xb[m] = (int)tex_x * s.smus;   // the node's block (see MakeLookup)
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
    if (active && kCols == 1) {
      // Consecutive samples of a ray lie in the same (mu, r) cell of the
      // delta-density LUT for 38% of the samples at the reference's shape:
      // their four rows, already in registers, are not loaded again (r00 and
      // r11 fix all four).  Predicated loads rather than a branch: a branch
      // around the loads measured slower than four loads per sample.  The
      // values, hence the LUTs, are the same as with four loads per sample.
      // The thread's column of the LUT, of its line and of its row's samples,
      // addressed once (row offsets are then 32-bit adds to a 64-bit base:
      // 7% fewer instructions than forming each address, 1.7% less time).
      int o00 = -1, o11 = -1;
      float4 a = make_float4(0.0f, 0.0f, 0.0f, 0.0f), b = a, p = a, q = a;
      const float4* col = in.dJ + x_t;
      float4* out_col = buf + rr * W + x_t;
      const RaySample* srow = samp + rr * kRaySamples + first;
      for (int g = 0; g < count; ++g) {
        const RaySample& sm = srow[g];
        const int fresh = (sm.r00 != o00) | (sm.r11 != o11);
        LoadIf(a, ATMO_LINE_PTR(col, sm.r00, 0, nS - x_t), fresh);
        LoadIf(b, ATMO_LINE_PTR(col, sm.r01, 0, nS - x_t), fresh);
        LoadIf(p, ATMO_LINE_PTR(col, sm.r10, 0, nS - x_t), fresh);
        LoadIf(q, ATMO_LINE_PTR(col, sm.r11, 0, nS - x_t), fresh);
        o00 = sm.r00;
        o11 = sm.r11;
        out_col[g * R * W] = make_float4(
            fmaf(q.x, sm.w11, fmaf(p.x, sm.w10, fmaf(b.x, sm.w01, a.x * sm.w00))),
            fmaf(q.y, sm.w11, fmaf(p.y, sm.w10, fmaf(b.y, sm.w01, a.y * sm.w00))),
            fmaf(q.z, sm.w11, fmaf(p.z, sm.w10, fmaf(b.z, sm.w01, a.z * sm.w00))), 0.0f);
      }
    } else if (active) {
      for (int g = 0; g < count; ++g) {
        const RaySample& sm = samp[rr * kRaySamples + first + g];
        float4* out = buf + (g * R + rr) * W;
#pragma unroll
        for (int m = 0; m < kCols; ++m) {
          const int x = x_t + m * kMultipleFastThreads;
          if (kCols > 1 && x >= W) break;
          const float4 a = __ldg(ATMO_LINE_PTR(in.dJ, sm.r00, x, nS));
          const float4 b = __ldg(ATMO_LINE_PTR(in.dJ, sm.r01, x, nS));
          const float4 p = __ldg(ATMO_LINE_PTR(in.dJ, sm.r10, x, nS));
          const float4 q = __ldg(ATMO_LINE_PTR(in.dJ, sm.r11, x, nS));
          out[x] = make_float4(
              fmaf(q.x, sm.w11, fmaf(p.x, sm.w10, fmaf(b.x, sm.w01, a.x * sm.w00))),
              fmaf(q.y, sm.w11, fmaf(p.y, sm.w10, fmaf(b.y, sm.w01, a.y * sm.w00))),
              fmaf(q.z, sm.w11, fmaf(p.z, sm.w10, fmaf(b.z, sm.w01, a.z * sm.w00))), 0.0f);
        }
      }
    }
    __syncthreads();
    if (active) {
      const RaySample* srow = samp + rr * kRaySamples + first;
      const float4* lrow = buf + rr * W;
      for (int g = 0; g < count; ++g) {
        const RaySample& sm = srow[g];
        const float4* L = lrow + g * R * W;
#pragma unroll
        for (int m = 0; m < kCols; ++m) {
          if (kCols > 1 && x_t + m * kMultipleFastThreads >= W) break;
          const float mu_s_i = clampf(fmaf(sm.d, nu[m], rmu_s[m]) * sm.inv_r, -1.0f, 1.0f);
          const float x0 =
              fmaf(UMuSFromMuSAlongRay(c, s, mu_s_i, inv_range, inv_A), smus_f, -0.5f);
          const float fx = floorf(x0);
          const float a = x0 - fx;
          const int i0 = xb[m] + (int)fx;
          const int c0 = min(max(i0, 0), nmax), c1 = min(max(i0 + 1, 0), nmax);
          const int c2 = min(max(i0 + s.smus, 0), nmax), c3 = min(max(i0 + s.smus + 1, 0), nmax);
          const float l1 = lnu[m], l0 = 1.0f - l1;
          const float v0 = (1.0f - a) * l0, v1 = a * l0;
          const float4 t0 = L[ATMO_CHECKED_INDEX(kCheckLineTap, c0, W)];
          const float4 t1 = L[ATMO_CHECKED_INDEX(kCheckLineTap, c1, W)];
          F3 S{fmaf(t1.x, v1, t0.x * v0), fmaf(t1.y, v1, t0.y * v0),
               fmaf(t1.z, v1, t0.z * v0)};
          if (l1 != 0.0f) {
            const float v2 = (1.0f - a) * l1, v3 = a * l1;
            const float4 t2 = L[ATMO_CHECKED_INDEX(kCheckLineTap, c2, W)];
            const float4 t3 = L[ATMO_CHECKED_INDEX(kCheckLineTap, c3, W)];
            S = F3{fmaf(t3.x, v3, fmaf(t2.x, v2, S.x)), fmaf(t3.y, v3, fmaf(t2.y, v2, S.y)),
                   fmaf(t3.z, v3, fmaf(t2.z, v2, S.z))};
          }
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
    const int texel = (int)ATMO_CHECKED_INDEX(kCheckOutput, rowi * W + x, nS);
    in.dR[texel] = to4(acc[m], 1.0f);   // delta multiple aliases delta Rayleigh
    const F3 add = MatVec(c.lum, acc[m]) * (1.0f / RayleighPhase(c, nu[m]));
    const float4 o = in.S[texel];
    in.S[texel] = make_float4(o.x + add.x, o.y + add.y, o.z + add.z, o.w);
  }
}

__global__ void __launch_bounds__(kMultipleFastThreads, 4)
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

// ---------------------------------------------------------------------------
// Single scattering, restructured (functions.glsl:650-730, :933-945).
//
// As for multiple scattering, a sample's r, altitude, densities and the
// transmittance from the texel to it depend on the texel's row only; the
// transmittance from the sample to the sun depends on mu_s at the sample,
// hence on the texel's column.  Its LUT lookup happens at the sample's
// (rho, r): a fixed pair of transmittance LUT rows.  Per sample the block
// interpolates those two rows into a line of W_T columns in shared memory; a
// texel computes the x_mu of its sun direction and reads 2 line entries.
// ---------------------------------------------------------------------------
constexpr int kSingleSamples = kSingleScatteringSamples + 1;

struct __align__(16) SunSample {
  int t0, t1;                // element offsets of the transmittance LUT rows j0, j1
  float b;                   // weight of row j1
  float rho, r, inv_r;       // the sample's rho, r and 1 / r
  float inv_2e;              // 1 / (2 sin(theta_h) alpha_s), sin(theta_h) = Rb / r
  float d;                   // distance from the texel's point along its ray
  float dens_r, dens_m;      // Rayleigh and Mie densities x trapezoid weight
  float tx, ty, tz;          // transmittance texel -> sample
  float inv_range;           // 1 / (d_max - d_min) of the transmittance mapping
  float pad[2];
};

__host__ __device__ inline MultipleFastDims SingleDims(const Shape& s) {
  int rows = kMultipleFastThreads / s.sw();
  rows = rows < 1 ? 1 : (rows > 4 ? 4 : rows);
  if (s.tune[2] > 0) rows = s.tune[2];
  int group = 32768 / (2 * 16 * rows * s.tw);
  group = group < 1 ? 1 : (group > 4 ? 4 : group);
  if (s.tune[3] > 0) group = s.tune[3];
  return MultipleFastDims{rows, group};
}
int SingleFastSmem(const Shape& s) {
  const MultipleFastDims d = SingleDims(s);
  return d.rows * kSingleSamples * (int)sizeof(SunSample) + 2 * d.group * d.rows * s.tw * 16;
}
bool SingleFastFits(const Shape& s) {
  return s.sw() <= kMultipleFastThreads * kMultipleFastMaxCols && SingleFastSmem(s) <= 48 * 1024;
}
int SingleFastTiles(const Shape& s) {
  const int rows = SingleDims(s).rows;
  return (s.sr * s.smu + rows - 1) / rows;
}

// Whether a (rows, group) block shape is launchable for shape s: one texel
// column per thread needs rows x W <= 256 (wider rows take one row per
// block), and the shared memory must stay within 48 KB.
bool FastTuningValid(const Shape& s, bool single, int rows, int group) {
  if (rows < 1 || rows > 4 || group < 1 || group > 8) return false;
  const int W = s.sw();
  if (W > kMultipleFastThreads * kMultipleFastMaxCols) return false;
  if (rows > 1 && rows * W > kMultipleFastThreads) return false;
  Shape t = s;
  t.tune[single ? 2 : 0] = rows;
  t.tune[single ? 3 : 1] = group;
  return (single ? SingleFastSmem(t) : MultipleFastSmem(t)) <= 48 * 1024;
}

// Sample i of the ray of LUT row `rowi` (the per-sample part of
// SingleScatteringTexel that does not depend on mu_s or nu).
__device__ SunSample MakeSunSample(const Instance& in, int rowi, int i) {
  const Consts& c = in.c;
  const Shape& s = in.s;
  const TexelRow row = in.tab.rows[rowi];
  const bool ground = row.ground != 0;
  const float dx = row.d / float(kSingleScatteringSamples);
  const float d = float(i) * dx;
  const float e = float(kSingleScatteringSamples - i) * dx;
  const RadialPoint p = PointFromRho2(c, RayRho2(row, d, e));
  const TStart start = MakeTStart(c, s, in.T, in.Tau, row.rho, row.r,
                                  ground ? -row.rmu : row.rmu, row.delta);
  const F3 t = SegmentTransmittance(c, s, in.T, in.Tau, row.rmu, row.delta, p, d, ground, start);
  const float w = (i == 0 || i == kSingleScatteringSamples) ? 0.5f : 1.0f;
  const float Y = p.rho / c.H * float(s.th - 1);
  const float fy = floorf(Y);
  const int j0 = ClampIdx((int)fy, s.th), j1 = ClampIdx((int)fy + 1, s.th);
  SunSample ss;
  ss.t0 = j0 * s.tw;
  ss.t1 = j1 * s.tw;
  ss.b = Y - fy;
  ss.rho = p.rho;
  ss.r = p.r;
  ss.inv_r = 1.0f / p.r;
  // 1 / 0 = +inf for a point sun: the smoothstep then becomes a step at 0.
  ss.inv_2e = 1.0f / (2.0f * (c.Rb / p.r * c.alpha_s));
  ss.d = d;
  ss.dens_r = ProfileDensity(c.prof_r, p.h) * w;
  ss.dens_m = ProfileDensity(c.prof_m, p.h) * w;
  ss.tx = t.x;
  ss.ty = t.y;
  ss.tz = t.z;
  const float d_min = (c.H - p.rho) * (c.H + p.rho) / (c.Rt + p.r);
  ss.inv_range = 1.0f / (p.rho + c.H - d_min);
  ss.pad[0] = ss.pad[1] = 0.0f;
  return ss;
}

template <int kCols>
__device__ __forceinline__ void SingleFastBlock(const Instance& in, int local, float4* smem) {
  const Shape s = in.s;
  const Consts& c = in.c;
  const MultipleFastDims dims = SingleDims(s);
  const int W = s.sw(), R = dims.rows, G = dims.group, TW = s.tw;
  const int rows_total = s.sr * s.smu;
  [[maybe_unused]] const long long nT = s.t_texels();   // checked build
  const int row0 = local * R;
  SunSample* samp = reinterpret_cast<SunSample*>(smem);                       // [R][51]
  float4* line = smem + R * kSingleSamples * (int)(sizeof(SunSample) / 16);   // [2][G][R][TW]

  for (int e = threadIdx.x; e < R * kSingleSamples; e += kMultipleFastThreads) {
    const int rr = e / kSingleSamples, i = e - rr * kSingleSamples;
    if (row0 + rr < rows_total) samp[e] = MakeSunSample(in, row0 + rr, i);
  }

  const int rr = kCols == 1 ? (int)threadIdx.x / W : 0;
  const int x_t = kCols == 1 ? (int)threadIdx.x - rr * W : (int)threadIdx.x;
  const int rowi = row0 + rr;
  const bool active = rr < R && rowi < rows_total;
  const int nmax = W - 1;
  float rmu_s[kCols], nu[kCols];
  F3 sum_r[kCols], sum_m[kCols];
  if (active) {
    const TexelRow row = in.tab.rows[rowi];
#pragma unroll
    for (int m = 0; m < kCols; ++m) {
      const int x = min(x_t + m * kMultipleFastThreads, nmax);
      const int n = x / s.smus, col = x - n * s.smus;
      const TexelAngles ang = MakeAngles(s, row, in.tab.cols[col], n);
      rmu_s[m] = row.r * ang.mu_s;
      nu[m] = ang.nu;
      sum_r[m] = f3(0.0f);
      sum_m[m] = f3(0.0f);
    }
  }
  __syncthreads();

  const float H = c.H, H2 = c.H * c.H;
  const float tw1 = float(TW - 1);
  const int line_stride = G * R * TW;
  const int stages = (kSingleSamples + G - 1) / G;
  for (int stage = 0; stage < stages; ++stage) {
    float4* buf = line + (stage & 1) * line_stride;
    const int first = stage * G;
    const int count = min(G, kSingleSamples - first);
    // Transmittance LUT rows j0, j1 of each sample, interpolated in rho.
    if (R == 1 && TW <= kMultipleFastThreads) {
      // One row per block, one line column per thread: consecutive samples
      // of the ray read the same two LUT rows 39% of the time at the
      // reference's shape, and those rows, already in registers, are not
      // loaded again (predicated loads: the same values, hence the same LUTs).
      // Handling the samples that share one row as well (another 53%) with
      // a branch per case, or with selects, measured slower.
      const int x = threadIdx.x;
      if (x < TW && row0 < rows_total) {
        // The thread's columns addressed once, as in multiple scattering.
        int o0 = -1, o1 = -1;
        float4 a = make_float4(0.0f, 0.0f, 0.0f, 0.0f), b = a;
        const float4* col = in.T + x;
        float4* out_col = buf + x;
        const SunSample* srow = samp + first;
        for (int g = 0; g < count; ++g) {
          const SunSample& sm = srow[g];
          const int fresh = (sm.t0 != o0) | (sm.t1 != o1);
          LoadIf(a, ATMO_LINE_PTR(col, sm.t0, 0, nT - x), fresh);
          LoadIf(b, ATMO_LINE_PTR(col, sm.t1, 0, nT - x), fresh);
          o0 = sm.t0;
          o1 = sm.t1;
          out_col[g * TW] = make_float4(fmaf(sm.b, b.x - a.x, a.x), fmaf(sm.b, b.y - a.y, a.y),
                                        fmaf(sm.b, b.z - a.z, a.z), 0.0f);
        }
      }
    } else {
      for (int g = 0; g < count; ++g) {
        for (int q = 0; q < R; ++q) {
          if (row0 + q >= rows_total) break;
          const SunSample& sm = samp[q * kSingleSamples + first + g];
          float4* out = buf + (g * R + q) * TW;
          for (int x = threadIdx.x; x < TW; x += kMultipleFastThreads) {
            const float4 a = __ldg(ATMO_LINE_PTR(in.T, sm.t0, x, nT));
            const float4 b = __ldg(ATMO_LINE_PTR(in.T, sm.t1, x, nT));
            out[x] = make_float4(fmaf(sm.b, b.x - a.x, a.x), fmaf(sm.b, b.y - a.y, a.y),
                                 fmaf(sm.b, b.z - a.z, a.z), 0.0f);
          }
        }
      }
    }
    __syncthreads();
    if (active) {
      for (int g = 0; g < count; ++g) {
        const SunSample& sm = samp[rr * kSingleSamples + first + g];
        const float4* L = buf + (g * R + rr) * TW;
#pragma unroll
        for (int m = 0; m < kCols; ++m) {
          if (kCols > 1 && x_t + m * kMultipleFastThreads >= W) break;
          // GetTransmittanceToSun (functions.glsl:552-563) at the sample, with
          // the lookup mapping of TransmittanceCoords.
          const float rmu = clampf(fmaf(sm.d, nu[m], rmu_s[m]), -sm.r, sm.r);
          // smoothstep(-e, e, mu_s - cos(theta_h)), cos(theta_h) = -rho / r.
          const float st = clampf((rmu + sm.rho) * sm.inv_r * sm.inv_2e + 0.5f, 0.0f, 1.0f);
          const float sun = st * st * fmaf(-2.0f, st, 3.0f);
          const float delta = (sm.rho - rmu) * (sm.rho + rmu);
          // H^2 - delta: zero, or a difference of floats far above FP32's
          // normal range (normal); delta and rho - rmu: zero, or sums and
          // products of lengths whose exact values are multiples of their
          // operands' ulps (normal); H + sq >= H.
          const float sq = SqrtFtz(fmaxf(H2 - delta, 0.0f));
          const float rho_minus_a =
              rmu < 0.0f ? (sm.rho - rmu > 0.0f ? DivFtz(delta, sm.rho - rmu) : 0.0f)
                         : sm.rho + rmu;
          const float omx =
              clampf((rho_minus_a + DivFtz(delta, H + sq)) * sm.inv_range, 0.0f, 1.0f);
          const float Xc = omx * tw1;
          const float f = floorf(Xc);
          const float gw = Xc - f;   // weight of the lower column
          const int i_hi = TW - 1 - (int)f;
          const int i_lo = max(i_hi - 1, 0);
          const float4 lo = L[ATMO_CHECKED_INDEX(kCheckLineTap, i_lo, TW)];
          const float4 hi = L[ATMO_CHECKED_INDEX(kCheckLineTap, max(i_hi, 0), TW)];
          const F3 tsun{fmaf(gw, lo.x - hi.x, hi.x), fmaf(gw, lo.y - hi.y, hi.y),
                        fmaf(gw, lo.z - hi.z, hi.z)};
          const F3 t = F3{sm.tx, sm.ty, sm.tz} * (tsun * sun);
          sum_r[m] = fma3(t, sm.dens_r, sum_r[m]);
          sum_m[m] = fma3(t, sm.dens_m, sum_m[m]);
        }
      }
    }
  }

  if (!active) return;
  const float dx = in.tab.rows[rowi].d / float(kSingleScatteringSamples);
#pragma unroll
  for (int m = 0; m < kCols; ++m) {
    const int x = x_t + m * kMultipleFastThreads;
    if (kCols > 1 && x >= W) break;
    StoreSingleScattering(in, (long long)rowi * W + x, sum_r[m] * dx * c.solar * c.rayleigh,
                          sum_m[m] * dx * c.solar * c.mie_sca);
  }
}

// 4 blocks per SM (64 registers, a few spills) beat 3 at 75 registers by 10%.
__global__ void __launch_bounds__(kMultipleFastThreads, 4)
k_single_fast(const Instance* __restrict__ insts, WorkList wl) {
  extern __shared__ float4 smem[];
  int local;
  const Instance& in = insts[FindEntry(wl, blockIdx.x, &local)];
  if (in.s.sw() <= kMultipleFastThreads) {
    SingleFastBlock<1>(in, local, smem);
  } else {
    SingleFastBlock<kMultipleFastMaxCols>(in, local, smem);
  }
}

cudaError_t LaunchSingleFast(const Instance* insts, WorkList wl, int tiles, int smem_bytes,
                             cudaStream_t st) {
  // smem_bytes: the largest SingleFastSmem of the work list's instances.
  k_single_fast<<<tiles, kMultipleFastThreads, (size_t)smem_bytes, st>>>(insts, wl);
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

ATMO_CHECK_WORD_ACCESSOR(CheckWordFast)

}  // namespace atmo
