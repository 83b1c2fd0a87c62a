// atmo_noalloc.cu -- atmo_precompute_noalloc: the one-group precomputation of
// atmo_precompute for callers that must not allocate device memory.
//
// Who needs it: code that runs inside a host application which owns and
// pre-reserves all device memory -- an engine plugin handed only its output
// textures, or a framework whose caching allocator holds the memory pool, so
// that a cudaMalloc behind its back fails or fragments the pool -- and code
// that must not pay cudaMalloc's implicit device synchronisation in a
// latency-bound loop.  atmo_precompute allocates its temporaries (the delta
// LUTs, the optical-depth LUT, the set-up tables, the launch descriptors)
// with cudaMallocAsync; this variant places them in a file-scope device
// array instead and calls no allocating routine.
//
// The array is a fixed kNoAllocScratchBytes (64 MiB) in every GPU that loads
// this library, held until the process exits.  It fits the reference's
// default LUT shape (256x64 / 8x32x128x32 / 64x16 needs ~49 MiB); larger
// shapes are rejected with ATMO_BUDGET.  All calls share it: calls whose GPU
// work overlaps (concurrent streams, or several host threads) race and must
// be serialised by the caller.  Nothing needs clearing between calls: every
// temporary is written in full by an earlier pass of the same call before any
// pass reads it.
//
// The array's memory is taken when this file's device code is loaded: with
// CUDA's default lazy module loading, by the first call on each device (the
// one that looks up the array's address), or at context creation with
// CUDA_MODULE_LOADING=EAGER.  A host application that reserves all device
// memory up front should make one call (or load eagerly) before reserving.
//
// Host code cannot use the array's symbol as a device address (it names a
// host-side stand-in); the device address comes from cudaGetSymbolAddress,
// looked up on the first call made in each CUDA context (a context that is
// destroyed and re-created, e.g. by cudaDeviceReset, gets a fresh lookup), so
// that first call should come before any stream capture.  The launch
// descriptors (the instance record and the per-pass work lists) reach the
// scratch array as by-value kernel parameters of a set-up kernel: a call
// copies nothing from host memory and does not wait for earlier work in the
// stream.
#include <cuda.h>
#include <cuda_runtime.h>

#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/atmo/atmo.h"
#include "atmo_consts.h"
#include "atmo_kernels.h"
#include "atmo_program.h"

namespace atmo {

constexpr size_t kNoAllocScratchBytes = size_t(64) << 20;
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

namespace {

constexpr int kMaxDevices = 64;
constexpr int kMaxOrders = 64;
constexpr int kMaxSteps = 4 + 3 * (kMaxOrders - 1);

// The launch descriptors of one call, passed by value to the set-up kernel.
struct NoAllocDescriptors {
  Instance in;
  int steps;
  int tiles[kMaxSteps];
};

// Writes the instance record and the work lists {inst = 0; start = 0,
// tiles} of every step into the scratch array.
__global__ void k_noalloc_setup(const NoAllocDescriptors d, Instance* in_dst, int* wl_dst) {
  const int* src = reinterpret_cast<const int*>(&d.in);
  int* dst = reinterpret_cast<int*>(in_dst);
  constexpr int kWords = (int)(sizeof(Instance) / sizeof(int));
  for (int i = threadIdx.x; i < kWords; i += blockDim.x) dst[i] = src[i];
  for (int i = threadIdx.x; i < d.steps; i += blockDim.x) {
    wl_dst[3 * i] = 0;
    wl_dst[3 * i + 1] = 0;
    wl_dst[3 * i + 2] = d.tiles[i];
  }
}
static_assert(sizeof(Instance) % sizeof(int) == 0, "the set-up kernel copies whole words");
static_assert(sizeof(NoAllocDescriptors) <= 4000, "the descriptors must fit a kernel's parameters");

// Per device: the CUDA context (its process-unique id) in which the scratch
// array's address was looked up, and that address.
struct ScratchAddress {
  unsigned long long ctx_id = 0;
  void* ptr = nullptr;
};
std::mutex g_noalloc_mutex;
ScratchAddress g_noalloc_addr[kMaxDevices];

using CtxGetCurrentFn = CUresult (*)(CUcontext*);
using CtxGetIdFn = CUresult (*)(CUcontext, unsigned long long*);

// The process-unique id of the calling thread's current context, or 0 when
// none is current (the driver entry points come through the runtime, so the
// library does not link libcuda).
unsigned long long CurrentContextId() {
  static CtxGetCurrentFn get_current = nullptr;
  static CtxGetIdFn get_id = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &fn, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_current = reinterpret_cast<CtxGetCurrentFn>(fn);
    fn = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &fn, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_id = reinterpret_cast<CtxGetIdFn>(fn);
  });
  if (!get_current || !get_id) return 0;
  CUcontext ctx = nullptr;
  unsigned long long id = 0;
  if (get_current(&ctx) != CUDA_SUCCESS || !ctx) return 0;
  if (get_id(ctx, &id) != CUDA_SUCCESS) return 0;
  return id;
}

// The scratch array's device address in the current context of device
// `dev`: looked up on the first call in each context.
atmo_status ScratchBase(int dev, unsigned char** base) {
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  ScratchAddress& a = g_noalloc_addr[dev];
  const unsigned long long ctx = CurrentContextId();
  if (a.ptr && ctx != 0 && ctx == a.ctx_id) {
    *base = static_cast<unsigned char*>(a.ptr);
    return ATMO_OK;
  }
  void* p = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
  if (e == cudaErrorMemoryAllocation) {
    cudaGetLastError();
    SetError("atmo_precompute_noalloc: loading its 64 MiB scratch array failed for lack of "
             "device memory; make one call (or set CUDA_MODULE_LOADING=EAGER) before "
             "reserving the device's memory");
    return ATMO_OOM;
  }
  if (e != cudaSuccess) return CudaFail(e, "cudaGetSymbolAddress(no-alloc scratch)");
  a.ptr = p;
  a.ctx_id = CurrentContextId();   // the lookup made the context current if none was
  *base = static_cast<unsigned char*>(p);
  return ATMO_OK;
}

size_t Align256(size_t x) { return (x + 255) & ~size_t(255); }

// The scratch layout of one call; offsets in bytes.
struct NoAllocLayout {
  size_t instance, worklists, dI, dR, dM, dJ, rows, cols, drows, irows, mus_i, tau, total;
};

NoAllocLayout Layout(const Shape& s, size_t worklist_ints) {
  NoAllocLayout L;
  size_t o = 0;
  auto take = [&](size_t bytes) {
    size_t at = o;
    o = Align256(o + bytes);
    return at;
  };
  const size_t nI = (size_t)s.i_texels(), nS = (size_t)s.s_texels(), nT = (size_t)s.t_texels();
  L.instance = take(sizeof(Instance));
  L.worklists = take(worklist_ints * sizeof(int));
  L.dI = take(nI * 16);
  L.dR = take(nS * 16);
  L.dM = take(nS * 16);
  L.dJ = take(nS * 16);
  L.rows = take((size_t)s.sr * s.smu * sizeof(TexelRow));
  L.cols = take((size_t)s.smus * sizeof(TexelCol));
  L.drows = take((size_t)s.sr * kDensityThetaSamples * sizeof(DensityRow));
  L.irows = take((size_t)s.ih * sizeof(IrrRow));
  L.mus_i = take((size_t)s.iw * sizeof(float));
  L.tau = take(nT * 16);
  L.total = o;
  return L;
}

}  // namespace
}  // namespace atmo

using namespace atmo;

extern "C" atmo_status atmo_precompute_noalloc(const atmo_atmosphere* atmosphere,
                                               const atmo_lut_shape* shape,
                                               unsigned num_scattering_orders,
                                               const float lum[9], int blend, int combined,
                                               float* transmittance, float* scattering,
                                               float* single_mie, float* irradiance,
                                               atmo_stream stream) {
  if (!atmosphere || !transmittance || !scattering || !irradiance) {
    SetError("NULL argument");
    return ATMO_INVALID_ARG;
  }
  if (!combined && !single_mie) {
    SetError("single_mie is required when combined == 0");
    return ATMO_INVALID_ARG;
  }
  if (num_scattering_orders < 1 || num_scattering_orders > (unsigned)kMaxOrders) {
    SetError("num_scattering_orders must be in [1, 64]");
    return ATMO_INVALID_ARG;
  }
  atmo_lut_shape ls = shape ? *shape : DefaultShape();
  std::string why;
  if (!ValidShape(ls, &why) || !ValidAtmosphere(*atmosphere, &why)) {
    SetError(why);
    return ATMO_INVALID_ARG;
  }
  const Shape s = ToShape(ls);
  const Consts consts = MakeConsts(*atmosphere, lum);

  // The pass sequence of atmosphere/model.cc:1048-1215 for one instance:
  // each step's work list is {inst = 0; start = 0, tiles}.
  struct PlannedStep {
    Pass pass;
    int order, tiles, smem;
    atmo_path path;
  };
  std::vector<PlannedStep> steps;
  auto add = [&](Pass p, int order) {
    const atmo_path path = PassPath(p, s, ATMO_PATH_FAST);
    steps.push_back(
        PlannedStep{p, order, Tiles(p, s, path), SharedBytes(p, s, consts, order, path), path});
  };
  add(Pass::kTables, 0);
  add(Pass::kTransmittance, 0);
  add(Pass::kDirect, 0);
  add(Pass::kSingle, 0);
  for (unsigned order = 2; order <= num_scattering_orders; ++order) {
    add(Pass::kDensity, (int)order);
    add(Pass::kIndirect, (int)order - 1);
    add(Pass::kMultiple, (int)order);
  }
  const NoAllocLayout L = Layout(s, 3 * steps.size());
  if (L.total > kNoAllocScratchBytes) {
    SetError("atmo_precompute_noalloc: this LUT shape needs " + std::to_string(L.total) +
             " bytes of temporaries, more than the fixed " +
             std::to_string(kNoAllocScratchBytes) + "-byte scratch array");
    return ATMO_BUDGET;
  }

  int dev = 0;
  ATMO_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) {
    SetError("device ordinal out of range");
    return ATMO_INVALID_ARG;
  }
  unsigned char* base = nullptr;
  const atmo_status found = ScratchBase(dev, &base);
  if (found != ATMO_OK) return found;

  NoAllocDescriptors d;
  std::memset(&d, 0, sizeof(d));
  Instance& in = d.in;
  in.c = consts;
  in.s = s;
  in.T = reinterpret_cast<float4*>(transmittance);
  in.S = reinterpret_cast<float4*>(scattering);
  in.M = combined ? nullptr : reinterpret_cast<float4*>(single_mie);
  in.I = reinterpret_cast<float4*>(irradiance);
  in.combined = combined ? 1 : 0;
  in.blend = blend ? 1 : 0;
  in.dI = reinterpret_cast<float4*>(base + L.dI);
  in.dR = reinterpret_cast<float4*>(base + L.dR);
  in.dM = reinterpret_cast<float4*>(base + L.dM);
  in.dJ = reinterpret_cast<float4*>(base + L.dJ);
  in.Tau = reinterpret_cast<float4*>(base + L.tau);
  in.tab.rows = reinterpret_cast<TexelRow*>(base + L.rows);
  in.tab.cols = reinterpret_cast<TexelCol*>(base + L.cols);
  in.tab.drows = reinterpret_cast<DensityRow*>(base + L.drows);
  in.tab.irows = reinterpret_cast<IrrRow*>(base + L.irows);
  in.tab.mus_i = reinterpret_cast<float*>(base + L.mus_i);
  d.steps = (int)steps.size();
  for (size_t i = 0; i < steps.size(); ++i) d.tiles[i] = steps[i].tiles;

  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  Instance* d_in = reinterpret_cast<Instance*>(base + L.instance);
  int* d_wl = reinterpret_cast<int*>(base + L.worklists);
  k_noalloc_setup<<<1, 256, 0, st>>>(d, d_in, d_wl);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return CudaFail(e, "no-alloc set-up launch");
  for (size_t i = 0; i < steps.size(); ++i) {
    WorkList wl;
    wl.inst = d_wl + 3 * i;
    wl.start = d_wl + 3 * i + 1;
    wl.count = 1;
    e = LaunchPass(steps[i].pass, steps[i].order, steps[i].smem, d_in, wl, steps[i].tiles,
                   steps[i].path, st);
    if (e != cudaSuccess) return CudaFail(e, "kernel launch");
  }
  return ATMO_OK;
}
