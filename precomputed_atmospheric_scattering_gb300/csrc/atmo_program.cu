// atmo_program.cu -- device storage and launch programs (see atmo_program.h).
#include "atmo_program.h"

#include <nvtx3/nvToolsExt.h>

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <tuple>

#include "atmo_kernels.h"
#include "atmo_tables.cuh"

namespace atmo {

namespace {
thread_local std::string g_last_error = "no error";

// Tuned block shapes by LUT sizes, for this process.
using SizeKey = std::tuple<int, int, int, int, int, int, int, int>;
std::mutex g_tuning_mutex;
std::map<SizeKey, std::array<int, 4>> g_tuning;

SizeKey KeyOf(const atmo_lut_shape& s) {
  return SizeKey(s.transmittance_width, s.transmittance_height, s.scattering_r,
                 s.scattering_mu, s.scattering_mu_s, s.scattering_nu, s.irradiance_width,
                 s.irradiance_height);
}
}  // namespace

void ApplyTuning(const atmo_lut_shape& sizes, Shape* s) {
  std::lock_guard<std::mutex> lk(g_tuning_mutex);
  auto it = g_tuning.find(KeyOf(sizes));
  if (it == g_tuning.end()) return;
  for (int i = 0; i < 4; ++i) s->tune[i] = it->second[i];
}

void SetTuning(const atmo_lut_shape& sizes, const int* tune) {
  std::lock_guard<std::mutex> lk(g_tuning_mutex);
  if (!tune) {
    g_tuning.erase(KeyOf(sizes));
    return;
  }
  g_tuning[KeyOf(sizes)] = {tune[0], tune[1], tune[2], tune[3]};
}

void SetError(const std::string& msg) { g_last_error = msg; }
const char* LastError() { return g_last_error.c_str(); }

atmo_status CudaFail(cudaError_t e, const char* what) {
  SetError(std::string(what) + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")");
  return e == cudaErrorMemoryAllocation ? ATMO_OOM : ATMO_CUDA_ERROR;
}

// ---------------------------------------------------------------------------
// Storage
// ---------------------------------------------------------------------------
// Whether the multiple-scattering blocks take the rows of an instance of
// this shape in the order of RowOrder: only where its delta density is a large
// part of the L2 (the high-resolution shape: 268 MB).  At the reference's
// shape (16 MB) the rows in flight already share the L2 and the reordered rows
// ran 0.2% slower; at the high-resolution shape the launch's DRAM reads fell
// from 3.8 GB to 0.54 GB and its time by 5%.
static bool UsesRowOrder(const Shape& s) {
  return double(s.s_texels()) * 16.0 >= 48.0 * (1 << 20);
}

atmo_status Storage::Allocate(const Shape& shape, bool combined_textures, bool half_precision) {
  Free();
  s = shape;
  combined = combined_textures;
  half = half_precision;
  const size_t nT = (size_t)s.t_texels(), nI = (size_t)s.i_texels(),
               nS = (size_t)s.s_texels();
  auto alloc = [&](void** p, size_t bytes) -> atmo_status {
    cudaError_t e = cudaMalloc(p, bytes);
    if (e != cudaSuccess) {
      *p = nullptr;
      Free();
      return CudaFail(e, "cudaMalloc");
    }
    owned.push_back(*p);
    return ATMO_OK;
  };
  atmo_status st;
#define ATMO_ALLOC(ptr, bytes)                                   \
  if ((st = alloc(reinterpret_cast<void**>(&(ptr)), (bytes))) != ATMO_OK) return st;
  ATMO_ALLOC(T, nT * sizeof(float4));
  ATMO_ALLOC(Tau, nT * sizeof(float4));
  ATMO_ALLOC(I, nI * sizeof(float4));
  ATMO_ALLOC(dI, nI * sizeof(float4));
  ATMO_ALLOC(dI2, nI * sizeof(float4));
  ATMO_ALLOC(dR, nS * sizeof(float4));
  ATMO_ALLOC(dM, nS * sizeof(float4));
  ATMO_ALLOC(dJ, nS * sizeof(float4));
  ATMO_ALLOC(S, nS * sizeof(float4));
  if (!combined) ATMO_ALLOC(M, nS * sizeof(float4));
  if (half) {
    ATMO_ALLOC(S_half, nS * 8);
    if (!combined) ATMO_ALLOC(M_half, nS * 8);
  }
  ATMO_ALLOC(tab.rows, (size_t)s.sr * s.smu * sizeof(TexelRow));
  ATMO_ALLOC(tab.cols, (size_t)s.smus * sizeof(TexelCol));
  ATMO_ALLOC(tab.drows, (size_t)s.sr * kDensityThetaSamples * sizeof(DensityRow));
  ATMO_ALLOC(tab.irows, (size_t)s.ih * sizeof(IrrRow));
  ATMO_ALLOC(tab.mus_i, (size_t)s.iw * sizeof(float));
  if (UsesRowOrder(s)) ATMO_ALLOC(tab.row_order, (size_t)s.sr * s.smu * sizeof(int));
#undef ATMO_ALLOC
  return ATMO_OK;
}

void Storage::Free() {
  for (void* p : owned) cudaFree(p);
  owned.clear();
  T = Tau = I = dI = dI2 = dR = dM = dJ = S = M = nullptr;
  S_half = M_half = nullptr;
  tab = Tables{};
}

size_t Storage::Bytes() const {
  const size_t nT = (size_t)s.t_texels(), nI = (size_t)s.i_texels(),
               nS = (size_t)s.s_texels();
  size_t b = (2 * nT + 3 * nI) * 16 + nS * 16 * (4 + (combined ? 0 : 1));
  if (half) b += nS * 8 * (combined ? 1 : 2);
  b += (size_t)s.sr * s.smu * sizeof(TexelRow) + s.smus * sizeof(TexelCol) +
       (size_t)s.sr * kDensityThetaSamples * sizeof(DensityRow) + s.ih * sizeof(IrrRow) +
       s.iw * sizeof(float) + (UsesRowOrder(s) ? (size_t)s.sr * s.smu * sizeof(int) : 0);
  return b;
}

// The rows of the scattering LUT sorted by the invariant of their rays,
// delta = rho^2 - (r mu)^2 (the squared impact parameter less Rb^2), ground
// rays first: the samples of a ray stay on its delta, so rows taken together
// in this order read the same delta-density rows.  From the texel-centre
// mapping of r and mu (functions.glsl:837-870) in FP64 at the given radii.
std::vector<int> RowOrder(const Shape& s, double Rb, double Rt) {
  const int rows = s.sr * s.smu, n = s.smu / 2;
  const double H = std::sqrt(std::max(Rt * Rt - Rb * Rb, 0.0));
  std::vector<double> delta(rows);
  std::vector<int> ground(rows), order(rows);
  for (int k = 0; k < s.sr; ++k) {
    const double rho = H * k / double(s.sr > 1 ? s.sr - 1 : 1);
    const double r = std::sqrt(rho * rho + Rb * Rb);
    for (int j = 0; j < s.smu; ++j) {
      const bool g = j < n;
      double d_min, d_max, x;
      if (g) {
        d_min = r - Rb;
        d_max = rho;
        x = double(n - 1 - j) / double(n - 1);
      } else {
        d_min = Rt - r;
        d_max = rho + H;
        x = double(j - n) / double(n - 1);
      }
      const double d = d_min + (d_max - d_min) * x;
      double mu = g ? -1.0 : 1.0;
      if (d > 0.0) mu = g ? -(rho * rho + d * d) / (2.0 * r * d) : (H * H - rho * rho - d * d) /
                                                                        (2.0 * r * d);
      mu = std::min(std::max(mu, -1.0), 1.0);
      const int i = k * s.smu + j;
      delta[i] = rho * rho - (r * mu) * (r * mu);
      ground[i] = g ? 0 : 1;
      order[i] = i;
    }
  }
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
    return ground[a] != ground[b] ? ground[a] < ground[b] : delta[a] < delta[b];
  });
  return order;
}

// ---------------------------------------------------------------------------
// Program
// ---------------------------------------------------------------------------
atmo_path PassPath(Pass pass, const Shape& s, atmo_path path) {
  if (path != ATMO_PATH_FAST) return path;
  if (pass == Pass::kMultiple && !MultipleFastFits(s)) return ATMO_PATH_PLAIN;
  if (pass == Pass::kSingle && !SingleFastFits(s)) return ATMO_PATH_PLAIN;
  if (pass == Pass::kDensity && !DensityFastFits(s)) return ATMO_PATH_PLAIN;
  return path;
}

int SharedBytes(Pass pass, const Shape& s, const Consts& c, int order, atmo_path path) {
  if (path != ATMO_PATH_FAST) return 0;
  if (pass == Pass::kDensity) return DensityFastSmem(s, c, order);
  if (pass == Pass::kMultiple) return MultipleFastSmem(s);
  if (pass == Pass::kSingle) return SingleFastSmem(s);
  if (pass == Pass::kIndirect) return IndirectSmem(s, order);
  return 0;
}

int Tiles(Pass pass, const Shape& s, atmo_path path) {
  auto cdiv = [](long long a, long long b) { return (int)((a + b - 1) / b); };
  switch (pass) {
    case Pass::kTables: return TableTiles(s);
    case Pass::kTransmittance: return cdiv(s.t_texels(), kTransmittanceTexelsPerTile);
    case Pass::kDirect: return cdiv(s.i_texels() + s.sr * kDensityThetaSamples, kTexelThreads);
    case Pass::kSingle:
      return path == ATMO_PATH_FAST ? SingleFastTiles(s) : cdiv(s.s_texels(), kTexelThreads);
    case Pass::kDensity:
      return path == ATMO_PATH_FAST ? DensityFastTiles(s) : cdiv(s.s_texels(), kTexelThreads);
    case Pass::kIndirect: return cdiv(s.i_texels(), kIndirectTexelsPerTile);
    case Pass::kMultiple:
      return path == ATMO_PATH_FAST ? MultipleFastTiles(s) : cdiv(s.s_texels(), kTexelThreads);
    case Pass::kToHalf: return cdiv(s.s_texels(), 256);
  }
  return 0;
}

Program::~Program() {
  if (graph_) cudaGraphExecDestroy(graph_);
  if (capture_stream_) cudaStreamDestroy(capture_stream_);
  if (side_stream_) cudaStreamDestroy(side_stream_);
  if (ev_fork_) cudaEventDestroy(ev_fork_);
  if (ev_join_) cudaEventDestroy(ev_join_);
  if (upload_done_) cudaEventDestroy(upload_done_);
  if (d_slots_) cudaFree(d_slots_);
  if (h_slots_pinned_) cudaFreeHost(h_slots_pinned_);
  if (d_blob_) cudaFree(d_blob_);
}

int Program::AddWorkList(const std::vector<int>& members, Pass pass, int order, int* tiles,
                         int* smem, atmo_path* step_path) {
  std::vector<int> inst, start;
  auto takes_part = [&](int m) {
    if ((pass == Pass::kDensity || pass == Pass::kMultiple) && orders[m] < (unsigned)order)
      return false;
    if (pass == Pass::kIndirect && orders[m] < (unsigned)order + 1) return false;
    return true;
  };
  // One kernel variant per launch: the fast one only if every member takes it.
  atmo_path p = path;
  for (int m : members)
    if (takes_part(m) && PassPath(pass, slots[m].s, path) != path) p = ATMO_PATH_PLAIN;
  if (step_path) *step_path = p;
  int t = 0;
  if (smem) *smem = 0;
  for (int m : members) {
    if (!takes_part(m)) continue;
    inst.push_back(m);
    start.push_back(t);
    t += Tiles(pass, slots[m].s, p);
    if (smem) {
      int b = SharedBytes(pass, slots[m].s, slots[m].c, order, p);
      *smem = b > *smem ? b : *smem;
    }
  }
  *tiles = t;
  if (inst.empty()) return -1;
  start.push_back(t);
  int offset = (int)blob_.size();
  blob_.insert(blob_.end(), inst.begin(), inst.end());
  blob_.insert(blob_.end(), start.begin(), start.end());
  wl_offsets_.push_back({offset, (int)inst.size()});
  return (int)wl_offsets_.size() - 1;
}

void Program::AddStage(const std::vector<int>& members, bool transmittance_only) {
  auto add = [&](Pass p, int order) {
    int tiles = 0, smem = 0;
    atmo_path step_path = path;
    int wl = AddWorkList(members, p, order, &tiles, &smem, &step_path);
    if (wl >= 0 && tiles > 0) steps_.push_back(Step{p, order, wl, tiles, smem, step_path});
  };
  if (transmittance_only) {
    add(Pass::kTransmittance, 0);
    return;
  }
  unsigned max_order = 1;
  for (int m : members) max_order = orders[m] > max_order ? orders[m] : max_order;
  add(Pass::kTables, 0);
  add(Pass::kTransmittance, 0);
  add(Pass::kDirect, 0);
  add(Pass::kSingle, 0);
  for (unsigned order = 2; order <= max_order; ++order) {
    add(Pass::kDensity, (int)order);
    add(Pass::kIndirect, (int)order - 1);
    add(Pass::kMultiple, (int)order);
  }
}

void Program::AddToHalf(const std::vector<int>& members) {
  for (int m : members) {
    int tiles = 0;
    int wl = AddWorkList({m}, Pass::kToHalf, 0, &tiles);
    if (wl >= 0) steps_.push_back(Step{Pass::kToHalf, 0, wl, tiles, 0, path});
  }
}

atmo_status Program::Finalize() {
  if (finalized_) return ATMO_OK;
  if (!blob_.empty()) {
    ATMO_CUDA_TRY(cudaMalloc(&d_blob_, blob_.size() * sizeof(int)));
    ATMO_CUDA_TRY(cudaMemcpy(d_blob_, blob_.data(), blob_.size() * sizeof(int),
                             cudaMemcpyHostToDevice));
  }
  wls_.clear();
  for (auto& o : wl_offsets_) {
    WorkList w;
    w.inst = d_blob_ + o.first;
    w.start = d_blob_ + o.first + o.second;
    w.count = o.second;
    wls_.push_back(w);
  }
  ATMO_CUDA_TRY(cudaMalloc(&d_slots_, slots.size() * sizeof(Instance)));
  ATMO_CUDA_TRY(cudaMallocHost(&h_slots_pinned_, slots.size() * sizeof(Instance)));
  // Row orders of the instances that have the table (slots of one model share
  // it; the radii of a later set_atmosphere leave the order stale, which
  // changes nothing in the LUTs).
  fork_indirect_ = !slots.empty();
  for (const Instance& in : slots)
    if (!in.dI2 || in.dI2 == in.dI) fork_indirect_ = false;
  std::vector<int*> done;
  for (const Instance& in : slots) {
    if (!in.tab.row_order ||
        std::find(done.begin(), done.end(), in.tab.row_order) != done.end())
      continue;
    const std::vector<int> order = RowOrder(in.s, in.c.dRb, in.c.dRt);
    ATMO_CUDA_TRY(cudaMemcpy(in.tab.row_order, order.data(),
                             order.size() * sizeof(int), cudaMemcpyHostToDevice));
    done.push_back(in.tab.row_order);
  }
  finalized_ = true;
  return ATMO_OK;
}

atmo_status Program::Upload(cudaStream_t st) {
  if (!upload_done_) {
    ATMO_CUDA_TRY(cudaEventCreateWithFlags(&upload_done_, cudaEventDisableTiming));
  } else {
    // The previous run's copy may still be reading the staging buffer.
    ATMO_CUDA_TRY(cudaEventSynchronize(upload_done_));
  }
  std::memcpy(h_slots_pinned_, slots.data(), slots.size() * sizeof(Instance));
  ATMO_CUDA_TRY(cudaMemcpyAsync(d_slots_, h_slots_pinned_, slots.size() * sizeof(Instance),
                                cudaMemcpyHostToDevice, st));
  ATMO_CUDA_TRY(cudaEventRecord(upload_done_, st));
  return ATMO_OK;
}

atmo_status Program::PrepareFork() {
  if (!fork_indirect_ || side_stream_) return ATMO_OK;
  ATMO_CUDA_TRY(cudaStreamCreateWithFlags(&side_stream_, cudaStreamNonBlocking));
  ATMO_CUDA_TRY(cudaEventCreateWithFlags(&ev_fork_, cudaEventDisableTiming));
  ATMO_CUDA_TRY(cudaEventCreateWithFlags(&ev_join_, cudaEventDisableTiming));
  return ATMO_OK;
}

atmo_status Program::Launch(cudaStream_t st) {
  for (size_t i = 0; i < steps_.size(); ++i) {
    // The indirect irradiance of order n - 1 runs beside the density pass of
    // order n: they write and read different delta-irradiance buffers and
    // both only read the previous order's scattering, which the multiple
    // scattering of order n overwrites after joining both.  The indirect
    // pass's small grid then fills the density launch's gaps.
    if (fork_indirect_ && steps_[i].pass == Pass::kDensity && i + 1 < steps_.size() &&
        steps_[i + 1].pass == Pass::kIndirect && steps_[i + 1].order == steps_[i].order - 1) {
      atmo_status s = PrepareFork();
      if (s != ATMO_OK) return s;
      ATMO_CUDA_TRY(cudaEventRecord(ev_fork_, st));
      ATMO_CUDA_TRY(cudaStreamWaitEvent(side_stream_, ev_fork_, 0));
      if ((s = LaunchStep(i + 1, side_stream_)) != ATMO_OK) return s;
      ATMO_CUDA_TRY(cudaEventRecord(ev_join_, side_stream_));
      if ((s = LaunchStep(i, st)) != ATMO_OK) return s;
      ATMO_CUDA_TRY(cudaStreamWaitEvent(st, ev_join_, 0));
      ++i;
      continue;
    }
    atmo_status s = LaunchStep(i, st);
    if (s != ATMO_OK) return s;
  }
  return ATMO_OK;
}

atmo_status Program::TimeSteps(cudaStream_t st, std::vector<float>* ms) {
  atmo_status s = Finalize();
  if (s != ATMO_OK) return s;
  if ((s = Upload(st)) != ATMO_OK) return s;
  std::vector<cudaEvent_t> ev(steps_.size() + 1);
  for (auto& e : ev) ATMO_CUDA_TRY(cudaEventCreate(&e));
  ATMO_CUDA_TRY(cudaEventRecord(ev[0], st));
  for (size_t i = 0; i < steps_.size(); ++i) {
    if ((s = LaunchStep(i, st)) != ATMO_OK) break;
    ATMO_CUDA_TRY(cudaEventRecord(ev[i + 1], st));
  }
  cudaError_t e = cudaEventSynchronize(ev.back());
  ms->assign(steps_.size(), 0.0f);
  for (size_t i = 0; s == ATMO_OK && e == cudaSuccess && i < steps_.size(); ++i)
    cudaEventElapsedTime(&(*ms)[i], ev[i], ev[i + 1]);
  for (auto& x : ev) cudaEventDestroy(x);
  if (s != ATMO_OK) return s;
  if (e != cudaSuccess) return CudaFail(e, "cudaEventSynchronize");
  return ATMO_OK;
}

cudaError_t LaunchPass(Pass pass, int order, int smem, const Instance* insts, WorkList wl,
                       int tiles, atmo_path path, cudaStream_t st) {
  switch (pass) {
    case Pass::kTables: return LaunchTables(insts, wl, tiles, st);
    case Pass::kTransmittance: return LaunchTransmittance(insts, wl, tiles, st);
    case Pass::kDirect: return LaunchDirectIrradiance(insts, wl, tiles, st);
    case Pass::kSingle:
      return path == ATMO_PATH_FAST ? LaunchSingleFast(insts, wl, tiles, smem, st)
                                    : LaunchSingleScattering(insts, wl, tiles, st);
    case Pass::kDensity:
      return path == ATMO_PATH_FAST ? LaunchDensityFast(insts, wl, tiles, order, smem, st)
                                    : LaunchDensityPlain(insts, wl, tiles, order, st);
    case Pass::kIndirect:
      return LaunchIndirectIrradiance(insts, wl, tiles, order, smem, st);
    case Pass::kMultiple:
      return path == ATMO_PATH_FAST ? LaunchMultipleFast(insts, wl, tiles, smem, st)
                                    : LaunchMultiplePlain(insts, wl, tiles, st);
    case Pass::kToHalf: return cudaErrorInvalidValue;   // handled by the program
  }
  return cudaErrorInvalidValue;
}

// The names of the NVTX ranges around the launches, "atmo:<pass>:<order>":
// a profiler selects one pass's launches with them (ncu --nvtx
// --nvtx-include "atmo:scattering_density:2/").  Ranges cost a pointer test
// when no tool is attached, and are recorded once when a graph is captured.
static const char* PassName(Pass p) {
  switch (p) {
    case Pass::kTables: return "tables";
    case Pass::kTransmittance: return "transmittance";
    case Pass::kDirect: return "direct_irradiance";
    case Pass::kSingle: return "single_scattering";
    case Pass::kDensity: return "scattering_density";
    case Pass::kIndirect: return "indirect_irradiance";
    case Pass::kMultiple: return "multiple_scattering";
    case Pass::kToHalf: return "to_half";
  }
  return "pass";
}

atmo_status Program::LaunchStep(size_t i, cudaStream_t st) {
  const Step& step = steps_[i];
  const WorkList& wl = wls_[step.wl];
  char label[48];
  std::snprintf(label, sizeof label, "atmo:%s:%d", PassName(step.pass), step.order);
  nvtxRangePushA(label);
  struct Pop {
    ~Pop() { nvtxRangePop(); }
  } pop;
  cudaError_t e = cudaSuccess;
  if (step.pass == Pass::kToHalf) {
    // One slot per step: convert its scattering (and single-Mie) outputs.
    int m = blob_[wl_offsets_[step.wl].first];
    const Instance& in = slots[m];
    if (in.S_half) e = LaunchToHalf(in.S, in.S_half, in.s.s_texels(), st);
    if (e == cudaSuccess && in.M && in.M_half)
      e = LaunchToHalf(in.M, in.M_half, in.s.s_texels(), st);
  } else {
    e = LaunchPass(step.pass, step.order, step.smem, d_slots_, wl, step.tiles, step.path, st);
  }
  if (e != cudaSuccess) return CudaFail(e, "kernel launch");
  return ATMO_OK;
}

atmo_status Program::Run(cudaStream_t st, bool use_graph) {
  atmo_status s = Finalize();
  if (s != ATMO_OK) return s;
  if ((s = Upload(st)) != ATMO_OK) return s;
  if (!use_graph) return Launch(st);
  if (!graph_) {
    if (!capture_stream_) {
      ATMO_CUDA_TRY(cudaStreamCreateWithFlags(&capture_stream_, cudaStreamNonBlocking));
    }
    cudaGraph_t g = nullptr;
    // Kernel attributes, the side stream and its events are set up before
    // the capture, not inside it.
    ATMO_CUDA_TRY(PrepareDensityFast());
    if ((s = PrepareFork()) != ATMO_OK) return s;
    ATMO_CUDA_TRY(cudaStreamBeginCapture(capture_stream_, cudaStreamCaptureModeThreadLocal));
    atmo_status ls = Launch(capture_stream_);
    cudaError_t ce = cudaStreamEndCapture(capture_stream_, &g);
    if (ls != ATMO_OK) {
      if (g) cudaGraphDestroy(g);
      return ls;
    }
    if (ce != cudaSuccess) return CudaFail(ce, "cudaStreamEndCapture");
    ce = cudaGraphInstantiate(&graph_, g, 0);
    cudaGraphDestroy(g);
    if (ce != cudaSuccess) {
      graph_ = nullptr;
      return CudaFail(ce, "cudaGraphInstantiate");
    }
  }
  ATMO_CUDA_TRY(cudaGraphLaunch(graph_, st));
  return ATMO_OK;
}

}  // namespace atmo
