// atmo_server.cu -- the serving engine: LUT sets resident on the device under
// an HBM budget with least-recently-used eviction, rebuild requests batched
// continuously at pass granularity, and shading requests overlapping them on
// their own streams.
//
// Continuous batching.  A rebuild is the pass sequence of
// atmosphere/model.cc:1048-1215 (tables, transmittance, direct irradiance,
// single scattering, then density / indirect irradiance / multiple
// scattering per order).  A worker thread runs rounds: each round launches,
// for every admitted instance, its next pass; instances at the same (pass,
// order, kernel variant) share one launch through a work list, whatever their
// LUT shapes and order counts.  A request that arrives while rounds are in
// flight is admitted at the next round, as soon as its memory fits the
// budget, and starts its passes beside instances that are further along.
// Each instance's arithmetic is the same in every grouping (the kernels
// assign tiles per instance), so a result does not depend on the mix.
//
// Memory.  A LUT set holds T, its optical depth, S, (single Mie) and I for as
// long as it is resident; the temporaries (delta LUTs, set-up tables) exist
// only while it is being built.  Both come from a private stream-ordered
// pool.  Admission charges the final and the scratch bytes against the
// budget; when they do not fit, idle ready sets (no shading pending) are
// evicted in least-recently-used order.
//
// Completion.  A host function enqueued behind an instance's last pass (or a
// shading kernel) stamps its ticket; latencies are measured on the host
// clock from submission to that stamp.  Every wait of the API is bounded.
// Each round (and each shading launch) is bracketed by timing events, so a
// ticket also reports the GPU time of the launches it took part in.
//
// Cancellation.  A queued request is dropped; a rebuild being built stops
// after the passes already enqueued: its memory goes back to the pool behind
// them (stream-ordered frees) and its instance row once the GPU has passed
// them.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <list>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <unordered_set>
#include <vector>

#include "../../include/atmo/atmo.h"
#include "atmo_consts.h"
#include "atmo_kernels.h"
#include "atmo_program.h"
#include "atmo_render.h"

namespace atmo {
namespace {

using Clock = std::chrono::steady_clock;

double MsSince(Clock::time_point t0, Clock::time_point t1) {
  return std::chrono::duration<double, std::milli>(t1 - t0).count();
}

size_t Align(size_t x) { return (x + 255) & ~size_t(255); }

// The pass sequence of one instance.
struct PassStep {
  Pass pass;
  int order;
};
std::vector<PassStep> PassSequence(unsigned orders) {
  std::vector<PassStep> seq = {
      {Pass::kTables, 0}, {Pass::kTransmittance, 0}, {Pass::kDirect, 0}, {Pass::kSingle, 0}};
  for (unsigned o = 2; o <= orders; ++o) {
    seq.push_back({Pass::kDensity, (int)o});
    seq.push_back({Pass::kIndirect, (int)o - 1});
    seq.push_back({Pass::kMultiple, (int)o});
  }
  return seq;
}

// Final and scratch bytes of one LUT set.
size_t FinalBytes(const Shape& s, bool combined) {
  const size_t nT = s.t_texels(), nI = s.i_texels(), nS = (size_t)s.s_texels();
  return Align(nT * 16) * 2 + Align(nI * 16) + Align(nS * 16) * (combined ? 1 : 2);
}
size_t ScratchBytes(const Shape& s) {
  const size_t nI = s.i_texels(), nS = (size_t)s.s_texels();
  return Align(nI * 16) + Align(nS * 16) * 3 + Align((size_t)s.sr * s.smu * sizeof(TexelRow)) +
         Align((size_t)s.smus * sizeof(TexelCol)) +
         Align((size_t)s.sr * kDensityThetaSamples * sizeof(DensityRow)) +
         Align((size_t)s.ih * sizeof(IrrRow)) + Align((size_t)s.iw * sizeof(float));
}

struct Ticket {
  enum State { kQueued = 0, kRunning = 1, kDone = 2, kFailed = 3 };
  std::atomic<int> state{kQueued};
  atmo_status status = ATMO_OK;
  Clock::time_point submitted, started, launched, finished;
  bool is_rebuild = false;
  bool has_launched = false;   // its first kernel has been enqueued
  double device_ms = 0.0;      // GPU time of the retired launches it took part in
  unsigned rounds = 0;         // those launches (rounds, or the shading kernel)
  uint64_t set_id = 0;
  std::string message;         // why it failed
};

// A resident (or building) LUT set.
struct LutSlot {
  uint64_t id = 0;                 // the rebuild ticket
  int index = -1;                  // row of the device instance array
  Shape s{};
  unsigned orders = 0;
  std::vector<PassStep> seq;
  size_t next = 0;                 // next pass of seq
  void* final_block = nullptr;
  void* scratch_block = nullptr;
  size_t final_bytes = 0, scratch_bytes = 0;
  bool ready = false;              // built and its last round completed
  int pins = 0;                    // shading requests not yet complete
  uint64_t last_use = 0;           // LRU clock
  atmo_lut_set view;
};

struct RebuildRequest {
  uint64_t ticket;
  atmo_atmosphere atm;
  Shape s;
  unsigned orders;
};

struct ShadeRequest {
  uint64_t ticket;
  uint64_t set_id;
  atmo_pinhole_view view;
  const float* depth;
  float* sky;
  float* shaded;
  int luminance;
};

struct Round {
  cudaEvent_t start = nullptr;         // timing events around the round's launches
  cudaEvent_t done = nullptr;
  std::vector<uint64_t> members;       // rebuild tickets with a pass in this round
  std::vector<uint64_t> finishing;     // sets whose last pass ran in this round
  std::vector<int> release_rows;       // instance rows freed once the round completes
  size_t ring_offset = 0, ring_ints = 0;
};

struct ShadeInFlight {
  cudaEvent_t start = nullptr, done = nullptr;
  uint64_t set_id = 0;
  uint64_t ticket = 0;
};

void StampDone(void* p) {
  Ticket* t = static_cast<Ticket*>(p);
  t->finished = Clock::now();
  t->state.store(Ticket::kDone, std::memory_order_release);
}

}  // namespace
}  // namespace atmo

using namespace atmo;

struct atmo_server {
  atmo_server_config cfg{};
  int device = 0;
  cudaStream_t build_stream = nullptr;
  std::vector<cudaStream_t> shade_streams;
  size_t next_shade_stream = 0;
  cudaMemPool_t pool = nullptr;

  // Device instance array and its pinned host mirror (one row per slot).
  unsigned capacity = 0;
  Instance* d_inst = nullptr;
  Instance* h_inst = nullptr;
  std::vector<int> free_rows;

  // Work-list ring: pinned staging and device copy.
  size_t ring_ints = 0, ring_head = 0;
  int* h_ring = nullptr;
  int* d_ring = nullptr;

  std::mutex mu;                        // guards everything below
  std::condition_variable cv;
  std::unordered_map<uint64_t, std::unique_ptr<Ticket>> tickets;
  std::map<uint64_t, std::unique_ptr<LutSlot>> slots;   // by set id
  std::deque<RebuildRequest> pending_rebuilds;
  std::deque<ShadeRequest> pending_shades;
  std::vector<uint64_t> building;       // admitted, not finished
  std::deque<Round> rounds;             // in flight, in order
  std::deque<ShadeInFlight> shades;     // in flight
  uint64_t next_ticket = 1, lru_clock = 0;
  size_t used_bytes = 0;
  atmo_server_stats stats{};
  bool stop = false;
  std::string worker_error;
  std::thread worker;

  atmo_status Init();
  void Shutdown();
  void WorkerLoop();
  bool Admit(std::unique_lock<std::mutex>& lk);
  bool EvictFor(size_t bytes);
  void FreeSlot(LutSlot* s);
  bool LaunchRound();
  bool RetireRounds();
  bool LaunchShades();
  bool RetireShades();
  atmo_status Cancel(uint64_t id);
  void FailTicket(uint64_t id, atmo_status st, const std::string& why) {
    auto it = tickets.find(id);
    if (it == tickets.end()) return;
    it->second->status = st;
    it->second->message = why;
    it->second->finished = Clock::now();
    it->second->state.store(Ticket::kFailed, std::memory_order_release);
  }
};

atmo_status atmo_server::Init() {
  ATMO_CUDA_TRY(cudaGetDevice(&device));
  // Rebuild rounds get the highest stream priority: their blocks are
  // scheduled ahead of pending shading blocks, so a rebuild's many small
  // rounds are not each queued behind a full-screen shading request.
  int least = 0, greatest = 0;
  ATMO_CUDA_TRY(cudaDeviceGetStreamPriorityRange(&least, &greatest));
  ATMO_CUDA_TRY(cudaStreamCreateWithPriority(&build_stream, cudaStreamNonBlocking, greatest));
  for (unsigned i = 0; i < cfg.shade_streams; ++i) {
    cudaStream_t st;
    ATMO_CUDA_TRY(cudaStreamCreateWithPriority(&st, cudaStreamNonBlocking, least));
    shade_streams.push_back(st);
  }
  cudaMemPoolProps props;
  std::memset(&props, 0, sizeof(props));
  props.allocType = cudaMemAllocationTypePinned;
  props.handleTypes = cudaMemHandleTypeNone;
  props.location.type = cudaMemLocationTypeDevice;
  props.location.id = device;
  props.maxSize = cfg.pool_max_bytes;   // 0: the device's default
  ATMO_CUDA_TRY(cudaMemPoolCreate(&pool, &props));
  uint64_t keep = UINT64_MAX;   // keep freed blocks for reuse
  ATMO_CUDA_TRY(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep));
  capacity = cfg.max_rebuilds_in_flight + 1;
  ATMO_CUDA_TRY(cudaMalloc(&d_inst, sizeof(Instance) * capacity));
  ATMO_CUDA_TRY(cudaMallocHost(&h_inst, sizeof(Instance) * capacity));
  for (int i = (int)capacity - 1; i >= 0; --i) free_rows.push_back(i);
  ring_ints = size_t(1) << 20;
  ATMO_CUDA_TRY(cudaMallocHost(&h_ring, ring_ints * sizeof(int)));
  ATMO_CUDA_TRY(cudaMalloc(&d_ring, ring_ints * sizeof(int)));
  worker = std::thread([this] { WorkerLoop(); });
  return ATMO_OK;
}

void atmo_server::Shutdown() {
  {
    std::lock_guard<std::mutex> lk(mu);
    stop = true;
  }
  cv.notify_all();
  if (worker.joinable()) worker.join();
  cudaSetDevice(device);
  if (build_stream) cudaStreamSynchronize(build_stream);
  for (cudaStream_t st : shade_streams) cudaStreamSynchronize(st);
  for (Round& r : rounds) {
    if (r.start) cudaEventDestroy(r.start);
    cudaEventDestroy(r.done);
  }
  for (ShadeInFlight& s : shades) {
    cudaEventDestroy(s.start);
    cudaEventDestroy(s.done);
  }
  for (auto& kv : slots) {
    if (kv.second->final_block) cudaFreeAsync(kv.second->final_block, build_stream);
    if (kv.second->scratch_block) cudaFreeAsync(kv.second->scratch_block, build_stream);
  }
  if (build_stream) cudaStreamSynchronize(build_stream);
  for (cudaStream_t st : shade_streams) cudaStreamDestroy(st);
  if (build_stream) cudaStreamDestroy(build_stream);
  if (pool) cudaMemPoolDestroy(pool);
  if (d_inst) cudaFree(d_inst);
  if (h_inst) cudaFreeHost(h_inst);
  if (d_ring) cudaFree(d_ring);
  if (h_ring) cudaFreeHost(h_ring);
}

void atmo_server::FreeSlot(LutSlot* s) {
  if (s->final_block) cudaFreeAsync(s->final_block, build_stream);
  if (s->scratch_block) cudaFreeAsync(s->scratch_block, build_stream);
  used_bytes -= s->final_bytes + (s->scratch_block ? s->scratch_bytes : 0);
  s->final_block = s->scratch_block = nullptr;
  if (s->index >= 0) free_rows.push_back(s->index);
  s->index = -1;
}

// Evicts idle ready sets (no shading queued or running), least recently
// used first, until `bytes` more fit.
bool atmo_server::EvictFor(size_t bytes) {
  if (used_bytes + bytes <= cfg.hbm_budget_bytes) return true;
  std::unordered_set<uint64_t> wanted;
  for (const ShadeRequest& r : pending_shades) wanted.insert(r.set_id);
  while (used_bytes + bytes > cfg.hbm_budget_bytes) {
    LutSlot* victim = nullptr;
    for (auto& kv : slots) {
      LutSlot* s = kv.second.get();
      if (s->ready && s->pins == 0 && s->final_block && !wanted.count(s->id) &&
          (!victim || s->last_use < victim->last_use))
        victim = s;
    }
    if (!victim) return false;
    FreeSlot(victim);
    victim->ready = false;
    ++stats.evictions;
    const uint64_t id = victim->id;
    slots.erase(id);
  }
  return true;
}

// Admits pending rebuilds while rows and memory allow; returns true if any.
bool atmo_server::Admit(std::unique_lock<std::mutex>&) {
  bool any = false;
  // The batching window: the oldest queued rebuild waits for company until
  // its window ends or a full batch is queued.
  if (cfg.admit_window_us > 0 && !pending_rebuilds.empty() &&
      pending_rebuilds.size() < free_rows.size()) {
    const auto waited = Clock::now() - tickets[pending_rebuilds.front().ticket]->submitted;
    if (waited < std::chrono::microseconds(cfg.admit_window_us)) return false;
  }
  while (!pending_rebuilds.empty() && !free_rows.empty()) {
    RebuildRequest& rq = pending_rebuilds.front();
    const size_t fb = FinalBytes(rq.s, cfg.combined != 0), sb = ScratchBytes(rq.s);
    if (fb + sb > cfg.hbm_budget_bytes) {
      FailTicket(rq.ticket, ATMO_BUDGET,
                 "a rebuild needs more than the whole device-memory budget");
      pending_rebuilds.pop_front();
      continue;
    }
    if (!EvictFor(fb + sb)) break;   // wait for sets to become idle or finish
    void* fblock = nullptr;
    void* sblock = nullptr;
    cudaError_t ae = cudaMallocFromPoolAsync(&fblock, fb, pool, build_stream);
    if (ae == cudaSuccess) ae = cudaMallocFromPoolAsync(&sblock, sb, pool, build_stream);
    if (ae != cudaSuccess) {
      // Not sticky: clear it, or the next launch check would report it.
      cudaGetLastError();
      if (fblock) cudaFreeAsync(fblock, build_stream);
      FailTicket(rq.ticket, ae == cudaErrorMemoryAllocation ? ATMO_OOM : ATMO_CUDA_ERROR,
                 std::string("the memory pool cannot serve the rebuild: ") +
                     cudaGetErrorString(ae));
      pending_rebuilds.pop_front();
      continue;
    }
    std::unique_ptr<LutSlot> slot(new LutSlot());
    slot->id = rq.ticket;
    slot->index = free_rows.back();
    free_rows.pop_back();
    slot->s = rq.s;
    slot->orders = rq.orders;
    slot->seq = PassSequence(rq.orders);
    slot->final_block = fblock;
    slot->scratch_block = sblock;
    slot->final_bytes = fb;
    slot->scratch_bytes = sb;
    used_bytes += fb + sb;
    // Carve the blocks.
    Instance& in = h_inst[slot->index];
    std::memset(&in, 0, sizeof(in));
    in.c = MakeConsts(rq.atm, nullptr);
    in.s = rq.s;
    in.combined = cfg.combined ? 1 : 0;
    in.blend = 0;
    const size_t nT = rq.s.t_texels(), nI = rq.s.i_texels(), nS = (size_t)rq.s.s_texels();
    char* f = static_cast<char*>(fblock);
    auto take_f = [&](size_t bytes) {
      char* p = f;
      f += Align(bytes);
      return p;
    };
    in.T = reinterpret_cast<float4*>(take_f(nT * 16));
    in.Tau = reinterpret_cast<float4*>(take_f(nT * 16));
    in.I = reinterpret_cast<float4*>(take_f(nI * 16));
    in.S = reinterpret_cast<float4*>(take_f(nS * 16));
    in.M = cfg.combined ? nullptr : reinterpret_cast<float4*>(take_f(nS * 16));
    char* sc = static_cast<char*>(sblock);
    auto take_s = [&](size_t bytes) {
      char* p = sc;
      sc += Align(bytes);
      return p;
    };
    in.dI = reinterpret_cast<float4*>(take_s(nI * 16));
    in.dR = reinterpret_cast<float4*>(take_s(nS * 16));
    in.dM = reinterpret_cast<float4*>(take_s(nS * 16));
    in.dJ = reinterpret_cast<float4*>(take_s(nS * 16));
    in.tab.rows = reinterpret_cast<TexelRow*>(take_s((size_t)rq.s.sr * rq.s.smu * sizeof(TexelRow)));
    in.tab.cols = reinterpret_cast<TexelCol*>(take_s((size_t)rq.s.smus * sizeof(TexelCol)));
    in.tab.drows = reinterpret_cast<DensityRow*>(
        take_s((size_t)rq.s.sr * kDensityThetaSamples * sizeof(DensityRow)));
    in.tab.irows = reinterpret_cast<IrrRow*>(take_s((size_t)rq.s.ih * sizeof(IrrRow)));
    in.tab.mus_i = reinterpret_cast<float*>(take_s((size_t)rq.s.iw * sizeof(float)));
    cudaMemcpyAsync(d_inst + slot->index, &in, sizeof(Instance), cudaMemcpyHostToDevice,
                    build_stream);
    slot->view.luts = LutsOf(in);
    slot->view.luminance_api = false;
    slot->view.radiance_api = true;
    for (int i = 0; i < 3; ++i) slot->view.solar[i] = rq.atm.solar_irradiance[i];
    slot->view.sun_angular_radius = rq.atm.sun_angular_radius;
    Ticket* t = tickets[rq.ticket].get();
    t->started = Clock::now();
    t->state.store(Ticket::kRunning, std::memory_order_release);
    building.push_back(rq.ticket);
    slots[rq.ticket] = std::move(slot);
    pending_rebuilds.pop_front();
    any = true;
  }
  return any;
}

// Launches one round: the next pass of every building instance.
bool atmo_server::LaunchRound() {
  if (building.empty()) return false;
  // Group by (pass, order, kernel variant).
  struct Group {
    Pass pass;
    int order;
    atmo_path path;
    std::vector<LutSlot*> members;
  };
  std::vector<Group> groups;
  for (uint64_t id : building) {
    LutSlot* s = slots[id].get();
    const PassStep ps = s->seq[s->next];
    const atmo_path path = PassPath(ps.pass, s->s, ATMO_PATH_FAST);
    Group* g = nullptr;
    for (Group& x : groups)
      if (x.pass == ps.pass && x.order == ps.order && x.path == path) g = &x;
    if (!g) {
      groups.push_back(Group{ps.pass, ps.order, path, {}});
      g = &groups.back();
    }
    g->members.push_back(s);
  }
  // Work lists into the ring.
  size_t need = 0;
  for (const Group& g : groups) need += 2 * g.members.size() + 1;
  if (ring_head + need > ring_ints) ring_head = 0;
  // The region must not overlap one still read by a round in flight.
  for (const Round& r : rounds) {
    const bool overlap = ring_head < r.ring_offset + r.ring_ints && r.ring_offset < ring_head + need;
    if (overlap) return false;   // retire rounds first
  }
  Round round;
  round.ring_offset = ring_head;
  round.ring_ints = need;
  int* h = h_ring + ring_head;
  struct Launch {
    Pass pass;
    int order, tiles, smem;
    atmo_path path;
    WorkList wl;
  };
  std::vector<Launch> launches;
  size_t off = 0;
  for (const Group& g : groups) {
    const size_t n = g.members.size();
    int t = 0, smem = 0;
    for (size_t i = 0; i < n; ++i) {
      h[off + i] = g.members[i]->index;
      h[off + n + i] = t;
      t += Tiles(g.pass, g.members[i]->s, g.path);
      smem = std::max(smem, SharedBytes(g.pass, g.members[i]->s, h_inst[g.members[i]->index].c,
                                        g.order, g.path));
    }
    h[off + 2 * n] = t;
    WorkList wl;
    wl.inst = d_ring + ring_head + off;
    wl.start = d_ring + ring_head + off + n;
    wl.count = (int)n;
    launches.push_back(Launch{g.pass, g.order, t, smem, g.path, wl});
    off += 2 * n + 1;
  }
  ring_head += need;
  cudaEventCreate(&round.start);
  cudaEventRecord(round.start, build_stream);
  cudaError_t e = cudaMemcpyAsync(d_ring + round.ring_offset, h, need * sizeof(int),
                                  cudaMemcpyHostToDevice, build_stream);
  for (const Launch& l : launches) {
    if (e != cudaSuccess) break;
    e = LaunchPass(l.pass, l.order, l.smem, d_inst, l.wl, l.tiles, l.path, build_stream);
    ++stats.kernels;
  }
  if (e != cudaSuccess) {
    worker_error = std::string("round launch: ") + cudaGetErrorString(e);
    for (uint64_t id : building) FailTicket(id, ATMO_CUDA_ERROR, worker_error);
    building.clear();
    return false;
  }
  // Advance; instances past their last pass complete with this round.
  std::vector<uint64_t> still;
  const Clock::time_point now = Clock::now();
  round.members = building;
  for (uint64_t id : building) {
    Ticket* t = tickets[id].get();
    if (!t->has_launched) {
      t->has_launched = true;
      t->launched = now;
    }
    LutSlot* s = slots[id].get();
    if (++s->next == s->seq.size()) {
      round.finishing.push_back(id);
      cudaLaunchHostFunc(build_stream, StampDone, tickets[id].get());
      // Temporaries go back to the pool behind the last pass.
      cudaFreeAsync(s->scratch_block, build_stream);
      s->scratch_block = nullptr;
      used_bytes -= s->scratch_bytes;
    } else {
      still.push_back(id);
    }
  }
  building.swap(still);
  cudaEventCreate(&round.done);
  cudaEventRecord(round.done, build_stream);
  rounds.push_back(round);
  ++stats.rounds;
  return true;
}

bool atmo_server::RetireRounds() {
  bool any = false;
  while (!rounds.empty() && cudaEventQuery(rounds.front().done) == cudaSuccess) {
    Round& r = rounds.front();
    if (r.start) {
      float ms = 0.0f;
      if (cudaEventElapsedTime(&ms, r.start, r.done) == cudaSuccess) {
        for (uint64_t id : r.members) {
          auto ti = tickets.find(id);
          if (ti == tickets.end()) continue;
          ti->second->device_ms += ms;
          ++ti->second->rounds;
        }
      }
      cudaEventDestroy(r.start);
    }
    for (int row : r.release_rows) free_rows.push_back(row);
    for (uint64_t id : r.finishing) {
      auto it = slots.find(id);
      if (it == slots.end()) continue;
      it->second->ready = true;
      it->second->last_use = ++lru_clock;
      free_rows.push_back(it->second->index);   // the instance row is no longer read
      it->second->index = -1;
    }
    cudaEventDestroy(r.done);
    rounds.pop_front();
    any = true;
  }
  return any;
}

bool atmo_server::LaunchShades() {
  bool any = false;
  for (auto it = pending_shades.begin(); it != pending_shades.end();) {
    if (cfg.max_shades_in_flight > 0 && shades.size() >= cfg.max_shades_in_flight) break;
    auto si = slots.find(it->set_id);
    if (si == slots.end()) {
      // A rebuild still queued for admission (batching window, budget) has
      // no slot yet: the shading request waits for it.
      auto ti = tickets.find(it->set_id);
      if (ti != tickets.end() && ti->second->state.load() == Ticket::kQueued) {
        ++it;
        continue;
      }
      FailTicket(it->ticket, ATMO_NOT_READY, "LUT set evicted, cancelled or unknown");
      it = pending_shades.erase(it);
      continue;
    }
    LutSlot* s = si->second.get();
    if (!s->ready) {
      ++it;
      continue;
    }
    cudaStream_t st = shade_streams[next_shade_stream++ % shade_streams.size()];
    PinholeView v;
    for (int i = 0; i < 3; ++i) {
      v.camera[i] = it->view.camera[i];
      v.right[i] = it->view.right[i];
      v.up[i] = it->view.up[i];
      v.forward[i] = it->view.forward[i];
      v.sun[i] = it->view.sun_direction[i];
      v.albedo[i] = it->view.albedo[i];
    }
    v.tan_half_fov_y = std::tan(0.5f * it->view.fov_y);
    v.width = it->view.width;
    v.height = it->view.height;
    v.depth = it->depth;
    v.luminance = 0;
    v.sky = reinterpret_cast<float4*>(it->sky);
    v.shaded = reinterpret_cast<float4*>(it->shaded);
    Ticket* t = tickets[it->ticket].get();
    t->started = t->launched = Clock::now();
    t->has_launched = true;
    t->state.store(Ticket::kRunning, std::memory_order_release);
    ShadeInFlight f;
    cudaEventCreate(&f.start);
    cudaEventRecord(f.start, st);
    cudaError_t e = LaunchShadeView(s->view.luts, v, st);
    if (e != cudaSuccess) {
      FailTicket(it->ticket, ATMO_CUDA_ERROR,
                 std::string("shading launch: ") + cudaGetErrorString(e));
      cudaEventDestroy(f.start);
    } else {
      cudaEventCreate(&f.done);
      cudaEventRecord(f.done, st);
      cudaLaunchHostFunc(st, StampDone, t);
      f.set_id = s->id;
      f.ticket = it->ticket;
      ++s->pins;
      s->last_use = ++lru_clock;
      shades.push_back(f);
      ++stats.shades_launched;
    }
    it = pending_shades.erase(it);
    any = true;
  }
  return any;
}

bool atmo_server::RetireShades() {
  bool any = false;
  for (auto it = shades.begin(); it != shades.end();) {
    if (cudaEventQuery(it->done) != cudaSuccess) {
      ++it;
      continue;
    }
    auto si = slots.find(it->set_id);
    if (si != slots.end()) --si->second->pins;
    float ms = 0.0f;
    auto ti = tickets.find(it->ticket);
    if (ti != tickets.end() && cudaEventElapsedTime(&ms, it->start, it->done) == cudaSuccess) {
      ti->second->device_ms += ms;
      ++ti->second->rounds;
    }
    cudaEventDestroy(it->start);
    cudaEventDestroy(it->done);
    it = shades.erase(it);
    any = true;
  }
  return any;
}

// Cancels ticket `id` (the lock is held).  A queued request is dropped.  A
// rebuild being built gets no further pass: its blocks are freed behind the
// passes already enqueued on the build stream (stream-ordered), its budget
// is released now, and its instance row once the GPU has passed the event
// recorded here (the rounds in flight still read the row).
atmo_status atmo_server::Cancel(uint64_t id) {
  auto ti = tickets.find(id);
  if (ti == tickets.end()) {
    SetError("unknown ticket");
    return ATMO_INVALID_ARG;
  }
  Ticket* t = ti->second.get();
  if (t->state.load() >= Ticket::kDone) {
    SetError("ticket already complete");
    return ATMO_INVALID_ARG;
  }
  if (!t->is_rebuild) {
    for (auto it = pending_shades.begin(); it != pending_shades.end(); ++it) {
      if (it->ticket != id) continue;
      pending_shades.erase(it);
      FailTicket(id, ATMO_CANCELLED, "cancelled");
      return ATMO_OK;
    }
    SetError("shading request already launched");
    return ATMO_INVALID_ARG;
  }
  for (auto it = pending_rebuilds.begin(); it != pending_rebuilds.end(); ++it) {
    if (it->ticket != id) continue;
    pending_rebuilds.erase(it);
    FailTicket(id, ATMO_CANCELLED, "cancelled");
    return ATMO_OK;
  }
  auto bi = std::find(building.begin(), building.end(), id);
  auto si = slots.find(id);
  if (bi == building.end() || si == slots.end()) {
    SetError("rebuild already complete on the GPU");
    return ATMO_INVALID_ARG;
  }
  int prev = 0;
  cudaGetDevice(&prev);
  cudaSetDevice(device);
  building.erase(bi);
  LutSlot* slot = si->second.get();
  const int row = slot->index;
  slot->index = -1;   // FreeSlot must not return the row yet
  FreeSlot(slot);
  Round release;
  release.release_rows.push_back(row);
  cudaEventCreateWithFlags(&release.done, cudaEventDisableTiming);
  cudaEventRecord(release.done, build_stream);
  rounds.push_back(release);
  slots.erase(si);
  FailTicket(id, ATMO_CANCELLED, "cancelled");
  cudaSetDevice(prev);
  return ATMO_OK;
}

void atmo_server::WorkerLoop() {
  cudaSetDevice(device);
  std::unique_lock<std::mutex> lk(mu);
  const int kMaxRoundsInFlight = 2;
  while (!stop) {
    bool progress = false;
    progress |= RetireRounds();
    progress |= RetireShades();
    progress |= Admit(lk);
    progress |= LaunchShades();
    if ((int)rounds.size() < kMaxRoundsInFlight) progress |= LaunchRound();
    stats.used_bytes = used_bytes;
    stats.resident_sets = 0;
    for (auto& kv : slots) stats.resident_sets += kv.second->ready ? 1 : 0;
    if (!progress) {
      // Nothing launched or retired: sleep until a submission or a short
      // timeout (the GPU work in flight completes on its own).
      cv.wait_for(lk, std::chrono::microseconds(100));
    }
  }
}

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
static atmo_status Fail(atmo_status s, const std::string& msg) {
  SetError(msg);
  return s;
}

extern "C" {

atmo_status atmo_server_create(const atmo_server_config* cfg, atmo_server** out) {
  if (!out) return Fail(ATMO_INVALID_ARG, "NULL argument");
  *out = nullptr;
  std::unique_ptr<atmo_server> s(new atmo_server());
  if (cfg) s->cfg = *cfg;
  if (s->cfg.hbm_budget_bytes == 0) s->cfg.hbm_budget_bytes = size_t(120) << 30;
  if (s->cfg.max_rebuilds_in_flight == 0) s->cfg.max_rebuilds_in_flight = 64;
  if (s->cfg.shade_streams == 0) s->cfg.shade_streams = 4;
  if (s->cfg.max_rebuilds_in_flight > 4096 || s->cfg.shade_streams > 64 ||
      s->cfg.admit_window_us > 10000000)
    return Fail(ATMO_INVALID_ARG,
                "max_rebuilds_in_flight <= 4096, shade_streams <= 64, admit_window_us <= 1e7");
  s->stats.budget_bytes = s->cfg.hbm_budget_bytes;
  atmo_status st = s->Init();
  if (st != ATMO_OK) {
    s->Shutdown();
    return st;
  }
  *out = s.release();
  return ATMO_OK;
}

atmo_status atmo_server_destroy(atmo_server* s) {
  if (!s) return ATMO_OK;
  s->Shutdown();
  delete s;
  return ATMO_OK;
}

atmo_status atmo_server_submit_rebuild(atmo_server* s, const atmo_atmosphere* atm,
                                       const atmo_lut_shape* shape, unsigned orders,
                                       uint64_t* ticket) {
  if (!s || !atm || !ticket) return Fail(ATMO_INVALID_ARG, "NULL argument");
  if (orders < 1 || orders > 64) return Fail(ATMO_INVALID_ARG, "orders must be in [1, 64]");
  std::string why;
  atmo_lut_shape ls = shape ? *shape : DefaultShape();
  if (!ValidShape(ls, &why) || !ValidAtmosphere(*atm, &why)) return Fail(ATMO_INVALID_ARG, why);
  {
    std::lock_guard<std::mutex> lk(s->mu);
    const uint64_t id = s->next_ticket++;
    std::unique_ptr<Ticket> t(new Ticket());
    t->submitted = Clock::now();
    t->is_rebuild = true;
    t->set_id = id;
    s->tickets[id] = std::move(t);
    s->pending_rebuilds.push_back(RebuildRequest{id, *atm, ToShape(ls), orders});
    *ticket = id;
  }
  s->cv.notify_all();
  return ATMO_OK;
}

atmo_status atmo_server_submit_shade(atmo_server* s, uint64_t set_id,
                                     const atmo_pinhole_view* view, const float* depth,
                                     float* sky_rgba, float* shaded_rgba, uint64_t* ticket) {
  if (!s || !view || !depth || !sky_rgba || !shaded_rgba || !ticket)
    return Fail(ATMO_INVALID_ARG, "NULL argument");
  if (view->width <= 0 || view->height <= 0 || !(view->fov_y > 0.0f && view->fov_y < 3.1f))
    return Fail(ATMO_INVALID_ARG, "bad view size or field of view");
  {
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->tickets.find(set_id);
    if (it == s->tickets.end() || !it->second->is_rebuild)
      return Fail(ATMO_INVALID_ARG, "unknown LUT set");
    const uint64_t id = s->next_ticket++;
    std::unique_ptr<Ticket> t(new Ticket());
    t->submitted = Clock::now();
    t->set_id = set_id;
    s->tickets[id] = std::move(t);
    s->pending_shades.push_back(
        ShadeRequest{id, set_id, *view, depth, sky_rgba, shaded_rgba, 0});
    *ticket = id;
  }
  s->cv.notify_all();
  return ATMO_OK;
}

static void FillInfo(const Ticket& t, atmo_ticket_info* info) {
  info->state = t.state.load(std::memory_order_acquire);
  info->status = t.status;
  const bool started = t.started != Clock::time_point{};   // admitted or launched
  info->queue_ms = started ? MsSince(t.submitted, t.started) : -1.0;
  info->latency_ms = info->state >= Ticket::kDone ? MsSince(t.submitted, t.finished) : -1.0;
  info->set_id = t.set_id;
  info->launch_ms = t.has_launched ? MsSince(t.submitted, t.launched) : -1.0;
  info->device_ms = t.device_ms;
  info->rounds = t.rounds;
}

atmo_status atmo_server_poll(atmo_server* s, uint64_t ticket, atmo_ticket_info* info) {
  if (!s || !info) return Fail(ATMO_INVALID_ARG, "NULL argument");
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->tickets.find(ticket);
  if (it == s->tickets.end()) return Fail(ATMO_INVALID_ARG, "unknown ticket");
  FillInfo(*it->second, info);
  return ATMO_OK;
}

atmo_status atmo_server_wait(atmo_server* s, uint64_t ticket, unsigned timeout_ms,
                             atmo_ticket_info* info) {
  if (!s || !info) return Fail(ATMO_INVALID_ARG, "NULL argument");
  const Clock::time_point deadline = Clock::now() + std::chrono::milliseconds(timeout_ms);
  for (;;) {
    {
      std::lock_guard<std::mutex> lk(s->mu);
      auto it = s->tickets.find(ticket);
      if (it == s->tickets.end()) return Fail(ATMO_INVALID_ARG, "unknown ticket");
      FillInfo(*it->second, info);
      if (info->state >= Ticket::kDone) {
        if (info->state == Ticket::kFailed) return Fail(info->status, it->second->message);
        // A rebuild's set is usable once its round has been retired.
        if (it->second->is_rebuild) {
          auto si = s->slots.find(ticket);
          if (si != s->slots.end() && si->second->ready) return ATMO_OK;
          if (si == s->slots.end()) return Fail(ATMO_NOT_READY, "LUT set evicted");
        } else {
          return ATMO_OK;
        }
      }
    }
    if (Clock::now() >= deadline) return Fail(ATMO_TIMEOUT, "ticket not complete");
    std::this_thread::sleep_for(std::chrono::microseconds(50));
  }
}

atmo_status atmo_server_cancel(atmo_server* s, uint64_t ticket) {
  if (!s) return Fail(ATMO_INVALID_ARG, "NULL server");
  atmo_status st;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    st = s->Cancel(ticket);
  }
  s->cv.notify_all();
  return st;
}

atmo_status atmo_server_release_ticket(atmo_server* s, uint64_t ticket) {
  if (!s) return Fail(ATMO_INVALID_ARG, "NULL server");
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->tickets.find(ticket);
  if (it == s->tickets.end()) return Fail(ATMO_INVALID_ARG, "unknown ticket");
  if (it->second->state.load() < Ticket::kDone)
    return Fail(ATMO_INVALID_ARG, "ticket still in flight");
  if (it->second->is_rebuild && s->slots.count(ticket))
    return Fail(ATMO_INVALID_ARG, "release the LUT set with atmo_server_evict first");
  s->tickets.erase(it);
  return ATMO_OK;
}

atmo_status atmo_server_lut_set(atmo_server* s, uint64_t set_id, const atmo_lut_set** out) {
  if (!s || !out) return Fail(ATMO_INVALID_ARG, "NULL argument");
  std::lock_guard<std::mutex> lk(s->mu);
  auto si = s->slots.find(set_id);
  if (si == s->slots.end()) return Fail(ATMO_NOT_READY, "LUT set evicted or unknown");
  if (!si->second->ready) return Fail(ATMO_NOT_READY, "LUT set not built yet");
  si->second->last_use = ++s->lru_clock;
  *out = &si->second->view;
  return ATMO_OK;
}

atmo_status atmo_server_evict(atmo_server* s, uint64_t set_id) {
  if (!s) return Fail(ATMO_INVALID_ARG, "NULL server");
  std::lock_guard<std::mutex> lk(s->mu);
  auto si = s->slots.find(set_id);
  if (si == s->slots.end()) return Fail(ATMO_INVALID_ARG, "LUT set evicted or unknown");
  if (!si->second->ready || si->second->pins > 0)
    return Fail(ATMO_INVALID_ARG, "LUT set is being built or shaded");
  s->FreeSlot(si->second.get());
  s->slots.erase(si);
  s->tickets.erase(set_id);
  return ATMO_OK;
}

atmo_status atmo_server_get_stats(atmo_server* s, atmo_server_stats* out) {
  if (!s || !out) return Fail(ATMO_INVALID_ARG, "NULL argument");
  std::lock_guard<std::mutex> lk(s->mu);
  *out = s->stats;
  out->used_bytes = s->used_bytes;
  out->building = (unsigned)s->building.size();
  out->pending = (unsigned)(s->pending_rebuilds.size() + s->pending_shades.size());
  return ATMO_OK;
}

}  // extern "C"
