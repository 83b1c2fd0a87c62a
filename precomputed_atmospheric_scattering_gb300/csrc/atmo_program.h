// atmo_program.h -- host-side launch programs: a sequence of passes over
// instance slots, with the per-pass work lists in device memory, replayed
// directly or through a CUDA graph.
#ifndef ATMO_PROGRAM_H_
#define ATMO_PROGRAM_H_

#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "../../include/atmo/atmo.h"
#include "atmo_instance.h"

namespace atmo {

// Registers the tuned block shapes (4 values, see Shape::tune) for LUTs of
// these sizes in this process; NULL removes them.  Shapes made afterwards by
// ToShape carry them.
void SetTuning(const atmo_lut_shape& sizes, const int* tune);

// Last error message of this host thread.
void SetError(const std::string& msg);
atmo_status CudaFail(cudaError_t e, const char* what);

#define ATMO_CUDA_TRY(expr)                                   \
  do {                                                        \
    cudaError_t atmo_err_ = (expr);                           \
    if (atmo_err_ != cudaSuccess) return CudaFail(atmo_err_, #expr); \
  } while (0)

// Device buffers of one instance storage (LUTs, temporaries, tables).
struct Storage {
  Shape s{};
  bool combined = true;
  bool half = false;
  float4 *T = nullptr, *Tau = nullptr, *I = nullptr, *dI = nullptr, *dI2 = nullptr,
         *dR = nullptr, *dM = nullptr, *dJ = nullptr, *S = nullptr, *M = nullptr;
  void *S_half = nullptr, *M_half = nullptr;   // half-precision outputs
  Tables tab{};
  std::vector<void*> owned;                    // what Free() releases
  atmo_status Allocate(const Shape& shape, bool combined_textures, bool half_precision);
  void Free();
  size_t Bytes() const;
};

enum class Pass { kTables, kTransmittance, kDirect, kSingle, kDensity, kIndirect, kMultiple,
                  kToHalf };

struct Step {
  Pass pass;
  int order;      // scattering order of density / multiple; order-1 for indirect
  int wl;         // work-list index
  int tiles;      // blocks of the launch
  int smem;       // dynamic shared memory bytes (fast kernels)
  atmo_path path; // kernel variant of this launch
};

// A program: a sequence of stages; a stage runs the full precomputation of a
// set of instance slots together (a batch), or only their transmittance.
class Program {
 public:
  ~Program();
  std::vector<Instance> slots;         // host copies, uploaded before each run
  std::vector<unsigned> orders;        // per slot
  atmo_path path = ATMO_PATH_FAST;

  // Appends the passes of atmosphere/model.cc:1048-1215 for `members`
  // (slot indices that run together), or only the transmittance pass.
  void AddStage(const std::vector<int>& members, bool transmittance_only = false);
  // Appends the FP32 -> FP16 conversion of the slots' scattering outputs.
  void AddToHalf(const std::vector<int>& members);
  atmo_status Finalize();              // uploads work lists
  atmo_status Upload(cudaStream_t st); // copies slots to the device
  atmo_status Launch(cudaStream_t st); // enqueues the steps
  atmo_status LaunchStep(size_t i, cudaStream_t st);
  // Runs the steps without a graph, timing each with CUDA events on `st`.
  atmo_status TimeSteps(cudaStream_t st, std::vector<float>* ms);
  // Upload + replay through a CUDA graph (captured on first use).
  atmo_status Run(cudaStream_t st, bool use_graph);
  int KernelCount() const { return (int)steps_.size(); }
  std::vector<Step> const& steps() const { return steps_; }

 private:
  int AddWorkList(const std::vector<int>& members, Pass pass, int order, int* tiles,
                  int* smem = nullptr, atmo_path* step_path = nullptr);
  std::vector<Step> steps_;
  std::vector<int> blob_;              // inst[] then start[] of every work list
  std::vector<std::pair<int, int>> wl_offsets_;  // (offset, count)
  std::vector<WorkList> wls_;
  Instance* d_slots_ = nullptr;
  Instance* h_slots_pinned_ = nullptr;
  int* d_blob_ = nullptr;
  cudaGraphExec_t graph_ = nullptr;
  cudaStream_t capture_stream_ = nullptr;
  cudaEvent_t upload_done_ = nullptr;    // guards reuse of the pinned staging copy
  bool finalized_ = false;
  // Indirect irradiance beside density (every slot has two delta-irradiance
  // buffers): the side stream and the fork / join events of Launch.
  bool fork_indirect_ = false;
  atmo_status PrepareFork();             // creates the side stream and events once
  cudaStream_t side_stream_ = nullptr;
  cudaEvent_t ev_fork_ = nullptr, ev_join_ = nullptr;
};

// The kernel variant that runs `pass` for shape s when `path` is requested:
// the fast single- and multiple-scattering kernels hold a LUT row of NU x MU_S
// texels per block and take shapes up to 1024 of them.
atmo_path PassPath(Pass pass, const Shape& s, atmo_path path);
// Blocks and dynamic shared memory of `pass` for shape s under the variant
// `path` (as PassPath returns it).
int Tiles(Pass pass, const Shape& s, atmo_path path);
// Dynamic shared memory of a pass's launch for one instance (shape and
// constants: the density pass sizes its merged tables from the radii).
int SharedBytes(Pass pass, const Shape& s, const Consts& c, int order, atmo_path path);
// Launches one pass over the instances of `wl` (device pointers); kToHalf is
// not a pass kernel and returns cudaErrorInvalidValue.
cudaError_t LaunchPass(Pass pass, int order, int smem, const Instance* insts, WorkList wl,
                       int tiles, atmo_path path, cudaStream_t st);

}  // namespace atmo

#endif  // ATMO_PROGRAM_H_
