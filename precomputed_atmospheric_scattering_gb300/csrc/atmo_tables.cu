// atmo_tables.cu -- FP64 set-up tables (see atmo_tables.cuh).  Built with
// --fmad=false so its double arithmetic rounds like the reference's CPU model.
#include "atmo_kernels.h"
#include "atmo_tables.cuh"

namespace atmo {

__global__ void __launch_bounds__(kTableThreads)
k_tables(const Instance* __restrict__ insts, WorkList wl) {
  int local;
  const Instance& in = insts[FindEntry(wl, blockIdx.x, &local)];
  int e = local * kTableThreads + threadIdx.x;
  if (e < dbl::TableEntries(in.s)) dbl::FillTableEntry(in.c, in.s, in.tab, e);
}

int TableTiles(const Shape& s) { return (dbl::TableEntries(s) + kTableThreads - 1) / kTableThreads; }

cudaError_t LaunchTables(const Instance* insts, WorkList wl, int tiles, cudaStream_t st) {
  k_tables<<<tiles, kTableThreads, 0, st>>>(insts, wl);
  return cudaGetLastError();
}

}  // namespace atmo
