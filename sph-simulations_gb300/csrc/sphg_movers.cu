// sphg_movers.cu -- incremental re-sort of a nearly sorted state.
//
// Between two main-loop iterations a particle moves a small fraction of a
// cell, so almost every particle keeps its cell key.  The stable sort of the
// new keys (GenericNeighborSearch::SortParticleIds,
// core/alg/GenericNeighborSearch.h:69-76, with ties in previous-slot order)
// is then a merge of two sorted sequences:
//   * stayers: slots whose key did not change -- already in (key, slot) order,
//     because the current state is sorted;
//   * movers: slots whose key changed -- few.
// Writing v_s = (key, slot) for the order of slot s:
//   final position of a stayer i = i - (movers with slot < i)
//                                    + (movers with v < v_i)
//   final position of a mover m  = (movers with v < v_m)
//                                    + (slots s with v_s < v_m in the current order)
//                                    - (movers among those slots)
// The force pass records every mover (key << 32 | slot, appended with one
// atomic per warp) and one bit per slot.  One kernel then places everything:
// each block of 512 consecutive slots counts, over the whole (short) mover
// list, the movers before its first slot and before its first stayer's key,
// keeps the few movers whose key falls inside its own key span in shared
// memory, and places its stayers; the movers go to leading blocks of their
// own, a warp each, which start with the launch.  When more than kMoverCap
// slots changed the kernel only records
// that and the full radix sort runs instead (under a conditional graph node,
// or its kernels skip themselves on the decision word).
#include <algorithm>
#include <cstdint>

#include <cuda_runtime.h>

#include "sphg_common.cuh"
#include "sphg_movers.cuh"
#include "sphg_movers_body.cuh"

namespace sphg {

namespace {

__global__ void __launch_bounds__(kMergeThreads) movers_merge(MoverArgs a) {
  cudaGridDependencySynchronize();  // the mover record of the previous force pass
  allow_next_kernel(a.early_next);
  uint32_t m = 0;
  if (!merge_decide(a, blockIdx.x == 0 && threadIdx.x == 0, &m)) return;
  constexpr uint32_t W = kMergeThreads / 32;
  if (blockIdx.x < a.mover_blocks)
    merge_movers<false>(a, blockIdx.x * W + (threadIdx.x >> 5), a.mover_blocks * W, m);
  else
    merge_block<false>(a, blockIdx.x - a.mover_blocks, 0, m);
}

}  // namespace

cudaError_t launch_movers(const MoverArgs& a, cudaStream_t st) {
  if (a.n <= 0) return cudaSuccess;
  const int64_t nb = (a.n + kMergeBlockSlots - 1) / kMergeBlockSlots;
  MoverArgs b = a;
  b.mover_blocks = (uint32_t)std::min<int64_t>(kMoverBlocks, std::max<int64_t>(8, nb / 4));
  const unsigned g = (unsigned)nb + b.mover_blocks;
  cudaError_t e = launch_pdl(movers_merge, dim3(g), dim3(kMergeThreads), 0, st, b);
  if (e != cudaSuccess) return e;
  return cudaGetLastError();
}

}  // namespace sphg
