// sphg_movers.cuh -- launch interface of the incremental re-sort (sphg_movers.cu).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace sphg {

constexpr int kMoverCap = 8192;   // largest mover set merged incrementally

struct MoverArgs {
  int64_t n;
  const uint32_t* keyA;    // sorted keys of the current state, slot order
  const uint32_t* mask;    // [ceil(n/32)] bit s%32 of word s/32: slot s changed key
  const unsigned long long* movers;  // [kMoverCap] key << 32 | slot of every changed slot, any order
  const uint32_t* count;   // changed slots the force pass recorded (may exceed kMoverCap)
  uint32_t* ctl;           // [0] = 1 when the incremental path ran, [1] = changed slots,
                           // [2] set to 1 if a record was inconsistent (never cleared here)
  uint32_t* epoch;         // step epoch of the cell-range table (bumped when the merge runs)
  const uint4* ranges;     // cell ranges {start, end, epoch, 0} of the current sorted order
  uint32_t* keyS;          // out: sorted keys
  uint32_t* perm;          // out: previous slot of each sorted position
  unsigned long long cond; // graph conditional handle of the full sort (0: none), set to
                           // 1 when it must run, 0 when the merge handled the iteration
  // the merge scatters the state into sorted order itself (the reorder then only
  // builds the cell ranges): sources in previous-slot order, destinations sorted
  const float2* posB;
  const float2* velB;
  const int32_t* idsB;     // null when creation indices are not tracked
  float2* posA;
  float4* velpA;
  int32_t* idsA;
  uint32_t mover_blocks;   // the stand-alone kernel's leading blocks that place the movers (set by launch_movers)
  int early_next;          // let the next kernel be scheduled at the start (allow_next_kernel)
};

// One launch: the decision (merge when at most kMoverCap slots changed, else
// leave ctl[0] = 0 for the full sort), the final position of every unchanged
// slot and of every changed one, and the scatter of the state.
cudaError_t launch_movers(const MoverArgs& a, cudaStream_t st);

}  // namespace sphg
