// sphg_movers.cuh -- launch interface of the incremental re-sort (sphg_movers.cu).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace sphg {

constexpr int kGroupShift = 13;   // slots per mover group count: 8,192
constexpr int kMoverCap = 8192;   // largest mover set merged incrementally

struct MoverArgs {
  int64_t n;
  const uint32_t* keyA;    // sorted keys of the current state, slot order
  const uint32_t* keyB;    // keys of the integrated state, per slot
  const uint32_t* mask;    // [ceil(n/32)] bit s%32 of word s/32: slot s changed key
  const uint32_t* gsum;    // [mover_groups(n)] changed slots per group of 8,192 slots
  uint32_t* wprefix;       // [ceil(n/32)] changed slots before each word
  unsigned long long* movers;   // [kMoverCap] key << 32 | slot, slot order
  unsigned long long* msorted;  // [kMoverCap] the same, ascending
  uint32_t* ctl;           // [0] = 1 when the incremental path ran, [1] = changed slots,
                           // [2] set to 1 if a record was inconsistent (never cleared here)
  uint32_t* epoch;         // step epoch of the cell-range table
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
};

int mover_groups(int64_t n);
// movers_compact, movers_rank_place, movers_merge; when more than kMoverCap
// slots changed they do nothing and leave ctl[0] = 0 for the full sort.
cudaError_t launch_movers(const MoverArgs& a, cudaStream_t st);

}  // namespace sphg
