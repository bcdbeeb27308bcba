// sphg_internal.cuh -- the handle behind the C ABI, shared by sphg_api.cu
// (single instances and fixed batches) and sphg_server.cu (continuous batching).
#pragma once
#include <cstdint>
#include <cstring>
#include <string>
#include <functional>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/sphg.h"
#include "sphg_movers.cuh"
#include "sphg_step.cuh"

using sphg::InstDesc;
using sphg::StepArgs;

namespace sphg_detail {

struct Arena {
  char* base = nullptr;
  size_t size = 0, used = 0;
  template <class T>
  T* take(size_t count) {
    size_t bytes = (count * sizeof(T) + 255) & ~(size_t)255;
    T* p = reinterpret_cast<T*>(base + used);
    used += bytes;
    return p;
  }
};

}  // namespace sphg_detail

struct sphg_sim {
  int ninst = 0;
  int64_t n = 0;
  sphg_options opt{};
  std::vector<sphg_params> params;
  std::vector<int64_t> counts;
  std::vector<InstDesc> hdesc;
  std::vector<int32_t> hbegins;
  std::vector<int32_t> hinst_tab;
  std::vector<uint32_t> hdiag_tab;  // several instances: (instance << 12 | chunk) of each diagnostics block
  uint64_t total_keys = 0;
  int key_bits = 1;
  int diag_chunks = 1;
  sphg_detail::Arena arena;
  // device buffers
  InstDesc* ddesc = nullptr;
  int32_t* dbegins = nullptr;
  int32_t* dinst_tab = nullptr;  // instance of the first slot of each 256-slot block
  uint32_t* ddiag_tab = nullptr;
  float2 *posA = nullptr, *posB = nullptr, *velB = nullptr, *acc = nullptr;
  float4* velpA = nullptr;
  float* rho = nullptr;
  uint32_t *keyA = nullptr, *keyB = nullptr, *keyTmp = nullptr, *perm = nullptr,
           *valTmp = nullptr, *scratch = nullptr, *flags = nullptr;
  uint4* ranges = nullptr;
  int32_t *idsA = nullptr, *idsB = nullptr;
  double *diag_partials = nullptr, *diag_out = nullptr;
  uint32_t* diag_tickets = nullptr;  // per instance: chunks done in the running diagnostics launch
  sphg::HeaderSlot* hslot = nullptr;  // step headers written into the caller's array
  uint2* tile_ranges = nullptr;
  uint32_t* tile_list = nullptr;
  uint32_t *nbr = nullptr, *ncount = nullptr;
  int nbr_slots = 0;
  // lists mode: CSR of each iteration; the index buffer is sized at the pre-loop
  // (twice the list total then) and an overflow past it is reported
  int32_t* csr_counts = nullptr;
  int64_t *csr_offs = nullptr, *csr_sums = nullptr;
  uint32_t* csr_idx = nullptr;
  int64_t csr_cap = 0, csr_total = 0;
  // incremental re-sort: mover bits and group counts written by the force pass
  bool movers_on = false;
  bool force_full_sort = false;  // the next iteration sorts fully (the slot record is stale)
  uint32_t* mmask = nullptr;
  unsigned long long* mlist = nullptr;
  size_t cap_n = 0;             // arena capacity (particles)
  uint64_t cap_keys = 0;        // arena capacity (cell keys)
  int cap_inst = 0;             // arena capacity (instances)
  int force_batched = 0;        // always use the per-instance-descriptor kernels
  int tile_bits = 0, tile_cap = 0, tile_grid = 0;
  bool uploaded = false, preloop_done = false;
  // 1: upload reads the caller's arrays from the device (pageable host memory
  // access); 2: download writes them from the device too; 0: both through the
  // pinned staging below
  int host_direct = 0;
  // pinned host staging of upload/download (grows on demand)
  char* hstage = nullptr;
  size_t hstage_bytes = 0;
  // CUDA graph of one step
  cudaStream_t cap_stream = nullptr, cap_stream2 = nullptr;
  bool cond_graph = true;       // full sort under a conditional graph node (when the merge is on)
  cudaGraphExec_t gexec = nullptr;
  cudaGraphExec_t gexec_hdr = nullptr;  // the same followed by the step header into hslot
  void drop_graphs() {
    if (gexec) cudaGraphExecDestroy(gexec);
    if (gexec_hdr) cudaGraphExecDestroy(gexec_hdr);
    gexec = gexec_hdr = nullptr;
  }

  StepArgs args() const {
    StepArgs a;
    std::memset(&a, 0, sizeof(a));
    a.n = n;
    a.ninst = ninst;
    a.track_ids = opt.track_ids;
    a.early_next = n <= sphg::kEarlyNextMaxN ? 1 : 0;
    if (!hdesc.empty()) a.d0 = hdesc[0];
    a.desc = ddesc;
    a.begins = dbegins;
    a.inst_tab = dinst_tab;
    a.diag_tab = hdiag_tab.empty() ? nullptr : ddiag_tab;
    a.diag_blocks = (int)hdiag_tab.size();
    a.posA = posA;
    a.velpA = velpA;
    a.rho = rho;
    a.keyA = keyA;
    a.ranges = ranges;
    a.epoch = flags + 2;
    a.idsA = idsA;
    a.posB = posB;
    a.velB = velB;
    a.keyB = keyB;
    a.idsB = idsB;
    a.perm = perm;
    a.acc = acc;
    a.flags = flags;
    a.tile_bits = tile_bits;
    a.tile_cap = tile_cap;
    a.tile_grid = tile_grid;
    a.tile_ranges = tile_ranges;
    a.tile_list = tile_list;
    a.tile_count = flags + 1;
    a.force_batched = force_batched;
    a.block = opt.block_threads > 0 ? opt.block_threads : 128;
    a.cell_pairs = opt.cell_pairs > 0 ? 1 : 0;
    a.nbr = tile_bits ? nullptr : nbr;  // the tile kernels walk the stencil in both passes
    a.ncount = ncount;
    a.nbr_slots = nbr_slots;
    a.csr_offs = csr_offs;
    a.csr_idx = csr_idx;
    a.csr_cap = csr_cap;
    a.csr_overflow = flags + 8;
    a.keyS = keyTmp;
    a.merged = movers_on ? flags + 3 : nullptr;
    a.mover_mask = movers_on ? mmask : nullptr;
    a.mover_list = movers_on ? mlist : nullptr;
    a.mover_count = movers_on ? flags + 7 : nullptr;
    return a;
  }
};

namespace sphg_detail {

sphg_status fail(sphg_status st, const std::string& msg);

#define SPHG_CUDA(expr)                                                                   \
  do {                                                                                    \
    cudaError_t e_ = (expr);                                                              \
    if (e_ != cudaSuccess)                                                                \
      return fail(SPHG_CUDA_ERROR, std::string(#expr) + ": " + cudaGetErrorString(e_));  \
  } while (0)

#define SPHG_TRY(expr)                   \
  do {                                   \
    sphg_status st_ = (expr);            \
    if (st_ != SPHG_OK) return st_;      \
  } while (0)


sphg_status make_desc(const sphg_params& p, int64_t begin, int64_t count, uint64_t cell_base,
                      InstDesc& d, uint64_t& span);
int host_cell(double x, double lo, double cs, int cmax);
// f(begin, end) over [0, n) split across host threads (one thread for small n).
void parallel_for(int64_t n, const std::function<void(int64_t, int64_t)>& f);
// Pinned host staging of at least `bytes` owned by the handle (nullptr: out of memory).
char* host_stage(sphg_sim* s, size_t bytes);
// In-cell offset o (FP64, in [0, cs)) as FP32, kept below cs after rounding.
float split_offset(double o, double cs);
// A lattice specification is valid for `count` particles (index: for the message).
sphg_status check_lattice(const sphg_lattice& L, int64_t count, int index);
// Instance holding particle i (instances are contiguous in particle order).
int instance_of(const sphg_sim* s, int64_t i);
uint32_t morton_host(uint32_t x, uint32_t y);
void demorton_host(uint32_t z, int& x, int& y);
// One main-loop iteration on st; ev (6 events, optional) records the phase boundaries.
// first: the iteration after an upload (cell keys computed; in lists mode the
// index buffer is sized from this iteration's list total, a host synchronisation).
sphg_status enqueue_step(sphg_sim* s, cudaStream_t st, bool first = false, cudaEvent_t* ev = nullptr);
// The single-launch iteration applies (sphg_options.fused, sorted mode, merge
// re-sort, no tiles, and the device can launch it cooperatively).
bool fused_on(sphg_sim* s);
// Captures (once per layout) the CUDA graph of one iteration (header: followed
// by its step header into the header slot).
sphg_status build_graph(sphg_sim* s, bool header = false);

struct Layout {
  std::vector<InstDesc> desc;
  std::vector<int32_t> begins;
  int64_t n = 0, max_n = 0;
  uint64_t keys = 0;
};
sphg_status check_options(sphg_sim* s, int ninst, const sphg_params* p);
sphg_status compute_layout(sphg_sim* s, int ninst, const sphg_params* p, const int64_t* counts,
                           uint64_t keys_cap, Layout& L);
sphg_status alloc_arena(sphg_sim* s, size_t N, uint64_t keys, int ninst, int diag_chunks);
sphg_status apply_layout(sphg_sim* s, int ninst, const sphg_params* p, const int64_t* counts,
                         const Layout& L, cudaStream_t* stream);
sphg_status destroy_impl(sphg_sim* s);

}  // namespace sphg_detail
