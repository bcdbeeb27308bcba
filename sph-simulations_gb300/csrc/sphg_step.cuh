// sphg_step.cuh -- launch interface of the per-step kernels (sphg_step.cu).
#pragma once
#include <cstdint>
#include <string>
#include <cuda_runtime.h>

#include "../../include/sphg.h"
#include "sphg_common.cuh"

namespace sphg {

// Everything a step kernel touches.  Passed by value (kernel parameter space).
constexpr int kInstTabShift = 8;  // slots per instance-table entry: 256

struct StepArgs {
  int64_t n;
  int ninst;
  int track_ids;
  int early_next;              // let the next kernel be scheduled at this kernel's start (allow_next_kernel)
  int force_batched;           // 1: per-instance descriptor kernels even for one instance
  int block;                   // threads per block of the density and force passes (64, 128, 256)
  int cell_pairs;              // 1: the density pass carries two particles of a cell per thread
  InstDesc d0;                 // copy of desc[0] (single-instance fast path)
  const InstDesc* desc;        // [ninst]
  const int32_t* begins;       // [ninst]
  const int32_t* inst_tab;     // [n >> kInstTabShift + 1] instance of the first slot of each block
  const uint32_t* diag_tab;    // several instances: instance << 12 | chunk of each diagnostics block (or null)
  int diag_blocks;             // entries of diag_tab
  // sorted ("current") state
  float2* posA;
  float4* velpA;               // (vx, vy, p/rho^2, 1/rho)
  float* rho;
  uint32_t* keyA;              // sorted global keys (written by the reorder)
  const uint32_t* keyS;        // sort output: sorted keys, read by the reorder
  uint4* ranges;               // [total keys] {start, end, epoch, 0}
  const uint32_t* epoch;       // current step's epoch (bumped by the sort)
  int32_t* idsA;
  // integrated ("next") state in the current slot order
  float2* posB;
  float2* velB;
  uint32_t* keyB;              // keys of the next state (sort input)
  int32_t* idsB;
  uint32_t* perm;              // sort output: previous slot of each new slot
  float2* acc;                 // forces (only written on request)
  uint32_t* nbr;               // [nbr_slots][n] neighbours found by the density pass: j << 5 | tag
  uint32_t* ncount;            // [n] neighbours of each particle (> nbr_slots: list overflowed)
  int nbr_slots;
  const int64_t* csr_offs;     // [n+1] CSR neighbour lists of this iteration (lists mode)
  const uint32_t* csr_idx;     // j << 5 | tag entries, self included, list order
  int64_t csr_cap;             // entries csr_idx holds (the passes read no further)
  uint32_t* csr_overflow;      // set by the fill when the lists exceed csr_cap
  const uint32_t* merged;      // non-null and set: this iteration's merge scattered the state (reorder: ranges only)
  uint32_t* mover_mask;        // [ceil(n/32)] force pass: bit per slot whose key changed (or null)
  unsigned long long* mover_list;  // [kMoverCap] force pass: key << 32 | slot of each changed slot
  uint32_t* mover_count;       // changed slots recorded (zeroed before the force pass)
  uint32_t* flags;             // [0] unused, [1] number of non-empty tiles this step
  // cell tiles (Morton order only; tile_bits == 0 disables them)
  int tile_bits;               // tiles of 2^tile_bits x 2^tile_bits cells
  int tile_cap;                // shared-memory staging capacity (particles)
  int tile_grid;               // CTAs of the tile kernels
  uint2* tile_ranges;          // [total keys >> 2*tile_bits] particle run of each tile
  uint32_t* tile_list;         // ids of this step's non-empty tiles
  uint32_t* tile_count;        // device counter (= flags + 1)
};

enum ForceMode { kForceIntegrate = 0, kForceOnly = 1 };

cudaError_t launch_keys(const StepArgs& a, int precision, cudaStream_t s);
// The iteration in one cooperative launch (merge -> ranges -> density -> forces;
// post: after a full sort, ranges -> density -> forces).  bar: two zeroed words,
// err: set when a grid barrier's wait gave up.  cudaErrorNotSupported when the
// device cannot launch it cooperatively.
struct MoverArgs;
cudaError_t launch_fused(const StepArgs& a, const MoverArgs& m, int precision, uint32_t* bar, uint32_t* err,
                         bool post, cudaStream_t s);
// Blocks of the fused launch for this handle (0: not available).
int fused_blocks(const StepArgs& a, int precision);
cudaError_t launch_reorder(const StepArgs& a, cudaStream_t s);
cudaError_t launch_density(const StepArgs& a, int precision, cudaStream_t s, bool csr = false);
cudaError_t launch_force(const StepArgs& a, int precision, int mode, cudaStream_t s, bool csr = false);
// Lists mode: per-particle counts, exclusive scan to int64 offsets (the total
// lands in sums[scan_tiles(n)]), fill of packed entries (at most cap).
int lists_scan_tiles(int64_t n);
cudaError_t launch_lists_count_scan(const StepArgs& a, int precision, int32_t* counts, int64_t* offs,
                                    int64_t* sums, cudaStream_t st);
cudaError_t launch_lists_fill_packed(const StepArgs& a, int precision, const int64_t* offs,
                                     uint32_t* idx, int64_t cap, uint32_t* overflow, cudaStream_t st);
// Per-instance diagnostics in one launch: float-float partials per (chunk,
// instance) block, then the last block of an instance (ticket counter) sums them
// in a fixed order; out[6*inst + {0..5}] = E_k, max|v|^2, inside, sum m vx,
// sum m vy, nonfinite.
// Where the step headers of sphg_step_headers go: the caller's host array
// (device-accessible), the index of the next step, and the count of instance
// blocks done with the current one.
struct HeaderSlot {
  double* out;
  uint32_t k;
  uint32_t done;
};
// Diagnostics of the current state written to slot->out[(k * ninst + inst) * 6 ..],
// then k advanced (by the last instance block to finish).
cudaError_t launch_diagnostics_slot(const StepArgs& a, int precision, double* partials, uint32_t* tickets,
                                    int chunks, HeaderSlot* slot, cudaStream_t s);
// The same into out[inst * 6 ..] (device-accessible).  partials: ninst x chunks
// 48-byte float-float records; tickets: ninst counters, zero between launches.
cudaError_t launch_diagnostics(const StepArgs& a, int precision, double* partials, uint32_t* tickets, int chunks,
                               double* out, cudaStream_t s);
// Diagnostics chunks of the largest instance (at most cap; the partial buffer
// holds ninst x chunks x 6 doubles).
int diag_chunks(int64_t max_inst_n, int ninst, int cap = 4096);
// Diagnostics blocks of one instance of `count` particles among several
// (about 4,096 particles a block -- 16 a thread --, at most `chunks`).
__host__ __device__ inline int diag_instance_chunks(int64_t count, int chunks) {
  const int64_t c = (count + 4095) / 4096;
  return (int)(c < 1 ? 1 : (c > chunks ? chunks : c));
}
// out[6*inst + {0, 1}] = max |v|^2, max |a|^2 of each instance (a.acc must hold the forces).
cudaError_t launch_cfl(const StepArgs& a, double* partials, int chunks, double* out, cudaStream_t s);
// CSR neighbour lists of the current state (sphg_lists.cu); returns an sphg_status.
int lists_impl(const StepArgs& a, int precision, int64_t* offs, int32_t* idx, int64_t* total,
               cudaStream_t st, std::string* err, bool encoded = false);
// Delta codec of CSR lists on device buffers (encode: in = ascending lists).
cudaError_t launch_delta(bool encode, const int64_t* offs, const int32_t* in, int64_t n, int32_t* out,
                         cudaStream_t st);
// Cell-tile density (force == false) or force + integration + next keys (force == true).
cudaError_t launch_tiled(const StepArgs& a, int precision, bool force, cudaStream_t s);
size_t tile_smem_bytes(int tb, int cap, bool force);
// Records the message returned by sphg_last_error_string() (sphg_api.cu).
void set_last_error(const std::string& msg);
// Upload / download through the caller's host arrays from the device (sphg_hostio.cu).
cudaError_t launch_upload_direct(const StepArgs& a, int precision, const double* x, const double* y,
                                 const double* vx, const double* vy, uint32_t* first_bad, cudaStream_t st);
cudaError_t launch_download_direct(const StepArgs& a, int precision, double* x, double* y, double* vx, double* vy,
                                   double* rho, double* fx, double* fy, int32_t* ids, cudaStream_t st);
// A served request's lattice initial state into the admission staging (sphg_init.cu).
cudaError_t launch_lattice_stage(const InstDesc& d, const sphg_lattice& L, int precision, int64_t n, float2* pos,
                                 float2* vel, uint32_t* key, int32_t* ids, cudaStream_t st);
cudaError_t launch_cell_keys_plain(const InstDesc& d, const float* x, const float* y, int64_t n,
                                   int32_t* keys, cudaStream_t s);

}  // namespace sphg
