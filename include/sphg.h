/*
 * sphg.h -- C ABI of the GB300 SPH step library (libsphg.so).
 *
 * One handle owns the device state of one or more independent 2-D SPH
 * simulations ("instances") and runs the reference's per-step pipeline on
 * them on one GPU:  Morton / row-major cell key -> stable key sort and cell
 * ranges -> density -> pressure -> forces -> symplectic-Euler integration
 * with reflecting (or periodic) walls.  Plain C types only: doubles at the
 * boundary, device pointers as void*, a CUDA stream as an opaque void*
 * (pass a cudaStream_t, or NULL for the legacy default stream).
 *
 * Every call returns an sphg_status; sphg_last_error_string() describes the
 * most recent failure of the calling thread.
 *
 * Reference interfaces these calls replace (paths inside
 * jose-pinzon0407/sph-simulations):
 *   sphg_create / sphg_create_batch  cudaConfigure + cudaSimulationSetup
 *                                    (app/cu_simulation_configuration.h:37-85),
 *                                    cuCreateContainer (core/acceleration/cuContainer.cu:31-48)
 *   sphg_upload                      cuReadContainer (core/acceleration/cuContainer.cu:50-68)
 *   sphg_preloop                     PreLoopComputationWithCellNeighbors
 *                                    (app/cu_simulation_configuration.h:88-164)
 *   sphg_step                        one iteration of MaiLoopComputationWithCellNeighbors
 *                                    (app/cu_simulation_configuration.h:166-259):
 *                                    cuCallbackIntegrate, cuCallbackFindNeighbors,
 *                                    cuCallbackApproximateDensitySorted, cuInvertBuffer,
 *                                    cuKernelComputePressureSorted, cuCallbackComputeForcesSorted
 *   sphg_download                    cuWriteContainer (core/acceleration/cuContainer.cu:70-88)
 *   sphg_diagnostics                 cuKernelMeasurementsPerStep (core/acceleration/utils/cuUtils.cu:33-60)
 *                                    and ComputeKineticEnergy/ComputeMaxVelocity/ParticlesInDomain
 *                                    (core/container/MeasuringFunctions.h:5-61)
 *   sphg_neighbor_lists              cuCallbackNeighborLists (core/acceleration/cuNeighborLists.cu:32-82)
 *                                    and MultipassNeighborLists::AssembleNeighborList
 *                                    (core/algorithmic/MultipassNeighborLists.h:10-14)
 *   sphg_sort_pairs                  the thrust::sort_by_key of cuSortContainerByCellID
 *                                    (core/acceleration/cuFindNeighbors.cu:82-100)
 *   sphg_cell_keys                   cuSetParticlesCellIndex (core/acceleration/cuFindNeighbors.cuh:6-24)
 */
#ifndef SPHG_H
#define SPHG_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum sphg_status {
  SPHG_OK = 0,
  SPHG_INVALID_ARG = 1,  /* bad size, parameter or call order */
  SPHG_OOM = 2,          /* device allocation failed */
  SPHG_NONFINITE = 3,    /* NaN/Inf found in an input or in the state */
  SPHG_TIMEOUT = 4,      /* a bounded device wait gave up */
  SPHG_CUDA_ERROR = 5,   /* a CUDA runtime call failed */
  SPHG_CAPACITY = 6,     /* a fixed capacity (cells, particles, list entries) was exceeded */
  SPHG_NOT_READY = 7     /* a served request has not finished yet */
} sphg_status;

enum { SPHG_ORDER_MORTON = 0, SPHG_ORDER_ROWMAJOR = 1 };
enum { SPHG_PRECISION_PLAIN = 0, SPHG_PRECISION_SPLIT = 1 };
/* compute_type of the reference driver (app/simulation_configuration.h:479-537):
 * SORTED  = `sorted`: the density pass walks the 3x3 cell stencil of the sorted
 *           state (GenericForceComputation, core/compute/GenericForceComputation.tpp:35-253)
 *           and hands the neighbours it accepts to the force pass;
 * LISTS   = `lists` / `mp-lists`: every iteration assembles CSR neighbour lists
 *           (count, scan, fill; MultipassNeighborLists,
 *           core/algorithmic/MultipassNeighborLists.h:47-181) and the density
 *           and force passes sum over them in list order
 *           (MPListsForceComputation, core/compute/MPListsForceComputation.cpp:3-147). */
enum { SPHG_COMPUTE_SORTED = 0, SPHG_COMPUTE_LISTS = 1 };

/* Physics and domain of one instance.  sphg_default_params() fills the
 * reference's values: core/ConfigVariables.hpp:9-15 (H=1, TOL=1e-12,
 * GAS_CONSTANT=30, RHO_0=25, MU=0.01), gravity -10 in y
 * (core/compute/GenericForceComputation.tpp:141), mass 1
 * (core/container/SoAContainer.cpp:10), and config/example.txt (dt=0.005,
 * domain 96x48, order=rowmajor).  alpha, periodic, gx, mass != 1 are
 * extensions; with their defaults the step is the reference's. */
typedef struct sphg_params {
  double h;        /* smoothing length H; also the cell size */
  double dt;       /* time step */
  double k;        /* GAS_CONSTANT: p = k (rho - rho0) */
  double rho0;     /* RHO_0 */
  double mu;       /* MU */
  double tol;      /* TOL: the pressure term needs r > tol */
  double gx, gy;   /* gravity */
  double mass;     /* particle mass */
  double alpha;    /* Monaghan artificial viscosity, 0 = off */
  double c0;       /* sound speed of the alpha term */
  double lo[2];    /* Domain::l_corner */
  double hi[2];    /* Domain::h_corner */
  int32_t order;   /* SPHG_ORDER_* */
  int32_t periodic;/* 0 = reflecting walls (reference), 1 = periodic */
} sphg_params;

typedef struct sphg_options {
  int32_t precision;   /* SPHG_PRECISION_PLAIN: FP32 positions;
                          SPHG_PRECISION_SPLIT: integer cell + FP32 in-cell offset,
                          compensated density/force sums */
  int32_t track_ids;   /* 1: carry each particle's creation index through the sorts */
  int32_t use_graph;   /* 1: replay each step from a captured CUDA graph */
  int32_t tile_bits;   /* density/force cell tiles of 2^b x 2^b cells staged in shared memory:
                          0 = default (off), 3..5 = that b (every instance in Morton order),
                          -1 = off (one thread per particle, L1-cached global loads) */
  int32_t compute;     /* SPHG_COMPUTE_*; LISTS sizes its list buffer at the pre-loop
                          (twice that iteration's total) and runs without cell tiles;
                          lists that later outgrow it make sphg_download /
                          sphg_diagnostics return SPHG_CAPACITY */
  int32_t resort;      /* 1 (default): when at most 8,192 particles changed cell since the
                          last iteration, re-sort by merging them into the unchanged
                          (already sorted) rest -- the same stable order as the full radix
                          sort, which runs otherwise; 0: full radix sort every iteration */
  int32_t block_threads;/* threads per block of the density and force passes: 0 = default
                          (128), 64, 128 or 256 */
  int32_t cell_pairs;  /* density pass: 0 (default) one particle per thread; 1 one thread
                          carries two particles of a cell (they share the stencil walk;
                          the same results) */
  int32_t fused;       /* 1: each iteration that merges is ONE cooperative launch (re-sort,
                          cell ranges, density, forces as phases between grid-wide
                          barriers) instead of four kernels -- for small and medium
                          workloads, whose kernel boundaries cost as much as their work;
                          the same results.  Sorted compute mode without cell tiles only;
                          its grid fills the GPU, so two handles must not run such
                          iterations at the same time on one GPU (different streams):
                          their barriers would wait on each other until their bounded
                          waits give up (SPHG_TIMEOUT).  0 (default): a graph of four
                          kernels */
} sphg_options;

typedef struct sphg_sim sphg_sim;

void sphg_default_params(sphg_params* p);
void sphg_default_options(sphg_options* o);
const char* sphg_last_error_string(void);
const char* sphg_version(void);
/* out[6]: compute capability major, minor, SM count, and whether the device can
 * read and write pageable host memory directly (cudaDevAttrPageableMemoryAccess,
 * ...UsesHostPageTables, cudaDevAttrConcurrentManagedAccess). */
sphg_status sphg_device_attributes(int32_t device, int32_t* out);
/* How upload and download reach the caller's FP64 arrays:
 *   0: through a pinned staging buffer, converted on the host;
 *   1: upload converts the caller's arrays on the device, reading them in place
 *      (the default when the device can access pageable host memory);
 *   2: download writes them from the device as well (fast when their pages are
 *      already resident: writes into untouched pages fault them in one by one).
 * The results are the same. */
sphg_status sphg_set_host_access(sphg_sim* s, int32_t mode);

/* One instance of n particles. */
sphg_status sphg_create(const sphg_params* p, const sphg_options* o, int64_t n, sphg_sim** out);
/* ninst independent instances; counts[i] particles each, laid out one after the other. */
sphg_status sphg_create_batch(int32_t ninst, const sphg_params* p, const int64_t* counts,
                              const sphg_options* o, sphg_sim** out);
sphg_status sphg_destroy(sphg_sim* s);

/* Host arrays of all instances' particles concatenated (instance order). */
sphg_status sphg_upload(sphg_sim* s, const double* x, const double* y, const double* vx,
                        const double* vy, void* stream);
/* Initial state generated on the device, one lattice per instance: the
 * reference's LatticeCreator (core/container/Lattice.h:12-35: x = x0 + i dx,
 * y = y0 + j dy, particle i + nx j) with an optional seeded uniform jitter of
 * +-jitter spacings and an optional Taylor-Green velocity field
 * (vx = u0 sin(2 pi x/Lx) cos(2 pi y/Ly), vy = -u0 cos(2 pi x/Lx) sin(2 pi y/Ly),
 * x and y measured from lo).  nx * ny must equal the instance's particle
 * count.  Replaces sphg_upload; no host arrays are involved. */
enum { SPHG_VEL_ZERO = 0, SPHG_VEL_TAYLOR_GREEN = 1 };
typedef struct sphg_lattice {
  double x0, y0;    /* first point */
  double dx, dy;    /* spacing */
  int64_t nx, ny;   /* points per direction */
  double jitter;    /* uniform jitter amplitude in spacings (0 = none) */
  uint64_t seed;    /* jitter stream */
  int32_t velocity; /* SPHG_VEL_* */
  int32_t pad;
  double u0;        /* Taylor-Green amplitude */
} sphg_lattice;
sphg_status sphg_upload_lattice(sphg_sim* s, const sphg_lattice* spec, void* stream);

/* FindNeighbors -> density -> pressure -> forces of the initial state. */
sphg_status sphg_preloop(sphg_sim* s, void* stream);
/* nsteps main-loop iterations: integrate -> FindNeighbors -> density -> pressure -> forces. */
sphg_status sphg_step(sphg_sim* s, int64_t nsteps, void* stream);
/* Current state in the current (cell-sorted) slot order; any pointer may be NULL.
 * fx/fy are the forces of the current state (GenericForceComputation::ComputeForces). */
sphg_status sphg_download(sphg_sim* s, double* x, double* y, double* vx, double* vy,
                          double* rho, double* fx, double* fy, int32_t* ids, void* stream);
/* Per instance, 6 doubles: E_k, max |v|^2, particles inside the domain,
 * sum m vx, sum m vy, non-finite count.  out has 6*ninst entries. */
sphg_status sphg_diagnostics(sphg_sim* s, double* out, void* stream);
/* The same without waiting: the values land in out (pinned host memory, kept
 * valid until the stream passes this point) in stream order, so a step loop
 * reads every step's header without a host synchronisation per step. */
sphg_status sphg_diagnostics_async(sphg_sim* s, double* out, void* stream);
/* nsteps main-loop iterations, each followed by its step header (the 6 values
 * of sphg_diagnostics per instance) written to out[(k * ninst + inst) * 6 ..]
 * for iteration k -- the reference's main loop, which prints a header after
 * every iteration (app/simulation_configuration.h:431-433).  out holds
 * nsteps * 6 * ninst doubles; the values land in stream order.  Where the
 * device can write out (pinned host memory, or pageable memory on a node with
 * pageable access) the kernels write it directly and the iterations replay as
 * one graph each; otherwise each header is copied. */
sphg_status sphg_step_headers(sphg_sim* s, int64_t nsteps, double* out, void* stream);
/* Waits for the work enqueued on stream (for hosts without a CUDA runtime of
 * their own, such as ctypes callers of the asynchronous entry points). */
sphg_status sphg_stream_synchronize(void* stream);

/* Adaptive time step per instance from the current state: FP64 maxima of the
 * speed and of the acceleration on the device, then
 *   dt = min(cfl * h / (c0 + max|v|), force_coef * sqrt(h / max|a|))
 * (infinite when both are zero).  out has ninst entries.  The reference steps
 * with a fixed dt (config/example.txt); apply a new one with sphg_set_dt. */
sphg_status sphg_cfl_dt(sphg_sim* s, double cfl, double force_coef, double* out, void* stream);
/* Time step of instance inst (every instance when inst < 0) from the next iteration on. */
sphg_status sphg_set_dt(sphg_sim* s, int32_t inst, double dt);

/* Debug / parity views (host copies, current slot order).  which: */
enum {
  SPHG_DBG_KEYS = 0,        /* int32[n]  sorted cell keys (instance-local codes) */
  SPHG_DBG_PERM = 1,        /* int32[n]  slot before the last sort of each slot */
  SPHG_DBG_UNSORTED_KEYS = 2,/* int32[n] keys of the integrated state awaiting the next sort */
  SPHG_DBG_POS_NEXT = 3,    /* double[2n] integrated positions awaiting the next sort */
  SPHG_DBG_VEL_NEXT = 4,    /* double[2n] integrated velocities awaiting the next sort */
  SPHG_DBG_RESORT = 5       /* int32[3]  last iteration: 1 if the incremental re-sort ran
                               (0: the full radix sort), particles that changed cell,
                               kernels of a full sort (histogram + radix passes) */
};
sphg_status sphg_get_debug(sphg_sim* s, int32_t which, void* host, void* stream);

/* CSR neighbour lists of the current state in the reference's stencil order
 * (self included, MultipassNeighborLists).  Call with idx == NULL to get the
 * total in *total; offs has n+1 entries. */
sphg_status sphg_neighbor_lists(sphg_sim* s, int64_t* offs, int32_t* idx, int64_t* total,
                                void* stream);

/* The same lists with each list sorted ascending and delta-coded as
 * Codifier::Encode does (core/encoders/Encoder.h:27-44: the first index, then
 * idx[k] - idx[k-1] - 1).  The reference never calls its encoder on the active
 * path (core/alg/GenericNeighborLists.tpp:75-78). */
sphg_status sphg_neighbor_lists_encoded(sphg_sim* s, int64_t* offs, int32_t* enc, int64_t* total,
                                        void* stream);
/* Stand-alone delta codec of n CSR lists on DEVICE buffers (offs[n+1]);
 * encode needs ascending lists; decode inverts it. */
sphg_status sphg_delta_encode(const int64_t* offs, const int32_t* idx, int64_t n, int32_t* enc,
                              void* stream);
sphg_status sphg_delta_decode(const int64_t* offs, const int32_t* enc, int64_t n, int32_t* idx,
                              void* stream);

/* Binary snapshot of the current state in the device representation (positions
 * or split cell + offset, velocities, cell keys, creation indices) so a run can
 * resume exactly: sphg_restore + sphg_preloop continues bit for bit where the
 * snapshot was taken.  buf == NULL: *bytes receives the size.  No reference
 * counterpart (CheckPointWriter writes positions only, core/utils/CheckPointWriter.cpp:11-27). */
sphg_status sphg_snapshot(sphg_sim* s, void* buf, uint64_t* bytes, void* stream);
sphg_status sphg_restore(sphg_sim* s, const void* buf, uint64_t bytes, void* stream);

/* ---- continuous batching ("serving").  A server owns one device arena sized
 * from an HBM budget and keeps every live simulation's state resident in it.
 * Submitted requests queue in order; every tick admits the queue head while
 * it fits (appended after the slots in use, so running simulations keep their
 * slots; the live set is compacted when the arena's end is reached or
 * finished simulations hold more slots than live ones), runs one batched
 * main-loop iteration of all live simulations from a CUDA graph (a newcomer's
 * first iteration is its pre-loop), and retires the ones that ran `steps`
 * iterations (the reference's `steps` key: the pre-loop plus steps-1 main-loop
 * iterations) by an asynchronous copy into pinned host memory.  A simulation
 * gives the same bits whatever else is live.  The serving loop runs either on
 * the caller's thread (sphg_server_tick) or on a thread and stream of the
 * server's own (sphg_server_start), which admits arrivals while earlier ticks
 * run on the GPU.  submit, result and stats may be called from any thread.
 * No reference counterpart: the reference runs one simulation per process
 * (app/main.cpp:20-56). */
typedef struct sphg_server sphg_server;
sphg_status sphg_server_create(double hbm_budget_bytes, int32_t max_instances,
                               const sphg_options* o, sphg_server** out);
sphg_status sphg_server_destroy(sphg_server* s);
sphg_status sphg_server_submit(sphg_server* s, const sphg_params* p, int64_t n, const double* x,
                               const double* y, const double* vx, const double* vy, int64_t steps,
                               int64_t* request_id);
/* The same for a state generated on the device at admission (sphg_upload_lattice's
 * lattice, nx * ny particles): no host arrays cross the boundary for it. */
sphg_status sphg_server_submit_lattice(sphg_server* s, const sphg_params* p, const sphg_lattice* spec,
                                       int64_t steps, int64_t* request_id);
/* Admit, step, retire on the caller's thread and stream.  *live = simulations
 * live after the tick, *finished = retired by it.  SPHG_INVALID_ARG while the
 * serving thread runs. */
sphg_status sphg_server_tick(sphg_server* s, void* stream, int32_t* live, int32_t* finished);
/* Starts the serving thread on `device` with a stream of its own: it ticks
 * while anything is live or queued (at most three ticks ahead of the GPU) and
 * waits for submissions otherwise. */
sphg_status sphg_server_start(sphg_server* s, int32_t device);
/* Stops and joins the serving thread (live and queued requests stay; ticks can
 * continue with sphg_server_tick).  Reports an error the thread stopped on. */
sphg_status sphg_server_stop(sphg_server* s);
/* Final state of a finished request (slot order, like sphg_download) and its
 * latency (time its result reached host memory - submission, seconds);
 * SPHG_NOT_READY until then (without the serving thread, a request retired by
 * the last tick waits for its copy here).  The result is released once fetched. */
sphg_status sphg_server_result(sphg_server* s, int64_t request_id, double* x, double* y, double* vx,
                               double* vy, double* rho, int32_t* ids, double* latency_s);
/* out[8]: live, queued, completed, particle-steps run, ticks, capacity (particles),
 * capacity (cell keys), live particles. */
sphg_status sphg_server_stats(sphg_server* s, double* out);
/* The first `count` of: appends, compactions, graph builds, slots of finished
 * simulations awaiting compaction, slots in use, result copies in flight,
 * serving thread running (1/0). */
sphg_status sphg_server_counters(sphg_server* s, double* out, int32_t count);

/* Autotuner: times every candidate launch configuration of this workload (the
 * cell-block shape: one thread per particle or Morton cell tiles of 2^b x 2^b
 * cells, b = 3..5; the re-sort strategy: incremental merge or full radix sort)
 * on handles of its own with the given state (pre-loop, 3 warm-up and `steps`
 * timed main-loop iterations on `stream`), and returns the fastest in *best
 * (precision, track_ids, use_graph and compute as in *base) with its
 * milliseconds per iteration.  Results are remembered per workload for the
 * process.  No reference counterpart (its block size is a config key,
 * gpu_threads_per_block, config/example.txt). */
sphg_status sphg_autotune(int32_t ninst, const sphg_params* p, const int64_t* counts, const double* x,
                          const double* y, const double* vx, const double* vy, const sphg_options* base,
                          int32_t steps, sphg_options* best, double* ms_per_step, void* stream);

/* Runs one main-loop iteration kernel by kernel with CUDA events between the
 * phases; ms[0..4] = keys, sort, reorder (+cell ranges), density, force+integrate
 * (milliseconds, summed over the instances of the handle). */
sphg_status sphg_profile_step(sphg_sim* s, float* ms, void* stream);
/* Kernel launches of a main-loop iteration that runs the full sort; in a graph,
 * an iteration that merges launches SPHG_DBG_RESORT[2] fewer. */
int32_t sphg_launches_per_step(const sphg_sim* s);

/* Stand-alone kernels on caller-owned DEVICE buffers. */
/* Stable LSD radix sort of (key, value) pairs on the low `bits` bits of the keys.
 * keys_out/vals_out must not alias the inputs; vals_in == NULL sorts the
 * identity 0..n-1.  Buffers need only 4-byte alignment.  n <= 2^30 - 1
 * (SPHG_CAPACITY otherwise).  Scratch is allocated by this call.  Every wait of
 * the sort's look-back is bounded; a wait that gives up (none does on a working
 * GPU: it only waits on tiles that started earlier) is not reported by this
 * stand-alone call. */
sphg_status sphg_sort_pairs(const uint32_t* keys_in, const uint32_t* vals_in, uint32_t* keys_out,
                            uint32_t* vals_out, int64_t n, int32_t bits, void* stream);
/* Largest n sphg_sort_pairs_noalloc accepts, and the size of its fixed scratch. */
#define SPHG_SORT_NOALLOC_MAX_PAIRS 262144
#define SPHG_SORT_NOALLOC_SCRATCH_BYTES 2626560
/* sphg_sort_pairs for callers that cannot allocate device memory when they
 * sort (allocation-free graph capture, fixed-budget allocators, hosts that
 * forbid cudaMalloc).  No counterpart in the reference.  Same arguments and
 * result as sphg_sort_pairs, but its scratch is a fixed device array inside
 * the library (SPHG_SORT_NOALLOC_SCRATCH_BYTES = 2,626,560 bytes, held on every GPU that loads the library until
 * the process exits), so n must be <= SPHG_SORT_NOALLOC_MAX_PAIRS
 * (SPHG_CAPACITY otherwise).  It calls no cudaMalloc/cudaFree.  The first
 * call on a device looks up the array's device address (cudaGetSymbolAddress);
 * make that first call before any stream capture.  The address is looked up
 * again when the device's context changes (after cudaDeviceReset the next call
 * is a first call again).  All calls share the one
 * array: calls that overlap on the GPU (different streams, or different host
 * threads on one device) race and corrupt each other's results. */
sphg_status sphg_sort_pairs_noalloc(const uint32_t* keys_in, const uint32_t* vals_in,
                                    uint32_t* keys_out, uint32_t* vals_out, int64_t n,
                                    int32_t bits, void* stream);
/* Cell key of each particle (SetParticleCellIds): float positions in, int32 keys out. */
sphg_status sphg_cell_keys(const sphg_params* p, const float* x, const float* y, int64_t n,
                           int32_t* keys, void* stream);

#ifdef __cplusplus
}
#endif
#endif
