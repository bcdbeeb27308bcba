/*
 * sph_oracle.h -- CPU restatement of the reference SPH step, used ONLY as a
 * test checker and as the timed CPU baseline.  Nothing in the product path
 * (the CUDA library and its host code) links or calls this.
 *
 * Parity: pinned against the reference's own C++ classes compiled from its
 * sources (oracle/_ref, built by oracle/Makefile) through the golden
 * fixtures under tests/golden/ (tests/test_oracle_golden.py).
 *
 * Everything is FP64 and follows the reference's expression order so that,
 * given the same sorted particle order, density, pressure, forces and the
 * integrator are bit-identical to the reference's FP64 build.
 *
 * Reference functions restated (paths inside jose-pinzon0407/sph-simulations):
 *   MortonOrder::Initialize/AddCellPadding/MortonCode2d  core/alg/orders/MortonOrder.h:11-43,92-103,117-126
 *   RowMajorOrder::MapThreeToOne/MapOneToThree           core/alg/orders/RowMajorOrder.h:48-59
 *   GenericNeighborSearch::SetParticleCellIds           core/alg/GenericNeighborSearch.h:201-231
 *   GenericNeighborSearch::SortParticleIds/SortContainer core/alg/GenericNeighborSearch.h:69-76,111-191
 *   GenericNeighborSearch::SetCellRanges                core/alg/GenericNeighborSearch.h:93-108
 *   GenericForceComputation::ApproximateDensity         core/compute/GenericForceComputation.tpp:35-130
 *   GenericForceComputation::CalculatePressure          core/compute/GenericForceComputation.tpp:23-32
 *   GenericForceComputation::ComputeForces              core/compute/GenericForceComputation.tpp:134-253
 *   Integrator::UpdateVelocities/UpdatePositions/BC      core/integrator/Integrator.cpp:7-46
 *   GenericNeighborLists::AssembleNeighborList          core/alg/GenericNeighborLists.tpp:10-81
 *   MultipassNeighborLists (count/offsets/fill)         core/algorithmic/MultipassNeighborLists.h:47-181
 *   MPListsForceComputation density/forces              core/compute/MPListsForceComputation.cpp:3-147
 *   Codifier::Encode                                    core/encoders/Encoder.h:27-44
 *   ComputeKineticEnergy/ComputeMaxVelocity/ParticlesInDomain core/container/MeasuringFunctions.h:5-61
 *   LatticeCreator::CreateLattice                       core/container/Lattice.h:12-35
 *
 * Deviations (documented, none reachable with the reference's defaults):
 *   - the sort is stable (reference: unstable std::sort); cell membership and
 *     cell ranges are identical, the order inside a cell is the canonical
 *     "by key, then by previous position".
 *   - cell coordinates are clamped to >= 0 (reference: prints "Out of domain"
 *     and produces an undefined key for negative positions).
 *   - extensions switched off by default: gravity (gx,gy), particle mass,
 *     Monaghan artificial viscosity alpha, periodic boundaries.
 */
#ifndef SPH_ORACLE_H
#define SPH_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_params {
  double h;      /* smoothing length H; also the cell size */
  double dt;     /* time step */
  double k;      /* GAS_CONSTANT (linear EOS stiffness) */
  double rho0;   /* RHO_0 */
  double mu;     /* MU (viscosity) */
  double tol;    /* TOL guard of the pressure term */
  double gx, gy; /* gravity; reference: (0,-10) */
  double mass;   /* particle mass; reference: 1 */
  double alpha;  /* artificial viscosity (extension, 0 = off) */
  double c0;     /* sound speed for the alpha term */
  double lo[2], hi[2]; /* Domain l_corner / h_corner */
  int32_t order;    /* 0 = morton, 1 = rowmajor */
  int32_t periodic; /* 0 = reflecting walls (reference), 1 = periodic (extension) */
} orc_params;

typedef struct orc_grid {
  double cs[2];      /* cell size per axis */
  int32_t nx, ny;    /* cells per axis (morton: padded to a power of two) */
  int32_t nx_real, ny_real; /* ceil(L/cs) before padding */
  int64_t ncells;    /* nx*ny */
} orc_grid;

void orc_default_params(orc_params* p);
void orc_grid_init(const orc_params* p, orc_grid* g);
int32_t orc_morton2d(int32_t x, int32_t y);
int32_t orc_flatten(const orc_params* p, const orc_grid* g, int32_t cx, int32_t cy);
void orc_unflatten(const orc_params* p, const orc_grid* g, int32_t key, int32_t* cx, int32_t* cy);

/* Per-particle cell key (SetParticleCellIds). */
void orc_cell_ids(const orc_params* p, const orc_grid* g, int64_t n,
                  const double* x, const double* y, int32_t* key);
/* Stable permutation by key: perm[i] = index (before sorting) of sorted slot i. */
void orc_sort_perm(int64_t n, const int32_t* key, int32_t* perm);
/* out[i] = in[perm[i]] (SortContainer gather), for double and int32 arrays. */
void orc_gather_f64(int64_t n, const int32_t* perm, const double* in, double* out);
void orc_gather_i32(int64_t n, const int32_t* perm, const int32_t* in, int32_t* out);
/* SetCellRanges: start/end of length g->ncells, -1 where empty, end exclusive. */
void orc_cell_ranges(const orc_grid* g, int64_t n, const int32_t* sorted_key,
                     int32_t* start, int32_t* end);

void orc_density(const orc_params* p, const orc_grid* g, int64_t n,
                 const double* x, const double* y, const int32_t* key,
                 const int32_t* start, const int32_t* end, double* rho);
void orc_pressure(const orc_params* p, int64_t n, const double* rho, double* pr);
void orc_forces(const orc_params* p, const orc_grid* g, int64_t n,
                const double* x, const double* y, const double* vx, const double* vy,
                const double* rho, const double* pr, const int32_t* key,
                const int32_t* start, const int32_t* end, double* fx, double* fy);
/* UpdateVelocities then UpdatePositions with the boundary condition. */
void orc_integrate(const orc_params* p, int64_t n, double* x, double* y,
                   double* vx, double* vy, const double* fx, const double* fy);

/* CSR neighbour list in stencil order (self included):
 * pass offs==NULL-free arrays: counts[n], offs[n+1]; idx sized offs[n].
 * orc_nlist_count fills counts and offs; orc_nlist_fill fills idx. */
int64_t orc_nlist_count(const orc_params* p, const orc_grid* g, int64_t n,
                        const double* x, const double* y, const int32_t* key,
                        const int32_t* start, const int32_t* end,
                        int32_t* counts, int64_t* offs);
void orc_nlist_fill(const orc_params* p, const orc_grid* g, int64_t n,
                    const double* x, const double* y, const int32_t* key,
                    const int32_t* start, const int32_t* end,
                    const int64_t* offs, int32_t* idx);
void orc_density_lists(const orc_params* p, int64_t n, const double* x, const double* y,
                       const int64_t* offs, const int32_t* idx, double* rho);
void orc_forces_lists(const orc_params* p, int64_t n, const double* x, const double* y,
                      const double* vx, const double* vy, const double* rho,
                      const double* pr, const int64_t* offs, const int32_t* idx,
                      double* fx, double* fy);
/* Codifier::Encode applied to each (ascending) CSR list; out sized offs[n]. */
void orc_delta_encode(int64_t n, const int64_t* offs, const int32_t* idx, int32_t* out);
void orc_delta_decode(int64_t n, const int64_t* offs, const int32_t* enc, int32_t* out);

/* Step-header diagnostics: out[0]=E_k, out[1]=max|v|^2, out[2]=N inside the
 * domain, out[3]=sum m*vx, out[4]=sum m*vy. */
void orc_diagnostics(const orc_params* p, int64_t n, const double* x, const double* y,
                     const double* vx, const double* vy, double* out);

/* LatticeCreator: returns the particle count; x/y may be NULL to query it. */
int64_t orc_lattice(double lx, double ly, double dX, double dY, double xvol, double yvol,
                    double* x, double* y);

/* ---- whole simulation state (pre-loop + main loop, app/simulation_configuration.h:168-440) */
typedef struct orc_sim orc_sim;
orc_sim* orc_sim_create(const orc_params* p, int64_t n, const double* x, const double* y,
                        const double* vx, const double* vy);
void orc_sim_destroy(orc_sim* s);
/* FindNeighbors -> density -> pressure -> forces. */
void orc_sim_preloop(orc_sim* s);
/* nsteps iterations of: integrate -> FindNeighbors -> density -> pressure -> forces. */
void orc_sim_steps(orc_sim* s, int64_t nsteps);
/* Copies the current (sorted) state; any pointer may be NULL.  ids[i] is the
 * creation index of the particle now in slot i. */
void orc_sim_get(const orc_sim* s, double* x, double* y, double* vx, double* vy,
                 double* fx, double* fy, double* rho, int32_t* key, int32_t* ids);
/* Overwrites x,y,vx,vy,fx,fy (in the current slot order). */
void orc_sim_set(orc_sim* s, const double* x, const double* y, const double* vx,
                 const double* vy, const double* fx, const double* fy);
int64_t orc_sim_size(const orc_sim* s);
void orc_set_threads(int32_t nthreads);
int32_t orc_get_threads(void);

#ifdef __cplusplus
}
#endif
#endif
