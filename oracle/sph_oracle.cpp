// sph_oracle.cpp -- test-only CPU restatement of the reference SPH step.
// See sph_oracle.h for the list of reference functions restated and the
// deviations.  Built with -O3 -fopenmp -ffp-contract=off (no fast-math) so the
// results are identical on x86-64 and aarch64 hosts.
#include "sph_oracle.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

struct Consts {  // GenericForceComputation constructor, GenericForceComputation.tpp:5-12
  double h1, h2, h6, dc, pc;
};

Consts make_consts(const orc_params* p) {
  Consts c;
  c.h1 = p->h;
  c.h2 = p->h * p->h;
  c.h6 = c.h2 * c.h2 * c.h2;
  c.dc = 315.0 / (64.0 * M_PI * std::pow(c.h1, 9.0));
  c.pc = 15.0 / (M_PI * std::pow(c.h1, 6.0));
  return c;
}

int next_pow2(int n) {  // MortonOrder::NexPowerOfTwo, MortonOrder.h:82-90
  int power = 1;
  while (power < n) power *= 2;
  return power;
}

inline double min_image(double d, double L) {
  if (d > 0.5 * L) return d - L;
  if (d < -0.5 * L) return d + L;
  return d;
}

// Visits the 3x3 stencil in the reference order (c1 = x offset outer,
// c2 = y offset inner; GenericForceComputation.tpp:56-70) and calls fn(cell).
template <class F>
inline void for_each_stencil_cell(const orc_params* p, const orc_grid* g, int32_t cx,
                                  int32_t cy, F&& fn) {
  for (int c1 = -1; c1 <= 1; ++c1) {
    for (int c2 = -1; c2 <= 1; ++c2) {
      int jx = cx + c1, jy = cy + c2;
      if (p->periodic) {
        jx = (jx + g->nx_real) % g->nx_real;
        jy = (jy + g->ny_real) % g->ny_real;
      } else {
        if (jx < 0 || jx >= g->nx) continue;
        if (jy < 0 || jy >= g->ny) continue;
      }
      fn(orc_flatten(p, g, jx, jy));
    }
  }
}

inline void pair_delta(const orc_params* p, double xi, double yi, double xj, double yj,
                       double* dx, double* dy) {
  *dx = xi - xj;
  *dy = yi - yj;
  if (p->periodic) {
    *dx = min_image(*dx, p->hi[0] - p->lo[0]);
    *dy = min_image(*dy, p->hi[1] - p->lo[1]);
  }
}

}  // namespace

extern "C" {

void orc_default_params(orc_params* p) {
  // core/ConfigVariables.hpp:9-15 and config/example.txt defaults
  p->h = 1.0;
  p->dt = 0.005;
  p->k = 30.0;
  p->rho0 = 25.0;
  p->mu = 0.01;
  p->tol = 1.0e-12;
  p->gx = 0.0;
  p->gy = -10.0;
  p->mass = 1.0;
  p->alpha = 0.0;
  p->c0 = std::sqrt(30.0);
  p->lo[0] = 0.0;
  p->lo[1] = 0.0;
  p->hi[0] = 96.0;
  p->hi[1] = 48.0;
  p->order = 1;
  p->periodic = 0;
}

void orc_grid_init(const orc_params* p, orc_grid* g) {
  // MortonOrder::Initialize (MortonOrder.h:11-43) / RowMajorOrder::Initialize (RowMajorOrder.h:12-25)
  for (int a = 0; a < 2; ++a) {
    double L = p->hi[a] - p->lo[a];
    int n;
    double cs;
    if (p->periodic) {
      n = (int)std::floor(L / p->h);
      if (n < 3) n = 3;
      cs = L / n;
    } else {
      cs = p->h;
      n = (int)std::ceil(L / cs);
    }
    g->cs[a] = cs;
    if (a == 0) g->nx_real = n; else g->ny_real = n;
  }
  g->nx = g->nx_real;
  g->ny = g->ny_real;
  if (p->order == 0) {  // AddCellPadding, MortonOrder.h:92-103
    g->nx = next_pow2(g->nx);
    g->ny = next_pow2(g->ny);
  }
  g->ncells = (int64_t)g->nx * g->ny;
}

int32_t orc_morton2d(int32_t x, int32_t y) {
  // MortonOrder::MortonCode2d, MortonOrder.h:117-126
  int z = 0;
  for (int i = 0; i < 21; ++i) {
    z |= (int)((x >> i) & 1) << (2 * i);
    z |= (int)((y >> i) & 1) << (2 * i + 1);
  }
  return z;
}

int32_t orc_flatten(const orc_params* p, const orc_grid* g, int32_t cx, int32_t cy) {
  if (p->order == 0) return orc_morton2d(cx, cy);
  return cx + cy * g->nx;  // RowMajorOrder::MapThreeToOne, RowMajorOrder.h:48-50
}

void orc_unflatten(const orc_params* p, const orc_grid* g, int32_t key, int32_t* cx,
                   int32_t* cy) {
  if (p->order == 0) {  // inverse of MortonCode2d (the cell_x/cell_y tables, MortonOrder.h:31-39)
    int32_t x = 0, y = 0;
    for (int i = 0; i < 16; ++i) {
      x |= ((key >> (2 * i)) & 1) << i;
      y |= ((key >> (2 * i + 1)) & 1) << i;
    }
    *cx = x;
    *cy = y;
    return;
  }
  *cx = key % g->nx;  // RowMajorOrder::MapOneToThree, RowMajorOrder.h:52-59
  *cy = (key / g->nx) % g->ny;
}

void orc_cell_ids(const orc_params* p, const orc_grid* g, int64_t n, const double* x,
                  const double* y, int32_t* key) {
  // GenericNeighborSearch::SetParticleCellIds, GenericNeighborSearch.h:201-231
  const int xmax = p->periodic ? g->nx_real - 1 : g->nx - 1;
  const int ymax = p->periodic ? g->ny_real - 1 : g->ny - 1;
#pragma omp parallel for schedule(runtime)
  for (int64_t i = 0; i < n; ++i) {
    int ci0 = (int)std::floor((x[i] - p->lo[0]) / g->cs[0]);
    int ci1 = (int)std::floor((y[i] - p->lo[1]) / g->cs[1]);
    ci0 = std::min(ci0, xmax);
    ci1 = std::min(ci1, ymax);
    ci0 = std::max(ci0, 0);
    ci1 = std::max(ci1, 0);
    key[i] = orc_flatten(p, g, ci0, ci1);
  }
}

void orc_sort_perm(int64_t n, const int32_t* key, int32_t* perm) {
  // SortParticleIds, GenericNeighborSearch.h:69-76 (made stable)
  std::iota(perm, perm + n, 0);
  std::stable_sort(perm, perm + n, [key](int32_t a, int32_t b) { return key[a] < key[b]; });
}

void orc_gather_f64(int64_t n, const int32_t* perm, const double* in, double* out) {
  for (int64_t i = 0; i < n; ++i) out[i] = in[perm[i]];
}

void orc_gather_i32(int64_t n, const int32_t* perm, const int32_t* in, int32_t* out) {
  for (int64_t i = 0; i < n; ++i) out[i] = in[perm[i]];
}

void orc_cell_ranges(const orc_grid* g, int64_t n, const int32_t* k, int32_t* start,
                     int32_t* end) {
  // SetCellRanges + RefillCellRanges, GenericNeighborSearch.h:93-108, MortonOrder.h:60-63
  std::fill(start, start + g->ncells, -1);
  std::fill(end, end + g->ncells, -1);
  for (int64_t i = 0; i < n; ++i) {
    int32_t c = k[i];
    if (i == 0 || c != k[i - 1]) start[c] = (int32_t)i;
    if (i == n - 1 || c != k[i + 1]) end[c] = (int32_t)(i + 1);
  }
}

void orc_density(const orc_params* p, const orc_grid* g, int64_t n, const double* x,
                 const double* y, const int32_t* key, const int32_t* start,
                 const int32_t* end, double* rho) {
  // GenericForceComputation::ApproximateDensity, GenericForceComputation.tpp:35-130
  const Consts c = make_consts(p);
  const double mass = p->mass;
#pragma omp parallel for schedule(runtime)
  for (int64_t i = 0; i < n; ++i) {
    double accum = 0.0;
    int32_t cx, cy;
    orc_unflatten(p, g, key[i], &cx, &cy);
    for_each_stencil_cell(p, g, cx, cy, [&](int32_t cell) {
      int32_t s = start[cell], e = end[cell];
      if (s < 0 || e < 0) return;
      for (int32_t j = s; j < e; ++j) {
        double dx, dy;
        pair_delta(p, x[i], y[i], x[j], y[j], &dx, &dy);
        double dz = 0.0;
        double r2 = dx * dx + dy * dy + dz * dz;
        if (r2 > c.h2) continue;
        accum += c.dc * (c.h2 - r2) * (c.h2 - r2) * (c.h2 - r2) * mass;
      }
    });
    rho[i] = accum;
  }
}

void orc_pressure(const orc_params* p, int64_t n, const double* rho, double* pr) {
  // CalculatePressure, GenericForceComputation.tpp:23-32
  for (int64_t i = 0; i < n; ++i) pr[i] = p->k * (rho[i] - p->rho0);
}

namespace {
// Per-pair contribution shared by the cell-stencil and list variants
// (GenericForceComputation.tpp:209-236 / MPListsForceComputation.cpp:80-110).
struct ForceAcc {
  double fpx = 0, fpy = 0, fvx = 0, fvy = 0, fax = 0, fay = 0;
};

inline void pair_force(const orc_params* p, const Consts& c, double dx, double dy,
                       double r2, double pi_, double rho_i, double pj, double rho_j,
                       double vix, double viy, double vjx, double vjy, ForceAcc& a) {
  const double mu = p->mu;
  const double mass = p->mass;
  double r1 = std::sqrt(r2);
  if (r1 > p->tol) {
    double pm = -0.5 * (pi_ / (rho_i * rho_i) + pj / (rho_j * rho_j)) * mass;
    double h_r12 = (c.h1 - r1) * (c.h1 - r1);
    a.fpx += -3.0 * c.pc * h_r12 / r1 * dx * pm;
    a.fpy += -3.0 * c.pc * h_r12 / r1 * dy * pm;
  }
  double dvx = vjx - vix;
  double dvy = vjy - viy;
  double vm = mu / (rho_j * M_PI * c.h6) * 45.0 * (c.h1 - r1) * mass;
  a.fvx += vm * dvx;
  a.fvy += vm * dvy;
  if (p->alpha > 0.0 && r1 > p->tol) {
    // Monaghan artificial viscosity (extension): a_i -= m * Pi_ij * grad_i W_spiky.
    double vr = (vix - vjx) * dx + (viy - vjy) * dy;
    if (vr < 0.0) {
      double muij = c.h1 * vr / (r2 + 0.01 * c.h2);
      double pij = -p->alpha * p->c0 * muij / (0.5 * (rho_i + rho_j));
      double s = 3.0 * c.pc * (c.h1 - r1) * (c.h1 - r1) / r1 * pij * mass;
      a.fax += s * dx;
      a.fay += s * dy;
    }
  }
}
}  // namespace

void orc_forces(const orc_params* p, const orc_grid* g, int64_t n, const double* x,
                const double* y, const double* vx, const double* vy, const double* rho,
                const double* pr, const int32_t* key, const int32_t* start,
                const int32_t* end, double* fx, double* fy) {
  // GenericForceComputation::ComputeForces, GenericForceComputation.tpp:134-253
  const Consts c = make_consts(p);
#pragma omp parallel for schedule(runtime)
  for (int64_t i = 0; i < n; ++i) {
    int32_t cx, cy;
    orc_unflatten(p, g, key[i], &cx, &cy);
    ForceAcc a;
    const double vix = vx[i], viy = vy[i], rho_i = rho[i];
    for_each_stencil_cell(p, g, cx, cy, [&](int32_t cell) {
      int32_t s = start[cell], e = end[cell];
      if (s < 0 || e < 0) return;
      for (int32_t j = s; j < e; ++j) {
        if (j == i) continue;
        double dx, dy;
        pair_delta(p, x[i], y[i], x[j], y[j], &dx, &dy);
        double dz = 0.0;
        double r2 = dx * dx + dy * dy + dz * dz;
        if (r2 > c.h2) continue;
        pair_force(p, c, dx, dy, r2, pr[i], rho_i, pr[j], rho[j], vix, viy, vx[j], vy[j], a);
      }
    });
    double fxi = p->gx, fyi = p->gy;
    fxi += a.fpx;
    fyi += a.fpy;
    fxi += a.fvx;
    fyi += a.fvy;
    if (p->alpha > 0.0) {
      fxi += a.fax;
      fyi += a.fay;
    }
    fx[i] = fxi;
    fy[i] = fyi;
  }
}

void orc_integrate(const orc_params* p, int64_t n, double* x, double* y, double* vx,
                   double* vy, const double* fx, const double* fy) {
  // Integrator::UpdateVelocities / UpdatePositions / ApplyBoundaryConditions,
  // Integrator.cpp:7-46 and SoAContainer.cpp:109-111,128-131
  const double dt = p->dt;
  for (int64_t i = 0; i < n; ++i) {
    vx[i] += dt * fx[i];
    vy[i] += dt * fy[i];
  }
  for (int64_t i = 0; i < n; ++i) {
    double r[2] = {x[i] + dt * vx[i], y[i] + dt * vy[i]};
    double v[2] = {vx[i], vy[i]};
    for (int a = 0; a < 2; ++a) {
      if (p->periodic) {
        double L = p->hi[a] - p->lo[a];
        if (r[a] >= p->hi[a]) r[a] -= L;
        if (r[a] < p->lo[a]) r[a] += L;
        continue;
      }
      if (r[a] > p->hi[a]) {
        r[a] = p->hi[a];
        v[a] *= -1;
      }
      if (r[a] < p->lo[a]) {
        r[a] = p->lo[a];
        v[a] *= -1;
      }
    }
    x[i] = r[0];
    y[i] = r[1];
    vx[i] = v[0];
    vy[i] = v[1];
  }
}

int64_t orc_nlist_count(const orc_params* p, const orc_grid* g, int64_t n, const double* x,
                        const double* y, const int32_t* key, const int32_t* start,
                        const int32_t* end, int32_t* counts, int64_t* offs) {
  // MultipassNeighborLists::CountNeighborsPerParticle + CalculateOffsets,
  // MultipassNeighborLists.h:47-121
  const double h2 = p->h * p->h;
#pragma omp parallel for schedule(runtime)
  for (int64_t i = 0; i < n; ++i) {
    int32_t cx, cy, cnt = 0;
    orc_unflatten(p, g, key[i], &cx, &cy);
    for_each_stencil_cell(p, g, cx, cy, [&](int32_t cell) {
      int32_t s = start[cell], e = end[cell];
      if (s < 0 || e < 0) return;
      for (int32_t j = s; j < e; ++j) {
        double dx, dy;
        pair_delta(p, x[i], y[i], x[j], y[j], &dx, &dy);
        double dz = 0.0;
        double r2 = dx * dx + dy * dy + dz * dz;
        if (r2 > h2) continue;
        ++cnt;
      }
    });
    counts[i] = cnt;
  }
  offs[0] = 0;
  for (int64_t i = 0; i < n; ++i) offs[i + 1] = offs[i] + counts[i];
  return offs[n];
}

void orc_nlist_fill(const orc_params* p, const orc_grid* g, int64_t n, const double* x,
                    const double* y, const int32_t* key, const int32_t* start,
                    const int32_t* end, const int64_t* offs, int32_t* idx) {
  // MultipassNeighborLists::AssignIndices, MultipassNeighborLists.h:123-181
  // (same order as GenericNeighborLists::AssembleNeighborList, GenericNeighborLists.tpp:10-81)
  const double h2 = p->h * p->h;
#pragma omp parallel for schedule(runtime)
  for (int64_t i = 0; i < n; ++i) {
    int32_t cx, cy;
    int64_t o = offs[i];
    orc_unflatten(p, g, key[i], &cx, &cy);
    for_each_stencil_cell(p, g, cx, cy, [&](int32_t cell) {
      int32_t s = start[cell], e = end[cell];
      if (s < 0 || e < 0) return;
      for (int32_t j = s; j < e; ++j) {
        double dx, dy;
        pair_delta(p, x[i], y[i], x[j], y[j], &dx, &dy);
        double dz = 0.0;
        double r2 = dx * dx + dy * dy + dz * dz;
        if (r2 > h2) continue;
        idx[o++] = j;
      }
    });
  }
}

void orc_density_lists(const orc_params* p, int64_t n, const double* x, const double* y,
                       const int64_t* offs, const int32_t* idx, double* rho) {
  // MPListsForceComputation::ApproximateDensity, MPListsForceComputation.cpp:3-38
  const Consts c = make_consts(p);
  const double mass = p->mass;
#pragma omp parallel for schedule(runtime)
  for (int64_t i = 0; i < n; ++i) {
    double accum = 0.0;
    for (int64_t q = offs[i]; q < offs[i + 1]; ++q) {
      int32_t j = idx[q];
      double dx, dy;
      pair_delta(p, x[i], y[i], x[j], y[j], &dx, &dy);
      double dz = 0.0;
      double r2 = dx * dx + dy * dy + dz * dz;
      accum += c.dc * (c.h2 - r2) * (c.h2 - r2) * (c.h2 - r2) * mass;
    }
    rho[i] = accum;
  }
}

void orc_forces_lists(const orc_params* p, int64_t n, const double* x, const double* y,
                      const double* vx, const double* vy, const double* rho,
                      const double* pr, const int64_t* offs, const int32_t* idx,
                      double* fx, double* fy) {
  // MPListsForceComputation::ComputeForces, MPListsForceComputation.cpp:58-147
  // (the list holds the particle itself; its pair adds zero)
  const Consts c = make_consts(p);
#pragma omp parallel for schedule(runtime)
  for (int64_t i = 0; i < n; ++i) {
    ForceAcc a;
    for (int64_t q = offs[i]; q < offs[i + 1]; ++q) {
      int32_t j = idx[q];
      double dx, dy;
      pair_delta(p, x[i], y[i], x[j], y[j], &dx, &dy);
      double dz = 0.0;
      double r2 = dx * dx + dy * dy + dz * dz;
      pair_force(p, c, dx, dy, r2, pr[i], rho[i], pr[j], rho[j], vx[i], vy[i], vx[j], vy[j], a);
    }
    double fxi = p->gx, fyi = p->gy;
    fxi += a.fpx;
    fyi += a.fpy;
    fxi += a.fvx;
    fyi += a.fvy;
    if (p->alpha > 0.0) {
      fxi += a.fax;
      fyi += a.fay;
    }
    fx[i] = fxi;
    fy[i] = fyi;
  }
}

void orc_delta_encode(int64_t n, const int64_t* offs, const int32_t* idx, int32_t* out) {
  // Codifier::Encode, Encoder.h:27-44 (first index verbatim, then idx[k]-idx[k-1]-1)
  for (int64_t i = 0; i < n; ++i) {
    int64_t b = offs[i], e = offs[i + 1];
    if (b == e) continue;
    out[b] = idx[b];
    for (int64_t q = b + 1; q < e; ++q) out[q] = idx[q] - idx[q - 1] - 1;
  }
}

void orc_delta_decode(int64_t n, const int64_t* offs, const int32_t* enc, int32_t* out) {
  for (int64_t i = 0; i < n; ++i) {
    int64_t b = offs[i], e = offs[i + 1];
    if (b == e) continue;
    out[b] = enc[b];
    for (int64_t q = b + 1; q < e; ++q) out[q] = out[q - 1] + enc[q] + 1;
  }
}

void orc_diagnostics(const orc_params* p, int64_t n, const double* x, const double* y,
                     const double* vx, const double* vy, double* out) {
  // ComputeKineticEnergy / ComputeMaxVelocity / ParticlesInDomain, MeasuringFunctions.h:5-61
  double ek = 0.0, vmax = 0.0, px = 0.0, py = 0.0;
  int64_t inside = 0;
  const double m = p->mass;
  for (int64_t i = 0; i < n; ++i) {
    double n2 = 0.0;
    n2 += vx[i] * vx[i];
    n2 += vy[i] * vy[i];
    n2 += 0.0 * 0.0;
    ek += 0.5 * n2 * m;
    vmax = std::max(n2, vmax);
    px += m * vx[i];
    py += m * vy[i];
    bool in = std::isfinite(x[i]) && std::isfinite(y[i]) && !(x[i] < p->lo[0] || x[i] > p->hi[0]) &&
              !(y[i] < p->lo[1] || y[i] > p->hi[1]);
    inside += in ? 1 : 0;
  }
  out[0] = ek;
  out[1] = vmax;
  out[2] = (double)inside;
  out[3] = px;
  out[4] = py;
}

int64_t orc_lattice(double lx, double ly, double dX, double dY, double xvol, double yvol,
                    double* x, double* y) {
  // LatticeCreator::CreateLattice, Lattice.h:12-35 (z extent 0 -> one layer)
  int nx = (int)std::ceil(xvol * lx / dX) + 1;
  int ny = (int)((double)std::ceil(yvol * ly / dY) + 1);
  int64_t n = (int64_t)nx * ny;
  if (x && y) {
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        int64_t idx = i + (int64_t)nx * j;
        x[idx] = dX * i;
        y[idx] = dY * j;
      }
  }
  return n;
}

// ---------------------------------------------------------------------------
struct orc_sim {
  orc_params p;
  orc_grid g;
  int64_t n;
  std::vector<double> x, y, vx, vy, fx, fy, rho, pr, tmp;
  std::vector<int32_t> key, ids, perm, itmp, start, end;
};

static void sim_find_neighbors(orc_sim* s) {
  // GenericNeighborSearch::FindNeighbors, GenericNeighborSearch.h:16-21
  const int64_t n = s->n;
  orc_cell_ids(&s->p, &s->g, n, s->x.data(), s->y.data(), s->key.data());
  orc_sort_perm(n, s->key.data(), s->perm.data());
  auto g64 = [&](std::vector<double>& a) {
    orc_gather_f64(n, s->perm.data(), a.data(), s->tmp.data());
    a.swap(s->tmp);
  };
  auto g32 = [&](std::vector<int32_t>& a) {
    orc_gather_i32(n, s->perm.data(), a.data(), s->itmp.data());
    a.swap(s->itmp);
  };
  g64(s->rho);
  g64(s->x);
  g64(s->y);
  g64(s->vx);
  g64(s->vy);
  g64(s->fx);
  g64(s->fy);
  g32(s->key);
  g32(s->ids);
  orc_cell_ranges(&s->g, n, s->key.data(), s->start.data(), s->end.data());
}

static void sim_compute(orc_sim* s) {
  const int64_t n = s->n;
  orc_density(&s->p, &s->g, n, s->x.data(), s->y.data(), s->key.data(), s->start.data(),
              s->end.data(), s->rho.data());
  orc_pressure(&s->p, n, s->rho.data(), s->pr.data());
  orc_forces(&s->p, &s->g, n, s->x.data(), s->y.data(), s->vx.data(), s->vy.data(),
             s->rho.data(), s->pr.data(), s->key.data(), s->start.data(), s->end.data(),
             s->fx.data(), s->fy.data());
}

orc_sim* orc_sim_create(const orc_params* p, int64_t n, const double* x, const double* y,
                        const double* vx, const double* vy) {
  orc_sim* s = new orc_sim();
  s->p = *p;
  orc_grid_init(p, &s->g);
  s->n = n;
  s->x.assign(x, x + n);
  s->y.assign(y, y + n);
  s->vx.assign(vx, vx + n);
  s->vy.assign(vy, vy + n);
  s->fx.assign(n, 0.0);
  s->fy.assign(n, 0.0);
  s->rho.assign(n, 0.0);
  s->pr.assign(n, 0.0);
  s->tmp.assign(n, 0.0);
  s->key.assign(n, 0);
  s->perm.assign(n, 0);
  s->itmp.assign(n, 0);
  s->ids.resize(n);
  std::iota(s->ids.begin(), s->ids.end(), 0);
  s->start.assign(s->g.ncells, -1);
  s->end.assign(s->g.ncells, -1);
  return s;
}

void orc_sim_destroy(orc_sim* s) { delete s; }

void orc_sim_preloop(orc_sim* s) {
  // PreLoopComputation, app/simulation_configuration.h:168-204
  sim_find_neighbors(s);
  sim_compute(s);
}

void orc_sim_steps(orc_sim* s, int64_t nsteps) {
  // MainLoopComputation, app/simulation_configuration.h:390-440 (without I/O)
  for (int64_t it = 0; it < nsteps; ++it) {
    orc_integrate(&s->p, s->n, s->x.data(), s->y.data(), s->vx.data(), s->vy.data(),
                  s->fx.data(), s->fy.data());
    sim_find_neighbors(s);
    sim_compute(s);
  }
}

void orc_sim_get(const orc_sim* s, double* x, double* y, double* vx, double* vy, double* fx,
                 double* fy, double* rho, int32_t* key, int32_t* ids) {
  const int64_t n = s->n;
  auto cp = [n](double* dst, const std::vector<double>& src) {
    if (dst) std::memcpy(dst, src.data(), n * sizeof(double));
  };
  cp(x, s->x);
  cp(y, s->y);
  cp(vx, s->vx);
  cp(vy, s->vy);
  cp(fx, s->fx);
  cp(fy, s->fy);
  cp(rho, s->rho);
  if (key) std::memcpy(key, s->key.data(), n * sizeof(int32_t));
  if (ids) std::memcpy(ids, s->ids.data(), n * sizeof(int32_t));
}

void orc_sim_set(orc_sim* s, const double* x, const double* y, const double* vx,
                 const double* vy, const double* fx, const double* fy) {
  const int64_t n = s->n;
  s->x.assign(x, x + n);
  s->y.assign(y, y + n);
  s->vx.assign(vx, vx + n);
  s->vy.assign(vy, vy + n);
  s->fx.assign(fx, fx + n);
  s->fy.assign(fy, fy + n);
}

int64_t orc_sim_size(const orc_sim* s) { return s->n; }

void orc_set_threads(int32_t nthreads) {
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
  omp_set_schedule(omp_sched_static, 0);
#else
  (void)nthreads;
#endif
}

int32_t orc_get_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

}  // extern "C"
