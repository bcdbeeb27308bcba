// ref_harness.cpp -- test-only harness that links the reference's own C++
// classes (compiled from their sources by oracle/Makefile into
// oracle/_ref/libsphref.so) and exposes them through a small C ABI, so the
// CPU restatement in sph_oracle.cpp and the golden fixtures can be checked
// against the reference itself.  Nothing here is part of the product.
//
// Reference classes driven (paths inside jose-pinzon0407/sph-simulations):
//   SoAContainer                      core/container/SoAContainer.{h,cpp}
//   GenericNeighborSearch<Order>      core/alg/GenericNeighborSearch.h
//   GenericForceComputation<Order>    core/compute/GenericForceComputation.{hpp,tpp}
//   GenericNeighborLists<Order>       core/alg/GenericNeighborLists.{hpp,tpp}
//   MultipassNeighborLists<Order>     core/algorithmic/MultipassNeighborLists.h
//   MPListsForceComputation           core/compute/MPListsForceComputation.cpp
//   Integrator                        core/integrator/Integrator.{h,cpp}
//   Codifier                          core/encoders/Encoder.h
//   MeasuringFunctions                core/container/MeasuringFunctions.h
//   LatticeCreator                    core/container/Lattice.h
//   MortonOrder                       core/alg/orders/MortonOrder.h
#include <cstdint>
#include <iostream>
#include <numeric>
#include <vector>

#include "alg/TypesNeighborSearch.h"
#include "alg/GenericNeighborLists.hpp"
#include "algorithmic/MultipassNeighborLists.h"
#include "compute/GenericForceComputation.hpp"
#include "compute/ListsForceComputation.h"
#include "container/Lattice.h"
#include "container/MeasuringFunctions.h"
#include "encoders/Encoder.h"
#include "integrator/Integrator.h"

double sphref_H = 1.0;
double sphref_GAS_CONSTANT = 30.0;
double sphref_RHO_0 = 25.0;
double sphref_MU = 0.01;

namespace {

struct RefBase {
  explicit RefBase(const Domain& d) : domain(d) {}
  virtual ~RefBase() {}
  virtual void find_neighbors(int32_t* perm) = 0;
  virtual void density() = 0;
  virtual void pressure_forces() = 0;
  virtual void integrate() = 0;
  virtual void cell_ranges(int32_t* start, int32_t* end) = 0;
  virtual void grid(int32_t* out) = 0;
  virtual int64_t nlists(int32_t which) = 0;
  virtual void mplists_compute() = 0;
  Domain domain;
  SoAContainer c;
  std::vector<int32_t> ids;
  std::vector<int64_t> offs;
  std::vector<int32_t> idx;
  double dt = 0.0;
};

Domain make_domain(double lox, double loy, double hix, double hiy) {
  Domain d;
  d.l_corner = Vec3d{lox, loy, 0};
  d.h_corner = Vec3d{hix, hiy, 0};
  return d;
}

template <class Order>
struct RefSim : RefBase {
  GenericNeighborSearch<Order> gns;
  GenericForceComputation<Order> comp;
  GenericNeighborLists<Order> lists;
  MultipassNeighborLists<Order> mpl;
  RefSim(const Domain& d, double h, int64_t n)
      : RefBase(d), gns(domain, h), comp(h, gns), lists(h), mpl(h) {
    c.Resize(n);
    ids.resize(n);
    std::iota(ids.begin(), ids.end(), 0);
    for (int64_t i = 0; i < n; ++i) c.SetParticleIndex(i, (uint)i);
  }
  void find_neighbors(int32_t* perm) override {
    // GenericNeighborSearch::FindNeighbors split into its public steps so the
    // permutation chosen by SortParticleIds can be recorded.
    const uint n = (uint)c.Size();
    gns.SetParticleCellIds(c);
    gns.SortParticleIds(c);
    auto& pid = c.GetParticles().particle_id;
    std::vector<int32_t> newids(n);
    for (uint i = 0; i < n; ++i) {
      if (perm) perm[i] = (int32_t)pid[i];
      newids[i] = ids[pid[i]];
    }
    ids.swap(newids);
    gns.SortContainer(c);
    gns.SetCellRanges(n, c);
  }
  void density() override { comp.ApproximateDensity(c); }
  void pressure_forces() override {
    comp.CalculatePressure(c);
    comp.ComputeForces(c);
  }
  void integrate() override {
    Integrator integ{dt, &domain};
    integ.UpdateVelocities(c);
    integ.UpdatePositions(c);
  }
  void cell_ranges(int32_t* start, int32_t* end) override {
    auto& s = gns.GetStart();
    auto& e = gns.GetEnd();
    for (size_t i = 0; i < s.size(); ++i) {
      start[i] = s[i];
      end[i] = e[i];
    }
  }
  void grid(int32_t* out) override {
    out[0] = gns.GetCellsInDirectionX();
    out[1] = gns.GetCellsInDirectionY();
    out[2] = (int32_t)gns.GetTotalCells();
  }
  int64_t nlists(int32_t which) override {
    const int64_t n = (int64_t)c.Size();
    offs.assign(n + 1, 0);
    idx.clear();
    if (which == 0) {  // GenericNeighborLists (vector of vectors)
      lists.AssembleNeighborList(c, gns);
      auto& nl = lists.GetNeighborList();
      for (int64_t i = 0; i < n; ++i) {
        offs[i + 1] = offs[i] + (int64_t)nl[i].size();
        for (int j : nl[i]) idx.push_back(j);
      }
    } else {  // MultipassNeighborLists (CSR)
      mpl.AssembleNeighborList(c, gns);
      auto& o = mpl.GetOffsetPerParticle();
      auto& l = mpl.GetNeighborList();
      for (int64_t i = 0; i <= n; ++i) offs[i] = o[i];
      idx.assign(l.begin(), l.begin() + offs[n]);
    }
    return offs[n];
  }
  void mplists_compute() override {
    mpl.AssembleNeighborList(c, gns);
    MPListsForceComputation mp{sphref_H, mpl.GetNeighborList(), mpl.GetOffsetPerParticle()};
    mp.ApproximateDensity(c);
    mp.CalculatePressure(c);
    mp.ComputeForces(c);
  }
};

}  // namespace

extern "C" {

void* ref_create(int32_t order, double lox, double loy, double hix, double hiy, double h,
                 double k, double rho0, double mu, double dt, int64_t n) {
  std::cout.setstate(std::ios_base::failbit);  // the reference prints a lot
  sphref_H = h;
  sphref_GAS_CONSTANT = k;
  sphref_RHO_0 = rho0;
  sphref_MU = mu;
  Domain d = make_domain(lox, loy, hix, hiy);
  RefBase* r;
  if (order == 0)
    r = new RefSim<MortonOrder>(d, h, n);
  else
    r = new RefSim<RowMajorOrder>(d, h, n);
  r->dt = dt;
  return r;
}

void ref_destroy(void* h) { delete (RefBase*)h; }

void ref_set(void* hnd, const double* x, const double* y, const double* vx, const double* vy,
             const double* fx, const double* fy, const double* rho) {
  RefBase* r = (RefBase*)hnd;
  const int64_t n = (int64_t)r->c.Size();
  for (int64_t i = 0; i < n; ++i) {
    r->c.SetPosition(i, x[i], y[i], 0.0);
    r->c.SetVelocity(i, vx[i], vy[i], 0.0);
    r->c.SetForce(i, fx ? fx[i] : 0.0, fy ? fy[i] : 0.0, 0.0);
    r->c.SetDensity(i, rho ? rho[i] : 0.0);
    r->c.SetParticleIndex(i, (uint)i);
  }
}

void ref_get(void* hnd, double* x, double* y, double* vx, double* vy, double* fx, double* fy,
             double* rho, int32_t* key, int32_t* ids) {
  RefBase* r = (RefBase*)hnd;
  auto& P = r->c.GetParticles();
  const int64_t n = (int64_t)r->c.Size();
  for (int64_t i = 0; i < n; ++i) {
    if (x) x[i] = P.rx[i];
    if (y) y[i] = P.ry[i];
    if (vx) vx[i] = P.vx[i];
    if (vy) vy[i] = P.vy[i];
    if (fx) fx[i] = P.fx[i];
    if (fy) fy[i] = P.fy[i];
    if (rho) rho[i] = P.density[i];
    if (key) key[i] = (int32_t)P.cell_id[i];
    if (ids) ids[i] = r->ids[i];
  }
}

void ref_set_params(double h, double k, double rho0, double mu) {
  sphref_H = h;
  sphref_GAS_CONSTANT = k;
  sphref_RHO_0 = rho0;
  sphref_MU = mu;
}

void ref_find_neighbors(void* h, int32_t* perm) { ((RefBase*)h)->find_neighbors(perm); }
void ref_density(void* h) { ((RefBase*)h)->density(); }
void ref_pressure_forces(void* h) { ((RefBase*)h)->pressure_forces(); }
void ref_integrate(void* h) { ((RefBase*)h)->integrate(); }
void ref_cell_ranges(void* h, int32_t* s, int32_t* e) { ((RefBase*)h)->cell_ranges(s, e); }
void ref_grid(void* h, int32_t* out) { ((RefBase*)h)->grid(out); }

int64_t ref_nlists(void* h, int32_t which) { return ((RefBase*)h)->nlists(which); }
void ref_nlists_get(void* h, int64_t* offs, int32_t* idx) {
  RefBase* r = (RefBase*)h;
  for (size_t i = 0; i < r->offs.size(); ++i) offs[i] = r->offs[i];
  for (size_t i = 0; i < r->idx.size(); ++i) idx[i] = r->idx[i];
}
void ref_mplists_compute(void* h) { ((RefBase*)h)->mplists_compute(); }

void ref_diagnostics(void* hnd, double* out) {
  RefBase* r = (RefBase*)hnd;
  out[0] = ComputeKineticEnergy(r->c);
  out[1] = ComputeMaxVelocity(r->c);
  out[2] = (double)ParticlesInDomain(r->domain, r->c);
}

int32_t ref_morton2d(int32_t x, int32_t y) {
  MortonOrder m;
  return m.MortonCode2d(x, y);
}

void ref_morton_table(int32_t nx, int32_t ny, int32_t* out) {
  // out[cx + nx*cy] = MortonOrder::MortonCode2d(cx, cy)
  MortonOrder m;
  for (int32_t cy = 0; cy < ny; ++cy)
    for (int32_t cx = 0; cx < nx; ++cx) out[cx + (int64_t)nx * cy] = m.MortonCode2d(cx, cy);
}

void ref_encode(int32_t n, const int32_t* list, int32_t* out) {
  Codifier enc;
  enc.Init(1);
  std::vector<int> v(list, list + n);
  enc.Encode(0, v);
  for (int32_t i = 0; i < n; ++i) out[i] = enc.neighbors_per_particle[0][i];
}

int64_t ref_lattice(double lx, double ly, double dX, double dY, double xvol, double yvol,
                    double* x, double* y) {
  std::cout.setstate(std::ios_base::failbit);
  Domain d = make_domain(0, 0, lx, ly);
  SoAContainer c;
  LatticeCreator lat;
  lat.dX = dX;
  lat.dY = dY;
  lat.xVol = xvol;
  lat.yVol = yvol;
  lat.CreateLattice(d, c);
  if (x && y) {
    for (size_t i = 0; i < c.Size(); ++i) {
      x[i] = c.pos(i)[0];
      y[i] = c.pos(i)[1];
    }
  }
  return (int64_t)c.Size();
}

}  // extern "C"
