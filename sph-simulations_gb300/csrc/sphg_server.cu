// sphg_server.cu -- continuous batching of independent SPH simulations.
//
// A server owns one device arena sized from an HBM budget.  Requests (an
// initial state, its parameters and a step count) wait in a FIFO queue.  Each
// tick:
//   1. admits queued requests, in order, while the live set still fits the
//      arena (particles, cell keys, instances);
//   2. when the live set changed, repacks it densely: retained instances' next
//      states are copied device to device into a staging area, newcomers'
//      initial states are uploaded into it from pinned host memory, the new
//      instance layout is made current and one gather kernel writes every live
//      particle to its new slot with its cell key moved to the instance's new
//      key range;
//   3. runs one batched main-loop iteration over every live instance (a
//      newcomer's first iteration is its pre-loop), with the per-instance
//      descriptor kernels for every batch size, so an instance computes the
//      same bits whatever else is live;
//   4. retires instances that ran their `steps` iterations: their state is
//      downloaded and kept until the caller fetches it.
// Latency of a request = completion time - submission time (steady clock).
#include <algorithm>
#include <chrono>
#include <cmath>
#include <deque>
#include <map>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "sphg_internal.cuh"

using namespace sphg_detail;

namespace {

struct RepackEntry {
  int64_t src_begin;  // first staged particle of the instance
  uint32_t key_delta; // added to the staged key (new cell base - old one)
  uint32_t pad;
};

__global__ void repack_kernel(int64_t n, int ninst, const int32_t* __restrict__ begins,
                              const RepackEntry* __restrict__ tab,
                              const float2* __restrict__ spos, const float2* __restrict__ svel,
                              const uint32_t* __restrict__ skey, const int32_t* __restrict__ sids,
                              float2* __restrict__ pos, float2* __restrict__ vel,
                              uint32_t* __restrict__ key, int32_t* __restrict__ ids) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int inst = sphg::find_instance(begins, ninst, (int)i);
  const RepackEntry e = tab[inst];
  const int64_t src = e.src_begin + (i - begins[inst]);
  pos[i] = spos[src];
  vel[i] = svel[src];
  key[i] = skey[src] + e.key_delta;
  if (ids) ids[i] = sids[src];
}

struct SrvReq {
  int64_t id = 0;
  sphg_params p{};
  int64_t n = 0, steps = 0, runs = 0;
  std::vector<double> x, y, vx, vy;           // initial state until admitted (host arrays) ...
  bool lattice = false;                        // ... or generated on the device at admission
  sphg_lattice spec{};
  std::vector<double> rx, ry, rvx, rvy, rrho;  // result once done
  std::vector<int32_t> rids;
  double t_submit = 0, t_done = 0;
  int state = 0;  // 0 queued, 1 live, 2 done
  int64_t begin = 0;
  uint32_t cell_base = 0;
};

double now_s(const std::chrono::steady_clock::time_point& t0) {
  return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

}  // namespace

struct sphg_server {
  sphg_sim* sim = nullptr;
  std::map<int64_t, SrvReq> reqs;
  std::deque<int64_t> queue;
  std::vector<int64_t> live;  // in layout order
  bool dirty = false;         // the live set changed since the last repack
  int64_t next_id = 1;
  double particle_steps = 0;
  int64_t ticks = 0, completed = 0;
  std::chrono::steady_clock::time_point t0 = std::chrono::steady_clock::now();
  float2 *hpos = nullptr, *hvel = nullptr;
  uint32_t* hkey = nullptr;
  int32_t* hids = nullptr;
  size_t hcap = 0;
  RepackEntry* htab = nullptr;
  RepackEntry* dtab = nullptr;
};

namespace {

sphg_status grow_staging(sphg_server* s, size_t n) {
  if (n <= s->hcap) return SPHG_OK;
  cudaFreeHost(s->hpos);
  cudaFreeHost(s->hvel);
  cudaFreeHost(s->hkey);
  cudaFreeHost(s->hids);
  s->hpos = s->hvel = nullptr;
  s->hkey = nullptr;
  s->hids = nullptr;
  s->hcap = 0;
  size_t cap = std::max(n, (size_t)1 << 20);
  if (cudaMallocHost((void**)&s->hpos, cap * sizeof(float2)) != cudaSuccess ||
      cudaMallocHost((void**)&s->hvel, cap * sizeof(float2)) != cudaSuccess ||
      cudaMallocHost((void**)&s->hkey, cap * sizeof(uint32_t)) != cudaSuccess ||
      cudaMallocHost((void**)&s->hids, cap * sizeof(int32_t)) != cudaSuccess)
    return fail(SPHG_OOM, "pinned staging buffers for admissions");
  s->hcap = cap;
  return SPHG_OK;
}

// Device representation of a newcomer's initial state: positions (plain: FP32
// position; split: FP32 offset in the cell), velocities, instance-local cell
// codes computed exactly as the key kernel would, creation indices.
void stage_newcomer(sphg_server* s, const SrvReq& r, const InstDesc& d, size_t at) {
  const sphg_sim* sim = s->sim;
  const int cmx = d.periodic ? d.nxr - 1 : d.nx - 1;
  const int cmy = d.periodic ? d.nyr - 1 : d.ny - 1;
  parallel_for(r.n, [&](int64_t b, int64_t e) {
  for (int64_t i = b; i < e; ++i) {
    int cx, cy;
    float2 pos;
    if (sim->opt.precision == SPHG_PRECISION_SPLIT) {
      cx = host_cell(r.x[i], d.lo_xd, d.cs_xd, cmx);
      cy = host_cell(r.y[i], d.lo_yd, d.cs_yd, cmy);
      pos = make_float2(split_offset((r.x[i] - d.lo_xd) - cx * d.cs_xd, d.cs_xd),
                        split_offset((r.y[i] - d.lo_yd) - cy * d.cs_yd, d.cs_yd));
    } else {
      const float fx = (float)r.x[i], fy = (float)r.y[i];
      cx = host_cell((double)fx, d.lo_xd, d.cs_xd, cmx);
      cy = host_cell((double)fy, d.lo_yd, d.cs_yd, cmy);
      pos = make_float2(fx, fy);
    }
    s->hpos[at + i] = pos;
    s->hvel[at + i] = make_float2((float)r.vx[i], (float)r.vy[i]);
    s->hkey[at + i] = d.order == 0 ? morton_host((uint32_t)cx, (uint32_t)cy) : (uint32_t)(cx + cy * d.nx);
    s->hids[at + i] = (int32_t)i;
  }
  });
}

// Layout of a candidate live list (fails with SPHG_CAPACITY when it does not fit).
sphg_status layout_of(sphg_server* s, const std::vector<int64_t>& ids, Layout& L,
                      std::vector<sphg_params>& p, std::vector<int64_t>& counts) {
  p.clear();
  counts.clear();
  for (int64_t id : ids) {
    const SrvReq& r = s->reqs[id];
    p.push_back(r.p);
    counts.push_back(r.n);
  }
  if ((int)ids.size() > s->sim->cap_inst) return fail(SPHG_CAPACITY, "instance slots full");
  if (ids.empty()) {
    L = Layout();
    return SPHG_OK;
  }
  SPHG_TRY(compute_layout(s->sim, (int)ids.size(), p.data(), counts.data(), s->sim->cap_keys, L));
  if ((size_t)L.n > s->sim->cap_n) return fail(SPHG_CAPACITY, "particle capacity full");
  return SPHG_OK;
}

sphg_status repack(sphg_server* s, const std::vector<int64_t>& newlive, size_t nadmit,
                   cudaStream_t st) {
  sphg_sim* sim = s->sim;
  Layout L;
  std::vector<sphg_params> p;
  std::vector<int64_t> counts;
  SPHG_TRY(layout_of(s, newlive, L, p, counts));
  const int64_t n_old = sim->n;
  // 1. retained instances' next states -> staging (the sorted-state buffers are free now)
  if (n_old > 0) {
    SPHG_CUDA(cudaMemcpyAsync(sim->posA, sim->posB, n_old * sizeof(float2), cudaMemcpyDeviceToDevice, st));
    SPHG_CUDA(cudaMemcpyAsync(sim->acc, sim->velB, n_old * sizeof(float2), cudaMemcpyDeviceToDevice, st));
    SPHG_CUDA(cudaMemcpyAsync(sim->keyTmp, sim->keyB, n_old * sizeof(uint32_t), cudaMemcpyDeviceToDevice, st));
    if (sim->opt.track_ids)
      SPHG_CUDA(cudaMemcpyAsync(sim->idsA, sim->idsB, n_old * sizeof(int32_t), cudaMemcpyDeviceToDevice, st));
  }
  // 2. newcomers (the last nadmit entries of newlive) -> pinned staging -> device staging
  size_t nnew = 0;
  for (size_t k = newlive.size() - nadmit; k < newlive.size(); ++k) nnew += s->reqs[newlive[k]].n;
  if ((size_t)n_old + nnew > sim->cap_n) return fail(SPHG_CAPACITY, "staging exceeds the particle capacity");
  SPHG_TRY(grow_staging(s, nnew));
  std::vector<int64_t> src(newlive.size());
  size_t at = 0;
  for (size_t k = 0; k < newlive.size(); ++k) {
    SrvReq& r = s->reqs[newlive[k]];
    if (k < newlive.size() - nadmit) {
      src[k] = r.begin;
    } else {
      if (!r.lattice) stage_newcomer(s, r, L.desc[k], at);
      src[k] = n_old + (int64_t)at;
      at += r.n;
    }
  }
  if (nnew) {
    SPHG_CUDA(cudaMemcpyAsync(sim->posA + n_old, s->hpos, nnew * sizeof(float2), cudaMemcpyHostToDevice, st));
    SPHG_CUDA(cudaMemcpyAsync(sim->acc + n_old, s->hvel, nnew * sizeof(float2), cudaMemcpyHostToDevice, st));
    SPHG_CUDA(cudaMemcpyAsync(sim->keyTmp + n_old, s->hkey, nnew * sizeof(uint32_t), cudaMemcpyHostToDevice, st));
    if (sim->opt.track_ids)
      SPHG_CUDA(cudaMemcpyAsync(sim->idsA + n_old, s->hids, nnew * sizeof(int32_t), cudaMemcpyHostToDevice, st));
    // lattice requests: generated in place on the device (after the copies above)
    size_t off = 0;
    for (size_t k = newlive.size() - nadmit; k < newlive.size(); ++k) {
      const SrvReq& r = s->reqs[newlive[k]];
      if (r.lattice)
        SPHG_CUDA(sphg::launch_lattice_stage(L.desc[k], r.spec, sim->opt.precision, r.n, sim->posA + n_old + off,
                                             sim->acc + n_old + off, sim->keyTmp + n_old + off,
                                             sim->opt.track_ids ? sim->idsA + n_old + off : nullptr, st));
      off += r.n;
    }
  }
  // 3. new layout + gather table, then the gather
  SPHG_TRY(apply_layout(sim, (int)newlive.size(), p.data(), counts.data(), L, &st));
  for (size_t k = 0; k < newlive.size(); ++k) {
    SrvReq& r = s->reqs[newlive[k]];
    const bool retained = k < newlive.size() - nadmit;
    s->htab[k].src_begin = src[k];
    s->htab[k].key_delta = L.desc[k].cell_base - (retained ? r.cell_base : 0u);
    r.begin = L.begins[k];
    r.cell_base = L.desc[k].cell_base;
  }
  if (!newlive.empty()) {
    SPHG_CUDA(cudaMemcpyAsync(s->dtab, s->htab, newlive.size() * sizeof(RepackEntry), cudaMemcpyHostToDevice, st));
    const unsigned g = (unsigned)((L.n + 255) / 256);
    repack_kernel<<<g, 256, 0, st>>>(L.n, (int)newlive.size(), sim->dbegins, s->dtab, sim->posA, sim->acc,
                                     sim->keyTmp, sim->idsA, sim->posB, sim->velB, sim->keyB,
                                     sim->opt.track_ids ? sim->idsB : nullptr);
    SPHG_CUDA(cudaGetLastError());
  }
  // the host arrays used by the copies must outlive them
  SPHG_CUDA(cudaStreamSynchronize(st));
  return SPHG_OK;
}

sphg_status retire(sphg_server* s, SrvReq& r, cudaStream_t st) {
  sphg_sim* sim = s->sim;
  const int64_t n = r.n, b = r.begin;
  std::vector<float2> pos(n);
  std::vector<float4> velp(n);
  std::vector<float> rho(n);
  std::vector<uint32_t> key(n);
  std::vector<int32_t> ids(n, -1);
  if (n > 0) {
    SPHG_CUDA(cudaMemcpyAsync(pos.data(), sim->posA + b, n * sizeof(float2), cudaMemcpyDeviceToHost, st));
    SPHG_CUDA(cudaMemcpyAsync(velp.data(), sim->velpA + b, n * sizeof(float4), cudaMemcpyDeviceToHost, st));
    SPHG_CUDA(cudaMemcpyAsync(rho.data(), sim->rho + b, n * sizeof(float), cudaMemcpyDeviceToHost, st));
    SPHG_CUDA(cudaMemcpyAsync(key.data(), sim->keyA + b, n * sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    if (sim->opt.track_ids)
      SPHG_CUDA(cudaMemcpyAsync(ids.data(), sim->idsA + b, n * sizeof(int32_t), cudaMemcpyDeviceToHost, st));
    SPHG_CUDA(cudaStreamSynchronize(st));
  }
  int k = 0;
  while (k < sim->ninst && sim->hbegins[k] != (int32_t)b) ++k;
  const InstDesc& d = sim->hdesc[k];
  r.rx.resize(n);
  r.ry.resize(n);
  r.rvx.resize(n);
  r.rvy.resize(n);
  r.rrho.resize(n);
  parallel_for(n, [&](int64_t lo, int64_t hi) {
  for (int64_t i = lo; i < hi; ++i) {
    double px = pos[i].x, py = pos[i].y;
    if (sim->opt.precision == SPHG_PRECISION_SPLIT) {
      int cx, cy;
      const uint32_t code = key[i] - d.cell_base;
      if (d.order == 0) demorton_host(code, cx, cy);
      else { cx = (int)(code % (uint32_t)d.nx); cy = (int)(code / (uint32_t)d.nx); }
      px = d.lo_xd + cx * d.cs_xd + px;
      py = d.lo_yd + cy * d.cs_yd + py;
    }
    r.rx[i] = px;
    r.ry[i] = py;
    r.rvx[i] = velp[i].x;
    r.rvy[i] = velp[i].y;
    r.rrho[i] = rho[i];
  }
  });
  r.rids = ids;
  r.t_done = now_s(s->t0);
  r.state = 2;
  r.x.clear(); r.y.clear(); r.vx.clear(); r.vy.clear();
  ++s->completed;
  return SPHG_OK;
}

}  // namespace

extern "C" {

sphg_status sphg_server_create(double hbm_budget_bytes, int32_t max_instances, const sphg_options* o,
                               sphg_server** out) {
  if (!out || !(hbm_budget_bytes > 0) || max_instances <= 0)
    return fail(SPHG_INVALID_ARG, "budget and max_instances must be positive");
  *out = nullptr;
  sphg_server* s = new sphg_server();
  s->sim = new sphg_sim();
  sphg_sim* sim = s->sim;
  if (o) sim->opt = *o; else sphg_default_options(&sim->opt);
  sim->opt.tile_bits = -1;   // layouts change every few ticks: per-particle kernels
  sim->opt.use_graph = 0;    // ... and direct launches
  sim->force_batched = 1;    // same kernels (and bits) whatever the batch size
  sim->opt.compute = SPHG_COMPUTE_SORTED;
  sphg_status st = check_options(sim, 0, nullptr);
  if (st != SPHG_OK) {
    delete sim;
    delete s;
    return st;
  }
  // split the budget: half for per-particle state (about 160 bytes a particle
  // with the neighbour slots), half for the cell-range table (16 bytes a key)
  const double per_particle = 160.0;
  size_t cap_n = (size_t)std::floor(0.5 * hbm_budget_bytes / per_particle);
  cap_n = std::min(cap_n, ((size_t)1 << 27) - 1);
  uint64_t cap_keys = (uint64_t)std::floor(0.5 * hbm_budget_bytes / 16.0);
  cap_keys = std::min<uint64_t>(cap_keys, 0xffffff00ull);
  const int chunks = sphg::diag_chunks((int64_t)cap_n, max_instances, 64);
  st = alloc_arena(sim, std::max<size_t>(cap_n, 1), cap_keys, max_instances, chunks);
  if (st == SPHG_OK) {
    if (cudaMallocHost((void**)&s->htab, sizeof(RepackEntry) * max_instances) != cudaSuccess ||
        cudaMalloc((void**)&s->dtab, sizeof(RepackEntry) * max_instances) != cudaSuccess)
      st = fail(SPHG_OOM, "repack tables");
  }
  if (st != SPHG_OK) {
    sphg_server_destroy(s);
    return st;
  }
  sim->ninst = 0;
  sim->n = 0;
  *out = s;
  return SPHG_OK;
}

sphg_status sphg_server_destroy(sphg_server* s) {
  if (!s) return SPHG_OK;
  cudaFreeHost(s->hpos);
  cudaFreeHost(s->hvel);
  cudaFreeHost(s->hkey);
  cudaFreeHost(s->hids);
  cudaFreeHost(s->htab);
  if (s->dtab) cudaFree(s->dtab);
  destroy_impl(s->sim);
  delete s;
  return SPHG_OK;
}

sphg_status sphg_server_submit(sphg_server* s, const sphg_params* p, int64_t n, const double* x,
                               const double* y, const double* vx, const double* vy, int64_t steps,
                               int64_t* id) {
  if (!s || !p || n <= 0 || !x || !y || !vx || !vy || steps < 1 || !id)
    return fail(SPHG_INVALID_ARG, "bad request (need n >= 1, steps >= 1, all arrays)");
  InstDesc d;
  uint64_t span = 0;
  SPHG_TRY(make_desc(*p, 0, n, 0, d, span));
  if ((size_t)n > s->sim->cap_n || span > s->sim->cap_keys)
    return fail(SPHG_CAPACITY, "request larger than the whole server capacity");
  for (int64_t i = 0; i < n; ++i)
    if (!std::isfinite(x[i]) || !std::isfinite(y[i]) || !std::isfinite(vx[i]) || !std::isfinite(vy[i]))
      return fail(SPHG_NONFINITE, "non-finite value in the submitted state");
  SrvReq r;
  r.id = s->next_id++;
  r.p = *p;
  r.n = n;
  r.steps = steps;
  r.x.assign(x, x + n);
  r.y.assign(y, y + n);
  r.vx.assign(vx, vx + n);
  r.vy.assign(vy, vy + n);
  r.t_submit = now_s(s->t0);
  s->reqs[r.id] = std::move(r);
  s->queue.push_back(*id = s->next_id - 1);
  return SPHG_OK;
}

sphg_status sphg_server_submit_lattice(sphg_server* s, const sphg_params* p, const sphg_lattice* spec,
                                       int64_t steps, int64_t* id) {
  if (!s || !p || !spec || steps < 1 || !id) return fail(SPHG_INVALID_ARG, "bad request (need steps >= 1)");
  const int64_t n = spec->nx * spec->ny;
  if (n <= 0) return fail(SPHG_INVALID_ARG, "empty lattice");
  SPHG_TRY(check_lattice(*spec, n, 0));
  InstDesc d;
  uint64_t span = 0;
  SPHG_TRY(make_desc(*p, 0, n, 0, d, span));
  if ((size_t)n > s->sim->cap_n || span > s->sim->cap_keys)
    return fail(SPHG_CAPACITY, "request larger than the whole server capacity");
  SrvReq r;
  r.id = s->next_id++;
  r.p = *p;
  r.n = n;
  r.steps = steps;
  r.lattice = true;
  r.spec = *spec;
  r.t_submit = now_s(s->t0);
  s->reqs[r.id] = std::move(r);
  s->queue.push_back(*id = s->next_id - 1);
  return SPHG_OK;
}

sphg_status sphg_server_tick(sphg_server* s, void* stream, int32_t* live_out, int32_t* finished_out) {
  if (!s) return fail(SPHG_INVALID_ARG, "null server");
  cudaStream_t st = (cudaStream_t)stream;
  // 1. admission, FIFO, while the live set fits
  std::vector<int64_t> newlive = s->live;
  size_t nadmit = 0;
  size_t staged = 0;  // newcomers' particles, staged after the current layout's
  while (!s->queue.empty()) {
    std::vector<int64_t> cand = newlive;
    cand.push_back(s->queue.front());
    Layout L;
    std::vector<sphg_params> p;
    std::vector<int64_t> counts;
    if (layout_of(s, cand, L, p, counts) != SPHG_OK) break;  // head does not fit yet
    // the repack stages the current layout (retired instances included until
    // then) plus the newcomers
    const size_t head_n = (size_t)s->reqs[s->queue.front()].n;
    if ((size_t)s->sim->n + staged + head_n > s->sim->cap_n) break;
    staged += head_n;
    newlive.swap(cand);
    s->reqs[s->queue.front()].state = 1;
    s->queue.pop_front();
    ++nadmit;
  }
  // 2. repack when the live set changed
  if (nadmit || s->dirty) {
    SPHG_TRY(repack(s, newlive, nadmit, st));
    s->live = newlive;
    s->dirty = false;
    s->sim->force_full_sort = true;  // the last force pass's changed-slot record is of the old layout
  }
  int32_t finished = 0;
  if (!s->live.empty()) {
    // 3. one iteration of every live instance
    SPHG_TRY(enqueue_step(s->sim, st, false));
    ++s->ticks;
    s->particle_steps += (double)s->sim->n;
    // 4. retire
    std::vector<int64_t> keep;
    for (int64_t id : s->live) {
      SrvReq& r = s->reqs[id];
      if (++r.runs >= r.steps) {
        SPHG_TRY(retire(s, r, st));
        ++finished;
        s->dirty = true;
      } else {
        keep.push_back(id);
      }
    }
    if (s->dirty) s->live.swap(keep);
  }
  if (live_out) *live_out = (int32_t)s->live.size();
  if (finished_out) *finished_out = finished;
  return SPHG_OK;
}

sphg_status sphg_server_result(sphg_server* s, int64_t id, double* x, double* y, double* vx,
                               double* vy, double* rho, int32_t* ids, double* latency_s) {
  if (!s) return fail(SPHG_INVALID_ARG, "null server");
  auto it = s->reqs.find(id);
  if (it == s->reqs.end()) return fail(SPHG_INVALID_ARG, "unknown request id");
  SrvReq& r = it->second;
  if (r.state != 2) return fail(SPHG_NOT_READY, "request not finished");
  const size_t bytes = (size_t)r.n * sizeof(double);
  if (x) std::memcpy(x, r.rx.data(), bytes);
  if (y) std::memcpy(y, r.ry.data(), bytes);
  if (vx) std::memcpy(vx, r.rvx.data(), bytes);
  if (vy) std::memcpy(vy, r.rvy.data(), bytes);
  if (rho) std::memcpy(rho, r.rrho.data(), bytes);
  if (ids) std::memcpy(ids, r.rids.data(), (size_t)r.n * sizeof(int32_t));
  if (latency_s) *latency_s = r.t_done - r.t_submit;
  s->reqs.erase(it);
  return SPHG_OK;
}

sphg_status sphg_server_stats(sphg_server* s, double* out) {
  if (!s || !out) return fail(SPHG_INVALID_ARG, "null argument");
  out[0] = (double)s->live.size();
  out[1] = (double)s->queue.size();
  out[2] = (double)s->completed;
  out[3] = s->particle_steps;
  out[4] = (double)s->ticks;
  out[5] = (double)s->sim->cap_n;
  out[6] = (double)s->sim->cap_keys;
  out[7] = (double)s->sim->n;
  return SPHG_OK;
}

}  // extern "C"
