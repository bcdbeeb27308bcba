// sphg_server.cu -- continuous batching of independent SPH simulations.
//
// A server owns one device arena sized from an HBM budget and keeps every live
// simulation's state resident in it.  Requests (an initial state or a lattice
// to generate, the parameters, a step count) wait in a FIFO queue.  Each tick:
//   1. admits queued requests, in order, while they fit;
//   2. places the newcomers: normally APPENDED after the last slot and the last
//      cell key in use -- their initial states are staged (pinned host copies,
//      or the device lattice generator), sorted among themselves by cell key,
//      and written as "integrated states awaiting the next sort" with no mover
//      bit, so the running instances keep their slots and the incremental
//      re-sort keeps merging; when the arena's end is reached, or finished
//      instances hold more slots than live ones, the live set is COMPACTED
//      (dense repack, one full radix sort);
//   3. runs one batched main-loop iteration of every live instance from a
//      CUDA graph replayed on the server's stream (rebuilt only when the slot
//      layout changes), with the per-instance-descriptor kernels for every
//      batch size, so an instance computes the same bits whatever else is live
//      (a newcomer's first iteration is its pre-loop);
//   4. retires the instances that ran their `steps` iterations: their state is
//      copied into pinned host memory behind an event (no host
//      synchronisation), their descriptor is switched off on the device (the
//      kernels skip its slots until the next compaction), and the result is
//      converted to FP64 when the caller fetches it.
// The serving loop runs on a thread of its own with a stream of its own
// (sphg_server_start), so arrivals are admitted while earlier ticks run on the
// GPU; sphg_server_tick runs the same tick on the caller's thread and stream.
// Latency of a request = time its result is in host memory - submission time.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <deque>
#include <map>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include <cuda_runtime.h>

#include "sphg_internal.cuh"
#include "sphg_sort.cuh"

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

// Appended newcomers, staged at [0, m) of the staging buffers: instance-local
// cell codes -> global keys (the instance's cell base), in place.
__global__ void append_keys_kernel(int64_t m, int nnew, const int64_t* __restrict__ starts,
                                   const uint32_t* __restrict__ bases, uint32_t* __restrict__ key) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= m) return;
  int lo = 0, hi = nnew - 1;  // newcomer holding staged particle t
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (starts[mid] <= t) lo = mid; else hi = mid - 1;
  }
  key[t] += bases[lo];
}

// The sorted newcomers into the "integrated state awaiting the next sort" of
// slots [n_old, n_old + m): positions, velocities, keys (also as the current
// sorted keys, so the merge sees them as unchanged), creation indices.
__global__ void append_place_kernel(int64_t m, int64_t n_old, const uint32_t* __restrict__ perm,
                                    const uint32_t* __restrict__ skey, const float2* __restrict__ spos,
                                    const float2* __restrict__ svel, const int32_t* __restrict__ sids,
                                    float2* __restrict__ posB, float2* __restrict__ velB,
                                    uint32_t* __restrict__ keyB, uint32_t* __restrict__ keyA,
                                    int32_t* __restrict__ idsB) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= m) return;
  const uint32_t src = perm[t];
  const uint32_t k = skey[t];
  posB[n_old + t] = spos[src];
  velB[n_old + t] = svel[src];
  keyB[n_old + t] = k;
  keyA[n_old + t] = k;
  if (idsB) idsB[n_old + t] = sids[src];
}

struct SrvReq {
  int64_t id = 0;
  sphg_params p{};
  int64_t n = 0, steps = 0, runs = 0;
  std::vector<double> x, y, vx, vy;  // initial state until admitted (host arrays) ...
  bool lattice = false;               // ... or generated on the device at admission
  sphg_lattice spec{};
  double t_submit = 0, t_done = 0;
  int state = 0;  // 0 queued, 1 live, 2 retiring (copy in flight), 3 done
  int64_t begin = 0;
  uint32_t cell_base = 0;
  InstDesc desc{};                    // descriptor at retirement (result conversion)
  char* rbuf = nullptr;               // pinned result: pos | velp | rho | key | ids
  size_t rbuf_bytes = 0;
  cudaEvent_t ev = nullptr;           // the result copy is done
};

double now_s(const std::chrono::steady_clock::time_point& t0) {
  return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

// Bytes of a retired instance's pinned result, per particle.
constexpr size_t kResultBytes = sizeof(float2) + sizeof(float4) + sizeof(float) + sizeof(uint32_t) + sizeof(int32_t);

// One entry of the slot layout: a live request, or a finished one whose slots
// stay until the next compaction.
struct SlotEntry {
  int64_t id;   // request id (dead entries keep it only for bookkeeping)
  bool live;
  sphg_params p;
  int64_t count;
};

}  // namespace

struct sphg_server {
  sphg_sim* sim = nullptr;
  std::mutex mu;                       // guards everything below that the caller's thread touches
  std::map<int64_t, SrvReq> reqs;
  std::deque<int64_t> queue;
  std::vector<SlotEntry> layout;       // instance order == slot order == key order
  int64_t live_slots = 0, dead_slots = 0;
  int64_t next_id = 1;
  double particle_steps = 0;
  int64_t ticks = 0, completed = 0, appends = 0, compactions = 0, graph_builds = 0;
  bool need_full_sort = false;         // the next iteration sorts fully (after a compaction)
  std::chrono::steady_clock::time_point t0 = std::chrono::steady_clock::now();
  // pinned staging of newcomers' host arrays
  float2 *hpos = nullptr, *hvel = nullptr;
  uint32_t* hkey = nullptr;
  int32_t* hids = nullptr;
  size_t hcap = 0;
  // small tables copied from pageable memory (the copy consumes the source
  // before it returns, so the next tick may rewrite them while it is queued)
  std::vector<RepackEntry> htab;
  RepackEntry* dtab = nullptr;
  std::vector<int64_t> hstarts;        // appended newcomers: staged start and cell base of each
  std::vector<uint32_t> hbases;
  int64_t* dstarts = nullptr;
  uint32_t* dbases = nullptr;
  // pinned result buffers by size class (power of two), reused once fetched
  std::map<size_t, std::vector<char*>> pool;
  std::vector<cudaEvent_t> free_events;
  std::vector<int64_t> retiring;       // requests whose result copy is in flight
  // serving thread
  std::thread worker;
  std::atomic<bool> running{false}, stop{false};
  std::condition_variable cv;
  cudaStream_t stream = nullptr;
  int device = 0;
  static constexpr int kDepth = 3;     // ticks in flight ahead of the host
  cudaEvent_t tick_ev[kDepth] = {};
  int64_t tick_seq = 0;
  sphg_status worker_status = SPHG_OK;
  std::string worker_error;
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

size_t size_class(size_t bytes) {
  size_t c = 4096;
  while (c < bytes) c <<= 1;
  return c;
}

char* take_buffer(sphg_server* s, size_t bytes, size_t* cls) {
  *cls = size_class(bytes);
  auto& v = s->pool[*cls];
  if (!v.empty()) {
    char* p = v.back();
    v.pop_back();
    return p;
  }
  char* p = nullptr;
  if (cudaMallocHost((void**)&p, *cls) != cudaSuccess) return nullptr;
  return p;
}

void give_buffer(sphg_server* s, char* p, size_t cls) {
  if (p) s->pool[cls].push_back(p);
}

cudaEvent_t take_event(sphg_server* s) {
  if (!s->free_events.empty()) {
    cudaEvent_t e = s->free_events.back();
    s->free_events.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) return nullptr;
  return e;
}

// Device representation of a newcomer's host-array initial state: positions
// (plain: FP32 position; split: FP32 offset in the cell), velocities,
// instance-local cell codes computed exactly as the key kernel would, creation
// indices.
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

// Layout of a list of slot entries (fails with SPHG_CAPACITY when it does not fit).
sphg_status layout_of(sphg_server* s, const std::vector<SlotEntry>& ents, Layout& L) {
  if ((int)ents.size() > s->sim->cap_inst) return fail(SPHG_CAPACITY, "instance slots full");
  if (ents.empty()) {
    L = Layout();
    return SPHG_OK;
  }
  std::vector<sphg_params> p;
  std::vector<int64_t> counts;
  for (const SlotEntry& e : ents) {
    p.push_back(e.p);
    counts.push_back(e.count);
  }
  SPHG_TRY(compute_layout(s->sim, (int)ents.size(), p.data(), counts.data(), s->sim->cap_keys, L));
  if ((size_t)L.n > s->sim->cap_n) return fail(SPHG_CAPACITY, "particle capacity full");
  for (size_t k = 0; k < ents.size(); ++k) L.desc[k].active = ents[k].live ? 1 : 0;
  return SPHG_OK;
}

sphg_status apply(sphg_server* s, const std::vector<SlotEntry>& ents, const Layout& L, cudaStream_t st) {
  std::vector<sphg_params> p;
  std::vector<int64_t> counts;
  for (const SlotEntry& e : ents) {
    p.push_back(e.p);
    counts.push_back(e.count);
  }
  return apply_layout(s->sim, (int)ents.size(), p.data(), counts.data(), L, &st);
}

// Stages the newcomers' initial states at [at, at + m) of the staging buffers
// (posA / acc / keyTmp / idsA: free between ticks beyond the slots in use):
// host arrays through pinned memory, lattices generated on the device.  Keys
// are instance-local codes.
sphg_status stage_all(sphg_server* s, const std::vector<int64_t>& ids, const std::vector<InstDesc>& descs,
                      int64_t at, cudaStream_t st) {
  sphg_sim* sim = s->sim;
  size_t host_n = 0;
  for (int64_t id : ids)
    if (!s->reqs[id].lattice) host_n += s->reqs[id].n;
  SPHG_TRY(grow_staging(s, host_n));
  // host-array newcomers: converted into pinned staging, then one copy per array
  size_t h = 0;
  int64_t off = 0;
  std::vector<std::pair<int64_t, size_t>> runs;  // (device offset, pinned offset) of each host newcomer
  for (size_t k = 0; k < ids.size(); ++k) {
    const SrvReq& r = s->reqs[ids[k]];
    if (!r.lattice) {
      stage_newcomer(s, r, descs[k], h);
      runs.emplace_back(at + off, h);
      h += r.n;
    }
    off += r.n;
  }
  for (size_t k = 0, q = 0; k < ids.size(); ++k) {
    const SrvReq& r = s->reqs[ids[k]];
    if (r.lattice) continue;
    const int64_t dst = runs[q].first;
    const size_t src = runs[q].second;
    ++q;
    SPHG_CUDA(cudaMemcpyAsync(sim->posA + dst, s->hpos + src, r.n * sizeof(float2), cudaMemcpyHostToDevice, st));
    SPHG_CUDA(cudaMemcpyAsync(sim->acc + dst, s->hvel + src, r.n * sizeof(float2), cudaMemcpyHostToDevice, st));
    SPHG_CUDA(cudaMemcpyAsync(sim->keyTmp + dst, s->hkey + src, r.n * sizeof(uint32_t), cudaMemcpyHostToDevice, st));
    if (sim->opt.track_ids)
      SPHG_CUDA(cudaMemcpyAsync(sim->idsA + dst, s->hids + src, r.n * sizeof(int32_t), cudaMemcpyHostToDevice, st));
  }
  off = 0;
  for (size_t k = 0; k < ids.size(); ++k) {
    const SrvReq& r = s->reqs[ids[k]];
    if (r.lattice)
      SPHG_CUDA(sphg::launch_lattice_stage(descs[k], r.spec, sim->opt.precision, r.n, sim->posA + at + off,
                                           sim->acc + at + off, sim->keyTmp + at + off,
                                           sim->opt.track_ids ? sim->idsA + at + off : nullptr, st));
    off += r.n;
  }
  // the pinned staging is reused by the next admission only after these copies
  if (host_n) SPHG_CUDA(cudaStreamSynchronize(st));
  return SPHG_OK;
}

// Appends newcomers after the last slot and key in use; the running instances
// keep their slots, keys and mover record.
sphg_status append(sphg_server* s, const std::vector<int64_t>& ids, cudaStream_t st) {
  sphg_sim* sim = s->sim;
  std::vector<SlotEntry> ents = s->layout;
  for (int64_t id : ids) ents.push_back({id, true, s->reqs[id].p, s->reqs[id].n});
  Layout L;
  SPHG_TRY(layout_of(s, ents, L));
  const int64_t n_old = sim->n;
  const int64_t m = L.n - n_old;
  const size_t k0 = s->layout.size();
  std::vector<InstDesc> descs(L.desc.begin() + k0, L.desc.end());
  SPHG_TRY(stage_all(s, ids, descs, n_old, st));
  // global keys, sorted among the newcomers (identity values = staged order,
  // i.e. creation order within each newcomer: the stable order of a full sort)
  s->hstarts.resize(ids.size());
  s->hbases.resize(ids.size());
  for (size_t k = 0; k < ids.size(); ++k) {
    s->hstarts[k] = L.begins[k0 + k] - n_old;
    s->hbases[k] = L.desc[k0 + k].cell_base;
  }
  SPHG_CUDA(cudaMemcpyAsync(s->dstarts, s->hstarts.data(), ids.size() * sizeof(int64_t), cudaMemcpyHostToDevice, st));
  SPHG_CUDA(cudaMemcpyAsync(s->dbases, s->hbases.data(), ids.size() * sizeof(uint32_t), cudaMemcpyHostToDevice, st));
  const unsigned g = (unsigned)((m + 255) / 256);
  append_keys_kernel<<<g, 256, 0, st>>>(m, (int)ids.size(), s->dstarts, s->dbases, sim->keyTmp + n_old);
  SPHG_CUDA(cudaGetLastError());
  int bits = 1;
  while (bits < 32 && ((uint64_t)1 << bits) < L.keys) ++bits;
  // ping-pong of the newcomer sort: the posB slots beyond n_old (two words a slot)
  uint32_t* ktmp = reinterpret_cast<uint32_t*>(sim->posB + n_old);
  uint32_t* vtmp = ktmp + m;
  SPHG_CUDA(sphg::radix_sort_pairs(sim->keyTmp + n_old, nullptr, sim->keyA + n_old, sim->perm + n_old,
                                   bits > 8 ? ktmp : nullptr, bits > 8 ? vtmp : nullptr, sim->scratch, m, bits,
                                   st));
  append_place_kernel<<<g, 256, 0, st>>>(m, n_old, sim->perm + n_old, sim->keyA + n_old, sim->posA + n_old,
                                         sim->acc + n_old, sim->opt.track_ids ? sim->idsA + n_old : nullptr,
                                         sim->posB, sim->velB, sim->keyB, sim->keyA,
                                         sim->opt.track_ids ? sim->idsB : nullptr);
  SPHG_CUDA(cudaGetLastError());
  // no mover bits for the new slots (the word holding slot n_old - 1 was
  // written by the last force pass with zeros above it)
  if (sim->movers_on) {
    const int64_t w0 = (n_old + 31) / 32, w1 = (L.n + 31) / 32;
    if (w1 > w0) SPHG_CUDA(cudaMemsetAsync(sim->mmask + w0, 0, (w1 - w0) * sizeof(uint32_t), st));
  }
  SPHG_TRY(apply(s, ents, L, st));
  for (size_t k = 0; k < ids.size(); ++k) {
    SrvReq& r = s->reqs[ids[k]];
    r.begin = L.begins[k0 + k];
    r.cell_base = L.desc[k0 + k].cell_base;
  }
  s->layout.swap(ents);
  for (int64_t id : ids) s->live_slots += s->reqs[id].n;
  ++s->appends;
  return SPHG_OK;
}

// Dense repack of the live instances followed by the newcomers (finished
// instances' slots and keys are reclaimed); the next iteration sorts fully.
sphg_status compact(sphg_server* s, const std::vector<int64_t>& ids, cudaStream_t st) {
  sphg_sim* sim = s->sim;
  std::vector<SlotEntry> ents;
  for (const SlotEntry& e : s->layout)
    if (e.live) ents.push_back(e);
  const size_t nret = ents.size();
  for (int64_t id : ids) ents.push_back({id, true, s->reqs[id].p, s->reqs[id].n});
  Layout L;
  SPHG_TRY(layout_of(s, ents, L));
  const int64_t n_old = sim->n;
  // 1. the whole current next state -> staging (the sorted-state buffers are free now)
  if (n_old > 0) {
    SPHG_CUDA(cudaMemcpyAsync(sim->posA, sim->posB, n_old * sizeof(float2), cudaMemcpyDeviceToDevice, st));
    SPHG_CUDA(cudaMemcpyAsync(sim->acc, sim->velB, n_old * sizeof(float2), cudaMemcpyDeviceToDevice, st));
    SPHG_CUDA(cudaMemcpyAsync(sim->keyTmp, sim->keyB, n_old * sizeof(uint32_t), cudaMemcpyDeviceToDevice, st));
    if (sim->opt.track_ids)
      SPHG_CUDA(cudaMemcpyAsync(sim->idsA, sim->idsB, n_old * sizeof(int32_t), cudaMemcpyDeviceToDevice, st));
  }
  // 2. newcomers after them
  int64_t nnew = 0;
  for (int64_t id : ids) nnew += s->reqs[id].n;
  if ((size_t)(n_old + nnew) > sim->cap_n) return fail(SPHG_CAPACITY, "staging exceeds the particle capacity");
  std::vector<InstDesc> descs(L.desc.begin() + nret, L.desc.end());
  SPHG_TRY(stage_all(s, ids, descs, n_old, st));
  // 3. new layout, then one gather of every live particle to its new slot
  std::vector<int64_t> src(ents.size());
  s->htab.resize(ents.size());
  int64_t at = n_old;
  for (size_t k = 0; k < ents.size(); ++k) {
    SrvReq& r = s->reqs[ents[k].id];
    const bool retained = k < nret;
    if (retained) {
      src[k] = r.begin;
    } else {
      src[k] = at;
      at += r.n;
    }
    s->htab[k].src_begin = src[k];
    s->htab[k].key_delta = L.desc[k].cell_base - (retained ? r.cell_base : 0u);
  }
  SPHG_TRY(apply(s, ents, L, st));
  for (size_t k = 0; k < ents.size(); ++k) {
    SrvReq& r = s->reqs[ents[k].id];
    r.begin = L.begins[k];
    r.cell_base = L.desc[k].cell_base;
  }
  if (!ents.empty()) {
    SPHG_CUDA(cudaMemcpyAsync(s->dtab, s->htab.data(), ents.size() * sizeof(RepackEntry), cudaMemcpyHostToDevice, st));
    const unsigned g = (unsigned)((L.n + 255) / 256);
    repack_kernel<<<g, 256, 0, st>>>(L.n, (int)ents.size(), sim->dbegins, s->dtab, sim->posA, sim->acc,
                                     sim->keyTmp, sim->idsA, sim->posB, sim->velB, sim->keyB,
                                     sim->opt.track_ids ? sim->idsB : nullptr);
    SPHG_CUDA(cudaGetLastError());
  }
  s->layout.swap(ents);
  s->live_slots = L.n;
  s->dead_slots = 0;
  s->need_full_sort = true;  // the last force pass's mover record is of the old layout
  ++s->compactions;
  return SPHG_OK;
}

// Retires a live request: its state (current slot order) into a pinned buffer
// behind an event, its descriptor switched off on the device.
sphg_status retire(sphg_server* s, int64_t id, cudaStream_t st) {
  sphg_sim* sim = s->sim;
  SrvReq& r = s->reqs[id];
  const int64_t n = r.n, b = r.begin;
  int k = 0;
  while (k < sim->ninst && sim->hbegins[k] != (int32_t)b) ++k;
  if (k >= sim->ninst) return fail(SPHG_CUDA_ERROR, "retired request not in the layout");
  r.desc = sim->hdesc[k];
  size_t cls = 0;
  r.rbuf = take_buffer(s, (size_t)n * kResultBytes, &cls);
  if (!r.rbuf) return fail(SPHG_OOM, "pinned result buffer");
  r.rbuf_bytes = cls;
  char* q = r.rbuf;
  SPHG_CUDA(cudaMemcpyAsync(q, sim->posA + b, n * sizeof(float2), cudaMemcpyDeviceToHost, st));
  q += n * sizeof(float2);
  SPHG_CUDA(cudaMemcpyAsync(q, sim->velpA + b, n * sizeof(float4), cudaMemcpyDeviceToHost, st));
  q += n * sizeof(float4);
  SPHG_CUDA(cudaMemcpyAsync(q, sim->rho + b, n * sizeof(float), cudaMemcpyDeviceToHost, st));
  q += n * sizeof(float);
  SPHG_CUDA(cudaMemcpyAsync(q, sim->keyA + b, n * sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
  q += n * sizeof(uint32_t);
  if (sim->opt.track_ids)
    SPHG_CUDA(cudaMemcpyAsync(q, sim->idsA + b, n * sizeof(int32_t), cudaMemcpyDeviceToHost, st));
  // the kernels skip the instance's slots from the next iteration on
  SPHG_CUDA(cudaMemsetAsync(&sim->ddesc[k].active, 0, sizeof(int32_t), st));
  sim->hdesc[k].active = 0;
  r.ev = take_event(s);
  if (!r.ev) return fail(SPHG_CUDA_ERROR, "event for a result copy");
  SPHG_CUDA(cudaEventRecord(r.ev, st));
  r.state = 2;
  for (SlotEntry& e : s->layout)
    if (e.id == id) e.live = false;
  s->live_slots -= n;
  s->dead_slots += n;
  s->retiring.push_back(id);
  ++s->completed;
  return SPHG_OK;
}

// Results whose copy has finished become fetchable (completion time stamped now).
void poll_retiring(sphg_server* s) {
  std::vector<int64_t> keep;
  for (int64_t id : s->retiring) {
    auto it = s->reqs.find(id);
    if (it == s->reqs.end()) continue;
    SrvReq& r = it->second;
    if (r.state == 2 && cudaEventQuery(r.ev) == cudaSuccess) {
      r.t_done = now_s(s->t0);
      r.state = 3;
      s->free_events.push_back(r.ev);
      r.ev = nullptr;
    } else if (r.state == 2) {
      keep.push_back(id);
    }
  }
  cudaGetLastError();  // cudaErrorNotReady of the queries
  s->retiring.swap(keep);
}

// One tick on stream st (caller holds s->mu).
sphg_status tick_impl(sphg_server* s, cudaStream_t st, int32_t* live_out, int32_t* finished_out) {
  sphg_sim* sim = s->sim;
  poll_retiring(s);
  // 1. admission, FIFO, while the head fits (appended, or after a compaction)
  std::vector<int64_t> admit;
  int64_t add_n = 0;
  bool do_compact = false;
  while (!s->queue.empty()) {
    const int64_t head = s->queue.front();
    const SrvReq& r = s->reqs[head];
    std::vector<SlotEntry> cand = s->layout;
    for (int64_t id : admit) cand.push_back({id, true, s->reqs[id].p, s->reqs[id].n});
    cand.push_back({head, true, r.p, r.n});
    Layout L;
    bool fits_append = !do_compact && layout_of(s, cand, L) == SPHG_OK;
    if (!fits_append) {
      // compacted: live instances + admitted + head
      std::vector<SlotEntry> dense;
      for (const SlotEntry& e : cand)
        if (e.live) dense.push_back(e);
      if (layout_of(s, dense, L) != SPHG_OK) break;  // does not fit even densely: wait
      do_compact = true;
      // staging of a compaction holds the current slots plus the newcomers: when
      // they do not fit, this tick compacts what is admitted so far and the head
      // follows once finished instances' slots are reclaimed
      if ((size_t)(sim->n + add_n + r.n) > sim->cap_n) break;
    }
    admit.push_back(head);
    add_n += r.n;
    s->reqs[head].state = 1;
    s->queue.pop_front();
  }
  // compaction also when finished instances hold more slots than live ones
  if (!do_compact && s->dead_slots > std::max<int64_t>(s->live_slots, (int64_t)1 << 18)) do_compact = true;
  if (do_compact) {
    SPHG_TRY(compact(s, admit, st));
  } else if (!admit.empty()) {
    SPHG_TRY(append(s, admit, st));
  }
  int32_t finished = 0;
  if (s->live_slots > 0) {
    // 2. one iteration of every live instance
    if (s->need_full_sort || !sim->opt.use_graph) {
      sim->force_full_sort = s->need_full_sort;
      SPHG_TRY(enqueue_step(sim, st, false));
      s->need_full_sort = false;
    } else {
      if (!sim->gexec) {
        SPHG_TRY(build_graph(sim));
        ++s->graph_builds;
      }
      SPHG_CUDA(cudaGraphLaunch(sim->gexec, st));
    }
    ++s->ticks;
    s->particle_steps += (double)s->live_slots;
    // 3. retire
    std::vector<int64_t> done;
    for (const SlotEntry& e : s->layout)
      if (e.live && ++s->reqs[e.id].runs >= s->reqs[e.id].steps) done.push_back(e.id);
    for (int64_t id : done) {
      SPHG_TRY(retire(s, id, st));
      ++finished;
    }
  }
  if (live_out) *live_out = (int32_t)std::count_if(s->layout.begin(), s->layout.end(),
                                                   [](const SlotEntry& e) { return e.live; });
  if (finished_out) *finished_out = finished;
  return SPHG_OK;
}

void serve_loop(sphg_server* s) {
  cudaSetDevice(s->device);
  while (!s->stop.load()) {
    // keep at most kDepth ticks in flight: wait for the one kDepth ticks back
    cudaEvent_t& ev = s->tick_ev[s->tick_seq % sphg_server::kDepth];
    if (s->tick_seq >= sphg_server::kDepth) cudaEventSynchronize(ev);
    std::unique_lock<std::mutex> lock(s->mu);
    int32_t live = 0, fin = 0;
    const sphg_status st = tick_impl(s, s->stream, &live, &fin);
    if (st != SPHG_OK) {
      s->worker_status = st;
      s->worker_error = sphg_last_error_string();
      break;
    }
    cudaEventRecord(ev, s->stream);
    ++s->tick_seq;
    if (live == 0 && s->queue.empty()) {
      // idle: results still in flight are polled every millisecond
      s->cv.wait_for(lock, std::chrono::milliseconds(s->retiring.empty() ? 20 : 1));
    }
  }
  cudaStreamSynchronize(s->stream);
  std::lock_guard<std::mutex> lock(s->mu);
  poll_retiring(s);
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
    if (cudaMalloc((void**)&s->dtab, sizeof(RepackEntry) * max_instances) != cudaSuccess ||
        cudaMalloc((void**)&s->dstarts, sizeof(int64_t) * max_instances) != cudaSuccess ||
        cudaMalloc((void**)&s->dbases, sizeof(uint32_t) * max_instances) != cudaSuccess)
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

sphg_status sphg_server_stop(sphg_server* s) {
  if (!s) return fail(SPHG_INVALID_ARG, "null server");
  if (!s->running.load()) return SPHG_OK;
  s->stop.store(true);
  s->cv.notify_all();
  if (s->worker.joinable()) s->worker.join();
  s->running.store(false);
  s->stop.store(false);
  if (s->worker_status != SPHG_OK) return fail(s->worker_status, "serving loop: " + s->worker_error);
  return SPHG_OK;
}

sphg_status sphg_server_destroy(sphg_server* s) {
  if (!s) return SPHG_OK;
  sphg_server_stop(s);
  if (s->stream) {
    cudaStreamSynchronize(s->stream);
    cudaStreamDestroy(s->stream);
  }
  for (cudaEvent_t e : s->tick_ev)
    if (e) cudaEventDestroy(e);
  cudaDeviceSynchronize();
  for (auto& kv : s->reqs) {
    if (kv.second.rbuf) cudaFreeHost(kv.second.rbuf);
    if (kv.second.ev) cudaEventDestroy(kv.second.ev);
  }
  for (auto& kv : s->pool)
    for (char* p : kv.second) cudaFreeHost(p);
  for (cudaEvent_t e : s->free_events) cudaEventDestroy(e);
  cudaFreeHost(s->hpos);
  cudaFreeHost(s->hvel);
  cudaFreeHost(s->hkey);
  cudaFreeHost(s->hids);
  if (s->dtab) cudaFree(s->dtab);
  if (s->dstarts) cudaFree(s->dstarts);
  if (s->dbases) cudaFree(s->dbases);
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
  r.p = *p;
  r.n = n;
  r.steps = steps;
  r.x.assign(x, x + n);
  r.y.assign(y, y + n);
  r.vx.assign(vx, vx + n);
  r.vy.assign(vy, vy + n);
  {
    std::lock_guard<std::mutex> lock(s->mu);
    r.id = s->next_id++;
    r.t_submit = now_s(s->t0);
    *id = r.id;
    s->queue.push_back(r.id);
    s->reqs[r.id] = std::move(r);
  }
  s->cv.notify_all();
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
  r.p = *p;
  r.n = n;
  r.steps = steps;
  r.lattice = true;
  r.spec = *spec;
  {
    std::lock_guard<std::mutex> lock(s->mu);
    r.id = s->next_id++;
    r.t_submit = now_s(s->t0);
    *id = r.id;
    s->queue.push_back(r.id);
    s->reqs[r.id] = std::move(r);
  }
  s->cv.notify_all();
  return SPHG_OK;
}

sphg_status sphg_server_tick(sphg_server* s, void* stream, int32_t* live_out, int32_t* finished_out) {
  if (!s) return fail(SPHG_INVALID_ARG, "null server");
  if (s->running.load()) return fail(SPHG_INVALID_ARG, "the serving thread is running (sphg_server_start)");
  std::lock_guard<std::mutex> lock(s->mu);
  return tick_impl(s, (cudaStream_t)stream, live_out, finished_out);
}

sphg_status sphg_server_start(sphg_server* s, int32_t device) {
  if (!s) return fail(SPHG_INVALID_ARG, "null server");
  if (s->running.load()) return SPHG_OK;
  SPHG_CUDA(cudaSetDevice(device));
  s->device = device;
  if (!s->stream) SPHG_CUDA(cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking));
  for (cudaEvent_t& e : s->tick_ev)
    if (!e) SPHG_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  s->tick_seq = 0;
  s->worker_status = SPHG_OK;
  s->stop.store(false);
  s->running.store(true);
  s->worker = std::thread(serve_loop, s);
  return SPHG_OK;
}

sphg_status sphg_server_result(sphg_server* s, int64_t id, double* x, double* y, double* vx,
                               double* vy, double* rho, int32_t* ids, double* latency_s) {
  if (!s) return fail(SPHG_INVALID_ARG, "null server");
  std::unique_lock<std::mutex> lock(s->mu);
  auto it = s->reqs.find(id);
  if (it == s->reqs.end()) return fail(SPHG_INVALID_ARG, "unknown request id");
  SrvReq& r = it->second;
  if (r.state < 2) {
    // a serving thread that stopped on an error will not finish it
    if (s->worker_status != SPHG_OK) return fail(s->worker_status, "serving loop stopped: " + s->worker_error);
    return fail(SPHG_NOT_READY, "request not finished");
  }
  if (r.state == 2) {
    if (s->running.load()) {
      poll_retiring(s);
      if (r.state == 2) return fail(SPHG_NOT_READY, "result copy in flight");
    } else {
      SPHG_CUDA(cudaEventSynchronize(r.ev));  // the caller's own ticks: wait for the copy
      poll_retiring(s);
    }
  }
  const int64_t n = r.n;
  const InstDesc& d = r.desc;
  const bool split = s->sim->opt.precision == SPHG_PRECISION_SPLIT;
  const float2* pos = reinterpret_cast<const float2*>(r.rbuf);
  const float4* velp = reinterpret_cast<const float4*>(pos + n);
  const float* rh = reinterpret_cast<const float*>(velp + n);
  const uint32_t* key = reinterpret_cast<const uint32_t*>(rh + n);
  const int32_t* rid = reinterpret_cast<const int32_t*>(key + n);
  const bool track = s->sim->opt.track_ids != 0;
  parallel_for(n, [&](int64_t lo, int64_t hi) {
    for (int64_t i = lo; i < hi; ++i) {
      double px = pos[i].x, py = pos[i].y;
      if (split) {
        int cx, cy;
        const uint32_t code = key[i] - d.cell_base;
        if (d.order == 0) demorton_host(code, cx, cy);
        else { cx = (int)(code % (uint32_t)d.nx); cy = (int)(code / (uint32_t)d.nx); }
        px = d.lo_xd + cx * d.cs_xd + px;
        py = d.lo_yd + cy * d.cs_yd + py;
      }
      if (x) x[i] = px;
      if (y) y[i] = py;
      if (vx) vx[i] = velp[i].x;
      if (vy) vy[i] = velp[i].y;
      if (rho) rho[i] = rh[i];
      if (ids) ids[i] = track ? rid[i] : -1;
    }
  });
  if (latency_s) *latency_s = r.t_done - r.t_submit;
  give_buffer(s, r.rbuf, r.rbuf_bytes);
  s->reqs.erase(it);
  return SPHG_OK;
}

sphg_status sphg_server_stats(sphg_server* s, double* out) {
  if (!s || !out) return fail(SPHG_INVALID_ARG, "null argument");
  std::lock_guard<std::mutex> lock(s->mu);
  out[0] = (double)std::count_if(s->layout.begin(), s->layout.end(), [](const SlotEntry& e) { return e.live; });
  out[1] = (double)s->queue.size();
  out[2] = (double)s->completed;
  out[3] = s->particle_steps;
  out[4] = (double)s->ticks;
  out[5] = (double)s->sim->cap_n;
  out[6] = (double)s->sim->cap_keys;
  out[7] = (double)s->live_slots;
  return SPHG_OK;
}

sphg_status sphg_server_counters(sphg_server* s, double* out, int32_t count) {
  if (!s || !out || count < 0) return fail(SPHG_INVALID_ARG, "null argument or negative count");
  std::lock_guard<std::mutex> lock(s->mu);
  const double v[7] = {(double)s->appends, (double)s->compactions, (double)s->graph_builds,
                       (double)s->dead_slots, (double)s->sim->n, (double)s->retiring.size(),
                       s->running.load() ? 1.0 : 0.0};
  for (int32_t k = 0; k < count && k < 7; ++k) out[k] = v[k];
  return SPHG_OK;
}

}  // extern "C"
