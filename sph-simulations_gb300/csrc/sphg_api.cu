// sphg_api.cu -- host side of the C ABI declared in include/sphg.h.
//
// A handle owns one device arena holding the state of all its instances
// (see sphg_common.cuh for the layout), the per-instance constants computed
// here in FP64, and optionally a captured CUDA graph of one step.  Nothing in
// here computes physics on the host; the host only converts the caller's
// doubles to the device representation and back.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <limits>
#include <string>
#include <thread>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/sphg.h"
#include "sphg_internal.cuh"
#include "sphg_sort.cuh"
#include "sphg_step.cuh"

using sphg::InstDesc;
using sphg::StepArgs;

namespace sphg_detail {

thread_local std::string g_err;

sphg_status fail(sphg_status st, const std::string& msg) {
  g_err = msg;
  return st;
}

int next_pow2(int n) {
  int p = 1;
  while (p < n) p *= 2;
  return p;
}

uint32_t morton_host(uint32_t x, uint32_t y) {
  uint32_t z = 0;
  for (int b = 0; b < 16; ++b) {
    z |= ((x >> b) & 1u) << (2 * b);
    z |= ((y >> b) & 1u) << (2 * b + 1);
  }
  return z;
}

void demorton_host(uint32_t z, int& x, int& y) {
  uint32_t a = 0, b = 0;
  for (int i = 0; i < 16; ++i) {
    a |= ((z >> (2 * i)) & 1u) << i;
    b |= ((z >> (2 * i + 1)) & 1u) << i;
  }
  x = (int)a;
  y = (int)b;
}

bool finite_params(const sphg_params& p) {
  const double v[] = {p.h, p.dt, p.k, p.rho0, p.mu, p.tol, p.gx, p.gy, p.mass, p.alpha, p.c0,
                      p.lo[0], p.lo[1], p.hi[0], p.hi[1]};
  for (double x : v)
    if (!std::isfinite(x)) return false;
  return true;
}

// Per-instance constants (FP64 on the host, rounded once to FP32).  Grid as
// MortonOrder::Initialize / RowMajorOrder::Initialize: cell size = H,
// n = ceil(L / H), Morton pads each axis to a power of two
// (core/alg/orders/MortonOrder.h:11-43,92-103).  Periodic boundaries (an
// extension) use floor(L / H) cells of size L / n >= H.
sphg_status make_desc(const sphg_params& p, int64_t begin, int64_t count, uint64_t cell_base,
                      InstDesc& d, uint64_t& span) {
  if (!finite_params(p)) return fail(SPHG_INVALID_ARG, "non-finite parameter");
  if (!(p.h > 0)) return fail(SPHG_INVALID_ARG, "h must be > 0");
  if (!(p.hi[0] > p.lo[0]) || !(p.hi[1] > p.lo[1]))
    return fail(SPHG_INVALID_ARG, "domain must have hi > lo on both axes");
  if (!(p.rho0 >= 0) || !(p.mass > 0) || !(p.mu >= 0) || !(p.alpha >= 0))
    return fail(SPHG_INVALID_ARG, "rho0, mu, alpha must be >= 0 and mass > 0");
  if (p.order != SPHG_ORDER_MORTON && p.order != SPHG_ORDER_ROWMAJOR)
    return fail(SPHG_INVALID_ARG, "order must be SPHG_ORDER_MORTON or SPHG_ORDER_ROWMAJOR");
  std::memset(&d, 0, sizeof(d));
  const double L[2] = {p.hi[0] - p.lo[0], p.hi[1] - p.lo[1]};
  int nr[2];
  double cs[2];
  for (int a = 0; a < 2; ++a) {
    double n;
    if (p.periodic) {
      n = std::floor(L[a] / p.h);
      if (n < 3) return fail(SPHG_INVALID_ARG, "periodic domain needs at least 3 cells of size >= h per axis");
      cs[a] = L[a] / n;
    } else {
      n = std::ceil(L[a] / p.h);
      cs[a] = p.h;
    }
    if (n > 65536.0) return fail(SPHG_CAPACITY, "more than 65536 cells along an axis");
    nr[a] = (int)n;
  }
  d.begin = (int32_t)begin;
  d.end = (int32_t)(begin + count);
  d.nxr = nr[0];
  d.nyr = nr[1];
  d.order = p.order;
  d.periodic = p.periodic ? 1 : 0;
  d.active = 1;
  d.wrap_f32 = (p.periodic && p.lo[0] == 0.0 && p.lo[1] == 0.0 && (double)(float)L[0] == L[0] &&
                (double)(float)L[1] == L[1]) ? 1 : 0;
  if (p.order == SPHG_ORDER_MORTON) {
    d.nx = next_pow2(nr[0]);
    d.ny = next_pow2(nr[1]);
    span = (uint64_t)morton_host((uint32_t)d.nx - 1, (uint32_t)d.ny - 1) + 1;
  } else {
    d.nx = nr[0];
    d.ny = nr[1];
    span = (uint64_t)d.nx * (uint64_t)d.ny;
  }
  d.cell_base = (uint32_t)cell_base;
  d.key_span = (uint32_t)span;
  d.lo_x = (float)p.lo[0];
  d.lo_y = (float)p.lo[1];
  d.hi_x = (float)p.hi[0];
  d.hi_y = (float)p.hi[1];
  d.cs_x = (float)cs[0];
  d.cs_y = (float)cs[1];
  d.inv_cs_x = (float)(1.0 / cs[0]);
  d.inv_cs_y = (float)(1.0 / cs[1]);
  d.Lx = (float)L[0];
  d.Ly = (float)L[1];
  const double h = p.h, h2 = h * h, h3 = h2 * h, h6 = h3 * h3;
  d.h = (float)h;
  d.inv_h2 = (float)(1.0 / h2);
  d.h2_lo = std::nextafter((float)(h2 * (1.0 - 1.0e-6)), 0.0f);
  d.h2_hi = std::nextafter((float)(h2 * (1.0 + 1.0e-6)), 3.0e38f);
  d.wd = (float)(p.mass * 315.0 / (64.0 * M_PI * h3));
  d.kp = (float)(p.mass * 1.5 * 15.0 / (M_PI * h6));
  d.kv = (float)(p.mass * 45.0 * p.mu / (M_PI * h6));
  d.ka = (float)(p.mass * 3.0 * 15.0 / (M_PI * h6));
  d.k = (float)p.k;
  d.rho0 = (float)p.rho0;
  d.tol2 = (float)(p.tol * p.tol);
  d.gx = (float)p.gx;
  d.gy = (float)p.gy;
  d.dt = (float)p.dt;
  d.alpha_c0 = (float)(p.alpha * p.c0);
  d.eps_h2 = (float)(0.01 * h2);
  d.lo_xd = p.lo[0];
  d.lo_yd = p.lo[1];
  d.cs_xd = cs[0];
  d.cs_yd = cs[1];
  d.Lx_d = L[0];
  d.Ly_d = L[1];
  d.h2_d = h2;
  d.mass_d = p.mass;
  d.hi_xd = p.hi[0];
  d.hi_yd = p.hi[1];
  d.inv_cs_xd = 1.0 / cs[0];
  d.inv_cs_yd = 1.0 / cs[1];
  d.half_Lx_d = 0.5 * L[0];
  d.half_Ly_d = 0.5 * L[1];
  if (!std::isfinite(d.wd) || !std::isfinite(d.kp) || !std::isfinite(d.kv) || !std::isfinite(d.ka) ||
      d.inv_h2 == 0.0f || !std::isfinite(d.inv_h2))
    return fail(SPHG_INVALID_ARG, "h out of the FP32 range of the kernel constants");
  return SPHG_OK;
}

// floor((x - lo)/cs) clamped exactly as the device computes it (FP64 on the host).
int host_cell(double x, double lo, double cs, int cmax) {
  double q = std::floor((x - lo) / cs);
  if (!(q < (double)cmax)) return cmax;
  if (q < 0) return 0;
  return (int)q;
}


void parallel_for(int64_t n, const std::function<void(int64_t, int64_t)>& f) {
  const int64_t grain = 1 << 16;
  int64_t t = std::min<int64_t>((int64_t)std::max(1u, std::thread::hardware_concurrency()), 32);
  t = std::min<int64_t>(t, (n + grain - 1) / grain);
  if (t <= 1) {
    if (n > 0) f(0, n);
    return;
  }
  std::vector<std::thread> pool;
  const int64_t per = (n + t - 1) / t;
  for (int64_t k = 1; k < t; ++k) {
    const int64_t b = k * per, e = std::min(n, b + per);
    if (b < e) pool.emplace_back([&f, b, e] { f(b, e); });
  }
  f(0, std::min(n, per));
  for (auto& th : pool) th.join();
}

char* host_stage(sphg_sim* s, size_t bytes) {
  if (bytes <= s->hstage_bytes) return s->hstage;
  if (s->hstage) cudaFreeHost(s->hstage);
  s->hstage = nullptr;
  s->hstage_bytes = 0;
  if (cudaMallocHost((void**)&s->hstage, bytes) != cudaSuccess) {
    s->hstage = nullptr;
    return nullptr;
  }
  s->hstage_bytes = bytes;
  return s->hstage;
}

float split_offset(double o, double cs) {
  float r = (float)o;
  if ((double)r >= cs) r = std::nextafter(r, 0.0f);  // stay inside the cell after rounding
  return r;
}

int instance_of(const sphg_sim* s, int64_t i) {
  const auto& b = s->hbegins;
  return (int)(std::upper_bound(b.begin(), b.end(), (int32_t)i) - b.begin()) - 1;
}

}  // namespace sphg_detail

namespace sphg {
void set_last_error(const std::string& msg) { sphg_detail::g_err = msg; }
}  // namespace sphg


namespace sphg_detail {

// The incremental re-sort's kernels (see sphg_movers.cu).  cond, when not 0,
// is the graph's conditional handle that guards the full sort: the decision
// kernel sets it to 0 when the merge handled the iteration.
static sphg::MoverArgs mover_args(sphg_sim* s, unsigned long long cond) {
  sphg::MoverArgs m = {};
  m.n = s->n;
  m.keyA = s->keyA;
  m.mask = s->mmask;
  m.movers = s->mlist;
  m.count = s->flags + 7;
  m.ctl = s->flags + 3;
  m.epoch = s->flags + 2;
  m.ranges = s->ranges;
  m.keyS = s->keyTmp;
  m.perm = s->perm;
  m.cond = cond;
  m.posB = s->posB;
  m.velB = s->velB;
  m.idsB = s->opt.track_ids ? s->idsB : nullptr;
  m.posA = s->posA;
  m.velpA = s->velpA;
  m.idsA = s->opt.track_ids ? s->idsA : nullptr;
  m.early_next = s->n <= sphg::kEarlyNextMaxN ? 1 : 0;
  return m;
}

sphg_status enqueue_movers(sphg_sim* s, cudaStream_t st, unsigned long long cond) {
  SPHG_CUDA(sphg::launch_movers(mover_args(s, cond), st));
  return SPHG_OK;
}

// The iteration as one cooperative launch (sphg_options.fused): available for
// the sorted compute mode with the merge re-sort and no cell tiles.
bool fused_on(sphg_sim* s) {
  if (s->opt.fused != 1 || !s->movers_on || s->tile_bits || s->opt.compute != SPHG_COMPUTE_SORTED || !s->nbr ||
      s->n == 0)
    return false;
  return sphg::fused_blocks(s->args(), s->opt.precision) > 0;
}

// post: after a full sort (ranges, density, forces); else the merge first.
sphg_status enqueue_fused(sphg_sim* s, cudaStream_t st, bool post, unsigned long long cond) {
  SPHG_CUDA(sphg::launch_fused(s->args(), mover_args(s, cond), s->opt.precision, s->flags + 10, s->flags + 12, post,
                               st));
  return SPHG_OK;
}

// The full stable radix sort of the next keys (skip: device word that makes
// its kernels return at once, or null).
sphg_status enqueue_full_sort(sphg_sim* s, cudaStream_t st, const uint32_t* skip) {
  SPHG_CUDA(sphg::radix_sort_pairs(s->keyB, nullptr, s->keyTmp, s->perm, s->keyA, s->valTmp,
                                   s->scratch, s->n, s->key_bits, st, s->flags + 2, nullptr, skip));
  return SPHG_OK;
}

// Reorder + cell ranges, density, forces + integration (ev: events 3..5).
// size_lists: (lists mode) size the index buffer from this iteration's total
// first -- a host synchronisation, done on the first iteration after an upload
// (never inside a graph capture).
sphg_status enqueue_after_sort(sphg_sim* s, cudaStream_t st, cudaEvent_t* ev, bool size_lists = false) {
  const StepArgs a = s->args();
  const int prec = s->opt.precision;
  if (s->tile_bits) SPHG_CUDA(cudaMemsetAsync(s->flags + 1, 0, sizeof(uint32_t), st));
  // (the reorder zeroes the mover count of this iteration's force pass)
  SPHG_CUDA(sphg::launch_reorder(a, st));
  if (ev) SPHG_CUDA(cudaEventRecord(ev[3], st));
  if (s->opt.compute == SPHG_COMPUTE_LISTS) {
    // AssembleNeighborList: count, offsets, fill -- then density and forces over the lists
    SPHG_CUDA(sphg::launch_lists_count_scan(a, prec, s->csr_counts, s->csr_offs, s->csr_sums, st));
    if (size_lists || !s->csr_idx) {
      cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
      SPHG_CUDA(cudaStreamIsCapturing(st, &cs));
      if (cs != cudaStreamCaptureStatusNone)
        return fail(SPHG_INVALID_ARG, "lists mode: the neighbour-list buffer is sized before any graph capture");
      SPHG_CUDA(cudaMemcpyAsync(&s->csr_total, s->csr_sums + sphg::lists_scan_tiles(s->n), sizeof(int64_t),
                                cudaMemcpyDeviceToHost, st));
      SPHG_CUDA(cudaStreamSynchronize(st));
      // twice this iteration's total (the lists of a compressing flow grow):
      // later iterations run without a host synchronisation and report an
      // overflow past it through the overflow word
      const int64_t cap = 2 * s->csr_total + 1024;
      if (cap > s->csr_cap) {
        if (s->csr_idx) SPHG_CUDA(cudaFree(s->csr_idx));
        s->csr_idx = nullptr;
        s->csr_cap = 0;
        s->drop_graphs();  // their kernels hold the old buffer
        cudaError_t e = cudaMalloc(&s->csr_idx, (size_t)cap * sizeof(uint32_t));
        if (e != cudaSuccess)
          return fail(SPHG_OOM, std::string("neighbour-list buffer: ") + cudaGetErrorString(e));
        s->csr_cap = cap;
      }
    }
    const StepArgs b = s->args();
    SPHG_CUDA(sphg::launch_lists_fill_packed(b, prec, s->csr_offs, s->csr_idx, s->csr_cap, s->flags + 8, st));
    SPHG_CUDA(sphg::launch_density(b, prec, st, true));
    if (ev) SPHG_CUDA(cudaEventRecord(ev[4], st));
    SPHG_CUDA(sphg::launch_force(b, prec, sphg::kForceIntegrate, st, true));
  } else if (s->tile_bits) {
    SPHG_CUDA(sphg::launch_tiled(a, prec, false, st));
    if (ev) SPHG_CUDA(cudaEventRecord(ev[4], st));
    SPHG_CUDA(sphg::launch_tiled(a, prec, true, st));
  } else {
    SPHG_CUDA(sphg::launch_density(a, prec, st));
    if (ev) SPHG_CUDA(cudaEventRecord(ev[4], st));
    SPHG_CUDA(sphg::launch_force(a, prec, sphg::kForceIntegrate, st));
  }
  if (ev) SPHG_CUDA(cudaEventRecord(ev[5], st));
  return SPHG_OK;
}

// One main-loop iteration.  The force kernel writes the keys of the integrated
// state, so the key pass only runs on the first iteration after an upload.
// With ev (6 events) the phase boundaries are recorded: start, keys, sort,
// reorder, density, force.
sphg_status enqueue_step(sphg_sim* s, cudaStream_t st, bool first, cudaEvent_t* ev) {
  if (!ev && fused_on(s)) {
    // one launch when the merge handles the iteration; else the full sort and
    // the launch's post part (the full sort's kernels and the post launch
    // return at once on the merge's decision word)
    if (first) SPHG_CUDA(sphg::launch_keys(s->args(), s->opt.precision, st));
    const bool inc = !first && !s->force_full_sort;
    s->force_full_sort = false;
    if (inc) SPHG_TRY(enqueue_fused(s, st, false, 0));
    else SPHG_CUDA(cudaMemsetAsync(s->flags + 3, 0, sizeof(uint32_t), st));
    SPHG_TRY(enqueue_full_sort(s, st, inc ? s->flags + 3 : nullptr));
    return enqueue_fused(s, st, true, 0);
  }
  if (ev) SPHG_CUDA(cudaEventRecord(ev[0], st));
  if (first) SPHG_CUDA(sphg::launch_keys(s->args(), s->opt.precision, st));
  if (ev) SPHG_CUDA(cudaEventRecord(ev[1], st));
  // the force pass of the previous iteration recorded which slots changed
  // cell: merge them in when few did (the full sort's kernels then skip)
  const bool inc = s->movers_on && !first && !s->force_full_sort;
  s->force_full_sort = false;
  if (inc) SPHG_TRY(enqueue_movers(s, st, 0));
  // without the merge this iteration, its decision word must read "full sort"
  else if (s->movers_on) SPHG_CUDA(cudaMemsetAsync(s->flags + 3, 0, sizeof(uint32_t), st));
  SPHG_TRY(enqueue_full_sort(s, st, inc ? s->flags + 3 : nullptr));
  if (ev) SPHG_CUDA(cudaEventRecord(ev[2], st));
  return enqueue_after_sort(s, st, ev, first);
}

// The step header of the current state into the header slot (graph-capturable).
sphg_status enqueue_header(sphg_sim* s, cudaStream_t st) {
  int64_t max_n = 0;
  for (const InstDesc& d : s->hdesc) max_n = std::max<int64_t>(max_n, d.end - d.begin);
  SPHG_CUDA(sphg::launch_diagnostics_slot(s->args(), s->opt.precision, s->diag_partials, s->diag_tickets,
                                          sphg::diag_chunks(max_n, s->ninst, s->diag_chunks), s->hslot, st));
  return SPHG_OK;
}

// Graph of one iteration with the full sort under a conditional node: the
// incremental re-sort's decision kernel switches it off, so iterations that
// merge launch none of the full sort's kernels.

sphg_status build_graph_conditional(sphg_sim* s, cudaGraphExec_t* exec, bool header) {
  if (!s->cap_stream2) SPHG_CUDA(cudaStreamCreateWithFlags(&s->cap_stream2, cudaStreamNonBlocking));
  cudaGraph_t g = nullptr;
  SPHG_CUDA(cudaGraphCreate(&g, 0));
  auto done = [&](sphg_status st) {
    cudaStreamCaptureStatus cs;
    if (cudaStreamIsCapturing(s->cap_stream, &cs) == cudaSuccess && cs != cudaStreamCaptureStatusNone) {
      cudaGraph_t junk = nullptr;
      cudaStreamEndCapture(s->cap_stream, &junk);
      if (junk && junk != g) cudaGraphDestroy(junk);
    }
    if (cudaStreamIsCapturing(s->cap_stream2, &cs) == cudaSuccess && cs != cudaStreamCaptureStatusNone) {
      cudaGraph_t junk = nullptr;
      cudaStreamEndCapture(s->cap_stream2, &junk);
    }
    if (g) cudaGraphDestroy(g);
    return st;
  };
  cudaGraphConditionalHandle h = 0;
  if (cudaGraphConditionalHandleCreate(&h, g, 1u, cudaGraphCondAssignDefault) != cudaSuccess)
    return done(fail(SPHG_CUDA_ERROR, "conditional handle"));
  if (cudaStreamBeginCaptureToGraph(s->cap_stream, g, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal) !=
      cudaSuccess)
    return done(fail(SPHG_CUDA_ERROR, "capture to graph"));
  const bool fused = fused_on(s);
  sphg_status st = fused ? enqueue_fused(s, s->cap_stream, false, (unsigned long long)h)
                         : enqueue_movers(s, s->cap_stream, (unsigned long long)h);
  if (st != SPHG_OK) return done(st);
  cudaStreamCaptureStatus cst;
  const cudaGraphNode_t* deps = nullptr;
  size_t ndeps = 0;
  if (cudaStreamGetCaptureInfo(s->cap_stream, &cst, nullptr, nullptr, &deps, nullptr, &ndeps) != cudaSuccess)
    return done(fail(SPHG_CUDA_ERROR, "capture info"));
  cudaGraphNodeParams cp = {};
  cp.type = cudaGraphNodeTypeConditional;
  cp.conditional.handle = h;
  cp.conditional.type = cudaGraphCondTypeIf;
  cp.conditional.size = 1;
  cudaGraphNode_t cnode = nullptr;
  if (cudaGraphAddNode(&cnode, g, deps, nullptr, ndeps, &cp) != cudaSuccess)
    return done(fail(SPHG_CUDA_ERROR, "conditional node"));
  cudaGraph_t body = cp.conditional.phGraph_out[0];
  if (cudaStreamBeginCaptureToGraph(s->cap_stream2, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal) !=
      cudaSuccess)
    return done(fail(SPHG_CUDA_ERROR, "capture of the conditional body"));
  st = enqueue_full_sort(s, s->cap_stream2, nullptr);
  if (st == SPHG_OK && fused) st = enqueue_fused(s, s->cap_stream2, true, 0);  // ranges, density, forces
  cudaGraph_t body_out = nullptr;
  const cudaError_t eb = cudaStreamEndCapture(s->cap_stream2, &body_out);
  if (st != SPHG_OK) return done(st);
  if (eb != cudaSuccess) return done(fail(SPHG_CUDA_ERROR, "end of the conditional body capture"));
  if (cudaStreamUpdateCaptureDependencies(s->cap_stream, &cnode, nullptr, 1, cudaStreamSetCaptureDependencies) != cudaSuccess)
    return done(fail(SPHG_CUDA_ERROR, "capture dependencies"));
  if (!fused) st = enqueue_after_sort(s, s->cap_stream, nullptr);
  if (st == SPHG_OK && header) st = enqueue_header(s, s->cap_stream);
  if (st != SPHG_OK) return done(st);
  cudaGraph_t out = nullptr;
  if (cudaStreamEndCapture(s->cap_stream, &out) != cudaSuccess) return done(fail(SPHG_CUDA_ERROR, "end capture"));
  const cudaError_t e = cudaGraphInstantiate(exec, g, 0);
  cudaGraphDestroy(g);
  g = nullptr;
  if (e != cudaSuccess) {
    *exec = nullptr;
    return fail(SPHG_CUDA_ERROR, std::string("instantiate: ") + cudaGetErrorString(e));
  }
  return SPHG_OK;
}

// The graph of one iteration (header: followed by its step header into the
// header slot).
sphg_status build_graph(sphg_sim* s, bool header) {
  cudaGraphExec_t* exec = header ? &s->gexec_hdr : &s->gexec;
  if (*exec) return SPHG_OK;
  if (!s->cap_stream) SPHG_CUDA(cudaStreamCreateWithFlags(&s->cap_stream, cudaStreamNonBlocking));
  if (s->movers_on && s->cond_graph) {
    if (build_graph_conditional(s, exec, header) == SPHG_OK) return SPHG_OK;
    s->cond_graph = false;  // not available here: the full sort's kernels skip themselves instead
    cudaGetLastError();
  }
  cudaGraph_t g = nullptr;
  SPHG_CUDA(cudaStreamBeginCapture(s->cap_stream, cudaStreamCaptureModeThreadLocal));
  sphg_status st = enqueue_step(s, s->cap_stream);
  if (st == SPHG_OK && header) st = enqueue_header(s, s->cap_stream);
  cudaError_t e = cudaStreamEndCapture(s->cap_stream, &g);
  if (st != SPHG_OK) {
    if (g) cudaGraphDestroy(g);
    return st;
  }
  SPHG_CUDA(e);
  e = cudaGraphInstantiate(exec, g, 0);
  cudaGraphDestroy(g);
  SPHG_CUDA(e);
  return SPHG_OK;
}

sphg_status run_steps(sphg_sim* s, int64_t k, cudaStream_t st, bool first = false) {
  if (s->n == 0) return SPHG_OK;
  if (first) {
    SPHG_TRY(enqueue_step(s, st, true));
    --k;
  }
  if (s->opt.use_graph) {
    SPHG_TRY(build_graph(s));
    for (int64_t i = 0; i < k; ++i) SPHG_CUDA(cudaGraphLaunch(s->gexec, st));
  } else {
    for (int64_t i = 0; i < k; ++i) SPHG_TRY(enqueue_step(s, st));
  }
  return SPHG_OK;
}


// Options shared by every handle: precision mode, cell tiles (Morton only).
sphg_status check_options(sphg_sim* s, int ninst, const sphg_params* p) {
  if (s->opt.precision != SPHG_PRECISION_PLAIN && s->opt.precision != SPHG_PRECISION_SPLIT)
    return fail(SPHG_INVALID_ARG, "unknown precision mode");
  bool all_morton = true;
  for (int i = 0; i < ninst; ++i) all_morton = all_morton && p[i].order == SPHG_ORDER_MORTON;
  int tb = s->opt.tile_bits;
  if (tb == 0) tb = -1;  // default: one thread per particle (faster than the tiles at these densities)
  if (tb > 0 && (!all_morton || tb < 3 || tb > 5))
    return fail(SPHG_INVALID_ARG, "cell tiles need Morton order on every instance and tile_bits in 3..5");
  if (s->opt.compute != SPHG_COMPUTE_SORTED && s->opt.compute != SPHG_COMPUTE_LISTS)
    return fail(SPHG_INVALID_ARG, "unknown compute mode");
  const int bt = s->opt.block_threads;
  if (bt != 0 && bt != 64 && bt != 128 && bt != 256)
    return fail(SPHG_INVALID_ARG, "block_threads must be 0 (default), 64, 128 or 256");
  if (s->opt.cell_pairs < 0 || s->opt.cell_pairs > 1) return fail(SPHG_INVALID_ARG, "cell_pairs must be 0 or 1");
  if (s->opt.fused < 0 || s->opt.fused > 1) return fail(SPHG_INVALID_ARG, "fused must be 0 or 1");
  if (s->opt.compute == SPHG_COMPUTE_LISTS) {
    if (tb > 0) return fail(SPHG_INVALID_ARG, "the lists compute mode runs without cell tiles");
    tb = -1;
  }
  s->tile_bits = tb > 0 ? tb : 0;
  // the tile kernels do not record which slots changed cell
  s->movers_on = s->opt.resort != 0 && s->tile_bits == 0;
  return SPHG_OK;
}

// Descriptors of ninst instances laid out one after the other; cell keys of
// instance i start at the sum of the previous spans (rounded to a tile block
// when tiles are on, so no tile spans two instances).  keys_cap > 0 bounds the
// key space.
sphg_status compute_layout(sphg_sim* s, int ninst, const sphg_params* p, const int64_t* counts,
                           uint64_t keys_cap, Layout& L) {
  const uint64_t key_align = s->tile_bits ? ((uint64_t)1 << (2 * 5)) : 1;
  L.desc.assign(ninst, InstDesc());
  L.begins.assign(ninst, 0);
  L.n = 0;
  L.keys = 0;
  L.max_n = 0;
  for (int i = 0; i < ninst; ++i) {
    if (counts[i] < 0) return fail(SPHG_INVALID_ARG, "negative particle count");
    uint64_t span = 0;
    SPHG_TRY(make_desc(p[i], L.n, counts[i], L.keys, L.desc[i], span));
    L.begins[i] = (int32_t)L.n;
    L.n += counts[i];
    L.keys += (span + key_align - 1) / key_align * key_align;
    L.max_n = std::max(L.max_n, counts[i]);
    if (L.n > sphg::kSortMaxKeys || L.keys >= (uint64_t)0xfffffff0u)
      return fail(SPHG_CAPACITY, "more than 2^30-1 particles or 2^32 cell keys in one handle");
  }
  if (keys_cap && L.keys > keys_cap) return fail(SPHG_CAPACITY, "cell keys exceed the handle's key capacity");
  return SPHG_OK;
}

// One device arena sized for N particles, `keys` cell keys and ninst instances.
sphg_status alloc_arena(sphg_sim* s, size_t N, uint64_t keys, int ninst, int diag_chunks) {
  s->cap_n = N;
  s->cap_keys = keys;
  s->cap_inst = ninst;
  s->diag_chunks = diag_chunks;
  // per-particle neighbour slots filled by the density pass and read by the
  // force pass (indices are packed as j << 5, so only below 2^27 particles)
  s->nbr_slots = (N < ((size_t)1 << 27) && s->opt.compute == SPHG_COMPUTE_SORTED) ? 12 : 0;
  auto layout = [&](Arena& A) {
    s->ddesc = A.take<InstDesc>(ninst);
    s->dbegins = A.take<int32_t>(ninst);
    s->dinst_tab = A.take<int32_t>((N >> sphg::kInstTabShift) + 2);
    s->posA = A.take<float2>(N + 1);  // one padding entry: the density walk prefetches one past its last candidate
    s->posB = A.take<float2>(N);
    s->velB = A.take<float2>(N);
    s->acc = A.take<float2>(N);
    s->velpA = A.take<float4>(N);
    s->rho = A.take<float>(N);
    s->keyA = A.take<uint32_t>(N);
    s->keyB = A.take<uint32_t>(N);
    s->keyTmp = A.take<uint32_t>(N);
    s->perm = A.take<uint32_t>(N);
    s->valTmp = A.take<uint32_t>(N);
    s->scratch = A.take<uint32_t>(sphg::sort_scratch_words(N));
    s->flags = A.take<uint32_t>(16);
    s->diag_partials = A.take<double>((size_t)ninst * s->diag_chunks * 6);
    s->diag_out = A.take<double>((size_t)ninst * 6);
    s->hslot = A.take<sphg::HeaderSlot>(1);
    s->diag_tickets = A.take<uint32_t>(ninst);
    // (instance, chunk) of every diagnostics block of several instances: at most
    // one per 4,096 particles plus one per instance
    s->ddiag_tab = A.take<uint32_t>(N / 4096 + (size_t)ninst + 1);
    if (s->opt.track_ids) {
      s->idsA = A.take<int32_t>(N);
      s->idsB = A.take<int32_t>(N);
    }
    if (s->nbr_slots) {
      s->nbr = A.take<uint32_t>(N * (size_t)s->nbr_slots);
      s->ncount = A.take<uint32_t>(N);
    }
    if (s->movers_on) {
      s->mmask = A.take<uint32_t>((N + 31) / 32);
      s->mlist = A.take<unsigned long long>(sphg::kMoverCap);
    }
    if (s->opt.compute == SPHG_COMPUTE_LISTS) {
      s->csr_counts = A.take<int32_t>(N);
      s->csr_offs = A.take<int64_t>(N + 1);
      s->csr_sums = A.take<int64_t>((size_t)sphg::lists_scan_tiles((int64_t)N) + 1);
    }
    if (s->tile_bits) {
      s->tile_ranges = A.take<uint2>((keys >> (2 * s->tile_bits)) + 1);
      s->tile_list = A.take<uint32_t>(std::min<uint64_t>(N, (keys >> (2 * s->tile_bits)) + 1));
    }
    s->ranges = A.take<uint4>(std::max<uint64_t>(keys, 1));
  };
  if (s->tile_bits) {
    const int fw = (1 << s->tile_bits) + 2;
    s->tile_cap = (3 * fw * fw + 127) / 128 * 128;
    const uint64_t max_tiles = std::min<uint64_t>(N, (keys >> (2 * s->tile_bits)) + 1);
    s->tile_grid = (int)std::min<uint64_t>(max_tiles, 4096);
  }
  Arena probe;
  layout(probe);
  cudaError_t e = cudaMalloc(&s->arena.base, probe.used);
  if (e != cudaSuccess)
    return fail(SPHG_OOM, std::string("cudaMalloc of the state arena failed: ") + cudaGetErrorString(e));
  s->arena.size = probe.used;
  layout(s->arena);
  // everything starts at zero: the step epoch (flags[2]) is bumped to 1 by the
  // first sort, so no range entry is valid before its cell is written; the
  // table is never cleared again
  e = cudaMemset(s->arena.base, 0, s->arena.size);
  if (e != cudaSuccess) return fail(SPHG_CUDA_ERROR, std::string("state init: ") + cudaGetErrorString(e));
  return SPHG_OK;
}

// Makes layout L current: host copies, key bits, descriptors on the device
// (stream-ordered when stream is given, else synchronous).
sphg_status apply_layout(sphg_sim* s, int ninst, const sphg_params* p, const int64_t* counts,
                         const Layout& L, cudaStream_t* stream) {
  if (ninst > s->cap_inst || (size_t)L.n > s->cap_n || L.keys > std::max<uint64_t>(s->cap_keys, 1))
    return fail(SPHG_CAPACITY, "layout exceeds the handle's capacity");
  s->ninst = ninst;
  s->params.assign(p, p + ninst);
  s->counts.assign(counts, counts + ninst);
  s->hdesc = L.desc;
  s->hbegins = L.begins;
  s->n = L.n;
  s->total_keys = L.keys;
  int bits = 1;
  while (bits < 32 && ((uint64_t)1 << bits) < L.keys) ++bits;
  s->key_bits = bits;
  s->drop_graphs();  // grid sizes depend on the layout
  // instance of the first slot of every 256-slot block
  const int64_t blocks = (s->n >> sphg::kInstTabShift) + 1;
  s->hinst_tab.assign((size_t)blocks, 0);
  for (int64_t b = 0, k = 0; b < blocks; ++b) {
    const int64_t slot = b << sphg::kInstTabShift;
    while (k + 1 < ninst && s->hbegins[k + 1] <= slot) ++k;
    s->hinst_tab[b] = (int32_t)k;
  }
  // step headers of several instances: one diagnostics block per (instance,
  // chunk) the instance uses (about 4,096 particles a block), as one 1-D grid
  s->hdiag_tab.clear();
  if (ninst > 1) {
    const int chunks = sphg::diag_chunks(L.max_n, ninst, s->diag_chunks);
    for (int k = 0; k < ninst; ++k)
      for (int c = 0, ck = sphg::diag_instance_chunks(s->hdesc[k].end - s->hdesc[k].begin, chunks); c < ck; ++c)
        s->hdiag_tab.push_back(((uint32_t)k << 12) | (uint32_t)c);
  }
  const size_t ntab = s->hdiag_tab.size();
  if (stream) {
    SPHG_CUDA(cudaMemcpyAsync(s->ddesc, s->hdesc.data(), sizeof(InstDesc) * ninst, cudaMemcpyHostToDevice, *stream));
    SPHG_CUDA(cudaMemcpyAsync(s->dbegins, s->hbegins.data(), sizeof(int32_t) * ninst, cudaMemcpyHostToDevice, *stream));
    SPHG_CUDA(cudaMemcpyAsync(s->dinst_tab, s->hinst_tab.data(), sizeof(int32_t) * blocks, cudaMemcpyHostToDevice, *stream));
    if (ntab)
      SPHG_CUDA(cudaMemcpyAsync(s->ddiag_tab, s->hdiag_tab.data(), sizeof(uint32_t) * ntab, cudaMemcpyHostToDevice, *stream));
  } else {
    SPHG_CUDA(cudaMemcpy(s->ddesc, s->hdesc.data(), sizeof(InstDesc) * ninst, cudaMemcpyHostToDevice));
    SPHG_CUDA(cudaMemcpy(s->dbegins, s->hbegins.data(), sizeof(int32_t) * ninst, cudaMemcpyHostToDevice));
    SPHG_CUDA(cudaMemcpy(s->dinst_tab, s->hinst_tab.data(), sizeof(int32_t) * blocks, cudaMemcpyHostToDevice));
    if (ntab) SPHG_CUDA(cudaMemcpy(s->ddiag_tab, s->hdiag_tab.data(), sizeof(uint32_t) * ntab, cudaMemcpyHostToDevice));
  }
  return SPHG_OK;
}

sphg_status destroy_impl(sphg_sim* s) {
  if (!s) return SPHG_OK;
  s->drop_graphs();
  if (s->cap_stream) cudaStreamDestroy(s->cap_stream);
  if (s->cap_stream2) cudaStreamDestroy(s->cap_stream2);
  if (s->arena.base) cudaFree(s->arena.base);
  if (s->csr_idx) cudaFree(s->csr_idx);
  if (s->hstage) cudaFreeHost(s->hstage);
  delete s;
  return SPHG_OK;
}

}  // namespace sphg_detail

using namespace sphg_detail;

extern "C" {

void sphg_default_params(sphg_params* p) {
  if (!p) return;
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
  p->order = SPHG_ORDER_ROWMAJOR;
  p->periodic = 0;
}

void sphg_default_options(sphg_options* o) {
  if (!o) return;
  o->precision = SPHG_PRECISION_PLAIN;
  o->track_ids = 1;
  o->use_graph = 1;
  o->tile_bits = 0;
  o->compute = SPHG_COMPUTE_SORTED;
  o->resort = 1;
  o->block_threads = 0;
  o->cell_pairs = 0;
  o->fused = 0;
}

const char* sphg_last_error_string(void) { return g_err.c_str(); }

const char* sphg_version(void) { return "sphg 0.1 (sm_103a)"; }

sphg_status sphg_set_host_access(sphg_sim* s, int32_t direct) {
  if (!s) return fail(SPHG_INVALID_ARG, "null handle");
  if (direct) {
    int dev = 0, pageable = 0;
    SPHG_CUDA(cudaGetDevice(&dev));
    SPHG_CUDA(cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, dev));
    if (!pageable) return fail(SPHG_INVALID_ARG, "this device cannot access pageable host memory");
  }
  s->host_direct = direct < 0 ? 0 : (direct > 2 ? 2 : direct);
  return SPHG_OK;
}

sphg_status sphg_device_attributes(int32_t device, int32_t* out) {
  if (!out) return fail(SPHG_INVALID_ARG, "null argument");
  const cudaDeviceAttr attrs[6] = {cudaDevAttrComputeCapabilityMajor, cudaDevAttrComputeCapabilityMinor,
                                   cudaDevAttrMultiProcessorCount, cudaDevAttrPageableMemoryAccess,
                                   cudaDevAttrPageableMemoryAccessUsesHostPageTables,
                                   cudaDevAttrConcurrentManagedAccess};
  for (int k = 0; k < 6; ++k) {
    int v = 0;
    SPHG_CUDA(cudaDeviceGetAttribute(&v, attrs[k], device));
    out[k] = v;
  }
  return SPHG_OK;
}

sphg_status sphg_create_batch(int32_t ninst, const sphg_params* p, const int64_t* counts,
                              const sphg_options* o, sphg_sim** out) {
  if (!out || !p || !counts || ninst <= 0) return fail(SPHG_INVALID_ARG, "null argument or ninst <= 0");
  *out = nullptr;
  sphg_sim* s = new sphg_sim();
  if (o) s->opt = *o; else sphg_default_options(&s->opt);
  sphg_status st = check_options(s, ninst, p);
  if (st != SPHG_OK) {
    delete s;
    return st;
  }
  Layout L;
  st = compute_layout(s, ninst, p, counts, 0, L);
  if (st != SPHG_OK) {
    delete s;
    return st;
  }
  st = alloc_arena(s, (size_t)std::max<int64_t>(L.n, 1), L.keys, ninst, sphg::diag_chunks(L.max_n, ninst));
  if (st != SPHG_OK) {
    delete s;
    return st;
  }
  st = apply_layout(s, ninst, p, counts, L, nullptr);
  if (st == SPHG_OK) {
    int dev = 0, pageable = 0;
    if (cudaGetDevice(&dev) == cudaSuccess &&
        cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, dev) == cudaSuccess)
      s->host_direct = pageable != 0 ? 1 : 0;
  }
  // set-up that would otherwise land on the first upload / step: the pinned
  // staging of upload and download, and the captured graph of an iteration
  if (st == SPHG_OK && s->n > 0 &&
      !host_stage(s, (size_t)s->n * (sizeof(float2) * 2 + sizeof(float4) + sizeof(float) + sizeof(uint32_t))))
    st = fail(SPHG_OOM, "pinned host staging");
  // (lists mode: captured after the pre-loop has sized the list buffer)
  const bool capture_now = s->opt.use_graph && s->opt.compute != SPHG_COMPUTE_LISTS;
  if (st == SPHG_OK && s->n > 0 && capture_now) st = build_graph(s);
  if (st == SPHG_OK && s->n > 0 && capture_now) st = build_graph(s, true);  // with step headers
  if (st != SPHG_OK) {
    destroy_impl(s);
    return st;
  }
  *out = s;
  return SPHG_OK;
}

sphg_status sphg_create(const sphg_params* p, const sphg_options* o, int64_t n, sphg_sim** out) {
  return sphg_create_batch(1, p, &n, o, out);
}

sphg_status sphg_destroy(sphg_sim* s) { return destroy_impl(s); }

sphg_status sphg_upload(sphg_sim* s, const double* x, const double* y, const double* vx,
                        const double* vy, void* stream) {
  if (!s || (s->n > 0 && (!x || !y || !vx || !vy))) return fail(SPHG_INVALID_ARG, "null argument");
  cudaStream_t st = (cudaStream_t)stream;
  const int64_t n = s->n;
  if (n > 0 && s->host_direct) {
    uint32_t first_bad = 0;
    SPHG_CUDA(cudaMemsetAsync(s->flags + 6, 0xff, sizeof(uint32_t), st));
    SPHG_CUDA(sphg::launch_upload_direct(s->args(), s->opt.precision, x, y, vx, vy, s->flags + 6, st));
    SPHG_CUDA(cudaMemsetAsync(s->scratch, 0, sizeof(uint32_t) * 4 * 256, st));
    SPHG_CUDA(cudaMemcpyAsync(&first_bad, s->flags + 6, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    SPHG_CUDA(cudaStreamSynchronize(st));
    if (first_bad != 0xffffffffu)
      return fail(SPHG_NONFINITE, "non-finite value in the uploaded state at particle " + std::to_string(first_bad));
  } else if (n > 0) {
    // pinned staging: positions (or split offsets), velocities, split cell keys, creation indices
    char* stg = host_stage(s, (size_t)n * (sizeof(float2) * 2 + sizeof(uint32_t) + sizeof(int32_t)));
    if (!stg) return fail(SPHG_OOM, "pinned host staging");
    float2* pos = reinterpret_cast<float2*>(stg);
    float2* vel = pos + n;
    uint32_t* key = reinterpret_cast<uint32_t*>(vel + n);
    int32_t* ids = reinterpret_cast<int32_t*>(key + n);
    const bool split = s->opt.precision == SPHG_PRECISION_SPLIT;
    std::atomic<int64_t> bad{n};
    parallel_for(n, [&](int64_t b, int64_t e) {
      int inst = instance_of(s, b);
      for (int64_t i = b; i < e; ++i) {
        while (i >= s->hdesc[inst].end) ++inst;
        const InstDesc& d = s->hdesc[inst];
        if (!std::isfinite(x[i]) || !std::isfinite(y[i]) || !std::isfinite(vx[i]) || !std::isfinite(vy[i])) {
          int64_t cur = bad.load();
          while (i < cur && !bad.compare_exchange_weak(cur, i)) {
          }
          return;
        }
        vel[i] = make_float2((float)vx[i], (float)vy[i]);
        ids[i] = (int32_t)i;
        if (split) {
          const int cmx = d.periodic ? d.nxr - 1 : d.nx - 1;
          const int cmy = d.periodic ? d.nyr - 1 : d.ny - 1;
          int cx = host_cell(x[i], d.lo_xd, d.cs_xd, cmx);
          int cy = host_cell(y[i], d.lo_yd, d.cs_yd, cmy);
          uint32_t code = d.order == 0 ? morton_host(cx, cy) : (uint32_t)(cx + cy * d.nx);
          key[i] = d.cell_base + code;
          pos[i] = make_float2(split_offset((x[i] - d.lo_xd) - cx * d.cs_xd, d.cs_xd),
                               split_offset((y[i] - d.lo_yd) - cy * d.cs_yd, d.cs_yd));
        } else {
          pos[i] = make_float2((float)x[i], (float)y[i]);
        }
      }
    });
    if (bad.load() < n)
      return fail(SPHG_NONFINITE, "non-finite value in the uploaded state at particle " + std::to_string(bad.load()));
    SPHG_CUDA(cudaMemcpyAsync(s->posB, pos, n * sizeof(float2), cudaMemcpyHostToDevice, st));
    SPHG_CUDA(cudaMemcpyAsync(s->velB, vel, n * sizeof(float2), cudaMemcpyHostToDevice, st));
    if (split) SPHG_CUDA(cudaMemcpyAsync(s->keyA, key, n * sizeof(uint32_t), cudaMemcpyHostToDevice, st));
    if (s->opt.track_ids) SPHG_CUDA(cudaMemcpyAsync(s->idsB, ids, n * sizeof(int32_t), cudaMemcpyHostToDevice, st));
    // digit histograms of the next sort restart with the uploaded state
    SPHG_CUDA(cudaMemsetAsync(s->scratch, 0, sizeof(uint32_t) * 4 * 256, st));
    SPHG_CUDA(cudaStreamSynchronize(st));
  }
  s->uploaded = true;
  s->preloop_done = false;
  return SPHG_OK;
}

sphg_status sphg_preloop(sphg_sim* s, void* stream) {
  if (!s || !s->uploaded) return fail(SPHG_INVALID_ARG, "upload a state before the pre-loop");
  // PreLoopComputation: FindNeighbors -> density -> pressure -> forces.  The
  // forces are consumed at once by the fused integration of the next state.
  SPHG_TRY(run_steps(s, 1, (cudaStream_t)stream, true));
  s->preloop_done = true;
  return SPHG_OK;
}

sphg_status sphg_step(sphg_sim* s, int64_t nsteps, void* stream) {
  if (!s || !s->preloop_done) return fail(SPHG_INVALID_ARG, "run sphg_preloop before sphg_step");
  if (nsteps < 0) return fail(SPHG_INVALID_ARG, "nsteps < 0");
  return run_steps(s, nsteps, (cudaStream_t)stream);
}

// Error words the kernels set instead of faulting or hanging: the radix sort's
// look-back (a wait that gave up) and the incremental re-sort's consistency
// word.  Read at the synchronising calls; both stay set.
static sphg_status device_errors(sphg_sim* s, cudaStream_t st) {
  uint32_t w[4] = {0, 0, 0, 0};
  SPHG_CUDA(cudaMemcpyAsync(&w[0], sphg::sort_error_word(s->scratch), sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
  SPHG_CUDA(cudaMemcpyAsync(&w[1], s->flags + 5, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
  SPHG_CUDA(cudaMemcpyAsync(&w[2], s->flags + 8, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
  SPHG_CUDA(cudaMemcpyAsync(&w[3], s->flags + 12, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
  SPHG_CUDA(cudaStreamSynchronize(st));
  if (w[3]) return fail(SPHG_TIMEOUT, "a grid-wide barrier of the single-launch iteration gave up; the state is not valid");
  if (w[0]) return fail(SPHG_TIMEOUT, "a radix-sort look-back wait gave up; the state is not valid");
  if (w[1]) return fail(SPHG_CUDA_ERROR, "inconsistent incremental re-sort record; the state is not valid");
  if (w[2]) return fail(SPHG_CAPACITY, "lists mode: the neighbour lists outgrew their buffer (twice the pre-loop's "
                                       "total); the state is not valid");
  return SPHG_OK;
}

sphg_status sphg_download(sphg_sim* s, double* x, double* y, double* vx, double* vy, double* rho,
                          double* fx, double* fy, int32_t* ids, void* stream) {
  if (!s || !s->preloop_done) return fail(SPHG_INVALID_ARG, "no computed state to download");
  cudaStream_t st = (cudaStream_t)stream;
  const int64_t n = s->n;
  if (n == 0) return SPHG_OK;
  const bool forces = fx || fy;
  if (s->host_direct == 2) {
    // writes from the device into pages the host has not touched yet fault them
    // in one by one, so the default download goes through the pinned staging
    if (forces) SPHG_CUDA(sphg::launch_force(s->args(), s->opt.precision, sphg::kForceOnly, st));
    SPHG_CUDA(sphg::launch_download_direct(s->args(), s->opt.precision, x, y, vx, vy, rho, fx, fy, ids, st));
    SPHG_CUDA(cudaStreamSynchronize(st));
    return device_errors(s, st);
  }
  char* stg = host_stage(s, (size_t)n * (sizeof(float2) * 2 + sizeof(float4) + sizeof(float) + sizeof(uint32_t)));
  if (!stg) return fail(SPHG_OOM, "pinned host staging");
  float4* velp = reinterpret_cast<float4*>(stg);
  float2* pos = reinterpret_cast<float2*>(velp + n);
  float2* acc = pos + n;
  float* r = reinterpret_cast<float*>(acc + n);
  uint32_t* key = reinterpret_cast<uint32_t*>(r + n);
  const bool split = s->opt.precision == SPHG_PRECISION_SPLIT;
  if (forces) {
    SPHG_CUDA(sphg::launch_force(s->args(), s->opt.precision, sphg::kForceOnly, st));
    SPHG_CUDA(cudaMemcpyAsync(acc, s->acc, n * sizeof(float2), cudaMemcpyDeviceToHost, st));
  }
  if (x || y) SPHG_CUDA(cudaMemcpyAsync(pos, s->posA, n * sizeof(float2), cudaMemcpyDeviceToHost, st));
  if (vx || vy) SPHG_CUDA(cudaMemcpyAsync(velp, s->velpA, n * sizeof(float4), cudaMemcpyDeviceToHost, st));
  if (rho) SPHG_CUDA(cudaMemcpyAsync(r, s->rho, n * sizeof(float), cudaMemcpyDeviceToHost, st));
  if (split && (x || y))
    SPHG_CUDA(cudaMemcpyAsync(key, s->keyA, n * sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
  if (ids && s->opt.track_ids)
    SPHG_CUDA(cudaMemcpyAsync(ids, s->idsA, n * sizeof(int32_t), cudaMemcpyDeviceToHost, st));
  SPHG_CUDA(cudaStreamSynchronize(st));
  SPHG_TRY(device_errors(s, st));
  if (ids && !s->opt.track_ids)
    for (int64_t i = 0; i < n; ++i) ids[i] = -1;
  parallel_for(n, [&](int64_t b, int64_t e) {
    int inst = instance_of(s, b);
    for (int64_t i = b; i < e; ++i) {
      while (i >= s->hdesc[inst].end) ++inst;
      const InstDesc& d = s->hdesc[inst];
      if (x || y) {
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
      }
      if (vx) vx[i] = velp[i].x;
      if (vy) vy[i] = velp[i].y;
      if (rho) rho[i] = r[i];
      if (fx) fx[i] = acc[i].x;
      if (fy) fy[i] = acc[i].y;
    }
  });
  return SPHG_OK;
}

sphg_status sphg_diagnostics(sphg_sim* s, double* out, void* stream) {
  if (!s || !out) return fail(SPHG_INVALID_ARG, "null argument");
  if (!s->preloop_done) return fail(SPHG_INVALID_ARG, "no computed state");
  cudaStream_t st = (cudaStream_t)stream;
  int64_t max_n = 0;
  for (const InstDesc& d : s->hdesc) max_n = std::max<int64_t>(max_n, d.end - d.begin);
  const int chunks = sphg::diag_chunks(max_n, s->ninst, s->diag_chunks);
  SPHG_CUDA(sphg::launch_diagnostics(s->args(), s->opt.precision, s->diag_partials, s->diag_tickets, chunks,
                                     s->diag_out, st));
  SPHG_CUDA(cudaMemcpyAsync(out, s->diag_out, sizeof(double) * 6 * s->ninst,
                            cudaMemcpyDeviceToHost, st));
  SPHG_CUDA(cudaStreamSynchronize(st));
  return device_errors(s, st);
}

sphg_status sphg_cfl_dt(sphg_sim* s, double cfl, double force_coef, double* out, void* stream) {
  if (!s || !out || !(cfl > 0) || !(force_coef > 0)) return fail(SPHG_INVALID_ARG, "null argument or coefficient <= 0");
  if (!s->preloop_done) return fail(SPHG_INVALID_ARG, "no computed state");
  cudaStream_t st = (cudaStream_t)stream;
  if (s->n > 0) {
    SPHG_CUDA(sphg::launch_force(s->args(), s->opt.precision, sphg::kForceOnly, st));
    int64_t max_n = 0;
    for (const InstDesc& d : s->hdesc) max_n = std::max<int64_t>(max_n, d.end - d.begin);
    const int chunks = sphg::diag_chunks(max_n, s->ninst, s->diag_chunks);
    SPHG_CUDA(sphg::launch_cfl(s->args(), s->diag_partials, chunks, s->diag_out, st));
  }
  std::vector<double> m((size_t)6 * s->ninst, 0.0);
  if (s->n > 0) {
    SPHG_CUDA(cudaMemcpyAsync(m.data(), s->diag_out, sizeof(double) * 6 * s->ninst, cudaMemcpyDeviceToHost, st));
    SPHG_CUDA(cudaStreamSynchronize(st));
  }
  for (int i = 0; i < s->ninst; ++i) {
    const sphg_params& p = s->params[i];
    const double vmax = std::sqrt(m[6 * i]), amax = std::sqrt(m[6 * i + 1]);
    double dt = std::numeric_limits<double>::infinity();
    if (p.c0 + vmax > 0) dt = std::min(dt, cfl * p.h / (p.c0 + vmax));
    if (amax > 0) dt = std::min(dt, force_coef * std::sqrt(p.h / amax));
    out[i] = dt;
  }
  return SPHG_OK;
}

sphg_status sphg_set_dt(sphg_sim* s, int32_t inst, double dt) {
  if (!s || !(dt > 0) || !std::isfinite(dt) || inst >= s->ninst) return fail(SPHG_INVALID_ARG, "bad handle, instance or dt");
  const int b = inst < 0 ? 0 : inst, e = inst < 0 ? s->ninst : inst + 1;
  for (int i = b; i < e; ++i) {
    s->params[i].dt = dt;
    s->hdesc[i].dt = (float)dt;
  }
  if (s->ninst > 0)
    SPHG_CUDA(cudaMemcpy(s->ddesc, s->hdesc.data(), sizeof(InstDesc) * s->ninst, cudaMemcpyHostToDevice));
  s->drop_graphs();  // the single-instance descriptor is a kernel argument of the captured graphs
  return SPHG_OK;
}

// A pointer through which kernels write the caller's array `out`, or null when
// they cannot (the values are then copied): device or managed memory, pinned
// host memory (mapped under unified addressing), or -- when host access is on
// and the device reads and writes pageable memory -- the array itself.
static double* device_view(sphg_sim* s, double* out) {
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, out) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  if (at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged) return out;
  if (at.type == cudaMemoryTypeHost) return static_cast<double*>(at.devicePointer);
  return s->host_direct ? out : nullptr;  // host_direct is set only where pageable access works
}

static int diag_chunk_count(const sphg_sim* s) {
  int64_t max_n = 0;
  for (const InstDesc& d : s->hdesc) max_n = std::max<int64_t>(max_n, d.end - d.begin);
  return sphg::diag_chunks(max_n, s->ninst, s->diag_chunks);
}

sphg_status sphg_diagnostics_async(sphg_sim* s, double* out, void* stream) {
  if (!s || !out) return fail(SPHG_INVALID_ARG, "null argument");
  if (!s->preloop_done) return fail(SPHG_INVALID_ARG, "no computed state");
  cudaStream_t st = (cudaStream_t)stream;
  const int chunks = diag_chunk_count(s);
  double* dv = device_view(s, out);
  SPHG_CUDA(sphg::launch_diagnostics(s->args(), s->opt.precision, s->diag_partials, s->diag_tickets, chunks, dv ? dv : s->diag_out,
                                     st));
  if (!dv) SPHG_CUDA(cudaMemcpyAsync(out, s->diag_out, sizeof(double) * 6 * s->ninst, cudaMemcpyDeviceToHost, st));
  return SPHG_OK;
}

sphg_status sphg_stream_synchronize(void* stream) {
  SPHG_CUDA(cudaStreamSynchronize((cudaStream_t)stream));
  return SPHG_OK;
}

sphg_status sphg_step_headers(sphg_sim* s, int64_t nsteps, double* out, void* stream) {
  if (!s || !s->preloop_done) return fail(SPHG_INVALID_ARG, "run sphg_preloop before sphg_step_headers");
  if (nsteps < 0) return fail(SPHG_INVALID_ARG, "nsteps < 0");
  if (nsteps == 0) return SPHG_OK;
  if (!out) return fail(SPHG_INVALID_ARG, "null argument");
  cudaStream_t st = (cudaStream_t)stream;
  const size_t per = (size_t)6 * s->ninst;
  double* dv = s->n > 0 ? device_view(s, out) : nullptr;
  if (!dv) {  // one copy per step
    const int chunks = diag_chunk_count(s);
    for (int64_t k = 0; k < nsteps; ++k) {
      SPHG_TRY(run_steps(s, 1, st));
      SPHG_CUDA(sphg::launch_diagnostics(s->args(), s->opt.precision, s->diag_partials, s->diag_tickets, chunks, s->diag_out, st));
      SPHG_CUDA(cudaMemcpyAsync(out + per * k, s->diag_out, sizeof(double) * per, cudaMemcpyDeviceToHost, st));
    }
    return SPHG_OK;
  }
  const sphg::HeaderSlot h = {dv, 0u, 0u};
  SPHG_CUDA(cudaMemcpyAsync(s->hslot, &h, sizeof(h), cudaMemcpyHostToDevice, st));
  if (s->opt.use_graph) {
    SPHG_TRY(build_graph(s, true));
    for (int64_t k = 0; k < nsteps; ++k) SPHG_CUDA(cudaGraphLaunch(s->gexec_hdr, st));
  } else {
    for (int64_t k = 0; k < nsteps; ++k) {
      SPHG_TRY(enqueue_step(s, st));
      SPHG_TRY(enqueue_header(s, st));
    }
  }
  return SPHG_OK;
}

sphg_status sphg_get_debug(sphg_sim* s, int32_t which, void* host, void* stream) {
  if (!s || !host) return fail(SPHG_INVALID_ARG, "null argument");
  cudaStream_t st = (cudaStream_t)stream;
  const int64_t n = s->n;
  if (n == 0) return SPHG_OK;
  auto local_keys = [&](const uint32_t* dev) -> sphg_status {
    std::vector<uint32_t> k(n);
    SPHG_CUDA(cudaMemcpyAsync(k.data(), dev, n * sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    SPHG_CUDA(cudaStreamSynchronize(st));
    int32_t* o = (int32_t*)host;
    for (int inst = 0; inst < s->ninst; ++inst) {
      const InstDesc& d = s->hdesc[inst];
      for (int64_t i = d.begin; i < d.end; ++i) o[i] = (int32_t)(k[i] - d.cell_base);
    }
    return SPHG_OK;
  };
  switch (which) {
    case SPHG_DBG_RESORT: {
      uint32_t c[3] = {0, 0, 0};
      if (s->movers_on) {
        SPHG_CUDA(cudaMemcpyAsync(c, s->flags + 3, 2 * sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
        SPHG_CUDA(cudaStreamSynchronize(st));
      }
      // histogram + radix passes of a full sort (+ the post part of the single-launch iteration)
      c[2] = (uint32_t)((s->key_bits + 7) / 8 + 1 + (fused_on(s) ? 1 : 0));
      std::memcpy(host, c, sizeof(c));
      return SPHG_OK;
    }
    case SPHG_DBG_KEYS: return local_keys(s->keyA);
    case SPHG_DBG_UNSORTED_KEYS: return local_keys(s->keyB);
    case SPHG_DBG_PERM:
      SPHG_CUDA(cudaMemcpyAsync(host, s->perm, n * sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
      SPHG_CUDA(cudaStreamSynchronize(st));
      return SPHG_OK;
    case SPHG_DBG_POS_NEXT:
    case SPHG_DBG_VEL_NEXT: {
      std::vector<float2> v(n);
      std::vector<uint32_t> k;
      const bool pos = which == SPHG_DBG_POS_NEXT;
      SPHG_CUDA(cudaMemcpyAsync(v.data(), pos ? s->posB : s->velB, n * sizeof(float2),
                                cudaMemcpyDeviceToHost, st));
      if (pos && s->opt.precision == SPHG_PRECISION_SPLIT) {
        k.resize(n);  // the integrated offsets are relative to their new cells
        SPHG_CUDA(cudaMemcpyAsync(k.data(), s->keyB, n * sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
      }
      SPHG_CUDA(cudaStreamSynchronize(st));
      double* o = (double*)host;
      for (int inst = 0; inst < s->ninst; ++inst) {
        const InstDesc& d = s->hdesc[inst];
        for (int64_t i = d.begin; i < d.end; ++i) {
          double a = v[i].x, b = v[i].y;
          if (!k.empty()) {
            int cx, cy;
            uint32_t code = k[i] - d.cell_base;
            if (d.order == 0) demorton_host(code, cx, cy);
            else { cx = (int)(code % (uint32_t)d.nx); cy = (int)(code / (uint32_t)d.nx); }
            a += d.lo_xd + cx * d.cs_xd;
            b += d.lo_yd + cy * d.cs_yd;
          }
          o[2 * i] = a;
          o[2 * i + 1] = b;
        }
      }
      return SPHG_OK;
    }
    default:
      return fail(SPHG_INVALID_ARG, "unknown debug view");
  }
}

sphg_status sphg_neighbor_lists(sphg_sim* s, int64_t* offs, int32_t* idx, int64_t* total,
                                void* stream) {
  if (!s || !s->preloop_done) return fail(SPHG_INVALID_ARG, "no computed state");
  std::string err;
  int st = sphg::lists_impl(s->args(), s->opt.precision, offs, idx, total, (cudaStream_t)stream, &err);
  if (st != SPHG_OK) return fail((sphg_status)st, err);
  return SPHG_OK;
}

sphg_status sphg_neighbor_lists_encoded(sphg_sim* s, int64_t* offs, int32_t* enc, int64_t* total,
                                        void* stream) {
  if (!s || !s->preloop_done) return fail(SPHG_INVALID_ARG, "no computed state");
  std::string err;
  int st = sphg::lists_impl(s->args(), s->opt.precision, offs, enc, total, (cudaStream_t)stream, &err, true);
  if (st != SPHG_OK) return fail((sphg_status)st, err);
  return SPHG_OK;
}

sphg_status sphg_delta_encode(const int64_t* offs, const int32_t* idx, int64_t n, int32_t* enc,
                              void* stream) {
  if (n < 0 || (n > 0 && (!offs || !idx || !enc))) return fail(SPHG_INVALID_ARG, "null buffer or n < 0");
  SPHG_CUDA(sphg::launch_delta(true, offs, idx, n, enc, (cudaStream_t)stream));
  return SPHG_OK;
}

sphg_status sphg_delta_decode(const int64_t* offs, const int32_t* enc, int64_t n, int32_t* idx,
                              void* stream) {
  if (n < 0 || (n > 0 && (!offs || !idx || !enc))) return fail(SPHG_INVALID_ARG, "null buffer or n < 0");
  SPHG_CUDA(sphg::launch_delta(false, offs, enc, n, idx, (cudaStream_t)stream));
  return SPHG_OK;
}

namespace {
struct SnapHeader {
  uint64_t magic;       // "SPHGSNAP"
  uint32_t version, precision;
  int64_t n;
  int32_t ninst, track_ids;
};
constexpr uint64_t kSnapMagic = 0x50414e5347485053ull;
}  // namespace

sphg_status sphg_snapshot(sphg_sim* s, void* buf, uint64_t* bytes, void* stream) {
  if (!s || !bytes) return fail(SPHG_INVALID_ARG, "null argument");
  if (!s->preloop_done) return fail(SPHG_INVALID_ARG, "no computed state to snapshot");
  const int64_t n = s->n;
  const uint64_t need = sizeof(SnapHeader) + (uint64_t)n * (sizeof(float2) * 2 + sizeof(uint32_t) + sizeof(int32_t));
  if (!buf) {
    *bytes = need;
    return SPHG_OK;
  }
  if (*bytes < need) return fail(SPHG_INVALID_ARG, "snapshot buffer too small");
  cudaStream_t st = (cudaStream_t)stream;
  SnapHeader h{kSnapMagic, 1u, (uint32_t)s->opt.precision, n, s->ninst, s->opt.track_ids};
  char* p = static_cast<char*>(buf);
  std::memcpy(p, &h, sizeof(h));
  p += sizeof(h);
  float2* pos = reinterpret_cast<float2*>(p);
  float2* vel = pos + n;
  uint32_t* key = reinterpret_cast<uint32_t*>(vel + n);
  int32_t* ids = reinterpret_cast<int32_t*>(key + n);
  if (n > 0) {
    std::vector<float4> velp(n);
    SPHG_CUDA(cudaMemcpyAsync(pos, s->posA, n * sizeof(float2), cudaMemcpyDeviceToHost, st));
    SPHG_CUDA(cudaMemcpyAsync(velp.data(), s->velpA, n * sizeof(float4), cudaMemcpyDeviceToHost, st));
    SPHG_CUDA(cudaMemcpyAsync(key, s->keyA, n * sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    if (s->opt.track_ids)
      SPHG_CUDA(cudaMemcpyAsync(ids, s->idsA, n * sizeof(int32_t), cudaMemcpyDeviceToHost, st));
    SPHG_CUDA(cudaStreamSynchronize(st));
    for (int64_t i = 0; i < n; ++i) vel[i] = make_float2(velp[i].x, velp[i].y);
    if (!s->opt.track_ids)
      for (int64_t i = 0; i < n; ++i) ids[i] = -1;
  }
  *bytes = need;
  return SPHG_OK;
}

sphg_status sphg_restore(sphg_sim* s, const void* buf, uint64_t bytes, void* stream) {
  if (!s || !buf || bytes < sizeof(SnapHeader)) return fail(SPHG_INVALID_ARG, "null or short snapshot");
  SnapHeader h;
  std::memcpy(&h, buf, sizeof(h));
  if (h.magic != kSnapMagic || h.version != 1u) return fail(SPHG_INVALID_ARG, "not an sphg snapshot");
  if (h.n != s->n || h.ninst != s->ninst || (int)h.precision != s->opt.precision)
    return fail(SPHG_INVALID_ARG, "snapshot of a different handle shape or precision");
  const int64_t n = s->n;
  if (bytes < sizeof(SnapHeader) + (uint64_t)n * (sizeof(float2) * 2 + sizeof(uint32_t) + sizeof(int32_t)))
    return fail(SPHG_INVALID_ARG, "truncated snapshot");
  cudaStream_t st = (cudaStream_t)stream;
  const char* p = static_cast<const char*>(buf) + sizeof(SnapHeader);
  const float2* pos = reinterpret_cast<const float2*>(p);
  const float2* vel = pos + n;
  const uint32_t* key = reinterpret_cast<const uint32_t*>(vel + n);
  const int32_t* ids = reinterpret_cast<const int32_t*>(key + n);
  if (n > 0) {
    // the saved (sorted) state becomes the uploaded state; split offsets stay
    // relative to the saved cells (keyA), exactly as after an upload
    SPHG_CUDA(cudaMemcpyAsync(s->posB, pos, n * sizeof(float2), cudaMemcpyHostToDevice, st));
    SPHG_CUDA(cudaMemcpyAsync(s->velB, vel, n * sizeof(float2), cudaMemcpyHostToDevice, st));
    SPHG_CUDA(cudaMemcpyAsync(s->keyA, key, n * sizeof(uint32_t), cudaMemcpyHostToDevice, st));
    if (s->opt.track_ids) SPHG_CUDA(cudaMemcpyAsync(s->idsB, ids, n * sizeof(int32_t), cudaMemcpyHostToDevice, st));
    SPHG_CUDA(cudaMemsetAsync(s->scratch, 0, sizeof(uint32_t) * 4 * 256, st));
    SPHG_CUDA(cudaStreamSynchronize(st));
  }
  s->uploaded = true;
  s->preloop_done = false;
  return SPHG_OK;
}

sphg_status sphg_profile_step(sphg_sim* s, float* ms, void* stream) {
  if (!s || !ms || !s->preloop_done) return fail(SPHG_INVALID_ARG, "no computed state or null output");
  cudaStream_t st = (cudaStream_t)stream;
  cudaEvent_t ev[6];
  for (int i = 0; i < 6; ++i) SPHG_CUDA(cudaEventCreate(&ev[i]));
  sphg_status res = enqueue_step(s, st, false, ev);
  if (res == SPHG_OK) {
    cudaError_t e = cudaEventSynchronize(ev[5]);
    for (int i = 0; i < 5 && e == cudaSuccess; ++i) e = cudaEventElapsedTime(&ms[i], ev[i], ev[i + 1]);
    if (e != cudaSuccess) res = fail(SPHG_CUDA_ERROR, std::string("profile events: ") + cudaGetErrorString(e));
  }
  for (int i = 0; i < 6; ++i) cudaEventDestroy(ev[i]);
  return res;
}

int32_t sphg_launches_per_step(const sphg_sim* s) {
  if (!s || s->n == 0) return 0;
  const int passes = (s->key_bits + 7) / 8;
  // an iteration that runs the full sort: its histogram kernel + radix passes +
  // reorder + density + force (+ the incremental re-sort's merge kernel; + list
  // count, three scan kernels and list fill in the lists mode).  An iteration
  // that merges launches (key_bits + 7) / 8 + 1 kernels fewer in a graph.
  // With the single-launch iteration: the launch (which only decides), the
  // histogram + radix passes and the launch's post part; an iteration that
  // merges is the one launch.
  if (fused_on(const_cast<sphg_sim*>(s))) return passes + 3;
  return passes + 4 + (s->movers_on ? 1 : 0) + (s->opt.compute == SPHG_COMPUTE_LISTS ? 5 : 0);
}

sphg_status sphg_sort_pairs(const uint32_t* keys_in, const uint32_t* vals_in, uint32_t* keys_out,
                            uint32_t* vals_out, int64_t n, int32_t bits, void* stream) {
  if (n < 0 || bits < 1 || bits > 32) return fail(SPHG_INVALID_ARG, "n < 0 or bits outside 1..32");
  if (n == 0) return SPHG_OK;
  if (!keys_in || !keys_out || !vals_out) return fail(SPHG_INVALID_ARG, "null buffer");
  if (n > sphg::kSortMaxKeys) return fail(SPHG_CAPACITY, "n above 2^30-1 (the sort's look-back counts)");
  cudaStream_t st = (cudaStream_t)stream;
  const size_t words = sphg::sort_scratch_words(n) + ((bits > 8) ? 2 * (size_t)n : 0);
  uint32_t* scratch = nullptr;
  SPHG_CUDA(cudaMallocAsync((void**)&scratch, words * sizeof(uint32_t), st));
  uint32_t* ktmp = scratch + sphg::sort_scratch_words(n);
  uint32_t* vtmp = ktmp + n;
  cudaError_t e = sphg::radix_sort_pairs(keys_in, vals_in, keys_out, vals_out,
                                         bits > 8 ? ktmp : nullptr, bits > 8 ? vtmp : nullptr,
                                         scratch, n, bits, st, nullptr, nullptr, nullptr, true);
  cudaError_t e2 = cudaFreeAsync(scratch, st);
  SPHG_CUDA(e);
  SPHG_CUDA(e2);
  return SPHG_OK;
}

sphg_status sphg_cell_keys(const sphg_params* p, const float* x, const float* y, int64_t n,
                           int32_t* keys, void* stream) {
  if (!p || n < 0) return fail(SPHG_INVALID_ARG, "null params or n < 0");
  if (n == 0) return SPHG_OK;
  if (!x || !y || !keys) return fail(SPHG_INVALID_ARG, "null buffer");
  InstDesc d;
  uint64_t span = 0;
  SPHG_TRY(make_desc(*p, 0, n, 0, d, span));
  SPHG_CUDA(sphg::launch_cell_keys_plain(d, x, y, n, keys, (cudaStream_t)stream));
  return SPHG_OK;
}

}  // extern "C"
