"""Benchmark of the GB300 SPH step (libsphg.so): batched vs plain GPU path,
the 1M-particle dam break against the HBM roofline, and serving latency.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--workload NAME] [--impl reference]

The default line is the metric's own configuration, batch_256: 256 independent
dam-break boxes (particle counts log-uniform in [2,000, 65,536] from the seed,
column aspect in [0.3, 2.0], artificial viscosity alpha in [0.05, 0.2]; about
4.4M particles), split-precision positions (integer cell + FP32 offset) with
compensated sums, stepped together in one handle from one CUDA graph per
iteration with the launch configuration the autotuner picks.
  value            batched particle-steps/s, device time (CUDA events on the
                   launching stream around each of K iterations, L2 flushed by a
                   256 MiB write between them, outside the events)
  plain_gpu_path   the same 256 instances each in its own handle, stepped one
                   after another (the plain drop-in path), and batched_vs_plain
  e2e              the batch through the C ABI from host FP64 arrays: upload,
                   pre-loop, K iterations each followed by its step headers
                   written into pinned host memory, final download
  config_run       all the configuration's iterations (1,000) timed as one
                   run, with the share that re-sorted by merging
  dam_break_12k,   nested records of the 12,800-particle dam break (plain FP32)
  tgv_262k         and of the periodic 512 x 512 Taylor-Green vortex
  dam_break_1m     nested record of the 1,000,000-particle dam break (1000 x
                   1000 particles, dx = 0.0005, split precision): device time,
                   roofline, re-sort mix of the timed steps and of its whole
                   2,000-step configuration
  serve            nested record of the serving workload: Poisson arrivals at
                   200 requests/s for 60 s of dam-break / Taylor-Green lattices
                   (50/50, 1,000-200,000 particles, 500 steps each) admitted by
                   a 120 GB HBM budget into one continuously batched server
                   running on its own thread and stream; p50/p99 completion
                   latency and aggregate particle-steps/s
One "step" is one main-loop iteration of the reference
(integrate -> cell keys -> sort -> cell ranges -> density -> pressure -> forces).
The dam breaks set the laminar MU = 0 and use the artificial viscosity their
configurations name (MU = 0.01 exceeds the explicit diffusion limit of
dt = 1e-5 at dx = 0.0005: the FP64 oracle diverges the same way).

--impl reference times the reference algorithm on the host cores: the CPU
restatement of the reference's OpenMP path (oracle/liboracle.so, FP64, all
threads), on a bounded sample of the same workload.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "sph-simulations_gb300")
sys.path.insert(0, PKG)

METRIC = ("particle-steps/s on 1 GB300, batched vs plain GPU path at ≤1e-5 rel err; "
          "p99 latency")
UNIT = "particle-steps/s"
BYTES_PER_PARTICLE_STEP = 80.0  # algorithmic: sweep A 44 B (state in/out, key, perm, rho) + sweep B 36 B
# DRAM bytes per particle-step measured by ncu (dram__bytes_read.sum + dram__bytes_write.sum
# summed over one merge-path iteration's kernels -- re-sort merge, reorder, density, force --
# caches flushed before each captured launch; profiles/traffic_dam_break_1m.md,
# profiles/launches_batch_256.md)
TRAFFIC_PER_PARTICLE_STEP = {"dam_break_1m": 104.3, "batch_256": 186.3}
L2_FLUSH_BYTES = 256 << 20
E2E_TRIALS = 3
DATA = "synthetic: seeded jittered-lattice initial states (no dataset)"


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


# ---------------------------------------------------------------- workloads
import workloads as W  # noqa: E402  (sph-simulations_gb300/workloads.py)

WORKLOADS = {
    # 256 independent dam-break boxes, 2,000-65,536 particles each (the metric's configuration)
    "batch_256": dict(kind="batch", count=256, steps_config=1000, precision="split"),
    # 1,000,000-particle dam break, split-precision positions
    "dam_break_1m": dict(kind="dam", nx=1000, ny=1000, dx=0.0005, steps_config=2000, precision="split"),
    # 12,800-particle dam break, plain FP32 positions
    "dam_break_12k": dict(kind="dam", nx=80, ny=160, dx=0.005, steps_config=1000, precision="plain"),
    # periodic Taylor-Green vortex, 512 x 512
    "tgv_262k": dict(kind="tgv", n=512, steps_config=5000, precision="plain"),
}


def make_workload(name):
    w = WORKLOADS[name]
    if w["kind"] == "dam":
        prm, x, y, vx, vy = W.dam_break(w["nx"], w["ny"], w["dx"], seed=0)
        return w, prm, x, y, vx, vy
    if w["kind"] == "tgv":
        prm, x, y, vx, vy, _ = W.taylor_green(w["n"], seed=0)
        return w, prm, x, y, vx, vy
    prms, counts, x, y, vx, vy = W.batch(w["count"], seed=0)
    w = dict(w, counts=counts)
    return w, prms, x, y, vx, vy


def workload_config(name, w, prm, n):
    """The `config` object of a workload (the same in both arms)."""
    cfg = {"workload": name, "particles": int(n), "precision": w["precision"],
           "steps_in_config": w["steps_config"], "replicas": "one per GPU",
           "l2": "flushed between timed steps (256 MiB write, outside the events)"}
    if w["kind"] == "batch":
        cfg.update(instances=len(prm), order="morton",
                   particles_per_instance="log-uniform [2000, 65536]",
                   physics="k=30 rho0=1000 alpha U[0.05,0.2] g=-9.81 mu=0 dt=1e-05")
    else:
        cfg.update(h=prm["h"], order=prm["order"],
                   physics="k=%g rho0=%g alpha=%g g=%g mu=%.4g dt=%g%s" % (
                       prm["k"], prm["rho0"], prm["alpha"], prm["gy"], prm["mu"], prm["dt"],
                       " periodic" if prm["periodic"] else ""))
    return cfg


# ---------------------------------------------------------------- clocks
class ClockSampler:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu=0):
        self.gpu = gpu
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.QUERY,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [v.strip() for v in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = max(smax, float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


# ---------------------------------------------------------------- CPU baseline (oracle port)
def cpu_baseline(prm, x, y, vx, vy, budget_s=15.0, max_steps=None, counts=None):
    """The CPU restatement of the reference's OpenMP path (FP64, all host threads)
    timed on a bounded sample of the workload: whole instances, main-loop
    iterations until the time budget is spent."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    O.build()
    O.set_threads(os.cpu_count() or 1)
    if counts is None:
        prms, counts = [prm], [len(x)]
    else:
        prms = prm
    off = np.concatenate([[0], np.cumsum(counts)])
    done_ps, el, steps_total, insts = 0, 0.0, 0, 0
    for k, p_k in enumerate(prms):
        sl = slice(off[k], off[k + 1])
        sim = O.Sim(O.params(**p_k), x[sl], y[sl], vx[sl], vy[sl])
        sim.preloop()
        insts += 1
        while True:
            t0 = time.perf_counter()
            sim.steps(1)
            el += time.perf_counter() - t0
            done_ps += int(counts[k])
            steps_total += 1
            if el >= budget_s or (max_steps and steps_total >= max_steps * (k + 1)):
                break
        if el >= budget_s:
            break
    rate = done_ps / el
    return {"value": rate, "unit": UNIT, "cores": O.get_threads(), "kind": "port",
            "sample": "%d particle-steps over %d instance(s) (%d main-loop iterations after the "
                      "pre-loop), FP64 CPU restatement of the reference's OpenMP path, %.1f s"
                      % (done_ps, insts, steps_total, el)}


# ---------------------------------------------------------------- GPU helpers
def time_steps(sim, steps, stream, flush, resort_log=None):
    """Per-step CUDA events around each graph launch; L2 flushed between steps
    (outside the events).  resort_log, when a list, receives each step's
    re-sort record (merged 1/0, particles that changed cell)."""
    import torch
    import sphg
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(steps)]
    sptr = stream.cuda_stream
    for k in range(steps):
        if flush is not None:
            flush.fill_(float(k))
        ev[k][0].record(stream)
        sim.step(1, stream=sptr)
        ev[k][1].record(stream)
        if resort_log is not None:
            resort_log.append(sim.debug(sphg.DBG_RESORT, stream=sptr)[:2].tolist())
    torch.cuda.synchronize()
    return float(sum(a.elapsed_time(b) for a, b in ev))


def max_over_ranks(x, device="cuda"):
    """The largest per-rank value over all ranks (the timed region of the slowest
    replica); the value itself when not running distributed."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(x)
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(particles_per_replica, world, steps, max_ms):
    """Whole-job particle-steps/s of `world` independent replicas (weak scaling)."""
    return particles_per_replica * world * steps / (max_ms * 1e-3)


def roofline_of(name, value, n):
    hbm, src = peaks()
    achieved = value * BYTES_PER_PARTICLE_STEP / 1e9
    tr = TRAFFIC_PER_PARTICLE_STEP.get(name)
    return {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
            "traffic": tr * n if tr is not None else None,
            "traffic_unit": "DRAM bytes per main-loop iteration (ncu)",
            "peak_source": src,
            "kernel": "one main-loop iteration (re-sort or radix sort + reorder + density + force)",
            "algorithmic_bytes_per_particle_step": BYTES_PER_PARTICLE_STEP}


def resort_summary(log):
    if not log:
        return None
    a = np.array(log, dtype=np.float64)
    return {"steps": len(log), "merged_fraction": float(a[:, 0].mean()),
            "full_sorts": int(len(log) - a[:, 0].sum()),
            "cell_changes_per_step": float(a[:, 1].mean())}


def device_record(name, args, opts, stream, steps, warmup, with_e2e=True, world=1, tune=False):
    """Device-resident timing of one workload (+ its whole configuration run and
    the end-to-end leg through the C ABI)."""
    import torch
    import sphg
    w, prm, x, y, vx, vy = make_workload(name)
    batched = w["kind"] == "batch"
    n = len(x)
    sptr = stream.cuda_stream
    sprm = [sphg.params(**p) for p in prm] if batched else sphg.params(**prm)
    counts = w["counts"] if batched else n
    tuned = None
    if tune:
        best, ms = sphg.autotune(sprm if batched else [sprm], counts if batched else [n], x, y, vx, vy,
                                 base=opts, steps=5, stream=sptr)
        opts = best
        tuned = {"ms_per_step": ms, "tile_bits": best.tile_bits, "resort": best.resort,
                 "block_threads": best.block_threads, "cell_pairs": best.cell_pairs, "fused": best.fused,
                 "searched": "tile_bits {off,3,4,5} x (untiled) re-sort {merge, full} x block {64,128,256} "
                             "x particles per density thread {2 of a cell, 1}; single cooperative launch per iteration"}
    sim = sphg.Sim(sprm, counts, opts)
    sim.upload(x, y, vx, vy, stream=sptr)
    sim.preloop(stream=sptr)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
    for _ in range(warmup):
        sim.step(1, stream=sptr)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    clocks = ClockSampler(torch.cuda.current_device())
    clocks.start()
    time.sleep(0.3)
    log = []
    total_ms = time_steps(sim, steps, stream, flush, resort_log=log)
    clk = clocks.stop()
    total_ms = max_over_ranks(total_ms)
    value = replica_throughput(n, world, steps, total_ms)
    full_sort_kernels = int(sim.debug(sphg.DBG_RESORT, stream=sptr)[2])
    per_step = sim.launches_per_step()
    rs = resort_summary(log)
    launches = int(round(steps * per_step - (rs["steps"] * rs["merged_fraction"]) * full_sort_kernels))
    # per-phase profile (CUDA events between the kernels of one iteration)
    phases = np.array([sim.profile_step(stream=sptr) for _ in range(10)])
    names = ["keys", "sort", "reorder", "density", "force_integrate"]
    pm = phases.mean(axis=0).tolist()
    tot = sum(pm)
    phases_out = {nm: {"ms": m, "share": m / tot if tot else 0.0} for nm, m in zip(names, pm)}
    sim.close()
    cfg = workload_config(name, w, prm, n)
    if opts.compute == sphg.LISTS:
        cfg["compute"] = "lists"
    rec = {"value": value, "unit": UNIT, "steps": steps, "ms_per_step": total_ms / steps,
           "config": cfg, "roofline": roofline_of(name + ("_lists" if opts.compute == sphg.LISTS else ""), value, n),
           "resort_timed": rs, "gpu_launches": launches, "clocks": clk, "phases_ms": phases_out}
    if tuned:
        rec["autotune"] = tuned
    # the whole configuration as one run (fresh handle: pre-loop + every iteration)
    sim = sphg.Sim(sprm, counts, opts)
    sim.upload(x, y, vx, vy, stream=sptr)
    sim.preloop(stream=sptr)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    cfg_steps = w["steps_config"]
    clog = []
    e0.record(stream)
    chunk = 50
    done = 0
    while done < cfg_steps:
        k = min(chunk, cfg_steps - done)
        sim.step(k, stream=sptr)
        done += k
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    diag = sim.diagnostics(stream=sptr)
    sim.close()
    rec["config_run"] = {"steps": cfg_steps, "ms_per_step": ms / cfg_steps,
                         "value": n * cfg_steps / (ms * 1e-3),
                         "note": "the configuration's whole run on the device (L2 warm), full sorts included",
                         "finite": bool(diag[:, 5].sum() == 0),
                         "inside": float(diag[:, 2].sum())}
    if with_e2e:
        rec["e2e"] = e2e_record(sphg, sprm, counts, n, batched, len(prm) if batched else 1, x, y, vx, vy,
                                opts, steps, sptr)
    return rec, (w, prm, x, y, vx, vy)


def e2e_record(sphg, sprm, counts, n, batched, ninst, x, y, vx, vy, opts, steps, sptr):
    """End to end through the C ABI from host buffers: upload of the initial
    state, pre-loop, every step followed by its step header (E_k, max|v|^2, N
    inside, momentum) written into pinned host memory (sphg_step_headers), final
    download into the caller's arrays.  The median of E2E_TRIALS runs, each on a
    fresh handle."""
    import torch
    headers = torch.empty((steps, 6 * ninst), dtype=torch.float64, pin_memory=True)
    result = {k: np.empty(n, np.float64) for k in ("x", "y", "vx", "vy", "rho")}
    result["ids"] = np.empty(n, np.int32)
    for arr in result.values():
        arr.fill(0)  # fault the pages in (np.zeros maps them lazily)
    host_mode = 2 if sphg.device_attributes()["pageable_access"] else 0
    walls = []
    for _ in range(E2E_TRIALS):
        sim = sphg.Sim(sprm, counts, opts)
        sim.set_host_access(host_mode)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        sim.upload(x, y, vx, vy, stream=sptr)
        sim.preloop(stream=sptr)
        sim.step_headers(steps, headers.data_ptr(), stream=sptr)
        out = sim.download(forces=False, stream=sptr, out=result)  # synchronises; checks the device error words
        walls.append(time.perf_counter() - t0)
        sim.close()
        hdr = headers.numpy()
        assert np.isfinite(hdr).all() and (hdr[:, 2::6].sum(axis=1) == n).all()
        assert np.isfinite(out["x"]).all()
    e2e_s = float(np.median(walls))
    state_h2d = 4 * 8   # the caller's FP64 x, y, vx, vy in
    state_d2h = 5 * 8 + 4  # FP64 x, y, vx, vy, rho and int32 ids out
    return {"value": n * steps / e2e_s, "unit": UNIT,
            "h2d_bytes_per_step": int(n * state_h2d / steps),
            "d2h_bytes_per_step": int(6 * 8 * ninst + n * state_d2h / steps),
            "wall_s": e2e_s, "trials_wall_s": walls,
            "host_access": {0: "pinned staging", 2: "device reads and writes the caller's arrays"}[host_mode]}


def plain_path(prm, counts, x, y, vx, vy, opts, stream, steps):
    """The plain GPU path: every instance in its own handle, stepped one after another."""
    import torch
    import sphg
    sptr = stream.cuda_stream
    off = np.concatenate([[0], np.cumsum(counts)])
    sims = []
    for k, p_k in enumerate(prm):
        sl = slice(off[k], off[k + 1])
        s_k = sphg.Sim(sphg.params(**p_k), int(counts[k]), opts)
        s_k.upload(x[sl], y[sl], vx[sl], vy[sl], stream=sptr)
        s_k.preloop(stream=sptr)
        sims.append(s_k)
    for s_k in sims:
        s_k.step(3, stream=sptr)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        for s_k in sims:
            s_k.step(1, stream=sptr)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    for s_k in sims:
        s_k.close()
    n = int(off[-1])
    return {"value": n * steps / (ms * 1e-3), "unit": UNIT, "steps": steps, "ms_per_step": ms / steps,
            "how": "one handle per instance (the plain drop-in path, CUDA graph per iteration), "
                   "stepped in turn on one stream; same options as the batched run"}


def serve_record(seconds, rate, steps, budget_gb, fused=0):
    """Serving: Poisson arrivals of dam-break / Taylor-Green lattice requests
    submitted at their arrival times to a server whose loop runs on its own
    thread and stream; latency = result in host memory - submission."""
    import torch
    import sphg
    reqs = W.lattice_requests(rate=rate, seconds=seconds, seed=0, steps=steps)
    srv = sphg.Server(budget_gb * 1e9, max_instances=8192,
                      opts=sphg.options(precision=sphg.SPLIT, track_ids=0, use_graph=1, fused=fused))
    srv.start(torch.cuda.current_device())
    clocks = ClockSampler(torch.cuda.current_device())
    clocks.start()
    live = {}
    lat = []
    done_ps = 0.0
    t0 = time.perf_counter()
    k = 0
    while k < len(reqs) or live:
        now = time.perf_counter() - t0
        while k < len(reqs) and reqs[k][0] <= now:
            arr, kind, prm, spec, st, npart = reqs[k]
            rid = srv.submit_lattice(sphg.params(**prm), sphg.lattice(**spec), st)
            live[rid] = npart * st
            k += 1
        for rid in list(live):
            r = srv.result(rid)
            if r is not None:
                lat.append(r["latency_s"])
                done_ps += live.pop(rid)
        nxt = reqs[k][0] - (time.perf_counter() - t0) if k < len(reqs) else 0.0005
        time.sleep(min(max(nxt, 0.0), 0.0005))
    wall = time.perf_counter() - t0
    st = srv.stats()
    srv.stop()
    srv.close()
    clk = clocks.stop()
    lat = np.array(lat)
    return {"value": done_ps / wall, "unit": UNIT,
            "latency_s": {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99)),
                          "max": float(lat.max()), "mean": float(lat.mean())},
            "requests": len(reqs), "completed": int(st["completed"]),
            "offered_particle_steps_per_s": sum(r[5] * r[4] for r in reqs) / seconds,
            "wall_s": wall, "ticks": int(st["ticks"]), "device_particle_steps": st["particle_steps"],
            "appends": int(st["appends"]), "compactions": int(st["compactions"]),
            "graph_builds": int(st["graph_builds"]),
            "config": {"workload": "serve", "rate_per_s": rate, "seconds": seconds, "steps_per_request": steps,
                       "single_launch_iterations": bool(fused),
                       "hbm_budget_gb": budget_gb, "particles_range": [1000, 200000], "precision": "split",
                       "mix": "dam-break / Taylor-Green 50/50, states generated on the device at admission",
                       "capacity_particles": st["cap_particles"], "capacity_cell_keys": st["cap_keys"]},
            "clocks": clk}


# ---------------------------------------------------------------- arms
def run_gpu(args):
    import torch
    import sphg

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    stream = torch.cuda.current_stream()
    name = args.workload
    prec = sphg.SPLIT if WORKLOADS[name]["precision"] == "split" else sphg.PLAIN
    opts = sphg.options(precision=prec, track_ids=0, use_graph=args.graph, compute=args.compute, fused=args.fused)
    is_batch = WORKLOADS[name]["kind"] == "batch"
    rec, (w, prm, x, y, vx, vy) = device_record(name, args, opts, stream, args.steps, args.warmup,
                                                world=world, tune=is_batch and args.graph == 1)
    extra = {}
    if is_batch:
        tuned_opts = opts
        if "autotune" in rec:
            t = rec["autotune"]
            tuned_opts = sphg.options(precision=prec, track_ids=0, use_graph=1, tile_bits=t["tile_bits"],
                                      resort=t["resort"], block_threads=t["block_threads"],
                                      cell_pairs=t["cell_pairs"], fused=t["fused"])
        plain = plain_path(prm, w["counts"], x, y, vx, vy, tuned_opts, stream, max(3, min(args.steps, 20)))
        extra = {"plain_gpu_path": plain, "batched_vs_plain": rec["value"] / plain["value"]}
    nested = {}
    if not args.no_nested and rank == 0:
        if name != "dam_break_1m":
            r1m, _ = device_record("dam_break_1m", args, sphg.options(precision=sphg.SPLIT, track_ids=0, use_graph=1),
                                   stream, args.steps, args.warmup, with_e2e=False)
            nested["dam_break_1m"] = r1m
        # the 12,800-particle dam break (plain FP32) and the periodic 512 x 512 Taylor-Green vortex
        for extra_name in ("dam_break_12k", "tgv_262k"):
            if extra_name != name:
                rx, _ = device_record(extra_name, args, sphg.options(precision=sphg.PLAIN, track_ids=0, use_graph=1),
                                      stream, args.steps, args.warmup, with_e2e=False)
                nested[extra_name] = rx
        # the lists compute mode (CSR neighbour lists assembled every iteration) on the same dam break
        rl, _ = device_record("dam_break_1m", args,
                              sphg.options(precision=sphg.SPLIT, track_ids=0, use_graph=1, compute="lists"),
                              stream, args.steps, args.warmup, with_e2e=False)
        nested["dam_break_1m_lists"] = rl
        if args.serve_seconds > 0:
            nested["serve"] = serve_record(args.serve_seconds, args.rate, args.serve_steps, args.budget_gb,
                                           args.serve_fused)
    if world > 1:
        torch.distributed.barrier()
    if rank == 0:
        cpu = None
        if args.cpu_budget > 0:
            cpu = cpu_baseline(prm, x, y, vx, vy, budget_s=args.cpu_budget,
                               counts=w["counts"] if w["kind"] == "batch" else None)
        line = {
            "metric": METRIC, "value": rec["value"], "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": rec["ms_per_step"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": DATA,
            "config": rec["config"], "roofline": rec["roofline"], "cpu_baseline": cpu, "e2e": rec["e2e"],
            "gpu_launches": rec["gpu_launches"], "clocks": rec["clocks"],
        }
        line.update(extra)
        for k in ("autotune", "resort_timed", "config_run", "phases_ms"):
            if k in rec:
                line[k] = rec[k]
        line.update(nested)
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    name = args.workload
    w, prm, x, y, vx, vy = make_workload(name)
    batched = w["kind"] == "batch"
    n = len(x)
    cpu = cpu_baseline(prm, x, y, vx, vy, budget_s=args.cpu_budget if args.cpu_budget > 0 else 15.0,
                       max_steps=max(args.steps, 1), counts=w["counts"] if batched else None)
    line = {"impl": "reference", "metric": METRIC, "value": cpu["value"], "unit": UNIT,
            "n_gpus": int(os.environ.get("WORLD_SIZE", "1")), "steps": args.steps,
            "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": DATA,
            "config": workload_config(name, w, prm, n),
            "cpu_baseline": cpu,
            "e2e": {"value": cpu["value"], "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--workload", default="batch_256", choices=sorted(WORKLOADS) + ["serve"])
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--cpu-budget", type=float, default=15.0,
                    help="seconds of CPU baseline sampling (0 = skip)")
    ap.add_argument("--compute", default="sorted", choices=["sorted", "lists"],
                    help="compute mode of the named workload (lists: CSR neighbour lists every iteration)")
    ap.add_argument("--fused", type=int, default=0,
                    help="1: the named workload's iterations as single cooperative launches")
    ap.add_argument("--graph", type=int, default=1,
                    help="1: every iteration replays a CUDA graph; 0: stream-launched kernels (for profilers)")
    ap.add_argument("--no-nested", action="store_true",
                    help="only the named workload (no nested dam_break_1m / serve records)")
    ap.add_argument("--rate", type=float, default=200.0, help="serve: arrivals per second")
    ap.add_argument("--serve-seconds", type=float, default=60.0, help="serve: arrival window (0 = skip)")
    ap.add_argument("--serve-steps", type=int, default=500, help="serve: steps per request")
    ap.add_argument("--budget-gb", type=float, default=120.0, help="serve: HBM budget")
    ap.add_argument("--serve-fused", type=int, default=0, help="serve: iterations as single cooperative launches")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        if args.workload == "serve":
            print(json.dumps({"impl": "reference", "unavailable": "the reference runs one simulation per process; serving has no reference counterpart"}))
            return
        run_reference(args)
    elif args.workload == "serve":
        import torch
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        rec = serve_record(args.serve_seconds, args.rate, args.serve_steps, args.budget_gb, args.serve_fused)
        line = {"metric": METRIC, "value": rec["value"], "unit": UNIT, "n_gpus": 1, "steps": args.serve_steps,
                "warmup": 0, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
                "data": "synthetic: seeded Poisson request stream of jittered lattices generated on the device"}
        line.update(rec)
        print(json.dumps(line))
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
