"""Benchmark of the GB300 SPH step (libsphg.so) on the 2-D dam-break workloads.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--workload NAME] [--impl reference]

Default workload: dam_break_1m -- 1000 x 1000 particles (dx = 0.0005, a 0.5 x 0.5
column at the left wall of the unit box, +-0.01 dx seeded jitter), h = 1.3 dx,
weakly compressible EOS with the reference's stiffness (k = 30), rest density
1000, artificial viscosity alpha = 0.1, gravity -9.81, dt = 1e-5, split-precision
positions (integer cell + FP32 offset) with compensated sums.  The dam-break
configurations name artificial viscosity as their only viscosity, so the
reference's laminar term is off (MU = 0): with MU = 0.01 its explicit diffusion
rate at dx = 0.0005 (MU m/rho 45/(pi h^6) (h - r), about 4e4 1/s per
neighbour) is at the 2/dt stability limit of dt = 1e-5 and the run diverges
(the FP64 oracle diverges the same way).

One "step" is one main-loop iteration of the reference
(integrate -> cell keys -> sort -> cell ranges -> density -> pressure -> forces).
`value` is device time with the state resident in HBM (CUDA events on the
launching stream, L2 flushed by a 256 MiB write between timed steps); `e2e` is
the same run driven through the C ABI from host buffers (upload, pre-loop, K
iterations each followed by its step-header diagnostics copied into pinned host
memory, final download), timed on the host around the whole sequence.

--impl reference times the reference algorithm on the host cores: the CPU
restatement of the reference's OpenMP path (oracle/liboracle.so, FP64, all
threads), on a bounded sample of the same workload.
"""
import argparse
import json
import math
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
# summed over one merge-path iteration's kernels, caches flushed before each captured
# launch): 104.9 MB per iteration of 1,000,000 particles
TRAFFIC_PER_PARTICLE_STEP = {"dam_break_1m": 104.9}
L2_FLUSH_BYTES = 256 << 20
E2E_TRIALS = 3


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
    # 1,000,000-particle dam break, split-precision positions (the headline)
    "dam_break_1m": dict(kind="dam", nx=1000, ny=1000, dx=0.0005, steps_config=2000, precision="split"),
    # 12,800-particle dam break, plain FP32 positions
    "dam_break_12k": dict(kind="dam", nx=80, ny=160, dx=0.005, steps_config=1000, precision="plain"),
    # periodic Taylor-Green vortex, 512 x 512
    "tgv_262k": dict(kind="tgv", n=512, steps_config=5000, precision="plain"),
    # 256 independent dam-break boxes, 2,000-65,536 particles each
    "batch_256": dict(kind="batch", count=256, steps_config=1000, precision="split"),
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


# ---------------------------------------------------------------- GPU arm
def time_steps(sim, sphg, steps, stream, flush):
    """Per-step CUDA events around each graph launch; L2 flushed between steps
    (outside the events) when flush is not None."""
    import torch
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(steps)]
    sptr = stream.cuda_stream
    for k in range(steps):
        if flush is not None:
            flush.fill_(float(k))
        ev[k][0].record(stream)
        sim.step(1, stream=sptr)
        ev[k][1].record(stream)
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
    w, prm, x, y, vx, vy = make_workload(args.workload)
    batched = w["kind"] == "batch"
    n = len(x)
    prec = sphg.SPLIT if w["precision"] == "split" else sphg.PLAIN
    opts = sphg.options(precision=prec, track_ids=0, use_graph=1)
    stream = torch.cuda.current_stream()
    sptr = stream.cuda_stream
    sprm = [sphg.params(**p) for p in prm] if batched else sphg.params(**prm)

    # ---- device-resident timing (inputs in HBM; L2 flushed between steps when
    #      the state fits in L2)
    sim = sphg.Sim(sprm, w["counts"] if batched else n, opts)
    sim.upload(x, y, vx, vy, stream=sptr)
    sim.preloop(stream=sptr)
    state_bytes = n * 100
    flush = None
    if state_bytes < L2_FLUSH_BYTES:
        flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
    for _ in range(args.warmup):
        sim.step(1, stream=sptr)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    total_ms = time_steps(sim, sphg, args.steps, stream, flush)
    clk = clocks.stop()
    total_ms = max_over_ranks(total_ms)
    ms_per_step = total_ms / args.steps
    value = replica_throughput(n, world, args.steps, total_ms)

    # ---- per-phase profile (CUDA events between the kernels of one iteration)
    phases, resort = [], []
    for _ in range(20):
        phases.append(sim.profile_step(stream=sptr))
        resort.append(sim.debug(sphg.DBG_RESORT, stream=sptr)[:2].tolist())
    phases = np.array(phases)
    phase_ms = phases.mean(axis=0).tolist()
    resort = np.array(resort)
    resort_out = {"incremental_fraction": float(resort[:, 0].mean()),
                  "cell_changes_per_step": float(resort[:, 1].mean())}
    diag = sim.diagnostics(stream=sptr)
    # kernels per timed iteration: the full sort's histogram + radix passes run only
    # on iterations that did not merge (they sit under a conditional graph node)
    full_sort_kernels = int(sim.debug(sphg.DBG_RESORT, stream=sptr)[2])
    per_step = sim.launches_per_step()
    merged = resort_out["incremental_fraction"]
    launches = int(round(args.steps * (per_step - merged * full_sort_kernels)))
    sim.close()

    extra = {}
    if batched:
        # the plain GPU path: every instance its own handle, stepped one after another
        counts = w["counts"]
        off = np.concatenate([[0], np.cumsum(counts)])
        sims = []
        for k, p_k in enumerate(prm):
            sl = slice(off[k], off[k + 1])
            s_k = sphg.Sim(sphg.params(**p_k), int(counts[k]), opts)
            s_k.upload(x[sl], y[sl], vx[sl], vy[sl], stream=sptr)
            s_k.preloop(stream=sptr)
            sims.append(s_k)
        psteps = max(3, min(args.steps, 20))
        for s_k in sims:
            s_k.step(2, stream=sptr)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(psteps):
            for s_k in sims:
                s_k.step(1, stream=sptr)
        e1.record(stream)
        torch.cuda.synchronize()
        plain = n * psteps / (e0.elapsed_time(e1) * 1e-3)
        for s_k in sims:
            s_k.close()
        extra = {"plain_gpu_path": {"value": plain, "unit": UNIT, "steps": psteps,
                                    "how": "one handle per instance, stepped in turn"},
                 "batched_vs_plain": value / plain}

    # ---- end to end through the C ABI from host buffers: upload of the initial
    #      state, pre-loop, every step followed by its step header (E_k, max|v|^2,
    #      N inside, momentum) written into pinned host memory (sphg_step_headers),
    #      final download.  The result arrays are the caller's, allocated and
    #      touched once before the timed region (like the pinned header buffer);
    #      where the GPU reads and writes pageable host memory the download writes
    #      them directly.
    #      The median of E2E_TRIALS runs, each on a fresh handle.
    ninst = len(prm) if batched else 1
    headers = torch.empty((args.steps, 6 * ninst), dtype=torch.float64, pin_memory=True)
    result = {k: np.empty(n, np.float64) for k in ("x", "y", "vx", "vy", "rho")}
    result["ids"] = np.empty(n, np.int32)
    for arr in result.values():
        arr.fill(0)  # fault the pages in (np.zeros maps them lazily)
    host_mode = 2 if sphg.device_attributes()["pageable_access"] else 0
    walls = []
    for _ in range(E2E_TRIALS):
        sim = sphg.Sim(sprm, w["counts"] if batched else n, opts)
        sim.set_host_access(host_mode)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        sim.upload(x, y, vx, vy, stream=sptr)
        sim.preloop(stream=sptr)
        sim.step_headers(args.steps, headers.data_ptr(), stream=sptr)  # every iteration + its header
        out = sim.download(forces=False, stream=sptr, out=result)  # synchronises; checks the device error words
        walls.append(time.perf_counter() - t0)
        sim.close()
        hdr = headers.numpy()
        assert np.isfinite(hdr).all() and (hdr[:, 2::6].sum(axis=1) == n).all()
        assert np.isfinite(out["x"]).all()
    e2e_s = float(np.median(walls))
    # bytes that cross between host and device per particle: the caller's FP64
    # x, y, vx, vy in; FP64 x, y, vx, vy, rho and int32 ids out (whether staged
    # or read and written by the device in place)
    state_h2d = 4 * 8
    state_d2h = 5 * 8 + 4
    e2e = {"value": n * args.steps / e2e_s, "unit": UNIT,
           "h2d_bytes_per_step": int(n * state_h2d / args.steps),
           "d2h_bytes_per_step": int(6 * 8 * ninst + n * state_d2h / args.steps),
           "wall_s": e2e_s, "trials_wall_s": walls,
           "host_access": {0: "pinned staging", 2: "device reads and writes the caller's arrays"}[host_mode]}

    hbm, src = peaks()
    achieved = value * BYTES_PER_PARTICLE_STEP / 1e9
    roofline = {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                "frac": achieved / hbm,
                "traffic": (TRAFFIC_PER_PARTICLE_STEP[args.workload] * n
                            if args.workload in TRAFFIC_PER_PARTICLE_STEP else None),
                "traffic_unit": "DRAM bytes per main-loop iteration (ncu)",
                "peak_source": src,
                "kernel": "one main-loop iteration (re-sort or radix sort + reorder + density + force)",
                "algorithmic_bytes_per_particle_step": BYTES_PER_PARTICLE_STEP}
    names = ["keys", "sort", "reorder", "density", "force_integrate"]
    tot = sum(phase_ms)
    phases_out = {nm: {"ms": m, "share": m / tot if tot else 0.0} for nm, m in zip(names, phase_ms)}
    dominant = max(phases_out, key=lambda k: phases_out[k]["ms"])

    if rank == 0:
        cpu = None
        if args.cpu_budget > 0:
            cpu = cpu_baseline(prm, x, y, vx, vy, budget_s=args.cpu_budget,
                               counts=w["counts"] if batched else None)
        cfg = {"workload": args.workload, "particles": n, "precision": w["precision"],
               "steps_in_config": w["steps_config"], "replicas": "one per GPU",
               "l2": ("flushed between timed steps (256 MiB write, outside the events)"
                      if flush is not None else "state larger than L2 (no flush)")}
        if batched:
            cfg.update(instances=len(prm), physics="k=30 rho0=1000 alpha U[0.05,0.2] g=-9.81 mu=0 dt=1e-5",
                       order="morton")
        else:
            cfg.update(h=prm["h"], order=prm["order"],
                       physics="k=%g rho0=%g alpha=%g g=%g mu=%.4g dt=%g%s" % (
                           prm["k"], prm["rho0"], prm["alpha"], prm["gy"], prm["mu"], prm["dt"],
                           " periodic" if prm["periodic"] else ""))
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic: seeded jittered-lattice initial states (no dataset)",
            "config": cfg, "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e,
            "gpu_launches": launches, "clocks": clk, "phases_ms": phases_out,
            "dominant_phase": dominant, "resort": resort_out,
            "diagnostics_after": {"E_k": float(diag[:, 0].sum()), "max_v2": float(diag[:, 1].max()),
                                  "inside": float(diag[:, 2].sum()), "nonfinite": float(diag[:, 5].sum())},
        }
        line.update(extra)
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()


def run_serve(args):
    """Serving: Poisson arrivals (200/s by default) of dam-break / Taylor-Green
    requests (50/50), 1e3-2e5 particles, 500 steps each, admitted by a fixed HBM
    budget into one continuously batched server; requests are generated before
    the clock starts and submitted at their arrival times."""
    import torch
    import sphg
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    reqs = W.requests(rate=args.rate, seconds=args.serve_seconds, seed=0, steps=args.serve_steps)
    srv = sphg.Server(args.budget_gb * 1e9, max_instances=8192,
                      opts=sphg.options(precision=sphg.SPLIT, track_ids=0, use_graph=0))
    stream = torch.cuda.current_stream().cuda_stream
    clocks = ClockSampler(int(os.environ.get("LOCAL_RANK", "0")))
    clocks.start()
    pending = list(reqs)
    ids = {}
    lat = []
    total_ps = 0.0
    t0 = time.perf_counter()
    while pending or ids:
        now = time.perf_counter() - t0
        while pending and pending[0][0] <= now:
            arr, kind, prm, x, y, vx, vy, steps = pending.pop(0)
            rid = srv.submit(sphg.params(**prm), x, y, vx, vy, steps)
            ids[rid] = (arr, len(x) * steps)
        live, fin = srv.tick(stream=stream)
        if fin:
            for rid in list(ids):
                r = srv.result(rid)
                if r is not None:
                    lat.append(r["latency_s"])
                    total_ps += ids[rid][1]
                    del ids[rid]
        if live == 0 and srv.stats()["queued"] == 0 and pending:
            wait = pending[0][0] - (time.perf_counter() - t0)
            if wait > 0:
                time.sleep(wait)
    wall = time.perf_counter() - t0
    st = srv.stats()
    srv.close()
    clk = clocks.stop()
    lat = np.array(lat)
    line = {
        "metric": METRIC, "value": total_ps / wall, "unit": UNIT, "n_gpus": 1,
        "steps": args.serve_steps, "warmup": 0, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32",
        "data": "synthetic: seeded Poisson request stream of jittered-lattice states",
        "config": {"workload": "serve", "rate_per_s": args.rate, "seconds": args.serve_seconds,
                   "requests": len(reqs), "hbm_budget_gb": args.budget_gb,
                   "particles_range": [1000, 200000], "precision": "split",
                   "capacity_particles": st["cap_particles"], "capacity_cell_keys": st["cap_keys"]},
        "latency_s": {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99)),
                      "max": float(lat.max()), "mean": float(lat.mean())},
        "offered_particle_steps_per_s": sum(len(r[3]) * r[7] for r in reqs) / args.serve_seconds,
        "wall_s": wall, "ticks": st["ticks"], "device_particle_steps": st["particle_steps"],
        "clocks": clk,
    }
    print(json.dumps(line))


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    w, prm, x, y, vx, vy = make_workload(args.workload)
    batched = w["kind"] == "batch"
    n = len(x)
    cpu = cpu_baseline(prm, x, y, vx, vy, budget_s=args.cpu_budget if args.cpu_budget > 0 else 15.0,
                       max_steps=max(args.steps, 1), counts=w["counts"] if batched else None)
    line = {"impl": "reference", "metric": METRIC, "value": cpu["value"], "unit": UNIT,
            "n_gpus": int(os.environ.get("WORLD_SIZE", "1")), "steps": args.steps,
            "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64",
            "data": "synthetic: seeded jittered-lattice initial states (no dataset)",
            "config": {"workload": args.workload, "particles": n},
            "cpu_baseline": cpu,
            "e2e": {"value": cpu["value"], "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--workload", default="dam_break_1m", choices=sorted(WORKLOADS) + ["serve"])
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--cpu-budget", type=float, default=15.0,
                    help="seconds of CPU baseline sampling (0 = skip)")
    ap.add_argument("--rate", type=float, default=200.0, help="serve: arrivals per second")
    ap.add_argument("--serve-seconds", type=float, default=10.0, help="serve: arrival window")
    ap.add_argument("--serve-steps", type=int, default=500, help="serve: steps per request")
    ap.add_argument("--budget-gb", type=float, default=120.0, help="serve: HBM budget")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        if args.workload == "serve":
            print(json.dumps({"impl": "reference", "unavailable": "the reference runs one simulation per process; serving has no reference counterpart"}))
            return
        run_reference(args)
    elif args.workload == "serve":
        run_serve(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
