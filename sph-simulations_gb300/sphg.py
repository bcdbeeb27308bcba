"""Python binding of libsphg.so (include/sphg.h) over ctypes.

This is the host-side mirror of the reference's GPU driver for the SPH step
(app/cu_simulation_configuration.h): ``Sim.preloop`` is
PreLoopComputationWithCellNeighbors, ``Sim.step`` one iteration of
MaiLoopComputationWithCellNeighbors, ``Sim.download`` cuWriteContainer.
There is no CPU fallback: if libsphg.so cannot be loaded, every call raises.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
# SPHG_LIB: another build of the library (for comparing builds side by side)
LIB_PATH = os.environ.get("SPHG_LIB") or os.path.join(HERE, "libsphg.so")

OK, INVALID_ARG, OOM, NONFINITE, TIMEOUT, CUDA_ERROR, CAPACITY, NOT_READY = range(8)
ORDER = {"morton": 0, "rowmajor": 1}
PLAIN, SPLIT = 0, 1
SORTED, LISTS = 0, 1
DBG_KEYS, DBG_PERM, DBG_UNSORTED_KEYS, DBG_POS_NEXT, DBG_VEL_NEXT, DBG_RESORT = range(6)


class SphgError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("sphg status %d: %s" % (status, msg))
        self.status = status


class Params(ctypes.Structure):
    _fields_ = [
        ("h", ctypes.c_double), ("dt", ctypes.c_double), ("k", ctypes.c_double),
        ("rho0", ctypes.c_double), ("mu", ctypes.c_double), ("tol", ctypes.c_double),
        ("gx", ctypes.c_double), ("gy", ctypes.c_double), ("mass", ctypes.c_double),
        ("alpha", ctypes.c_double), ("c0", ctypes.c_double),
        ("lo", ctypes.c_double * 2), ("hi", ctypes.c_double * 2),
        ("order", ctypes.c_int32), ("periodic", ctypes.c_int32),
    ]


class Lattice(ctypes.Structure):
    _fields_ = [("x0", ctypes.c_double), ("y0", ctypes.c_double), ("dx", ctypes.c_double),
                ("dy", ctypes.c_double), ("nx", ctypes.c_int64), ("ny", ctypes.c_int64),
                ("jitter", ctypes.c_double), ("seed", ctypes.c_uint64), ("velocity", ctypes.c_int32),
                ("pad", ctypes.c_int32), ("u0", ctypes.c_double)]


VEL_ZERO, VEL_TAYLOR_GREEN = 0, 1


def lattice(x0, y0, dx, dy, nx, ny, jitter=0.0, seed=0, velocity=VEL_ZERO, u0=0.0):
    return Lattice(float(x0), float(y0), float(dx), float(dy), int(nx), int(ny), float(jitter),
                   int(seed) & 0xFFFFFFFFFFFFFFFF, int(velocity), 0, float(u0))


class Options(ctypes.Structure):
    _fields_ = [("precision", ctypes.c_int32), ("track_ids", ctypes.c_int32),
                ("use_graph", ctypes.c_int32), ("tile_bits", ctypes.c_int32),
                ("compute", ctypes.c_int32), ("resort", ctypes.c_int32),
                ("block_threads", ctypes.c_int32), ("cell_pairs", ctypes.c_int32),
                ("fused", ctypes.c_int32)]


_lib = None
_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int32)
_lp = ctypes.POINTER(ctypes.c_int64)
_vp = ctypes.c_void_p


def lib():
    """Loads libsphg.so (built by build.py); raises if it is missing."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("libsphg.so not built (run __graft_entry__.build()); "
                               "there is no CPU fallback")
        L = ctypes.CDLL(LIB_PATH)
        PP = ctypes.POINTER(Params)
        OP = ctypes.POINTER(Options)
        SP = ctypes.c_void_p
        L.sphg_default_params.argtypes = [PP]
        L.sphg_default_options.argtypes = [OP]
        L.sphg_last_error_string.restype = ctypes.c_char_p
        L.sphg_version.restype = ctypes.c_char_p
        L.sphg_create.argtypes = [PP, OP, ctypes.c_int64, ctypes.POINTER(SP)]
        L.sphg_create_batch.argtypes = [ctypes.c_int32, PP, _lp, OP, ctypes.POINTER(SP)]
        L.sphg_destroy.argtypes = [SP]
        L.sphg_upload.argtypes = [SP, _dp, _dp, _dp, _dp, _vp]
        L.sphg_preloop.argtypes = [SP, _vp]
        L.sphg_step.argtypes = [SP, ctypes.c_int64, _vp]
        L.sphg_download.argtypes = [SP] + [_dp] * 7 + [_ip, _vp]
        L.sphg_diagnostics.argtypes = [SP, _dp, _vp]
        L.sphg_get_debug.argtypes = [SP, ctypes.c_int32, _vp, _vp]
        L.sphg_neighbor_lists.argtypes = [SP, _lp, _ip, _lp, _vp]
        L.sphg_profile_step.argtypes = [SP, ctypes.POINTER(ctypes.c_float), _vp]
        L.sphg_profile_step.restype = ctypes.c_int
        L.sphg_launches_per_step.argtypes = [SP]
        L.sphg_launches_per_step.restype = ctypes.c_int32
        L.sphg_snapshot.argtypes = [SP, _vp, ctypes.POINTER(ctypes.c_uint64), _vp]
        L.sphg_restore.argtypes = [SP, _vp, ctypes.c_uint64, _vp]
        L.sphg_snapshot.restype = ctypes.c_int
        L.sphg_restore.restype = ctypes.c_int
        L.sphg_server_create.argtypes = [ctypes.c_double, ctypes.c_int32, OP, ctypes.POINTER(SP)]
        L.sphg_server_destroy.argtypes = [SP]
        L.sphg_server_submit.argtypes = [SP, PP, ctypes.c_int64, _dp, _dp, _dp, _dp, ctypes.c_int64, _lp]
        L.sphg_server_tick.argtypes = [SP, _vp, _ip, _ip]
        L.sphg_server_result.argtypes = [SP, ctypes.c_int64] + [_dp] * 5 + [_ip, _dp]
        L.sphg_server_stats.argtypes = [SP, _dp]
        L.sphg_server_start.argtypes = [SP, ctypes.c_int32]
        L.sphg_server_stop.argtypes = [SP]
        L.sphg_server_counters.argtypes = [SP, _dp, ctypes.c_int32]
        for f in ("sphg_server_create", "sphg_server_destroy", "sphg_server_submit",
                  "sphg_server_tick", "sphg_server_result", "sphg_server_stats", "sphg_server_start",
                  "sphg_server_stop", "sphg_server_counters"):
            getattr(L, f).restype = ctypes.c_int
        L.sphg_sort_pairs.argtypes = [_vp, _vp, _vp, _vp, ctypes.c_int64, ctypes.c_int32, _vp]
        L.sphg_cell_keys.argtypes = [PP, _vp, _vp, ctypes.c_int64, _vp, _vp]
        L.sphg_neighbor_lists_encoded.argtypes = [SP, _lp, _ip, _lp, _vp]
        L.sphg_delta_encode.argtypes = [_vp, _vp, ctypes.c_int64, _vp, _vp]
        L.sphg_delta_decode.argtypes = [_vp, _vp, ctypes.c_int64, _vp, _vp]
        L.sphg_autotune.argtypes = [ctypes.c_int32, PP, _lp, _dp, _dp, _dp, _dp, OP, ctypes.c_int32, OP,
                                    _dp, _vp]
        L.sphg_server_submit_lattice.argtypes = [SP, PP, ctypes.POINTER(Lattice), ctypes.c_int64, _lp]
        L.sphg_server_submit_lattice.restype = ctypes.c_int
        L.sphg_diagnostics_async.argtypes = [SP, _vp, _vp]
        L.sphg_diagnostics_async.restype = ctypes.c_int
        L.sphg_step_headers.argtypes = [SP, ctypes.c_int64, _vp, _vp]
        L.sphg_step_headers.restype = ctypes.c_int
        L.sphg_stream_synchronize.argtypes = [_vp]
        L.sphg_stream_synchronize.restype = ctypes.c_int
        L.sphg_set_host_access.argtypes = [SP, ctypes.c_int32]
        L.sphg_set_host_access.restype = ctypes.c_int
        L.sphg_device_attributes.argtypes = [ctypes.c_int32, _ip]
        L.sphg_device_attributes.restype = ctypes.c_int
        L.sphg_upload_lattice.argtypes = [SP, ctypes.POINTER(Lattice), _vp]
        L.sphg_upload_lattice.restype = ctypes.c_int
        L.sphg_cfl_dt.argtypes = [SP, ctypes.c_double, ctypes.c_double, _dp, _vp]
        L.sphg_set_dt.argtypes = [SP, ctypes.c_int32, ctypes.c_double]
        for f in ("sphg_neighbor_lists_encoded", "sphg_delta_encode", "sphg_delta_decode", "sphg_autotune",
                  "sphg_cfl_dt", "sphg_set_dt"):
            getattr(L, f).restype = ctypes.c_int
        for f in ("sphg_create", "sphg_create_batch", "sphg_destroy", "sphg_upload",
                  "sphg_preloop", "sphg_step", "sphg_download", "sphg_diagnostics",
                  "sphg_get_debug", "sphg_neighbor_lists", "sphg_sort_pairs", "sphg_cell_keys"):
            getattr(L, f).restype = ctypes.c_int
        _lib = L
    return _lib


def check(status):
    if status != OK:
        raise SphgError(status, lib().sphg_last_error_string().decode())


def params(**kw):
    """The reference's defaults (core/ConfigVariables.hpp, config/example.txt), overridable."""
    p = Params()
    lib().sphg_default_params(ctypes.byref(p))
    for k, v in kw.items():
        if k in ("lo", "hi"):
            getattr(p, k)[0], getattr(p, k)[1] = v
        elif k == "order" and isinstance(v, str):
            p.order = ORDER[v]
        else:
            setattr(p, k, v)
    return p


def options(precision=PLAIN, track_ids=1, use_graph=1, tile_bits=0, compute=None, resort=None,
            block_threads=None, cell_pairs=None, fused=None):
    o = Options()
    lib().sphg_default_options(ctypes.byref(o))
    if resort is not None:
        o.resort = int(resort)
    if block_threads is not None:
        o.block_threads = int(block_threads)
    if cell_pairs is not None:
        o.cell_pairs = int(cell_pairs)
    if fused is not None:
        o.fused = int(fused)
    o.precision = precision
    o.track_ids = track_ids
    o.use_graph = use_graph
    o.tile_bits = tile_bits
    if compute is not None:
        o.compute = {"sorted": SORTED, "lists": LISTS, "mp-lists": LISTS}.get(compute, compute)
    return o


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _ptr(a, t=_dp):
    return a.ctypes.data_as(t)


def _stream(stream):
    if stream is None:
        return None
    if isinstance(stream, int):
        return stream
    return getattr(stream, "cuda_stream", stream)


class Sim:
    """One handle: a single instance (params) or a batch (list of params)."""

    def __init__(self, prm, n, opts=None):
        L = lib()
        self._h = ctypes.c_void_p()
        if opts is None:
            opts = options()
        self.opts = opts
        if isinstance(prm, (list, tuple)):
            counts = np.ascontiguousarray(n, dtype=np.int64)
            arr = (Params * len(prm))(*prm)
            check(L.sphg_create_batch(len(prm), arr, _ptr(counts, _lp), ctypes.byref(opts),
                                      ctypes.byref(self._h)))
            self.counts = counts
            self.n = int(counts.sum())
            self.ninst = len(prm)
        else:
            check(L.sphg_create(ctypes.byref(prm), ctypes.byref(opts), int(n), ctypes.byref(self._h)))
            self.counts = np.array([n], np.int64)
            self.n = int(n)
            self.ninst = 1

    def upload(self, x, y, vx, vy, stream=None):
        x, y, vx, vy = _f64(x), _f64(y), _f64(vx), _f64(vy)
        assert len(x) == self.n
        check(lib().sphg_upload(self._h, _ptr(x), _ptr(y), _ptr(vx), _ptr(vy), _stream(stream)))

    def upload_lattice(self, specs, stream=None):
        """Device-generated initial state: one Lattice per instance."""
        if isinstance(specs, Lattice):
            specs = [specs]
        arr = (Lattice * len(specs))(*specs)
        check(lib().sphg_upload_lattice(self._h, arr, _stream(stream)))

    def preloop(self, stream=None):
        check(lib().sphg_preloop(self._h, _stream(stream)))

    def step(self, k=1, stream=None):
        check(lib().sphg_step(self._h, int(k), _stream(stream)))

    def step_headers(self, k, out=None, stream=None):
        """k iterations, each followed by its step header (the 6 values of
        diagnostics() per instance).  out: the caller's buffer of k * ninst * 6
        doubles -- a float64 array, or the address of pinned host memory -- filled
        in stream order; without it an array is allocated and returned after the
        stream is synchronised, shaped (k, ninst, 6)."""
        k = int(k)
        if out is None:
            arr = np.empty((k, self.ninst, 6), np.float64)
            check(lib().sphg_step_headers(self._h, k, arr.ctypes.data_as(_vp), _stream(stream)))
            check(lib().sphg_stream_synchronize(_stream(stream)))
            return arr
        if isinstance(out, np.ndarray):
            if out.dtype != np.float64 or out.size != k * self.ninst * 6 or not out.flags.c_contiguous:
                raise ValueError("step_headers: out must be a contiguous float64 array of k * ninst * 6")
            check(lib().sphg_step_headers(self._h, k, out.ctypes.data_as(_vp), _stream(stream)))
            return out
        check(lib().sphg_step_headers(self._h, k, ctypes.c_void_p(int(out)), _stream(stream)))
        return out

    def download(self, forces=True, stream=None, out=None):
        """Current state as FP64 arrays in slot order.  out: optional dict of the
        caller's arrays to fill (x, y, vx, vy, rho, ids, and fx, fy with forces),
        each C-contiguous with n entries of the right type; reused buffers whose
        pages are resident let host-access mode 2 write them from the device."""
        n = self.n
        names = ("x", "y", "vx", "vy", "rho") + (("fx", "fy") if forces else ())
        if out is None:
            out = {k: np.empty(n, np.float64) for k in names}
            ids = np.empty(n, np.int32)
        else:
            for k in names:
                a = out[k]
                if a.dtype != np.float64 or a.shape != (n,) or not a.flags.c_contiguous:
                    raise ValueError(f"download: out[{k!r}] must be a contiguous float64 array of {n}")
            ids = out.get("ids")
            if ids is None or ids.dtype != np.int32 or ids.shape != (n,) or not ids.flags.c_contiguous:
                raise ValueError(f"download: out['ids'] must be a contiguous int32 array of {n}")
        check(lib().sphg_download(self._h, _ptr(out["x"]), _ptr(out["y"]), _ptr(out["vx"]),
                                  _ptr(out["vy"]), _ptr(out["rho"]),
                                  _ptr(out["fx"]) if forces else None,
                                  _ptr(out["fy"]) if forces else None, _ptr(ids, _ip),
                                  _stream(stream)))
        out["ids"] = ids
        return out

    def diagnostics(self, stream=None):
        out = np.zeros(6 * self.ninst, np.float64)
        check(lib().sphg_diagnostics(self._h, _ptr(out), _stream(stream)))
        return out.reshape(self.ninst, 6)

    def debug(self, which, stream=None):
        if which in (DBG_POS_NEXT, DBG_VEL_NEXT):
            out = np.empty(2 * self.n, np.float64)
        elif which == DBG_RESORT:
            out = np.zeros(3, np.int32)
        else:
            out = np.empty(self.n, np.int32)
        check(lib().sphg_get_debug(self._h, which, out.ctypes.data_as(_vp), _stream(stream)))
        if which in (DBG_POS_NEXT, DBG_VEL_NEXT):
            return out[0::2].copy(), out[1::2].copy()
        return out

    def neighbor_lists(self, stream=None):
        total = ctypes.c_int64(0)
        offs = np.empty(self.n + 1, np.int64)
        check(lib().sphg_neighbor_lists(self._h, _ptr(offs, _lp), None, ctypes.byref(total),
                                        _stream(stream)))
        idx = np.empty(max(total.value, 1), np.int32)
        check(lib().sphg_neighbor_lists(self._h, _ptr(offs, _lp), _ptr(idx, _ip),
                                        ctypes.byref(total), _stream(stream)))
        return offs, idx[:total.value]

    def neighbor_lists_encoded(self, stream=None):
        """Ascending lists, delta-coded (Codifier::Encode)."""
        total = ctypes.c_int64(0)
        offs = np.empty(self.n + 1, np.int64)
        check(lib().sphg_neighbor_lists_encoded(self._h, _ptr(offs, _lp), None, ctypes.byref(total),
                                                _stream(stream)))
        enc = np.empty(max(total.value, 1), np.int32)
        check(lib().sphg_neighbor_lists_encoded(self._h, _ptr(offs, _lp), _ptr(enc, _ip),
                                                ctypes.byref(total), _stream(stream)))
        return offs, enc[:total.value]

    def set_host_access(self, mode):
        """0: pinned staging; 1: upload reads the caller's arrays from the device;
        2: download writes them from the device as well."""
        check(lib().sphg_set_host_access(self._h, int(mode)))

    def diagnostics_async(self, out_ptr, stream=None):
        """Enqueues the step header into pinned host memory at out_ptr (6 doubles per instance)."""
        check(lib().sphg_diagnostics_async(self._h, out_ptr, _stream(stream)))

    def cfl_dt(self, cfl=0.25, force_coef=0.25, stream=None):
        out = np.zeros(self.ninst, np.float64)
        check(lib().sphg_cfl_dt(self._h, float(cfl), float(force_coef), _ptr(out), _stream(stream)))
        return out

    def set_dt(self, dt, inst=-1):
        check(lib().sphg_set_dt(self._h, int(inst), float(dt)))

    def snapshot(self, stream=None):
        """bytes of an exact-resume snapshot of the current state."""
        size = ctypes.c_uint64(0)
        check(lib().sphg_snapshot(self._h, None, ctypes.byref(size), _stream(stream)))
        buf = ctypes.create_string_buffer(size.value)
        check(lib().sphg_snapshot(self._h, buf, ctypes.byref(size), _stream(stream)))
        return buf.raw

    def restore(self, blob, stream=None):
        buf = ctypes.create_string_buffer(blob, len(blob))
        check(lib().sphg_restore(self._h, buf, len(blob), _stream(stream)))

    def profile_step(self, stream=None):
        """Milliseconds of keys, sort, reorder, density, force+integrate for one iteration."""
        ms = (ctypes.c_float * 5)()
        check(lib().sphg_profile_step(self._h, ms, _stream(stream)))
        return list(ms)

    def launches_per_step(self):
        return int(lib().sphg_launches_per_step(self._h))

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            lib().sphg_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Server:
    """Continuous batching of independent simulations (sphg_server_*)."""

    def __init__(self, budget_bytes, max_instances=4096, opts=None):
        self._h = ctypes.c_void_p()
        self.opts = opts if opts is not None else options()
        check(lib().sphg_server_create(float(budget_bytes), int(max_instances),
                                       ctypes.byref(self.opts), ctypes.byref(self._h)))
        self.sizes = {}

    def submit(self, prm, x, y, vx, vy, steps):
        x, y, vx, vy = _f64(x), _f64(y), _f64(vx), _f64(vy)
        rid = ctypes.c_int64(0)
        check(lib().sphg_server_submit(self._h, ctypes.byref(prm), len(x), _ptr(x), _ptr(y),
                                       _ptr(vx), _ptr(vy), int(steps), ctypes.byref(rid)))
        self.sizes[rid.value] = len(x)
        return rid.value

    def submit_lattice(self, prm, spec, steps):
        """A request whose initial state the device generates at admission."""
        rid = ctypes.c_int64(0)
        check(lib().sphg_server_submit_lattice(self._h, ctypes.byref(prm), ctypes.byref(spec), int(steps),
                                               ctypes.byref(rid)))
        self.sizes[rid.value] = int(spec.nx * spec.ny)
        return rid.value

    def tick(self, stream=None):
        live = ctypes.c_int32(0)
        fin = ctypes.c_int32(0)
        check(lib().sphg_server_tick(self._h, _stream(stream), ctypes.byref(live), ctypes.byref(fin)))
        return live.value, fin.value

    def result(self, rid):
        """dict of the final state and latency, or None while the request runs."""
        n = self.sizes[rid]
        out = {k: np.empty(n, np.float64) for k in ("x", "y", "vx", "vy", "rho")}
        ids = np.empty(n, np.int32)
        lat = ctypes.c_double(0)
        st = lib().sphg_server_result(self._h, rid, _ptr(out["x"]), _ptr(out["y"]), _ptr(out["vx"]),
                                      _ptr(out["vy"]), _ptr(out["rho"]), _ptr(ids, _ip),
                                      ctypes.byref(lat))
        if st == NOT_READY:
            return None
        check(st)
        out["ids"] = ids
        out["latency_s"] = lat.value
        del self.sizes[rid]
        return out

    def stats(self):
        out = np.zeros(8, np.float64)
        check(lib().sphg_server_stats(self._h, _ptr(out)))
        keys = ("live", "queued", "completed", "particle_steps", "ticks", "cap_particles",
                "cap_keys", "live_particles")
        d = dict(zip(keys, out.tolist()))
        c = np.zeros(7, np.float64)
        check(lib().sphg_server_counters(self._h, _ptr(c), 7))
        d.update(zip(("appends", "compactions", "graph_builds", "finished_slots", "slots_in_use",
                      "copies_in_flight", "thread_running"), c.tolist()))
        return d

    def start(self, device=0):
        """Serving thread with its own stream: ticks while work is live or queued."""
        check(lib().sphg_server_start(self._h, int(device)))

    def stop(self):
        check(lib().sphg_server_stop(self._h))

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            lib().sphg_server_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def sort_pairs(keys_in_ptr, vals_in_ptr, keys_out_ptr, vals_out_ptr, n, bits, stream=None):
    """Stand-alone radix sort on caller-owned device buffers (raw pointers)."""
    check(lib().sphg_sort_pairs(keys_in_ptr, vals_in_ptr, keys_out_ptr, vals_out_ptr, int(n),
                                int(bits), _stream(stream)))


def autotune(prms, counts, x, y, vx, vy, base=None, steps=10, stream=None):
    """Fastest launch configuration of this workload: (Options, ms per iteration)."""
    if not isinstance(prms, (list, tuple)):
        prms = [prms]
    counts = np.ascontiguousarray(counts if np.ndim(counts) else [counts], dtype=np.int64)
    arr = (Params * len(prms))(*prms)
    x, y, vx, vy = _f64(x), _f64(y), _f64(vx), _f64(vy)
    best = Options()
    ms = ctypes.c_double(0.0)
    check(lib().sphg_autotune(len(prms), arr, _ptr(counts, _lp), _ptr(x), _ptr(y), _ptr(vx), _ptr(vy),
                              ctypes.byref(base if base is not None else options()), int(steps),
                              ctypes.byref(best), ctypes.byref(ms), _stream(stream)))
    return best, ms.value


def device_attributes(device=0):
    out = np.zeros(6, np.int32)
    check(lib().sphg_device_attributes(int(device), _ptr(out, _ip)))
    keys = ("cc_major", "cc_minor", "sms", "pageable_access", "pageable_uses_host_tables", "concurrent_managed")
    return dict(zip(keys, out.tolist()))


def delta_encode(offs_ptr, idx_ptr, n, enc_ptr, stream=None):
    """Delta codec of n CSR lists on caller-owned device buffers (raw pointers)."""
    check(lib().sphg_delta_encode(offs_ptr, idx_ptr, int(n), enc_ptr, _stream(stream)))


def delta_decode(offs_ptr, enc_ptr, n, idx_ptr, stream=None):
    check(lib().sphg_delta_decode(offs_ptr, enc_ptr, int(n), idx_ptr, _stream(stream)))


def cell_keys(prm, x_ptr, y_ptr, n, keys_ptr, stream=None):
    check(lib().sphg_cell_keys(ctypes.byref(prm), x_ptr, y_ptr, int(n), keys_ptr, _stream(stream)))
