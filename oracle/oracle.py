"""Test-only Python bindings of the CPU checkers.

* ``liboracle.so`` -- the FP64 CPU restatement of the reference step
  (``sph_oracle.cpp``).  Used by the tests, by ``__graft_entry__.smoke`` and by
  ``bench.py``'s CPU-baseline leg, never by the product path.
* ``_ref/libsphref.so`` -- the reference's own classes compiled from their
  sources (``Makefile`` target ``ref``); only present on a machine that has the
  reference checkout.  Used to pin the restatement and to write the golden
  fixtures under ``tests/golden``.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "liboracle.so")
REF_SO = os.path.join(HERE, "_ref", "libsphref.so")
# The reference checkout: SPH_REFERENCE_SRC, else a checkout named "reference"
# beside this repository.
REF_SRC = os.environ.get("SPH_REFERENCE_SRC") or os.path.normpath(os.path.join(HERE, "..", "..", "reference"))

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int32)
_lp = ctypes.POINTER(ctypes.c_int64)


class Params(ctypes.Structure):
    _fields_ = [
        ("h", ctypes.c_double), ("dt", ctypes.c_double), ("k", ctypes.c_double),
        ("rho0", ctypes.c_double), ("mu", ctypes.c_double), ("tol", ctypes.c_double),
        ("gx", ctypes.c_double), ("gy", ctypes.c_double), ("mass", ctypes.c_double),
        ("alpha", ctypes.c_double), ("c0", ctypes.c_double),
        ("lo", ctypes.c_double * 2), ("hi", ctypes.c_double * 2),
        ("order", ctypes.c_int32), ("periodic", ctypes.c_int32),
    ]


class Grid(ctypes.Structure):
    _fields_ = [("cs", ctypes.c_double * 2), ("nx", ctypes.c_int32), ("ny", ctypes.c_int32),
                ("nx_real", ctypes.c_int32), ("ny_real", ctypes.c_int32),
                ("ncells", ctypes.c_int64)]


def build(force=False):
    """Compiles liboracle.so with the host compiler (no make needed)."""
    src = os.path.join(HERE, "sph_oracle.cpp")
    if (not force and os.path.exists(ORACLE_SO)
            and os.path.getmtime(ORACLE_SO) >= os.path.getmtime(src)
            and os.path.getmtime(ORACLE_SO) >= os.path.getmtime(os.path.join(HERE, "sph_oracle.h"))):
        return ORACLE_SO
    cmd = ["g++", "-std=c++17", "-O3", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
           src, "-o", ORACLE_SO]
    subprocess.check_call(cmd, cwd=HERE)
    return ORACLE_SO


def build_ref():
    """Builds _ref/libsphref.so from the reference sources when they are present."""
    if not os.path.isdir(REF_SRC):
        return None
    subprocess.check_call(["make", "-s", "-C", HERE, "ref", "REF=" + REF_SRC])
    return REF_SO


_lib = None
_ref = None


def _p(a, t):
    return a.ctypes.data_as(t) if a is not None else None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(ORACLE_SO)
        PP = ctypes.POINTER(Params)
        GP = ctypes.POINTER(Grid)
        L.orc_default_params.argtypes = [PP]
        L.orc_grid_init.argtypes = [PP, GP]
        L.orc_morton2d.argtypes = [ctypes.c_int32, ctypes.c_int32]
        L.orc_morton2d.restype = ctypes.c_int32
        L.orc_cell_ids.argtypes = [PP, GP, ctypes.c_int64, _dp, _dp, _ip]
        L.orc_sort_perm.argtypes = [ctypes.c_int64, _ip, _ip]
        L.orc_cell_ranges.argtypes = [GP, ctypes.c_int64, _ip, _ip, _ip]
        L.orc_density.argtypes = [PP, GP, ctypes.c_int64, _dp, _dp, _ip, _ip, _ip, _dp]
        L.orc_pressure.argtypes = [PP, ctypes.c_int64, _dp, _dp]
        L.orc_forces.argtypes = [PP, GP, ctypes.c_int64, _dp, _dp, _dp, _dp, _dp, _dp, _ip,
                                 _ip, _ip, _dp, _dp]
        L.orc_integrate.argtypes = [PP, ctypes.c_int64, _dp, _dp, _dp, _dp, _dp, _dp]
        L.orc_nlist_count.argtypes = [PP, GP, ctypes.c_int64, _dp, _dp, _ip, _ip, _ip, _ip, _lp]
        L.orc_nlist_count.restype = ctypes.c_int64
        L.orc_nlist_fill.argtypes = [PP, GP, ctypes.c_int64, _dp, _dp, _ip, _ip, _ip, _lp, _ip]
        L.orc_density_lists.argtypes = [PP, ctypes.c_int64, _dp, _dp, _lp, _ip, _dp]
        L.orc_forces_lists.argtypes = [PP, ctypes.c_int64, _dp, _dp, _dp, _dp, _dp, _dp, _lp,
                                       _ip, _dp, _dp]
        L.orc_delta_encode.argtypes = [ctypes.c_int64, _lp, _ip, _ip]
        L.orc_delta_decode.argtypes = [ctypes.c_int64, _lp, _ip, _ip]
        L.orc_diagnostics.argtypes = [PP, ctypes.c_int64, _dp, _dp, _dp, _dp, _dp]
        L.orc_lattice.argtypes = [ctypes.c_double] * 6 + [_dp, _dp]
        L.orc_lattice.restype = ctypes.c_int64
        L.orc_sim_create.argtypes = [PP, ctypes.c_int64, _dp, _dp, _dp, _dp]
        L.orc_sim_create.restype = ctypes.c_void_p
        L.orc_sim_destroy.argtypes = [ctypes.c_void_p]
        L.orc_sim_preloop.argtypes = [ctypes.c_void_p]
        L.orc_sim_steps.argtypes = [ctypes.c_void_p, ctypes.c_int64]
        L.orc_sim_get.argtypes = [ctypes.c_void_p] + [_dp] * 7 + [_ip, _ip]
        L.orc_sim_set.argtypes = [ctypes.c_void_p] + [_dp] * 6
        L.orc_set_threads.argtypes = [ctypes.c_int32]
        L.orc_get_threads.restype = ctypes.c_int32
        _lib = L
    return _lib


def params(**kw):
    """Reference defaults (core/ConfigVariables.hpp, config/example.txt), overridable."""
    p = Params()
    lib().orc_default_params(ctypes.byref(p))
    for k, v in kw.items():
        if k in ("lo", "hi"):
            getattr(p, k)[0], getattr(p, k)[1] = v
        elif k == "order" and isinstance(v, str):
            p.order = {"morton": 0, "rowmajor": 1}[v]
        else:
            setattr(p, k, v)
    return p


def grid(p):
    g = Grid()
    lib().orc_grid_init(ctypes.byref(p), ctypes.byref(g))
    return g


def f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def cell_ids(p, x, y):
    g = grid(p)
    x, y = f64(x), f64(y)
    key = np.empty(len(x), np.int32)
    lib().orc_cell_ids(ctypes.byref(p), ctypes.byref(g), len(x), _p(x, _dp), _p(y, _dp),
                       _p(key, _ip))
    return key


def sort_perm(key):
    key = i32(key)
    perm = np.empty(len(key), np.int32)
    lib().orc_sort_perm(len(key), _p(key, _ip), _p(perm, _ip))
    return perm


def cell_ranges(p, sorted_key):
    g = grid(p)
    k = i32(sorted_key)
    s = np.empty(g.ncells, np.int32)
    e = np.empty(g.ncells, np.int32)
    lib().orc_cell_ranges(ctypes.byref(g), len(k), _p(k, _ip), _p(s, _ip), _p(e, _ip))
    return s, e


def find_neighbors(p, x, y):
    """Keys -> stable permutation -> sorted keys -> cell ranges."""
    key = cell_ids(p, x, y)
    perm = sort_perm(key)
    sk = key[perm]
    s, e = cell_ranges(p, sk)
    return key, perm, sk, s, e


def density(p, x, y, sk, s, e):
    g = grid(p)
    x, y, sk = f64(x), f64(y), i32(sk)
    rho = np.empty(len(x), np.float64)
    lib().orc_density(ctypes.byref(p), ctypes.byref(g), len(x), _p(x, _dp), _p(y, _dp),
                      _p(sk, _ip), _p(s, _ip), _p(e, _ip), _p(rho, _dp))
    return rho


def pressure(p, rho):
    rho = f64(rho)
    pr = np.empty_like(rho)
    lib().orc_pressure(ctypes.byref(p), len(rho), _p(rho, _dp), _p(pr, _dp))
    return pr


def forces(p, x, y, vx, vy, rho, sk, s, e):
    g = grid(p)
    x, y, vx, vy, rho, sk = f64(x), f64(y), f64(vx), f64(vy), f64(rho), i32(sk)
    pr = pressure(p, rho)
    fx = np.empty_like(x)
    fy = np.empty_like(x)
    lib().orc_forces(ctypes.byref(p), ctypes.byref(g), len(x), _p(x, _dp), _p(y, _dp),
                     _p(vx, _dp), _p(vy, _dp), _p(rho, _dp), _p(pr, _dp), _p(sk, _ip),
                     _p(s, _ip), _p(e, _ip), _p(fx, _dp), _p(fy, _dp))
    return fx, fy


def integrate(p, x, y, vx, vy, fx, fy):
    x, y, vx, vy = f64(x).copy(), f64(y).copy(), f64(vx).copy(), f64(vy).copy()
    fx, fy = f64(fx), f64(fy)
    lib().orc_integrate(ctypes.byref(p), len(x), _p(x, _dp), _p(y, _dp), _p(vx, _dp),
                        _p(vy, _dp), _p(fx, _dp), _p(fy, _dp))
    return x, y, vx, vy


def neighbor_lists(p, x, y, sk, s, e):
    g = grid(p)
    x, y, sk = f64(x), f64(y), i32(sk)
    n = len(x)
    counts = np.empty(n, np.int32)
    offs = np.empty(n + 1, np.int64)
    tot = lib().orc_nlist_count(ctypes.byref(p), ctypes.byref(g), n, _p(x, _dp), _p(y, _dp),
                                _p(sk, _ip), _p(s, _ip), _p(e, _ip), _p(counts, _ip),
                                _p(offs, _lp))
    idx = np.empty(max(tot, 1), np.int32)
    lib().orc_nlist_fill(ctypes.byref(p), ctypes.byref(g), n, _p(x, _dp), _p(y, _dp),
                         _p(sk, _ip), _p(s, _ip), _p(e, _ip), _p(offs, _lp), _p(idx, _ip))
    return offs, idx[:tot]


def density_lists(p, x, y, offs, idx):
    x, y = f64(x), f64(y)
    offs = np.ascontiguousarray(offs, np.int64)
    idx = i32(idx)
    rho = np.empty_like(x)
    lib().orc_density_lists(ctypes.byref(p), len(x), _p(x, _dp), _p(y, _dp), _p(offs, _lp),
                            _p(idx, _ip), _p(rho, _dp))
    return rho


def forces_lists(p, x, y, vx, vy, rho, offs, idx):
    x, y, vx, vy, rho = f64(x), f64(y), f64(vx), f64(vy), f64(rho)
    offs = np.ascontiguousarray(offs, np.int64)
    idx = i32(idx)
    pr = pressure(p, rho)
    fx = np.empty_like(x)
    fy = np.empty_like(x)
    lib().orc_forces_lists(ctypes.byref(p), len(x), _p(x, _dp), _p(y, _dp), _p(vx, _dp),
                           _p(vy, _dp), _p(rho, _dp), _p(pr, _dp), _p(offs, _lp), _p(idx, _ip),
                           _p(fx, _dp), _p(fy, _dp))
    return fx, fy


def delta_encode(offs, idx):
    offs = np.ascontiguousarray(offs, np.int64)
    idx = i32(idx)
    out = np.zeros(max(len(idx), 1), np.int32)
    lib().orc_delta_encode(len(offs) - 1, _p(offs, _lp), _p(idx, _ip), _p(out, _ip))
    return out[:len(idx)]


def delta_decode(offs, enc):
    offs = np.ascontiguousarray(offs, np.int64)
    enc = i32(enc)
    out = np.zeros(max(len(enc), 1), np.int32)
    lib().orc_delta_decode(len(offs) - 1, _p(offs, _lp), _p(enc, _ip), _p(out, _ip))
    return out[:len(enc)]


def diagnostics(p, x, y, vx, vy):
    x, y, vx, vy = f64(x), f64(y), f64(vx), f64(vy)
    out = np.zeros(5, np.float64)
    lib().orc_diagnostics(ctypes.byref(p), len(x), _p(x, _dp), _p(y, _dp), _p(vx, _dp),
                          _p(vy, _dp), _p(out, _dp))
    return out


def lattice(lx, ly, dX, dY, xvol, yvol):
    n = lib().orc_lattice(lx, ly, dX, dY, xvol, yvol, None, None)
    x = np.empty(n, np.float64)
    y = np.empty(n, np.float64)
    lib().orc_lattice(lx, ly, dX, dY, xvol, yvol, _p(x, _dp), _p(y, _dp))
    return x, y


class Sim:
    """Whole pre-loop + main loop (app/simulation_configuration.h:168-440)."""

    def __init__(self, p, x, y, vx, vy):
        x, y, vx, vy = f64(x), f64(y), f64(vx), f64(vy)
        self.n = len(x)
        self.h = lib().orc_sim_create(ctypes.byref(p), self.n, _p(x, _dp), _p(y, _dp),
                                      _p(vx, _dp), _p(vy, _dp))

    def preloop(self):
        lib().orc_sim_preloop(self.h)

    def steps(self, k):
        lib().orc_sim_steps(self.h, k)

    def get(self):
        n = self.n
        a = {k: np.empty(n, np.float64) for k in ("x", "y", "vx", "vy", "fx", "fy", "rho")}
        key = np.empty(n, np.int32)
        ids = np.empty(n, np.int32)
        lib().orc_sim_get(self.h, *[_p(a[k], _dp) for k in ("x", "y", "vx", "vy", "fx", "fy", "rho")],
                          _p(key, _ip), _p(ids, _ip))
        a["key"] = key
        a["ids"] = ids
        return a

    def set(self, x, y, vx, vy, fx, fy):
        arrs = [f64(v) for v in (x, y, vx, vy, fx, fy)]
        lib().orc_sim_set(self.h, *[_p(v, _dp) for v in arrs])

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_sim_destroy(self.h)
            self.h = None


def set_threads(n):
    lib().orc_set_threads(n)


def get_threads():
    return lib().orc_get_threads()


# ---------------------------------------------------------------- reference harness
def ref_lib():
    """The reference's own classes (None when not built on this machine)."""
    global _ref
    if _ref is None:
        if not os.path.exists(REF_SO):
            return None
        R = ctypes.CDLL(REF_SO)
        R.ref_create.argtypes = [ctypes.c_int32] + [ctypes.c_double] * 9 + [ctypes.c_int64]
        R.ref_create.restype = ctypes.c_void_p
        R.ref_destroy.argtypes = [ctypes.c_void_p]
        R.ref_set.argtypes = [ctypes.c_void_p] + [_dp] * 7
        R.ref_get.argtypes = [ctypes.c_void_p] + [_dp] * 7 + [_ip, _ip]
        R.ref_set_params.argtypes = [ctypes.c_double] * 4
        for f in ("ref_density", "ref_pressure_forces", "ref_integrate", "ref_mplists_compute"):
            getattr(R, f).argtypes = [ctypes.c_void_p]
        R.ref_find_neighbors.argtypes = [ctypes.c_void_p, _ip]
        R.ref_cell_ranges.argtypes = [ctypes.c_void_p, _ip, _ip]
        R.ref_grid.argtypes = [ctypes.c_void_p, _ip]
        R.ref_nlists.argtypes = [ctypes.c_void_p, ctypes.c_int32]
        R.ref_nlists.restype = ctypes.c_int64
        R.ref_nlists_get.argtypes = [ctypes.c_void_p, _lp, _ip]
        R.ref_diagnostics.argtypes = [ctypes.c_void_p, _dp]
        R.ref_morton2d.argtypes = [ctypes.c_int32, ctypes.c_int32]
        R.ref_morton2d.restype = ctypes.c_int32
        R.ref_encode.argtypes = [ctypes.c_int32, _ip, _ip]
        R.ref_morton_table.argtypes = [ctypes.c_int32, ctypes.c_int32, _ip]
        R.ref_lattice.argtypes = [ctypes.c_double] * 6 + [_dp, _dp]
        R.ref_lattice.restype = ctypes.c_int64
        _ref = R
    return _ref


class RefSim:
    """One reference simulation object (SoAContainer + GenericNeighborSearch +
    GenericForceComputation + Integrator) driven step by step."""

    def __init__(self, p, n):
        R = ref_lib()
        self.R = R
        self.p = p
        self.n = n
        self.h = R.ref_create(p.order, p.lo[0], p.lo[1], p.hi[0], p.hi[1], p.h, p.k, p.rho0,
                              p.mu, p.dt, n)

    def _params(self):
        self.R.ref_set_params(self.p.h, self.p.k, self.p.rho0, self.p.mu)

    def set(self, x, y, vx, vy, fx=None, fy=None, rho=None):
        arrs = [f64(a) if a is not None else None for a in (x, y, vx, vy, fx, fy, rho)]
        self.R.ref_set(self.h, *[_p(a, _dp) for a in arrs])

    def get(self):
        n = self.n
        a = {k: np.empty(n, np.float64) for k in ("x", "y", "vx", "vy", "fx", "fy", "rho")}
        key = np.empty(n, np.int32)
        ids = np.empty(n, np.int32)
        self.R.ref_get(self.h, *[_p(a[k], _dp) for k in ("x", "y", "vx", "vy", "fx", "fy", "rho")],
                       _p(key, _ip), _p(ids, _ip))
        a["key"] = key
        a["ids"] = ids
        return a

    def find_neighbors(self):
        self._params()
        perm = np.empty(self.n, np.int32)
        self.R.ref_find_neighbors(self.h, _p(perm, _ip))
        return perm

    def grid(self):
        out = np.zeros(3, np.int32)
        self.R.ref_grid(self.h, _p(out, _ip))
        return out

    def cell_ranges(self):
        nc = int(self.grid()[2])
        s = np.empty(nc, np.int32)
        e = np.empty(nc, np.int32)
        self.R.ref_cell_ranges(self.h, _p(s, _ip), _p(e, _ip))
        return s, e

    def density(self):
        self._params()
        self.R.ref_density(self.h)

    def pressure_forces(self):
        self._params()
        self.R.ref_pressure_forces(self.h)

    def integrate(self):
        self.R.ref_integrate(self.h)

    def preloop(self):
        self.find_neighbors()
        self.density()
        self.pressure_forces()

    def step(self):
        self.integrate()
        self.find_neighbors()
        self.density()
        self.pressure_forces()

    def nlists(self, which):
        self._params()
        tot = self.R.ref_nlists(self.h, which)
        offs = np.empty(self.n + 1, np.int64)
        idx = np.empty(max(tot, 1), np.int32)
        self.R.ref_nlists_get(self.h, _p(offs, _lp), _p(idx, _ip))
        return offs, idx[:tot]

    def mplists_compute(self):
        self._params()
        self.R.ref_mplists_compute(self.h)

    def diagnostics(self):
        out = np.zeros(3, np.float64)
        self.R.ref_diagnostics(self.h, _p(out, _dp))
        return out

    def __del__(self):
        if getattr(self, "h", None):
            self.R.ref_destroy(self.h)
            self.h = None
