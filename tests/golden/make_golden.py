"""Writes the golden fixtures in this directory from the REFERENCE's own code.

The reference (jose-pinzon0407/sph-simulations) has no tests or golden vectors
of its own, so these are produced by running its C++ classes, compiled from
their sources by ``oracle/Makefile`` (target ``ref``) into
``oracle/_ref/libsphref.so``, on seeded synthetic inputs.  All inputs are
float32-representable so the same values can be fed to the CUDA path.

Run from the repository root on a machine with the reference checkout:
    python tests/golden/make_golden.py
"""
import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import oracle as O  # noqa: E402


def jittered_lattice(nx, ny, dx, seed, origin=0.5):
    rng = np.random.default_rng(seed)
    gx, gy = np.meshgrid(np.arange(nx), np.arange(ny), indexing="xy")
    x = (gx.ravel() + origin) * dx + rng.uniform(-0.01 * dx, 0.01 * dx, gx.size)
    y = (gy.ravel() + origin) * dx + rng.uniform(-0.01 * dx, 0.01 * dx, gx.size)
    return x.astype(np.float32).astype(np.float64), y.astype(np.float32).astype(np.float64)


def snapshot(R, prefix, out, keys=("x", "y", "vx", "vy", "fx", "fy", "rho", "key", "ids")):
    a = R.get()
    for k in keys:
        out[prefix + k] = a[k]


def ranges_compact(R):
    s, e = R.cell_ranges()
    occ = np.nonzero(s >= 0)[0].astype(np.int32)
    return occ, s[occ], e[occ], np.int64(len(s))


def morton_kat():
    R = O.ref_lib()
    table = np.empty(2048 * 2048, np.int32)
    R.ref_morton_table(2048, 2048, table.ctypes.data_as(O._ip))
    rng = np.random.default_rng(7)
    cx = rng.integers(0, 2048, 4096).astype(np.int32)
    cy = rng.integers(0, 2048, 4096).astype(np.int32)
    cx = np.concatenate([cx, [0, 2047, 0, 2047, 1, 1024, 1023]]).astype(np.int32)
    cy = np.concatenate([cy, [0, 0, 2047, 2047, 1, 1024, 1023]]).astype(np.int32)
    code = table[cx + 2048 * cy]
    np.savez_compressed(os.path.join(HERE, "morton_kat.npz"), cx=cx, cy=cy, code=code,
                        sha256_2048=np.frombuffer(hashlib.sha256(table.tobytes()).digest(), np.uint8))


def default_rowmajor():
    # config/example.txt: domain 96x48, lattice 0.5 spacing, 0.4 x 0.8 volume, dt 0.005,
    # order=rowmajor, compute_type=sorted; H=1 (core/ConfigVariables.hpp:9)
    p = O.params(order="rowmajor", h=1.0, dt=0.005, lo=(0, 0), hi=(96, 48))
    x, y = O.lattice(96, 48, 0.5, 0.5, 0.4, 0.8)
    n = len(x)
    R = O.RefSim(p, n)
    R.set(x, y, np.zeros(n), np.zeros(n))
    out = {"x_in": x, "y_in": y}
    R.preloop()
    snapshot(R, "s0_", out)
    out["s0_occ"], out["s0_start"], out["s0_end"], out["ncells"] = ranges_compact(R)
    R.step()
    R.step()
    snapshot(R, "s2_", out)
    out["s2_diag"] = R.diagnostics()
    np.savez_compressed(os.path.join(HERE, "default_rowmajor.npz"), **out)


def dam12k_morton():
    # dam-break column geometry of the 12,800-particle case: 80 x 160 lattice,
    # dx = 0.005 from (dx/2, dx/2), +-0.01 dx jitter, h = 1.3 dx, box [0,1]^2.
    dx = 0.005
    x, y = jittered_lattice(80, 160, dx, seed=0)
    rng = np.random.default_rng(1)
    vx = rng.uniform(-0.1, 0.1, len(x)).astype(np.float32).astype(np.float64)
    vy = rng.uniform(-0.1, 0.1, len(x)).astype(np.float32).astype(np.float64)
    p = O.params(order="morton", h=1.3 * dx, dt=1e-5, lo=(0, 0), hi=(1, 1))
    n = len(x)
    R = O.RefSim(p, n)
    R.set(x, y, vx, vy)
    perm = R.find_neighbors()
    R.density()
    R.pressure_forces()
    a = R.get()
    key_in = O.cell_ids(p, x, y)
    np.savez_compressed(os.path.join(HERE, "dam12k_morton.npz"), x_in=x, y_in=y, vx_in=vx,
                        vy_in=vy, key_in=key_in, perm=perm, key=a["key"], rho=a["rho"],
                        fx=a["fx"], fy=a["fy"], h=p.h, dt=p.dt)


def small_multistep():
    dx = 0.01
    x, y = jittered_lattice(30, 60, dx, seed=2)
    n = len(x)
    rng = np.random.default_rng(3)
    vx = rng.uniform(-0.05, 0.05, n).astype(np.float32).astype(np.float64)
    vy = rng.uniform(-0.05, 0.05, n).astype(np.float32).astype(np.float64)
    out = {"x_in": x, "y_in": y, "vx_in": vx, "vy_in": vy}
    for order in ("morton", "rowmajor"):
        p = O.params(order=order, h=1.3 * dx, dt=1e-5, lo=(0, 0), hi=(1, 1))
        R = O.RefSim(p, n)
        R.set(x, y, vx, vy)
        R.preloop()
        snapshot(R, order + "_s0_", out)
        R.step()
        snapshot(R, order + "_s1_", out)
        for _ in range(9):
            R.step()
        snapshot(R, order + "_s10_", out)
        out[order + "_s10_diag"] = R.diagnostics()
    out["h"] = 1.3 * dx
    out["dt"] = 1e-5
    np.savez_compressed(os.path.join(HERE, "small_multistep.npz"), **out)


def lists():
    dx = 0.01
    x, y = jittered_lattice(30, 60, dx, seed=2)
    n = len(x)
    rng = np.random.default_rng(4)
    vx = rng.uniform(-0.05, 0.05, n).astype(np.float32).astype(np.float64)
    vy = rng.uniform(-0.05, 0.05, n).astype(np.float32).astype(np.float64)
    out = {}
    p = O.params(order="morton", h=1.3 * dx, dt=1e-5, lo=(0, 0), hi=(1, 1))
    R = O.RefSim(p, n)
    R.set(x, y, vx, vy)
    R.find_neighbors()
    a = R.get()
    out.update(x=a["x"], y=a["y"], vx=a["vx"], vy=a["vy"], key=a["key"])
    out["gnl_offs"], out["gnl_idx"] = R.nlists(0)
    out["mpl_offs"], out["mpl_idx"] = R.nlists(1)
    R.mplists_compute()
    b = R.get()
    out.update(mpl_rho=b["rho"], mpl_fx=b["fx"], mpl_fy=b["fy"])
    # Codifier::Encode on ascending lists
    offs, idx = out["gnl_offs"], out["gnl_idx"]
    enc_lists, enc_out = [], []
    for i in range(0, n, 37):
        lst = np.sort(idx[offs[i]:offs[i + 1]]).astype(np.int32)
        res = np.empty(len(lst), np.int32)
        O.ref_lib().ref_encode(len(lst), lst.ctypes.data_as(O._ip), res.ctypes.data_as(O._ip))
        enc_lists.append(lst)
        enc_out.append(res)
    lens = np.array([len(v) for v in enc_lists], np.int64)
    out["enc_offs"] = np.concatenate([[0], np.cumsum(lens)]).astype(np.int64)
    out["enc_in"] = np.concatenate(enc_lists)
    out["enc_out"] = np.concatenate(enc_out)
    out["h"] = p.h
    np.savez_compressed(os.path.join(HERE, "lists.npz"), **out)


def tiny():
    """Hand-checkable cases: 2 to 9 particles, both orders, H = 1."""
    cases = {
        "pair": ([1.2, 1.7], [1.5, 1.5], [0.1, -0.1], [0.0, 0.2]),
        "line3": ([1.1, 1.6, 2.05], [1.3, 1.3, 1.3], [0.0, 0.0, 0.0], [0.0, 0.1, -0.1]),
        "grid9": ([1.0 + 0.7 * (i % 3) for i in range(9)], [1.0 + 0.7 * (i // 3) for i in range(9)],
                  [0.01 * i for i in range(9)], [-0.02 * i for i in range(9)]),
        "wall": ([0.001, 3.999, 2.0], [0.001, 2.0, 3.999], [-1.0, 1.0, 0.0], [-1.0, 0.0, 1.0]),
    }
    out = {}
    for name, (x, y, vx, vy) in cases.items():
        x = np.array(x, np.float32).astype(np.float64)
        y = np.array(y, np.float32).astype(np.float64)
        vx = np.array(vx, np.float32).astype(np.float64)
        vy = np.array(vy, np.float32).astype(np.float64)
        out[name + "_x_in"], out[name + "_y_in"] = x, y
        out[name + "_vx_in"], out[name + "_vy_in"] = vx, vy
        for order in ("morton", "rowmajor"):
            p = O.params(order=order, h=1.0, dt=0.005, lo=(0, 0), hi=(4, 4))
            R = O.RefSim(p, len(x))
            R.set(x, y, vx, vy)
            R.preloop()
            snapshot(R, f"{name}_{order}_s0_", out)
            R.step()
            snapshot(R, f"{name}_{order}_s1_", out)
    np.savez_compressed(os.path.join(HERE, "tiny.npz"), **out)


def main():
    if O.ref_lib() is None:
        O.build_ref()
    assert O.ref_lib() is not None, "reference harness not built (needs the reference sources)"
    morton_kat()
    default_rowmajor()
    dam12k_morton()
    small_multistep()
    lists()
    tiny()
    for f in sorted(os.listdir(HERE)):
        if f.endswith(".npz"):
            print(f, os.path.getsize(os.path.join(HERE, f)))


if __name__ == "__main__":
    main()
