"""Parity of the CUDA path (through the C ABI of libsphg.so) with the oracle
and with the reference's own golden fixtures.

Tolerances (the CUDA path computes in FP32, the oracle and the reference in FP64):
  * cell keys, sorted permutation, cell membership, neighbour lists: bit-exact
    (same FP32-representable positions in; the FP64 decision is reproduced);
  * density: per particle |drho| / rho <= 1e-5;
  * acceleration: max_i |da_i| / max_i |a_i| <= 1e-5 (norm-wise, per instance);
  * integrated positions/velocities: within a few FP32 ulp of the FP64 update.
"""
import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu

RHO_TOL = 1e-5
ACC_TOL = 1e-5


def _sphg():
    import sphg
    return sphg


def jittered(nx, ny, dx, seed, vel=0.0):
    rng = np.random.default_rng(seed)
    gx, gy = np.meshgrid(np.arange(nx), np.arange(ny), indexing="xy")
    x = (gx.ravel() + 0.5) * dx + rng.uniform(-0.01 * dx, 0.01 * dx, gx.size)
    y = (gy.ravel() + 0.5) * dx + rng.uniform(-0.01 * dx, 0.01 * dx, gx.size)
    vx = rng.uniform(-vel, vel, gx.size)
    vy = rng.uniform(-vel, vel, gx.size)
    f = lambda a: a.astype(np.float32).astype(np.float64)  # noqa: E731
    return f(x), f(y), f(vx), f(vy)


def rel_rho(got, ref):
    return float(np.max(np.abs(got - ref) / np.abs(ref)))


def rel_acc(gx, gy, rx, ry):
    scale = max(np.abs(rx).max(), np.abs(ry).max())
    return float(max(np.abs(gx - rx).max(), np.abs(gy - ry).max()) / scale)


def oracle_state(p, g):
    """Oracle density/forces on the GPU's own current (sorted) state."""
    sk = O.cell_ids(p, g["x"], g["y"])
    s, e = O.cell_ranges(p, sk)
    rho = O.density(p, g["x"], g["y"], sk, s, e)
    fx, fy = O.forces(p, g["x"], g["y"], g["vx"], g["vy"], rho, sk, s, e)
    return sk, s, e, rho, fx, fy


# ---------------------------------------------------------------- stand-alone kernels
@pytest.mark.parametrize("order", ["morton", "rowmajor"])
def test_cell_keys_exact_at_cell_edges(order):
    torch = pytest.importorskip("torch")
    S = _sphg()
    h = 0.0065
    kw = dict(order=order, h=h, lo=(0, 0), hi=(1, 1))
    rng = np.random.default_rng(5)
    # random positions plus positions on and next to every cell edge
    edges = np.arange(0, 155) * h
    near = np.concatenate([edges, np.nextafter(edges.astype(np.float32), 2).astype(np.float64),
                           np.nextafter(edges.astype(np.float32), -1).astype(np.float64)])
    near = near[(near >= 0) & (near <= 1)]
    x = np.concatenate([rng.uniform(0, 1, 200000), near, np.full(near.size, 0.5), [0.0, 1.0]])
    y = np.concatenate([rng.uniform(0, 1, 200000), np.full(near.size, 0.25), near, [1.0, 0.0]])
    x = x.astype(np.float32)
    y = y.astype(np.float32)
    ref = O.cell_ids(O.params(**kw), x.astype(np.float64), y.astype(np.float64))
    dx = torch.from_numpy(x).cuda()
    dy = torch.from_numpy(y).cuda()
    dk = torch.empty(len(x), dtype=torch.int32, device="cuda")
    S.cell_keys(S.params(**kw), dx.data_ptr(), dy.data_ptr(), len(x), dk.data_ptr())
    torch.cuda.synchronize()
    assert (dk.cpu().numpy() == ref).all()


@pytest.mark.parametrize("n,bits", [(0, 8), (1, 8), (2047, 8), (2048, 16), (2049, 22),
                                    (100003, 22), (1 << 20, 25), (300000, 32)])
def test_sort_pairs_stable(n, bits):
    torch = pytest.importorskip("torch")
    S = _sphg()
    rng = np.random.default_rng(n + bits)
    hi = (1 << bits) if bits < 32 else (1 << 32)
    keys = rng.integers(0, min(hi, 1 << 12) if n > 1000 and bits > 16 else hi, n,
                        dtype=np.uint64).astype(np.uint32)
    vals = rng.permutation(n).astype(np.uint32)
    order = np.argsort(keys, kind="stable")
    if n == 0:
        S.sort_pairs(0, 0, 0, 0, 0, bits)
        return
    ki = torch.from_numpy(keys.view(np.int32)).cuda()
    vi = torch.from_numpy(vals.view(np.int32)).cuda()
    ko = torch.empty_like(ki)
    vo = torch.empty_like(vi)
    S.sort_pairs(ki.data_ptr(), vi.data_ptr(), ko.data_ptr(), vo.data_ptr(), n, bits)
    torch.cuda.synchronize()
    assert (ko.cpu().numpy().view(np.uint32) == keys[order]).all()
    assert (vo.cpu().numpy().view(np.uint32) == vals[order]).all()


@pytest.mark.parametrize("offset", [1, 2, 3])
def test_sort_pairs_from_unaligned_views(offset):
    """Caller buffers that start at any 4-byte boundary (keys[offset:]): the
    histogram pass takes 16-byte loads only where the address allows them."""
    torch = pytest.importorskip("torch")
    S = _sphg()
    n = 100003
    rng = np.random.default_rng(offset)
    keys = rng.integers(0, 1 << 20, n + offset, dtype=np.uint64).astype(np.uint32)
    keys[offset: offset + n // 4] = 7  # runs of equal keys
    base = torch.from_numpy(keys.view(np.int32)).cuda()
    ki = base[offset:]
    assert ki.data_ptr() % 16 != 0
    ko = torch.empty(n, dtype=torch.int32, device="cuda")
    vo = torch.empty(n, dtype=torch.int32, device="cuda")
    S.sort_pairs(ki.data_ptr(), 0, ko.data_ptr(), vo.data_ptr(), n, 20)
    torch.cuda.synchronize()
    order = np.argsort(keys[offset:], kind="stable")
    assert (ko.cpu().numpy().view(np.uint32) == keys[offset:][order]).all()
    assert (vo.cpu().numpy() == order).all()


# ---------------------------------------------------------------- whole step vs reference goldens
def test_preloop_matches_reference_dam12k(golden):
    """12,800-particle dam-break geometry, reference physics (k=30, rho0=25, mu=0.01,
    g=-10, m=1), h = 0.0065, Morton: keys, cell membership, density and forces
    against the reference's own FP64 output."""
    S = _sphg()
    g = golden("dam12k_morton")
    kw = dict(order="morton", h=float(g["h"]), dt=float(g["dt"]), lo=(0, 0), hi=(1, 1))
    sim = S.Sim(S.params(**kw), len(g["x_in"]))
    sim.upload(g["x_in"], g["y_in"], g["vx_in"], g["vy_in"])
    sim.preloop()
    out = sim.download()
    keys = sim.debug(S.DBG_KEYS)
    assert (keys == g["key"]).all()
    # same particles in every cell as the reference's (unstable) sort
    cells = np.unique(keys)
    starts = np.searchsorted(keys, cells)
    ends = np.searchsorted(keys, cells, side="right")
    for c, b, e in zip(cells, starts, ends):
        assert set(out["ids"][b:e]) == set(g["perm"][b:e])
    # density and forces by particle identity
    ref_rho = np.empty_like(g["rho"]); ref_rho[g["perm"]] = g["rho"]
    ref_fx = np.empty_like(g["fx"]); ref_fx[g["perm"]] = g["fx"]
    ref_fy = np.empty_like(g["fy"]); ref_fy[g["perm"]] = g["fy"]
    assert rel_rho(out["rho"], ref_rho[out["ids"]]) <= RHO_TOL
    assert rel_acc(out["fx"], out["fy"], ref_fx[out["ids"]], ref_fy[out["ids"]]) <= ACC_TOL
    sim.close()


@pytest.mark.parametrize("case", ["pair", "line3", "grid9", "wall"])
@pytest.mark.parametrize("order", ["morton", "rowmajor"])
def test_tiny_cases(golden, case, order):
    S = _sphg()
    g = golden("tiny")
    kw = dict(order=order, h=1.0, dt=0.005, lo=(0, 0), hi=(4, 4))
    sim = S.Sim(S.params(**kw), len(g[case + "_x_in"]))
    sim.upload(g[case + "_x_in"], g[case + "_y_in"], g[case + "_vx_in"], g[case + "_vy_in"])
    sim.preloop()
    for step in (0, 1):
        if step:
            sim.step(1)
        out = sim.download()
        pre = f"{case}_{order}_s{step}_"
        assert (sim.debug(S.DBG_KEYS) == g[pre + "key"]).all()
        by = lambda a, ids: a[np.argsort(ids)]  # noqa: E731
        for k in ("x", "y", "vx", "vy", "rho"):
            ref = by(g[pre + k], g[pre + "ids"])
            got = by(out[k], out["ids"])
            np.testing.assert_allclose(got, ref, rtol=2e-6, atol=1e-6 * max(np.abs(ref).max(), 1e-30))
        rx, ry = by(g[pre + "fx"], g[pre + "ids"]), by(g[pre + "fy"], g[pre + "ids"])
        gx, gy = by(out["fx"], out["ids"]), by(out["fy"], out["ids"])
        assert rel_acc(gx, gy, rx, ry) <= 2e-6
    sim.close()


def test_default_config_rowmajor(golden):
    """The reference's own config/example.txt run (6,084 particles, H=1, rowmajor)."""
    S = _sphg()
    g = golden("default_rowmajor")
    kw = dict(order="rowmajor", h=1.0, dt=0.005, lo=(0, 0), hi=(96, 48))
    n = len(g["x_in"])
    sim = S.Sim(S.params(**kw), n)
    sim.upload(g["x_in"], g["y_in"], np.zeros(n), np.zeros(n))
    sim.preloop()
    out = sim.download()
    assert (sim.debug(S.DBG_KEYS) == g["s0_key"]).all()
    ref_rho = np.empty(n); ref_rho[g["s0_ids"]] = g["s0_rho"]
    ref_fx = np.empty(n); ref_fx[g["s0_ids"]] = g["s0_fx"]
    ref_fy = np.empty(n); ref_fy[g["s0_ids"]] = g["s0_fy"]
    assert rel_rho(out["rho"], ref_rho[out["ids"]]) <= RHO_TOL
    assert rel_acc(out["fx"], out["fy"], ref_fx[out["ids"]], ref_fy[out["ids"]]) <= ACC_TOL
    sim.step(2)
    out = sim.download()
    ref = {k: np.empty(n) for k in ("x", "y", "vx", "vy", "rho")}
    for k in ref:
        ref[k][g["s2_ids"]] = g["s2_" + k]
    for k in ("x", "y"):
        np.testing.assert_allclose(out[k], ref[k][out["ids"]], rtol=1e-6, atol=1e-5)
    assert rel_rho(out["rho"], ref["rho"][out["ids"]]) <= 1e-5
    d = sim.diagnostics()[0]
    np.testing.assert_allclose(d[0], g["s2_diag"][0], rtol=1e-4)
    assert d[2] == g["s2_diag"][2]
    sim.close()


# ---------------------------------------------------------------- teacher-forced step chain
@pytest.mark.parametrize("order", ["morton", "rowmajor"])
def test_step_chain_teacher_forced(order):
    """Every stage of a main-loop iteration against the oracle fed with the GPU's
    own previous-stage output: integrate -> keys -> stable sort -> density -> forces."""
    S = _sphg()
    dx = 0.005
    x, y, vx, vy = jittered(80, 160, dx, seed=3, vel=0.5)
    kw = dict(order=order, h=1.3 * dx, dt=1e-5, lo=(0, 0), hi=(1, 1))
    p = O.params(**kw)
    sim = S.Sim(S.params(**kw), len(x))
    sim.upload(x, y, vx, vy)
    sim.preloop()
    for it in range(3):
        a = sim.download()
        sk, s, e, rho, fx, fy = oracle_state(p, a)
        assert (sim.debug(S.DBG_KEYS) == sk).all()
        assert rel_rho(a["rho"], rho) <= RHO_TOL
        assert rel_acc(a["fx"], a["fy"], fx, fy) <= ACC_TOL
        # integration of the next state with the GPU's own forces
        nx_, ny_ = sim.debug(S.DBG_POS_NEXT)
        nvx, nvy = sim.debug(S.DBG_VEL_NEXT)
        ox, oy, ovx, ovy = O.integrate(p, a["x"], a["y"], a["vx"], a["vy"], a["fx"], a["fy"])
        for got, ref in ((nx_, ox), (ny_, oy)):
            assert np.all(np.abs(got - ref) <= 4 * np.spacing(np.abs(ref).astype(np.float32)) + 1e-12)
        for got, ref in ((nvx, ovx), (nvy, ovy)):
            assert np.all(np.abs(got - ref) <= 4 * np.spacing(np.abs(ref).astype(np.float32)) + 1e-9)
        # keys of the integrated state, computed from the same FP32 positions
        assert (sim.debug(S.DBG_UNSORTED_KEYS) == O.cell_ids(p, nx_, ny_)).all()
        sim.step(1)
        perm = sim.debug(S.DBG_PERM)
        assert (perm == O.sort_perm(O.cell_ids(p, nx_, ny_))).all()
        b = sim.download(forces=False)
        assert (b["x"] == nx_[perm]).all() and (b["y"] == ny_[perm]).all()
    sim.close()


def test_neighbor_lists_exact():
    S = _sphg()
    dx = 0.005
    x, y, vx, vy = jittered(80, 160, dx, seed=4)
    for order in ("morton", "rowmajor"):
        kw = dict(order=order, h=1.3 * dx, dt=1e-5, lo=(0, 0), hi=(1, 1))
        p = O.params(**kw)
        sim = S.Sim(S.params(**kw), len(x))
        sim.upload(x, y, vx, vy)
        sim.preloop()
        a = sim.download(forces=False)
        sk = O.cell_ids(p, a["x"], a["y"])
        s, e = O.cell_ranges(p, sk)
        offs, idx = O.neighbor_lists(p, a["x"], a["y"], sk, s, e)
        goffs, gidx = sim.neighbor_lists()
        assert (goffs == offs).all() and (gidx == idx).all()
        sim.close()


def test_lists_golden(golden):
    """CSR lists of the reference's MultipassNeighborLists on its own sorted state."""
    S = _sphg()
    g = golden("lists")
    kw = dict(order="morton", h=float(g["h"]), dt=1e-5, lo=(0, 0), hi=(1, 1))
    sim = S.Sim(S.params(**kw), len(g["x"]))
    # the fixture state is already sorted by cell: the stable sort keeps its order
    sim.upload(g["x"], g["y"], g["vx"], g["vy"])
    sim.preloop()
    assert (sim.debug(S.DBG_PERM) == np.arange(len(g["x"]))).all()
    offs, idx = sim.neighbor_lists()
    assert (offs == g["mpl_offs"]).all() and (idx == g["mpl_idx"]).all()
    sim.close()


def test_diagnostics_vs_oracle():
    S = _sphg()
    dx = 0.005
    x, y, vx, vy = jittered(40, 80, dx, seed=6, vel=1.0)
    kw = dict(order="morton", h=1.3 * dx, dt=1e-5, lo=(0, 0), hi=(1, 1))
    sim = S.Sim(S.params(**kw), len(x))
    sim.upload(x, y, vx, vy)
    sim.preloop()
    a = sim.download(forces=False)
    d = sim.diagnostics()[0]
    ref = O.diagnostics(O.params(**kw), a["x"], a["y"], a["vx"], a["vy"])
    np.testing.assert_allclose(d[:2], ref[:2], rtol=1e-12)
    assert d[2] == ref[2] == len(x)
    np.testing.assert_allclose(d[3:5], ref[3:5], rtol=1e-9, atol=1e-9)
    assert d[5] == 0
    sim.close()


def test_empty_and_single_particle():
    S = _sphg()
    kw = dict(order="morton", h=0.1, dt=1e-3, lo=(0, 0), hi=(1, 1))
    sim = S.Sim(S.params(**kw), 0)
    sim.upload([], [], [], [])
    sim.preloop()
    sim.step(3)
    sim.close()
    sim = S.Sim(S.params(**kw), 1)
    sim.upload([0.5], [0.5], [0.0], [0.0])
    sim.preloop()
    out = sim.download()
    p = O.params(**kw)
    assert abs(out["fy"][0] - (-10.0)) < 1e-6  # gravity only
    wd = 315.0 / (64 * np.pi * 0.1 ** 3)
    assert abs(out["rho"][0] - wd) / wd < 1e-6  # self term only
    sim.step(10)
    out = sim.download()
    oy, ovy = 0.5, 0.0
    for _ in range(10):  # ten main-loop iterations, each one integration
        ovy += p.dt * -10.0
        oy += p.dt * ovy
    assert abs(out["y"][0] - oy) < 1e-6 and abs(out["vy"][0] - ovy) < 1e-6
    sim.close()


def test_invalid_arguments_fail_loudly():
    S = _sphg()
    with pytest.raises(S.SphgError):
        S.Sim(S.params(h=-1.0), 10)
    with pytest.raises(S.SphgError):
        S.Sim(S.params(hi=(0.0, 1.0), lo=(0.0, 0.0)), 10)
    sim = S.Sim(S.params(h=0.1, lo=(0, 0), hi=(1, 1)), 2)
    with pytest.raises(S.SphgError):
        sim.step(1)  # before the pre-loop
    with pytest.raises(S.SphgError) as ei:
        sim.upload([0.1, np.nan], [0.1, 0.2], [0, 0], [0, 0])
    assert ei.value.status == S.NONFINITE
    sim.close()


# ---------------------------------------------------------------- split-precision positions
@pytest.mark.parametrize("order", ["morton", "rowmajor"])
def test_split_precision_step_chain(order):
    """Integer cell + FP32 offset positions with compensated sums: density and
    forces against the oracle on the reconstructed positions, keys exact."""
    S = _sphg()
    dx = 0.005
    x, y, vx, vy = jittered(80, 160, dx, seed=7, vel=0.5)
    kw = dict(order=order, h=1.3 * dx, dt=1e-5, lo=(0, 0), hi=(1, 1))
    p = O.params(**kw)
    sim = S.Sim(S.params(**kw), len(x), S.options(precision=S.SPLIT))
    sim.upload(x, y, vx, vy)
    sim.preloop()
    for it in range(4):
        a = sim.download()
        # reconstructed positions within float rounding of the uploaded ones at step 0
        if it == 0:
            ix = np.argsort(a["ids"])
            assert np.max(np.abs(a["x"][ix] - x)) < 1e-9 and np.max(np.abs(a["y"][ix] - y)) < 1e-9
        sk, s, e, rho, fx, fy = oracle_state(p, a)
        assert (sim.debug(S.DBG_KEYS) == sk).all()
        assert rel_rho(a["rho"], rho) <= RHO_TOL
        assert rel_acc(a["fx"], a["fy"], fx, fy) <= ACC_TOL
        nx_, ny_ = sim.debug(S.DBG_POS_NEXT)
        ox, oy, ovx, ovy = O.integrate(p, a["x"], a["y"], a["vx"], a["vy"], a["fx"], a["fy"])
        assert np.max(np.abs(nx_ - ox)) < 1e-9 and np.max(np.abs(ny_ - oy)) < 1e-9
        sim.step(1)
    sim.close()


def test_split_and_plain_agree_over_many_steps():
    """Both position representations follow the same trajectory (FP32 noise only)."""
    S = _sphg()
    dx = 0.005
    x, y, vx, vy = jittered(40, 80, dx, seed=8)
    kw = dict(order="morton", h=1.3 * dx, dt=1e-5, k=30.0, rho0=1000.0, gy=-9.81,
              mass=1.0e-4, alpha=0.1, lo=(0, 0), hi=(1, 1))
    out = []
    for prec in (S.PLAIN, S.SPLIT):
        sim = S.Sim(S.params(**kw), len(x), S.options(precision=prec))
        sim.upload(x, y, vx, vy)
        sim.preloop()
        sim.step(200)
        a = sim.download(forces=False)
        ix = np.argsort(a["ids"])
        out.append((a["x"][ix], a["y"][ix], sim.diagnostics()[0]))
        sim.close()
    # 200 steps of FP32 rounding in different position representations: << dx = 5e-3
    assert np.max(np.abs(out[0][0] - out[1][0])) < 1e-5
    assert np.max(np.abs(out[0][1] - out[1][1])) < 1e-5
    assert out[1][2][2] == len(x) and out[1][2][5] == 0


# ---------------------------------------------------------------- cell-tile kernels
@pytest.mark.parametrize("prec", ["plain", "split"])
@pytest.mark.parametrize("tb", [3, 4, 5])
def test_tiled_kernels_match_oracle_and_untiled(prec, tb):
    S = _sphg()
    dx = 0.005
    x, y, vx, vy = jittered(80, 160, dx, seed=9, vel=0.3)
    kw = dict(order="morton", h=1.3 * dx, dt=1e-5, k=30.0, rho0=1000.0, gy=-9.81,
              mass=1.3e-4, alpha=0.1, lo=(0, 0), hi=(1, 1))
    p = O.params(**kw)
    P = S.SPLIT if prec == "split" else S.PLAIN
    res = {}
    for t in (tb, -1):
        sim = S.Sim(S.params(**kw), len(x), S.options(precision=P, tile_bits=t))
        sim.upload(x, y, vx, vy)
        sim.preloop()
        sim.step(3)
        a = sim.download()
        nxt = sim.debug(S.DBG_POS_NEXT)
        res[t] = (a, nxt, sim.debug(S.DBG_UNSORTED_KEYS))
        sk, s, e, rho, fx, fy = oracle_state(p, a)
        assert rel_rho(a["rho"], rho) <= RHO_TOL
        assert rel_acc(a["fx"], a["fy"], fx, fy) <= ACC_TOL
        sim.close()
    a, b = res[tb][0], res[-1][0]
    assert (a["ids"] == b["ids"]).all()
    # both within ACC_TOL of the oracle, in different summation orders: velocities
    # agree to 3 steps x dt x 2 ACC_TOL x max|a|
    amax = max(np.abs(b["fx"]).max(), np.abs(b["fy"]).max())
    for k in ("x", "y", "vx", "vy"):
        np.testing.assert_allclose(a[k], b[k], rtol=1e-6, atol=max(1e-9, 3 * 1e-5 * 2 * ACC_TOL * amax * 2))
    np.testing.assert_allclose(a["rho"], b["rho"], rtol=1e-6)


def test_tile_overflow_falls_back_to_global_walk():
    """A clump far denser than the shared-memory staging capacity."""
    S = _sphg()
    rng = np.random.default_rng(12)
    h = 0.01
    n = 3000
    x = (0.5 + rng.uniform(-1.5 * h, 1.5 * h, n)).astype(np.float32).astype(np.float64)
    y = (0.5 + rng.uniform(-1.5 * h, 1.5 * h, n)).astype(np.float32).astype(np.float64)
    z = np.zeros(n)
    kw = dict(order="morton", h=h, dt=1e-6, lo=(0, 0), hi=(1, 1))
    p = O.params(**kw)
    sim = S.Sim(S.params(**kw), n, S.options(tile_bits=3))
    sim.upload(x, y, z, z)
    sim.preloop()
    a = sim.download()
    sk, s, e, rho, fx, fy = oracle_state(p, a)
    assert rel_rho(a["rho"], rho) <= RHO_TOL
    assert rel_acc(a["fx"], a["fy"], fx, fy) <= ACC_TOL
    sim.close()


# ---------------------------------------------------------------- batches of instances
def _instances(seed=5):
    import workloads as W
    rng = np.random.default_rng(seed)
    out = []
    for npart, aspect, alpha, order in ((900, 0.5, 0.1, "morton"), (2500, 1.7, 0.05, "morton"),
                                        (400, 1.0, 0.2, "rowmajor"), (3000, 0.3, 0.15, "morton")):
        prm, x, y = W.dam_break_sized(npart, aspect, 0.005, rng, alpha, order=order)
        x = x.astype(np.float32).astype(np.float64)
        y = y.astype(np.float32).astype(np.float64)
        vx = rng.uniform(-0.2, 0.2, len(x)).astype(np.float32).astype(np.float64)
        vy = rng.uniform(-0.2, 0.2, len(x)).astype(np.float32).astype(np.float64)
        out.append((prm, x, y, vx, vy))
    return out


@pytest.mark.parametrize("prec", ["plain", "split"])
def test_batch_equals_each_instance_alone(prec):
    """Instances stepped together in one handle give each instance's result
    alone (every per-particle computation is instance-local)."""
    S = _sphg()
    P = S.SPLIT if prec == "split" else S.PLAIN
    inst = _instances()
    prms = [S.params(**i[0]) for i in inst]
    counts = [len(i[1]) for i in inst]
    cat = [np.concatenate([i[k] for i in inst]) for k in (1, 2, 3, 4)]
    b = S.Sim(prms, counts, S.options(precision=P))
    b.upload(*cat)
    b.preloop()
    b.step(30)
    bo = b.download()
    bd = b.diagnostics()
    off = np.concatenate([[0], np.cumsum(counts)])
    for k, (prm, x, y, vx, vy) in enumerate(inst):
        s = S.Sim(S.params(**prm), len(x), S.options(precision=P))
        s.upload(x, y, vx, vy)
        s.preloop()
        s.step(30)
        so = s.download()
        sl = slice(off[k], off[k + 1])
        assert (bo["ids"][sl] - off[k] == so["ids"]).all()
        for f in ("x", "y", "vx", "vy", "rho", "fx", "fy"):
            np.testing.assert_allclose(bo[f][sl], so[f], rtol=1e-6, atol=1e-7 * np.abs(so[f]).max())
        np.testing.assert_allclose(bd[k], s.diagnostics()[0], rtol=1e-6)
        s.close()
    b.close()


def test_batch_order_independent_bitwise():
    """An instance gives bit-identical results whatever other instances share its batch."""
    S = _sphg()
    inst = _instances()
    def run(sel):
        prms = [S.params(**inst[i][0]) for i in sel]
        counts = [len(inst[i][1]) for i in sel]
        cat = [np.concatenate([inst[i][k] for i in sel]) for k in (1, 2, 3, 4)]
        b = S.Sim(prms, counts)
        b.upload(*cat)
        b.preloop()
        b.step(25)
        o = b.download()
        off = np.concatenate([[0], np.cumsum(counts)])
        res = {i: {f: o[f][off[q]:off[q + 1]] for f in ("x", "y", "vx", "vy", "rho")}
               for q, i in enumerate(sel)}
        b.close()
        return res
    a = run([0, 1, 2, 3])
    c = run([3, 1, 0])
    for i in (0, 1, 3):
        for f in ("x", "y", "vx", "vy", "rho"):
            assert (a[i][f] == c[i][f]).all(), (i, f)


# ---------------------------------------------------------------- periodic boundaries
@pytest.mark.parametrize("prec", ["plain", "split"])
@pytest.mark.parametrize("order", ["morton", "rowmajor"])
def test_periodic_taylor_green_vs_oracle(prec, order):
    S = _sphg()
    import workloads as W
    prm, x, y, vx, vy, rate = W.taylor_green(48, seed=2, order=order)
    f32 = lambda a: np.asarray(a).astype(np.float32).astype(np.float64)  # noqa: E731
    x, y, vx, vy = f32(x), f32(y), f32(vx), f32(vy)
    p = O.params(**prm)
    P = S.SPLIT if prec == "split" else S.PLAIN
    sim = S.Sim(S.params(**prm), len(x), S.options(precision=P))
    sim.upload(x, y, vx, vy)
    sim.preloop()
    for it in range(3):
        a = sim.download()
        sk, s, e, rho, fx, fy = oracle_state(p, a)
        assert (sim.debug(S.DBG_KEYS) == sk).all()
        assert rel_rho(a["rho"], rho) <= RHO_TOL
        assert rel_acc(a["fx"], a["fy"], fx, fy) <= ACC_TOL
        offs, idx = O.neighbor_lists(p, a["x"], a["y"], sk, s, e)
        goffs, gidx = sim.neighbor_lists()
        assert (goffs == offs).all() and (gidx == idx).all()
        sim.step(7)
    # kinetic energy after the first 500 steps follows exp(-16 pi^2 nu t) closely
    e0 = 0.5 * prm["mass"] * np.sum(vx ** 2 + vy ** 2)
    sim.step(500 - 21)
    d = sim.diagnostics()[0]
    t = 500 * prm["dt"]
    assert abs(d[0] / e0 - np.exp(-rate * t)) < 0.01
    assert d[2] == len(x) and d[5] == 0
    sim.close()


@pytest.mark.parametrize("order", ["morton", "rowmajor"])
@pytest.mark.parametrize("side,h", [(1.0, 0.05), (0.25, 0.08)])
def test_periodic_minimum_image_at_the_wrap(order, side, h):
    """Plain positions in a periodic box that starts at 0 and whose side is
    exact in FP32: pairs reached through the boundary form their minimum image
    in FP32 (FP64 only near the cut-off, for operands near 0 below 2^-28 of
    the side, or near a separation of half the side).  Particles placed on
    both faces, a few ulp from them, at tiny offsets and (in the 3-cell box)
    near half-side separations: neighbour lists equal the oracle's, densities
    and forces within the tolerances."""
    S = _sphg()
    rng = np.random.default_rng(7)
    f32 = lambda a: np.asarray(a, np.float64).astype(np.float32).astype(np.float64)  # noqa: E731
    L = side
    one_ulp = float(np.spacing(np.float32(L)))
    edge = [0.0, 2.0 ** -40, 2.0 ** -30, 2.0 ** -27 * L, 3 * 2.0 ** -24, 1e-4 * L,
            L - one_ulp, L - 3 * one_ulp, L - 1e-4 * L, L - h, h, 0.5 * L, 0.5 * L - one_ulp]
    pts = set()
    for ex in edge:
        for ey in edge:
            pts.add((ex, ey))
        for _ in range(3):
            pts.add((ex, float(rng.uniform(0, L))))
            pts.add((float(rng.uniform(0, L)), ex))
    x = np.array([p[0] for p in pts])
    y = np.array([p[1] for p in pts])
    x = np.concatenate([x, rng.uniform(0, L, 400)])
    y = np.concatenate([y, rng.uniform(0, L, 400)])
    x, y = f32(np.mod(x, L)), f32(np.mod(y, L))
    keep = (x < L) & (y < L)
    x, y = x[keep], y[keep]
    vx, vy = f32(rng.normal(0, 0.1, len(x))), f32(rng.normal(0, 0.1, len(x)))
    prm = dict(order=order, h=h, dt=1e-5, k=30.0, rho0=1000.0, mu=0.01, gx=0.0, gy=0.0,
               mass=2e-3 * side * side, alpha=0.0, c0=5.0, lo=(0.0, 0.0), hi=(L, L), periodic=1)
    p = O.params(**prm)
    sim = S.Sim(S.params(**prm), len(x), S.options(precision=S.PLAIN))
    sim.upload(x, y, vx, vy)
    sim.preloop()
    a = sim.download()
    sk, s_, e_, rho, fx, fy = oracle_state(p, a)
    assert (sim.debug(S.DBG_KEYS) == sk).all()
    offs, idx = O.neighbor_lists(p, a["x"], a["y"], sk, s_, e_)
    goffs, gidx = sim.neighbor_lists()
    assert (goffs == offs).all() and (gidx == idx).all()
    assert rel_rho(a["rho"], rho) <= RHO_TOL
    assert rel_acc(a["fx"], a["fy"], fx, fy) <= ACC_TOL
    sim.close()


@pytest.mark.parametrize("prec", ["plain", "split"])
def test_snapshot_resume_is_exact(prec):
    """sphg_snapshot -> sphg_restore on a fresh handle -> sphg_preloop continues
    bit for bit: the resumed state and every later step equal the original run."""
    S = _sphg()
    P = S.SPLIT if prec == "split" else S.PLAIN
    inst = _instances(seed=11)
    prms = [S.params(**i[0]) for i in inst]
    counts = [len(i[1]) for i in inst]
    cat = [np.concatenate([i[k] for i in inst]) for k in (1, 2, 3, 4)]
    a = S.Sim(prms, counts, S.options(precision=P))
    a.upload(*cat)
    a.preloop()
    a.step(20)
    at_snap = a.download()
    blob = a.snapshot()
    a.step(15)
    later = a.download()
    b = S.Sim(prms, counts, S.options(precision=P))
    b.restore(blob)
    b.preloop()
    resumed = b.download()
    for f in ("x", "y", "vx", "vy", "rho", "fx", "fy", "ids"):
        assert (resumed[f] == at_snap[f]).all(), f
    b.step(15)
    cont = b.download()
    for f in ("x", "y", "vx", "vy", "rho", "fx", "fy", "ids"):
        assert (cont[f] == later[f]).all(), f
    # a snapshot of another shape is refused
    c = S.Sim(prms[:2], counts[:2], S.options(precision=P))
    with pytest.raises(S.SphgError):
        c.restore(blob)
    for h in (a, b, c):
        h.close()


# ---------------------------------------------------------------- lists compute mode + delta codec
def test_lists_mode_matches_reference_lists_golden(golden):
    """compute=lists on the fixture's sorted state: the reference's
    MPListsForceComputation density and forces (FP64) within the FP32 tolerances."""
    S = _sphg()
    g = golden("lists")
    n = len(g["x"])
    prm = S.params(order="morton", h=float(g["h"]), dt=1e-5, lo=(0, 0), hi=(1, 1))
    sim = S.Sim(prm, n, S.options(compute="lists"))
    sim.upload(g["x"], g["y"], g["vx"], g["vy"])
    sim.preloop()
    out = sim.download()
    ids = out["ids"]
    assert rel_rho(out["rho"], g["mpl_rho"][ids]) <= RHO_TOL
    assert rel_acc(out["fx"], out["fy"], g["mpl_fx"][ids], g["mpl_fy"][ids]) <= ACC_TOL
    offs, idx = sim.neighbor_lists()
    assert (offs == g["mpl_offs"]).all() and (idx == g["mpl_idx"]).all()
    sim.close()


@pytest.mark.parametrize("prec", ["plain", "split"])
@pytest.mark.parametrize("order", ["morton", "rowmajor"])
def test_lists_mode_steps_match_oracle_and_sorted_mode(prec, order):
    S = _sphg()
    P = S.SPLIT if prec == "split" else S.PLAIN
    x, y, vx, vy = jittered(48, 40, 0.005, seed=21, vel=0.3)
    kw = dict(order=order, h=0.0065, dt=1e-5, lo=(0, 0), hi=(0.4, 0.3))
    prm = S.params(**kw)
    p = O.params(**kw)
    lists = S.Sim(prm, len(x), S.options(precision=P, compute="lists"))
    srt = S.Sim(prm, len(x), S.options(precision=P))
    for s in (lists, srt):
        s.upload(x, y, vx, vy)
        s.preloop()
    for k in (0, 7):
        if k:
            lists.step(k)
            srt.step(k)
        a = lists.download()
        b = srt.download()
        _, _, _, rho, fx, fy = oracle_state(p, a)
        assert rel_rho(a["rho"], rho) <= RHO_TOL
        assert rel_acc(a["fx"], a["fy"], fx, fy) <= ACC_TOL
        oa, ob = np.argsort(a["ids"]), np.argsort(b["ids"])  # slot orders may differ at cell edges
        for f in ("x", "y", "vx", "vy", "rho"):
            np.testing.assert_allclose(a[f][oa], b[f][ob], rtol=1e-5, atol=1e-6 * np.abs(b[f]).max())
    assert lists.launches_per_step() == srt.launches_per_step() + 5
    lists.close()
    srt.close()


def test_lists_mode_graph_equals_stream_launches():
    """Lists mode replays a CUDA graph per iteration (the list buffer is sized at
    the pre-loop, no per-iteration host synchronisation): the same bits as the
    stream-launched iterations."""
    S = _sphg()
    x, y, vx, vy = jittered(48, 40, 0.005, seed=22, vel=0.3)
    kw = dict(order="morton", h=0.0065, dt=1e-5, lo=(0, 0), hi=(0.4, 0.3))
    out = []
    for graph in (1, 0):
        sim = S.Sim(S.params(**kw), len(x), S.options(precision=S.SPLIT, compute="lists", use_graph=graph))
        sim.upload(x, y, vx, vy)
        sim.preloop()
        sim.step(12)
        out.append(sim.download())
        sim.close()
    for f in ("x", "y", "vx", "vy", "rho", "fx", "fy", "ids"):
        assert (out[0][f] == out[1][f]).all(), f


def test_lists_mode_reports_lists_outgrowing_their_buffer():
    """A collapsing cloud: isolated particles (the pre-loop's lists hold only
    each particle itself) driven together until every particle has four
    neighbours -- more than the buffer sized at the pre-loop (twice that
    total): the overflow is reported as SPHG_CAPACITY, nothing is written past
    the buffer."""
    S = _sphg()
    h = 0.005
    g = (np.arange(64) - 31.5) * 2 * h + 0.5
    x, y = [a.ravel().astype(np.float32).astype(np.float64) for a in np.meshgrid(g, g, indexing="xy")]
    vx, vy = -300.0 * (x - 0.5), -300.0 * (y - 0.5)
    kw = dict(order="morton", h=h, dt=1e-4, lo=(0, 0), hi=(1, 1), gy=0.0)
    sim = S.Sim(S.params(**kw), len(x), S.options(compute="lists"))
    sim.upload(x, y, vx, vy)
    sim.preloop()
    sim.step(35)
    with pytest.raises(S.SphgError) as e:
        sim.download()
    assert e.value.status == S.CAPACITY
    sim.close()


@pytest.mark.parametrize("opt", [dict(cell_pairs=1), dict(block_threads=64), dict(block_threads=256),
                                 dict(cell_pairs=1, block_threads=64), dict(fused=1), dict(fused=1, use_graph=0)])
def test_launch_shapes_give_identical_results(opt):
    """The autotuner's launch shapes (threads per block, two particles of a cell
    per density thread) visit the same pairs in the same order: the same bits."""
    S = _sphg()
    inst = _instances()
    prms = [S.params(**i[0]) for i in inst]
    counts = [len(i[1]) for i in inst]
    cat = [np.concatenate([i[k] for i in inst]) for k in (1, 2, 3, 4)]
    out = []
    for o in ({}, opt):
        o = dict(o)
        g = o.pop("use_graph", 1)
        b = S.Sim(prms, counts, S.options(precision=S.SPLIT, use_graph=g, **o))
        b.upload(*cat)
        b.preloop()
        b.step(20)
        out.append(b.download())
        b.close()
    for f in ("x", "y", "vx", "vy", "rho", "fx", "fy", "ids"):
        assert (out[0][f] == out[1][f]).all(), f


@pytest.mark.parametrize("graph", [1, 0])
@pytest.mark.parametrize("prec", ["plain", "split"])
def test_single_launch_iteration_equals_kernel_graph(prec, graph):
    """The iteration as one cooperative launch (merge, ranges, density, forces
    between grid-wide barriers) gives the bits of the four-kernel iteration --
    also on iterations where more than 8,192 particles change cell and the full
    radix sort runs between the launch's decision and its post part."""
    S = _sphg()
    P = S.SPLIT if prec == "split" else S.PLAIN
    # ballistic particles (no pressure, viscosity or gravity: the forces are exactly zero) fast enough that
    # about a third change cell every step
    x, y, vx, vy = jittered(240, 200, 0.004, seed=31, vel=80.0)
    kw = dict(order="morton", h=0.0052, dt=2e-5, lo=(0, 0), hi=(1.2, 1.0), k=0.0, mu=0.0, gx=0.0, gy=0.0, alpha=0.0)
    out, resort = [], []
    for fused in (0, 1):
        sim = S.Sim(S.params(**kw), len(x), S.options(precision=P, fused=fused, use_graph=graph))
        sim.upload(x, y, vx, vy)
        sim.preloop()
        merged = []
        for _ in range(12):
            sim.step(1)
            merged.append(int(sim.debug(S.DBG_RESORT)[0]))
        out.append(sim.download())
        resort.append(merged)
        sim.close()
    assert resort[0] == resort[1]
    assert 0 in resort[1], "the case must exercise the full sort"
    for f in ("x", "y", "vx", "vy", "rho", "fx", "fy", "ids"):
        assert (out[0][f] == out[1][f]).all(), f


def test_lists_mode_periodic_and_batched():
    """Lists mode over a batch holding a periodic Taylor-Green box and a walled box."""
    import workloads as W
    S = _sphg()
    prm1, x1, y1, vx1, vy1, _ = W.taylor_green(24, seed=3)
    rng = np.random.default_rng(4)
    prm2, x2, y2 = W.dam_break_sized(700, 1.0, 0.005, rng, alpha=0.1)
    prms = [S.params(**prm1), S.params(**prm2)]
    counts = [len(x1), len(x2)]
    cat = [np.concatenate(v) for v in ((x1, x2), (y1, y2), (vx1, np.zeros(len(x2))), (vy1, np.zeros(len(x2))))]
    outs = []
    for mode in ("lists", "sorted"):
        sim = S.Sim(prms, counts, S.options(precision=S.SPLIT, compute=mode))
        sim.upload(*cat)
        sim.preloop()
        sim.step(10)
        outs.append(sim.download())
        sim.close()
    oa, ob = np.argsort(outs[0]["ids"]), np.argsort(outs[1]["ids"])
    for f in ("x", "y", "vx", "vy", "rho"):
        np.testing.assert_allclose(outs[0][f][oa], outs[1][f][ob], rtol=1e-5,
                                   atol=1e-6 * np.abs(outs[1][f]).max())
    # accelerations: the two summation orders differ by rounding, which the
    # pressure k (rho - rho0) amplifies by rho / (rho - rho0)
    assert rel_acc(outs[0]["fx"][oa], outs[0]["fy"][oa], outs[1]["fx"][ob], outs[1]["fy"][ob]) <= 1e-4


def test_encoded_lists_round_trip(golden):
    """GPU delta codec: encoded lists equal Codifier::Encode of the ascending lists,
    the device decoder inverts the device encoder, and the reference's own
    encoder output (fixture) is reproduced."""
    import torch
    S = _sphg()
    x, y, vx, vy = jittered(30, 30, 0.005, seed=8)
    prm = S.params(order="morton", h=0.0065, dt=1e-5, lo=(0, 0), hi=(0.2, 0.2))
    sim = S.Sim(prm, len(x))
    sim.upload(x, y, vx, vy)
    sim.preloop()
    offs, idx = sim.neighbor_lists()
    eoffs, enc = sim.neighbor_lists_encoded()
    assert (eoffs == offs).all()
    asc = idx.copy()
    for i in range(len(offs) - 1):
        asc[offs[i]:offs[i + 1]] = np.sort(idx[offs[i]:offs[i + 1]])
    assert (enc == O.delta_encode(offs, asc)).all()
    sim.close()
    dev = torch.device("cuda:0")
    for o_, a_, want in ((offs, asc, O.delta_encode(offs, asc)),
                         (golden("lists")["enc_offs"], golden("lists")["enc_in"], golden("lists")["enc_out"])):
        d_offs = torch.from_numpy(np.ascontiguousarray(o_, np.int64)).to(dev)
        d_in = torch.from_numpy(np.ascontiguousarray(a_, np.int32)).to(dev)
        d_enc = torch.empty_like(d_in)
        d_dec = torch.empty_like(d_in)
        n = len(o_) - 1
        S.delta_encode(d_offs.data_ptr(), d_in.data_ptr(), n, d_enc.data_ptr())
        S.delta_decode(d_offs.data_ptr(), d_enc.data_ptr(), n, d_dec.data_ptr())
        torch.cuda.synchronize()
        assert (d_enc.cpu().numpy() == want).all()
        assert (d_dec.cpu().numpy() == a_).all()


# ---------------------------------------------------------------- incremental re-sort
@pytest.mark.parametrize("prec", ["plain", "split"])
@pytest.mark.parametrize("vel", [0.3, 400.0])
def test_incremental_resort_equals_full_sort_bitwise(prec, vel):
    """resort=1 merges the particles that changed cell into the rest; it must give
    the full radix sort's order and therefore the same bits.  vel=400 moves more
    than 8,192 particles in the first iterations, so the device falls back to the
    full sort there (and merges again once the particles pile up at the walls)."""
    S = _sphg()
    P = S.SPLIT if prec == "split" else S.PLAIN
    x, y, vx, vy = jittered(160, 120, 0.005, seed=31, vel=vel)
    prm = S.params(order="morton", h=0.0065, dt=1e-5, lo=(0, 0), hi=(0.8, 0.6))
    outs = []
    for resort in (1, 0):
        sim = S.Sim(prm, len(x), S.options(precision=P, resort=resort))
        sim.upload(x, y, vx, vy)
        sim.preloop()
        moved = []
        for _ in range(6):
            before = sim.debug(S.DBG_KEYS).copy()
            nxt = sim.debug(S.DBG_UNSORTED_KEYS)
            moved.append(int((before != nxt).sum()))
            sim.step(4)
        o = sim.download()
        o["keys"] = sim.debug(S.DBG_KEYS)
        o["perm"] = sim.debug(S.DBG_PERM)
        rs = sim.debug(S.DBG_RESORT)
        if resort and vel < 1:
            assert rs[0] == 1 and 0 <= rs[1] <= 8192
        if not resort:
            assert rs[0] == 0
        outs.append((o, moved))
        sim.close()
    (a, moved), (b, _) = outs
    if vel < 1:
        assert 0 < max(moved) <= 8192
    else:
        assert max(moved) > 8192  # at least one iteration took the full sort
    for f in ("x", "y", "vx", "vy", "rho", "fx", "fy", "ids", "keys", "perm"):
        assert np.array_equal(a[f], b[f], equal_nan=True), f


# ---------------------------------------------------------------- autotuner, adaptive dt
def test_autotune_returns_a_working_configuration():
    S = _sphg()
    inst = _instances(seed=13)
    prms = [S.params(**i[0]) for i in inst]
    counts = [len(i[1]) for i in inst]
    cat = [np.concatenate([i[k] for i in inst]) for k in (1, 2, 3, 4)]
    best, ms = S.autotune(prms, counts, *cat, base=S.options(precision=S.SPLIT), steps=5)
    assert ms > 0 and best.precision == S.SPLIT
    assert best.tile_bits == -1  # one instance is row-major: no cell tiles
    again, ms2 = S.autotune(prms, counts, *cat, base=S.options(precision=S.SPLIT), steps=5)
    assert ms2 == ms and again.resort == best.resort  # remembered
    morton = [i for i in inst if i[0]["order"] == "morton"]
    best_m, _ = S.autotune([S.params(**i[0]) for i in morton], [len(i[1]) for i in morton],
                           *[np.concatenate([i[k] for i in morton]) for k in (1, 2, 3, 4)], steps=5)
    assert best_m.tile_bits in (-1, 3, 4, 5)
    a = S.Sim(prms, counts, best)
    b = S.Sim(prms, counts, S.options(precision=S.SPLIT))
    for s in (a, b):
        s.upload(*cat)
        s.preloop()
        s.step(10)
    oa, ob = a.download(), b.download()
    ia, ib = np.argsort(oa["ids"]), np.argsort(ob["ids"])
    np.testing.assert_allclose(oa["x"][ia], ob["x"][ib], rtol=0, atol=1e-9)
    a.close()
    b.close()


def test_cfl_dt_and_set_dt():
    S = _sphg()
    x, y, vx, vy = jittered(60, 50, 0.005, seed=17, vel=0.4)
    kw = dict(order="morton", h=0.0065, dt=1e-5, lo=(0, 0), hi=(0.4, 0.3), c0=5.0)
    sim = S.Sim(S.params(**kw), len(x), S.options(precision=S.SPLIT))  # positions to ~1e-10
    sim.upload(x, y, vx, vy)
    sim.preloop()
    sim.step(3)
    o = sim.download()
    dt = sim.cfl_dt(cfl=0.3, force_coef=0.2)
    vmax = np.sqrt((o["vx"] ** 2 + o["vy"] ** 2).max())
    amax = np.sqrt((o["fx"] ** 2 + o["fy"] ** 2).max())
    want = min(0.3 * 0.0065 / (5.0 + vmax), 0.2 * np.sqrt(0.0065 / amax))
    np.testing.assert_allclose(dt[0], want, rtol=1e-6)
    # a new dt applies from the next iteration on (graph rebuilt)
    sim.set_dt(2.5e-5)
    sim.step(1)
    a = sim.download()
    nx_, ny_ = sim.debug(S.DBG_POS_NEXT)
    p = O.params(**dict(kw, dt=2.5e-5))
    ox, oy, _, _ = O.integrate(p, a["x"], a["y"], a["vx"], a["vy"], a["fx"], a["fy"])
    assert np.max(np.abs(nx_ - ox)) < 1e-9 and np.max(np.abs(ny_ - oy)) < 1e-9
    sim.close()


# ---------------------------------------------------------------- device initial states
def _splitmix_uniform(seed, counters):
    z = (np.uint64(seed) + (counters.astype(np.uint64) + np.uint64(1)) * np.uint64(0x9E3779B97F4A7C15))
    z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
    z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
    z = z ^ (z >> np.uint64(31))
    return (z >> np.uint64(11)).astype(np.float64) * 2.0 ** -52 - 1.0


def _lattice_host(x0, y0, dx, dy, nx, ny, jitter, seed):
    p = np.arange(nx * ny, dtype=np.int64)
    gi, gj = p % nx, p // nx
    ox = jitter * _splitmix_uniform(seed, 2 * p) if jitter else 0.0
    oy = jitter * _splitmix_uniform(seed, 2 * p + 1) if jitter else 0.0
    return x0 + (gi + ox) * dx, y0 + (gj + oy) * dy


@pytest.mark.parametrize("prec", ["plain", "split"])
def test_device_lattice_equals_host_lattice(prec):
    S = _sphg()
    P = S.SPLIT if prec == "split" else S.PLAIN
    # the reference's own lattice (LatticeCreator, no jitter) of config/example.txt
    x0, y0 = O.lattice(96, 48, 0.5, 0.5, 0.4, 0.8)
    kw = dict(order="rowmajor", h=1.0, dt=0.005, lo=(0, 0), hi=(96, 48))
    a = S.Sim(S.params(**kw), len(x0), S.options(precision=P))
    a.upload_lattice(S.lattice(0.0, 0.0, 0.5, 0.5, 78, 78))
    b = S.Sim(S.params(**kw), len(x0), S.options(precision=P))
    b.upload(x0, y0, np.zeros(len(x0)), np.zeros(len(x0)))
    for s in (a, b):
        s.preloop()
        s.step(3)
    oa, ob = a.download(), b.download()
    for f in ("x", "y", "vx", "vy", "rho", "ids"):
        assert (oa[f] == ob[f]).all(), f
    # jittered lattice in a batch, against the same generator restated on the host
    specs = [S.lattice(0.0025, 0.0025, 0.005, 0.005, 40, 30, jitter=0.01, seed=7),
             S.lattice(0.01, 0.02, 0.004, 0.004, 25, 50, jitter=0.02, seed=2 ** 63 + 5)]
    prms = [S.params(order="morton", h=0.0065, dt=1e-5, lo=(0, 0), hi=(0.4, 0.3)),
            S.params(order="morton", h=0.0052, dt=1e-5, lo=(0, 0), hi=(0.2, 0.3))]
    counts = [1200, 1250]
    hx, hy = zip(*[_lattice_host(L.x0, L.y0, L.dx, L.dy, L.nx, L.ny, L.jitter, L.seed) for L in specs])
    hx, hy = np.concatenate(hx), np.concatenate(hy)
    c = S.Sim(prms, counts, S.options(precision=P))
    c.upload_lattice(specs)
    c.preloop()
    oc = c.download()
    ix = oc["ids"]
    if prec == "plain":
        assert (oc["x"] == hx.astype(np.float32)[ix]).all() and (oc["y"] == hy.astype(np.float32)[ix]).all()
    else:
        assert np.max(np.abs(oc["x"] - hx[ix])) < 1e-9 and np.max(np.abs(oc["y"] - hy[ix])) < 1e-9
    for s in (a, b, c):
        s.close()


def test_device_taylor_green_lattice():
    import workloads as W
    S = _sphg()
    prm, x, y, vx, vy, _ = W.taylor_green(32, seed=3)
    n = 32
    sim = S.Sim(S.params(**prm), n * n)
    sim.upload_lattice(S.lattice(0.5 / n, 0.5 / n, 1.0 / n, 1.0 / n, n, n, velocity=S.VEL_TAYLOR_GREEN, u0=1.0))
    sim.preloop()
    o = sim.download()
    np.testing.assert_allclose(o["vx"], np.sin(2 * np.pi * o["x"]) * np.cos(2 * np.pi * o["y"]), atol=1e-6)
    np.testing.assert_allclose(o["vy"], -np.cos(2 * np.pi * o["x"]) * np.sin(2 * np.pi * o["y"]), atol=1e-6)
    with pytest.raises(S.SphgError):
        sim.upload_lattice(S.lattice(0, 0, 0.1, 0.1, 10, 10))  # 100 != 1024 particles
    sim.close()


def test_diagnostics_async_equals_sync():
    import torch
    S = _sphg()
    x, y, vx, vy = jittered(40, 40, 0.005, seed=23, vel=0.3)
    sim = S.Sim(S.params(order="morton", h=0.0065, dt=1e-5, lo=(0, 0), hi=(0.3, 0.3)), len(x))
    sim.upload(x, y, vx, vy)
    sim.preloop()
    buf = torch.zeros((5, 6), dtype=torch.float64, pin_memory=True)
    sync = []
    for k in range(5):
        sim.step(2)
        sim.diagnostics_async(buf[k].data_ptr())
        torch.cuda.synchronize()
        sync.append(sim.diagnostics()[0])
    assert (buf.numpy() == np.array(sync)).all()
    sim.close()


@pytest.mark.parametrize("case", ["graph-pageable", "graph-pinned", "stream", "copies", "batched"])
def test_step_headers_equal_step_then_diagnostics(case):
    """sphg_step_headers = the reference's main loop with a header after every
    iteration: the same values as sphg_step(1) + sphg_diagnostics per iteration,
    whether the kernels write the caller's array (pageable or pinned) or the
    headers are copied (host access off), with and without the step graph."""
    import torch
    S = _sphg()
    x, y, vx, vy = jittered(40, 40, 0.005, seed=31, vel=0.3)
    kw = dict(order="morton", h=0.0065, dt=1e-5, lo=(0, 0), hi=(0.3, 0.3))
    opts = S.options(precision=S.SPLIT, use_graph=(case != "stream"))
    if case == "batched":
        x2, y2, vx2, vy2 = jittered(30, 20, 0.005, seed=37, vel=0.2)
        prm = [S.params(**kw), S.params(**kw)]
        counts = [len(x), len(x2)]
        x, y, vx, vy = (np.concatenate(p) for p in ((x, x2), (y, y2), (vx, vx2), (vy, vy2)))
        make = lambda: S.Sim(prm, counts, opts)  # noqa: E731
    else:
        make = lambda: S.Sim(S.params(**kw), len(x), opts)  # noqa: E731
    K = 12
    a, b = make(), make()
    for sim in (a, b):
        sim.upload(x, y, vx, vy)
        sim.preloop()
    if case == "copies":
        a.set_host_access(0)
    if case == "graph-pinned":
        buf = torch.zeros((K, a.ninst, 6), dtype=torch.float64, pin_memory=True)
        a.step_headers(K, buf.data_ptr())
        torch.cuda.synchronize()
        got = buf.numpy().copy()
    else:
        got = a.step_headers(K)
    ref = []
    for _ in range(K):
        b.step(1)
        ref.append(b.diagnostics())
    ref = np.array(ref)
    assert got.shape == ref.shape
    assert (got == ref).all()
    assert (ref[:, :, 2] == np.asarray(a.counts)[None, :]).all()  # every particle inside
    sa, sb = a.download(), b.download()
    for f in ("x", "y", "vx", "vy", "rho"):
        assert (sa[f] == sb[f]).all(), f
    # a second call continues from the state and restarts its own header index
    got2 = a.step_headers(3)
    b.step(3)
    assert (got2[-1] == b.diagnostics()).all()
    a.close()
    b.close()


@pytest.mark.parametrize("prec", ["plain", "split"])
def test_particles_outside_the_high_walls(prec):
    """Particles beyond the high walls at upload: their cells clamp to the last
    cell (GenericNeighborSearch::SetParticleCellIds clamps ci <= n - 1) and the
    first integration puts them on the walls with reflected velocity
    (Integrator::ApplyBoundaryConditions)."""
    S = _sphg()
    x, y, vx, vy = jittered(30, 30, 0.005, seed=29, vel=0.2)
    x[:5] = 0.3 + np.array([1e-4, 2e-3, 5e-3, 0.0, 3e-4])  # hi = 0.3
    y[5:10] = 0.3 + np.array([1e-4, 2e-3, 5e-3, 0.0, 3e-4])
    x = x.astype(np.float32).astype(np.float64)
    y = y.astype(np.float32).astype(np.float64)
    kw = dict(order="morton", h=0.0065, dt=1e-5, lo=(0, 0), hi=(0.3, 0.3))
    p = O.params(**kw)
    P = S.SPLIT if prec == "split" else S.PLAIN
    sim = S.Sim(S.params(**kw), len(x), S.options(precision=P))
    sim.upload(x, y, vx, vy)
    sim.preloop()
    a = sim.download()
    sk, s, e, rho, fx, fy = oracle_state(p, a)
    assert (sim.debug(S.DBG_KEYS) == sk).all()
    assert rel_rho(a["rho"], rho) <= RHO_TOL
    nx_, ny_ = sim.debug(S.DBG_POS_NEXT)
    ox, oy, _, _ = O.integrate(p, a["x"], a["y"], a["vx"], a["vy"], a["fx"], a["fy"])
    assert np.max(np.abs(nx_ - ox)) < 1e-7 and np.max(np.abs(ny_ - oy)) < 1e-7
    assert (nx_ <= 0.3 + 1e-7).all() and (ny_ <= 0.3 + 1e-7).all()  # on the walls, within FP32 rounding
    sim.close()


@pytest.mark.parametrize("prec", ["split", "plain"])
def test_direct_host_access_vector_and_scalar_paths(prec):
    """The device-side conversion of the caller's arrays reads and writes two
    particles a thread with 16-byte accesses when every array is 16-byte
    aligned, one a thread otherwise: both equal the pinned staging path bit for
    bit, for an odd particle count (the last particle alone), and report the
    first non-finite particle of a pair or of the odd tail."""
    S = _sphg()
    if not S.device_attributes(0)["pageable_access"]:
        pytest.skip("the device cannot access pageable host memory")
    import workloads as W
    P = S.SPLIT if prec == "split" else S.PLAIN
    prm, x, y, vx, vy = W.dam_break(13, 77, 0.01, seed=5)  # 1,001 particles
    n = len(x)
    assert n % 2 == 1
    vx = np.linspace(-0.2, 0.3, n)
    vy = np.linspace(0.1, -0.4, n)

    def views(offset):
        out = []
        for a in (x, y, vx, vy):
            buf = np.zeros(n + 2, np.float64)
            buf[offset:offset + n] = a
            out.append(buf[offset:offset + n])
        return out

    def out_views(offset):
        d = {}
        for k in ("x", "y", "vx", "vy", "rho", "fx", "fy"):
            d[k] = np.zeros(n + 2, np.float64)[offset:offset + n]
        d["ids"] = np.zeros(n + 2, np.int32)[offset:offset + n]
        return d

    results = []
    for mode, offset in ((0, 0), (2, 0), (2, 1), (1, 0), (1, 1)):
        arrs = views(offset)
        assert (arrs[0].ctypes.data % 16 == 0) == (offset == 0)
        sim = S.Sim(S.params(**prm), n, S.options(precision=P))
        sim.set_host_access(mode)
        sim.upload(*arrs)
        sim.preloop()
        sim.step(3)
        results.append(sim.download(out=out_views(offset)))
        for bad_at in (0, 5, n - 1):
            bad = [a.copy() for a in arrs] if offset == 0 else views(offset)
            bad[2][bad_at] = np.inf
            if bad_at == 0:
                bad[3][1] = np.nan  # both of the first pair: the first is reported
            with pytest.raises(S.SphgError) as ei:
                sim.upload(*bad)
            assert ei.value.status == S.NONFINITE and ("particle %d" % bad_at) in str(ei.value), (mode, offset, bad_at)
        sim.close()
    ref = results[0]
    for r in results[1:]:
        for f in ("x", "y", "vx", "vy", "rho", "fx", "fy", "ids"):
            assert np.array_equal(r[f], ref[f]), f


@pytest.mark.parametrize("prec", ["plain", "split"])
def test_direct_host_access_equals_staging(prec):
    """Upload/download converting the caller's arrays on the device (pageable host
    memory access) give the staging path's results."""
    S = _sphg()
    if not S.device_attributes(0)["pageable_access"]:
        pytest.skip("the device cannot access pageable host memory")
    P = S.SPLIT if prec == "split" else S.PLAIN
    inst = _instances(seed=41)
    prms = [S.params(**i[0]) for i in inst]
    counts = [len(i[1]) for i in inst]
    cat = [np.concatenate([i[k] for i in inst]) for k in (1, 2, 3, 4)]
    outs = []
    for direct in (2, 1, 0):
        sim = S.Sim(prms, counts, S.options(precision=P))
        sim.set_host_access(direct)
        sim.upload(*cat)
        sim.preloop()
        sim.step(7)
        outs.append(sim.download())
        bad = [c.copy() for c in cat]
        bad[1][17] = np.nan
        with pytest.raises(S.SphgError) as ei:
            sim.upload(*bad)
        assert ei.value.status == S.NONFINITE and "particle 17" in str(ei.value)
        sim.close()
    for a in outs[:2]:
        b = outs[2]
        for f in ("x", "y", "vx", "vy", "rho", "fx", "fy", "ids"):
            np.testing.assert_allclose(a[f], b[f], rtol=0, atol=1e-15 * max(1.0, np.abs(b[f]).max()))
