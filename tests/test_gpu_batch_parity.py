"""The batched kernels against the oracle at the sizes of the 256-instance
mixed-size batch (dam-break boxes of 2,000-65,536 particles, column aspect in
[0.3, 2.0], alpha in [0.05, 0.2], split precision).

Sixteen instances from the batch's seeded distribution, the 65,536-particle
maximum among them, half in Morton and half in row-major order, stepped in one
handle.  For three iterations every instance of the batch is checked against
the oracle fed with the GPU's own previous-stage output (teacher forcing):
  * cell keys: the oracle's own keys of the downloaded positions, equal except
    where the position lies within 1e-9 of a cell edge (split reconstruction);
  * the stable sort: the permutation equals the oracle's stable order of the
    GPU's unsorted keys, bit for bit;
  * density per particle and acceleration norm-wise within 1e-5 of the oracle
    evaluated on the instance's own state (FP64 against the FP32 path);
  * the integrated positions within 1e-9 of the oracle's FP64 update;
  * the neighbour lists of every instance bit for bit (first iteration).
"""
import math

import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu

RHO_TOL = 1e-5
ACC_TOL = 1e-5
EDGE_TOL = 1e-9


def _instances(count=16, seed=11):
    import workloads as W
    rng = np.random.default_rng(seed)
    out = []
    for q in range(count):
        npart = 65536 if q == 5 else int(round(math.exp(rng.uniform(math.log(2000), math.log(65536)))))
        aspect = 1.0 if q == 5 else rng.uniform(0.3, 2.0)  # 256 x 256: the maximum exactly
        alpha = rng.uniform(0.05, 0.2)
        order = "rowmajor" if q % 2 else "morton"
        prm, x, y = W.dam_break_sized(npart, aspect, 0.005, rng, alpha, order=order)
        f32 = lambda a: np.asarray(a).astype(np.float32).astype(np.float64)  # noqa: E731
        vx = f32(rng.uniform(-0.3, 0.3, len(x)))
        vy = f32(rng.uniform(-0.3, 0.3, len(x)))
        out.append((prm, f32(x), f32(y), vx, vy))
    return out


def _edge(prm, x, y):
    cs = prm["h"]
    fx = (np.asarray(x) - prm["lo"][0]) / cs
    fy = (np.asarray(y) - prm["lo"][1]) / cs
    return np.minimum(np.abs(fx - np.round(fx)), np.abs(fy - np.round(fy)))


def _keys_match(prm, p, x, y, keys):
    own = O.cell_ids(p, x, y)
    off = np.nonzero(own != keys)[0]
    if len(off):
        assert np.all(_edge(prm, x[off], y[off]) < EDGE_TOL), (len(off), off[:5])
    return len(off)


def test_batched_kernels_teacher_forced_vs_oracle():
    import sphg as S
    inst = _instances()
    counts = np.array([len(i[1]) for i in inst])
    assert counts.max() == 65536 and counts.min() >= 1900 and counts.sum() > 300000
    off = np.concatenate([[0], np.cumsum(counts)])
    cat = [np.concatenate([i[k] for i in inst]) for k in (1, 2, 3, 4)]
    sim = S.Sim([S.params(**i[0]) for i in inst], counts, S.options(precision=S.SPLIT))
    sim.upload(*cat)
    sim.preloop()
    edges = 0
    for it in range(3):
        a = sim.download()
        keys = sim.debug(S.DBG_KEYS)
        nxt_x, nxt_y = sim.debug(S.DBG_POS_NEXT)
        nkeys = sim.debug(S.DBG_UNSORTED_KEYS)
        if it == 0:
            go, gi = sim.neighbor_lists()
        for q, (prm, *_rest) in enumerate(inst):
            p = O.params(**prm)
            sl = slice(off[q], off[q + 1])
            g = {f: a[f][sl] for f in ("x", "y", "vx", "vy", "rho", "fx", "fy")}
            k_gpu = keys[sl]
            edges += _keys_match(prm, p, g["x"], g["y"], k_gpu)
            s_, e_ = O.cell_ranges(p, k_gpu)
            rho = O.density(p, g["x"], g["y"], k_gpu, s_, e_)
            fx, fy = O.forces(p, g["x"], g["y"], g["vx"], g["vy"], rho, k_gpu, s_, e_)
            assert np.max(np.abs(g["rho"] - rho) / rho) <= RHO_TOL, (it, q)
            scale = max(np.abs(fx).max(), np.abs(fy).max())
            dacc = max(np.abs(g["fx"] - fx).max(), np.abs(g["fy"] - fy).max()) / scale
            assert dacc <= ACC_TOL, (it, q, dacc)
            if it == 0:
                ro, ri = O.neighbor_lists(p, g["x"], g["y"], k_gpu, s_, e_)
                lo_, hi_ = go[off[q]], go[off[q + 1]]
                assert np.array_equal(go[off[q]:off[q + 1] + 1] - lo_, ro), (q, "offsets")
                assert np.array_equal(gi[lo_:hi_] - off[q], ri), (q, "entries")
            # integration with the GPU's own forces, FP64 update of the oracle
            ox, oy, _, _ = O.integrate(p, g["x"], g["y"], g["vx"], g["vy"], g["fx"], g["fy"])
            assert np.max(np.abs(nxt_x[sl] - ox)) < 1e-9 and np.max(np.abs(nxt_y[sl] - oy)) < 1e-9, (it, q)
            edges += _keys_match(prm, p, nxt_x[sl], nxt_y[sl], nkeys[sl])
        sim.step(1)
        perm = sim.debug(S.DBG_PERM)
        for q in range(len(inst)):
            sl = slice(off[q], off[q + 1])
            want = O.sort_perm(nkeys[sl]) + off[q]
            assert np.array_equal(perm[sl], want), (it, q, "permutation")
    sim.close()
    print("BATCH_PARITY instances=%d particles=%d edge_cases=%d" % (len(inst), int(off[-1]), edges))
