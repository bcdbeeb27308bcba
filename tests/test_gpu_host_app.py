"""The host driver (sph_gb300_app, compute_type=gb300) against the oracle run of
the same configuration: checkpoint files, step headers, cell files, and an
exact resume from a binary snapshot."""
import os
import re
import subprocess

import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu


def _app():
    import build as B
    B.build()
    return B.HOST_APP


def _cfg(path, **kv):
    base = dict(steps=13, dt=0.005, domain_x=96, domain_y=48, lattice_dx=0.5, lattice_dy=0.5,
                lattice_xvol=0.4, lattice_yvol=0.8, checkpoint_write_frequency=4, order="rowmajor",
                compute_type="gb300", bool_output_first_step=1, bool_measure_neighborhood=0)
    base.update(kv)
    with open(path, "w") as f:
        for k, v in base.items():
            f.write("%s = %s\n" % (k, v))
    return base


def _run(app, cfg, cwd):
    r = subprocess.run([app, cfg], capture_output=True, text=True, timeout=300, cwd=cwd)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    return r.stdout


def _headers(out):
    rows = {}
    for m in re.finditer(r"Step= (\d+)\t N=(\d+)\t E_k=(\S+)\t \|v\|_max=(\S+)", out):
        rows[int(m.group(1))] = (int(m.group(2)), float(m.group(3)), float(m.group(4)))
    return rows


def _match(points, ref):
    """Nearest-neighbour matching of checkpoint rows to oracle particles."""
    from scipy.spatial import cKDTree
    d, idx = cKDTree(ref).query(points)
    assert len(np.unique(idx)) == len(idx)
    return d


@pytest.mark.parametrize("order,ctype", [("rowmajor", "gb300"), ("morton", "sorted"), ("morton", "mp-lists")])
def test_driver_matches_oracle_run(tmp_path, order, ctype):
    app = _app()
    cfg = str(tmp_path / "example.txt")
    kv = _cfg(cfg, order=order, compute_type=ctype, bool_measure_neighborhood=1)
    out = _run(app, cfg, str(tmp_path))
    heads = _headers(out)
    assert sorted(heads) == list(range(kv["steps"]))
    x0, y0 = O.lattice(96, 48, 0.5, 0.5, 0.4, 0.8)
    p = O.params(order=order, h=1.0, dt=0.005, lo=(0, 0), hi=(96, 48))
    sim = O.Sim(p, x0, y0, np.zeros(len(x0)), np.zeros(len(x0)))
    sim.preloop()
    done = 0
    for step in range(kv["steps"]):
        if step > done:
            sim.steps(step - done)
            done = step
        st = sim.get()
        n_in, ek, vmax2 = heads[step]
        diag = O.diagnostics(p, st["x"], st["y"], st["vx"], st["vy"])
        assert n_in == int(diag[2])
        assert ek == pytest.approx(diag[0], rel=2e-4, abs=1e-9)
        assert vmax2 == pytest.approx(diag[1], rel=2e-4, abs=1e-9)
        if step % kv["checkpoint_write_frequency"] == 0:
            rows = np.loadtxt(tmp_path / ("positions_step_%d.txt" % step))
            assert rows.shape == (len(x0), 3) and (rows[:, 2] == 0).all()
            d = _match(rows[:, :2], np.stack([st["x"], st["y"]], 1))
            assert d.max() < 1e-3  # six significant digits of coordinates up to 96
        if step == 0:
            # cells_0.txt: the reference's [start, end) table of the sorted state
            text = open(tmp_path / "cells_0.txt").read()
            cells = re.findall(r"cell:(\d+)\[(-?\d+),(-?\d+)\)", text)
            start = {int(c): int(s) for c, s, e in cells}
            end = {int(c): int(e) for c, s, e in cells}
            k = st["key"]
            for c in np.unique(k):
                w = np.nonzero(k == c)[0]
                assert start[int(c)] == w[0] and end[int(c)] == w[-1] + 1
            assert sum(1 for c in start if start[c] >= 0) == len(np.unique(k))
    assert os.path.exists(tmp_path / "timer_manager.data")
    # neighbour and cell statistics of the last iteration (AvgNeighborsPerParticle columns)
    lines = open(tmp_path / "neighborhood_and_cells.data").read().splitlines()
    assert len(lines) == 2 and lines[0].split()[0] == "avg_npp"
    vals = [float(v) for v in lines[1].split()]
    r = sim.get()
    sk = O.cell_ids(p, r["x"], r["y"])
    s_, e_ = O.cell_ranges(p, sk)
    offs, _ = O.neighbor_lists(p, r["x"], r["y"], sk, s_, e_)
    npp = np.diff(offs)
    assert vals[0] == int(npp.sum() // len(npp)) and vals[1] == npp.min() and vals[2] == npp.max()


def test_driver_resume_from_snapshot_is_exact(tmp_path):
    app = _app()
    a = tmp_path / "a"
    b = tmp_path / "b"
    a.mkdir()
    b.mkdir()
    _cfg(str(a / "c.txt"), order="morton", snapshot_write_frequency=5, precision="split")
    out_a = _run(app, str(a / "c.txt"), str(a))
    _cfg(str(b / "c.txt"), order="morton", precision="split", resume_from=str(a / "snapshot_step_5.bin"))
    out = _run(app, str(b / "c.txt"), str(b))
    assert "Resumed after step 5" in out
    for step in (8, 12):
        assert open(a / ("positions_step_%d.txt" % step)).read() == \
            open(b / ("positions_step_%d.txt" % step)).read()
    ha, hb = _headers(out_a), _headers(out)
    assert sorted(hb) == list(range(6, 13))
    for step in hb:
        assert ha[step] == hb[step]
    assert not os.path.exists(b / "positions_step_4.txt")
