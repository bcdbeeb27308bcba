"""Continuous batching (sphg_server_*): results are the same alone and in the
mix, admission respects the capacity, latency is reported."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _requests(seed, count):
    import workloads as W
    rng = np.random.default_rng(seed)
    out = []
    for k in range(count):
        if k % 2 == 0:
            npart = int(rng.integers(300, 3000))
            prm, x, y = W.dam_break_sized(npart, rng.uniform(0.3, 2.0), 0.005, rng, alpha=0.1)
            vx = np.zeros(len(x))
            vy = np.zeros(len(x))
        else:
            prm, x, y, vx, vy, _ = W.taylor_green(int(rng.integers(12, 40)), seed=int(rng.integers(1 << 20)))
        out.append((prm, x, y, vx, vy, int(rng.integers(5, 25))))
    return out


def _serve(S, reqs, budget=2e9, stagger=True):
    srv = S.Server(budget)
    ids = []
    pending = list(reqs)
    results = {}
    while pending or len(results) < len(reqs):
        # submit a couple of requests per tick so arrivals overlap running work
        for _ in range(2 if stagger else len(pending)):
            if pending:
                prm, x, y, vx, vy, steps = pending.pop(0)
                ids.append(srv.submit(S.params(**prm), x, y, vx, vy, steps))
        srv.tick()
        for rid in ids:
            if rid not in results:
                r = srv.result(rid)
                if r is not None:
                    results[rid] = r
    stats = srv.stats()
    srv.close()
    return [results[i] for i in ids], stats


def test_served_results_equal_alone_and_in_the_mix():
    import sphg as S
    reqs = _requests(1, 10)
    mixed, stats = _serve(S, reqs)
    assert stats["completed"] == len(reqs) and stats["live"] == 0
    for k, req in enumerate(reqs):
        alone, _ = _serve(S, [req])
        for f in ("x", "y", "vx", "vy", "rho"):
            assert (alone[0][f] == mixed[k][f]).all(), (k, f)  # same bits
        assert mixed[k]["latency_s"] > 0
        # and the same state as a plain single-instance handle run (pre-loop + steps-1)
        prm, x, y, vx, vy, steps = req
        sim = S.Sim(S.params(**prm), len(x))
        sim.upload(x, y, vx, vy)
        sim.preloop()
        sim.step(steps - 1)
        o = sim.download(forces=False)
        sim.close()
        assert (o["ids"] == mixed[k]["ids"]).all()
        for f in ("x", "y", "vx", "vy", "rho"):
            np.testing.assert_allclose(mixed[k][f], o[f], rtol=1e-6, atol=1e-7 * np.abs(o[f]).max())


def test_admission_respects_capacity_fifo():
    import sphg as S
    reqs = _requests(2, 8)
    # a budget for ~6,000 particles (160 B/particle for state, the rest for cell keys)
    budget = 2 * 160.0 * 6000
    srv = S.Server(budget)
    cap = srv.stats()["cap_particles"]
    ids = [srv.submit(S.params(**r[0]), *r[1:5], r[5]) for r in reqs if len(r[1]) <= cap]
    done = {}
    order = []
    max_live_particles = 0
    for _ in range(10000):
        srv.tick()
        st = srv.stats()
        max_live_particles = max(max_live_particles, st["live_particles"])
        for rid in ids:
            if rid not in done:
                r = srv.result(rid)
                if r is not None:
                    done[rid] = r
                    order.append(rid)
        if len(done) == len(ids):
            break
    assert len(done) == len(ids)
    assert max_live_particles <= cap
    srv.close()


def test_server_rejects_bad_requests():
    import sphg as S
    srv = S.Server(1e6)
    prm = S.params(h=0.01, lo=(0, 0), hi=(1, 1))
    with pytest.raises(S.SphgError):
        srv.submit(prm, [0.5], [0.5], [0.0], [0.0], 0)  # steps < 1
    with pytest.raises(S.SphgError) as ei:
        srv.submit(prm, [0.5, np.inf], [0.5, 0.5], [0, 0], [0, 0], 3)
    assert ei.value.status == S.NONFINITE
    big = np.linspace(0.1, 0.9, 100000)
    with pytest.raises(S.SphgError) as ei:
        srv.submit(prm, big, big, big * 0, big * 0, 3)
    assert ei.value.status == S.CAPACITY
    srv.close()


@pytest.mark.parametrize("prec", ["plain", "split"])
def test_lattice_requests_equal_host_array_requests(prec):
    """A request generated on the device at admission gives the same result as the
    same lattice submitted as host arrays (and mixes with other requests)."""
    import sphg as S
    import workloads as W
    from test_gpu_parity import _lattice_host
    P = S.SPLIT if prec == "split" else S.PLAIN
    prm, x, y = W.dam_break_sized(1500, 1.2, 0.005, np.random.default_rng(3), alpha=0.1)
    spec = S.lattice(0.0025, 0.0025, 0.005, 0.005, 30, 40, jitter=0.01, seed=77)
    hx, hy = _lattice_host(spec.x0, spec.y0, spec.dx, spec.dy, spec.nx, spec.ny, spec.jitter, spec.seed)
    out = []
    for mode in ("lattice", "arrays"):
        srv = S.Server(2e9, opts=S.options(precision=P))
        other = srv.submit(S.params(**prm), x, y, np.zeros(len(x)), np.zeros(len(x)), 9)
        if mode == "lattice":
            rid = srv.submit_lattice(S.params(**prm), spec, 12)
        else:
            rid = srv.submit(S.params(**prm), hx, hy, np.zeros(len(hx)), np.zeros(len(hx)), 12)
        res = None
        for _ in range(100):
            srv.tick()
            res = srv.result(rid)
            if res is not None:
                break
        assert res is not None
        out.append(res)
        srv.close()
    a, b = out
    assert (a["ids"] == b["ids"]).all()
    for f in ("x", "y", "vx", "vy", "rho"):
        if prec == "plain":
            assert (a[f] == b[f]).all(), f
        else:
            np.testing.assert_allclose(a[f], b[f], rtol=1e-6, atol=1e-7 * np.abs(b[f]).max())


def _alone_map(S, reqs):
    return [_serve(S, [r])[0][0] for r in reqs]


def test_serving_thread_overlaps_arrivals_and_matches_alone():
    """The serving thread (own thread and stream) admits requests that arrive
    while others run; every result equals the same request served alone, bit
    for bit, and newcomers were appended without moving the running ones."""
    import time

    import sphg as S
    reqs = _requests(4, 12)
    srv = S.Server(2e9)
    srv.start()
    ids = []
    for k, (prm, x, y, vx, vy, steps) in enumerate(reqs):
        ids.append(srv.submit(S.params(**prm), x, y, vx, vy, steps))
        time.sleep(0.002 * (k % 3))
    results = {}
    t0 = time.time()
    while len(results) < len(ids) and time.time() - t0 < 60:
        for rid in ids:
            if rid not in results:
                r = srv.result(rid)
                if r is not None:
                    results[rid] = r
        time.sleep(0.001)
    st = srv.stats()
    srv.stop()
    srv.close()
    assert len(results) == len(ids)
    assert st["thread_running"] == 1 and st["appends"] >= 1
    alone = _alone_map(S, reqs)
    for k, rid in enumerate(ids):
        for f in ("x", "y", "vx", "vy", "rho", "ids"):
            assert (results[rid][f] == alone[k][f]).all(), (k, f)
        assert results[rid]["latency_s"] > 0


def test_compaction_keeps_every_result_bitwise():
    """A budget small enough that finished requests' slots must be reclaimed:
    the live set is compacted (dense repack + full sort) and every result still
    equals the request served alone."""
    import sphg as S
    reqs = _requests(5, 14)
    budget = 2 * 160.0 * 9000
    srv = S.Server(budget)
    cap = srv.stats()["cap_particles"]
    reqs = [r for r in reqs if len(r[1]) <= cap]
    ids = [srv.submit(S.params(**r[0]), *r[1:5], r[5]) for r in reqs]
    done = {}
    for _ in range(20000):
        srv.tick()
        for rid in ids:
            if rid not in done:
                r = srv.result(rid)
                if r is not None:
                    done[rid] = r
        if len(done) == len(ids):
            break
    st = srv.stats()
    srv.close()
    assert len(done) == len(ids)
    assert st["compactions"] >= 1 and st["appends"] >= 1
    alone = _alone_map(S, reqs)
    for k, rid in enumerate(ids):
        for f in ("x", "y", "vx", "vy", "rho", "ids"):
            assert (done[rid][f] == alone[k][f]).all(), (k, f)


def test_served_results_equal_with_the_single_launch_iteration():
    """A server whose iterations are single cooperative launches gives the same
    bits as one running the four-kernel graph."""
    import sphg as S
    reqs = _requests(6, 8)
    outs = []
    for fused in (0, 1):
        srv = S.Server(2e9, opts=S.options(fused=fused))
        ids = [srv.submit(S.params(**r[0]), *r[1:5], r[5]) for r in reqs]
        done = {}
        for _ in range(5000):
            srv.tick()
            for rid in ids:
                if rid not in done:
                    r = srv.result(rid)
                    if r is not None:
                        done[rid] = r
            if len(done) == len(ids):
                break
        srv.close()
        outs.append([done[i] for i in ids])
    for a, b in zip(*outs):
        for f in ("x", "y", "vx", "vy", "rho", "ids"):
            assert (a[f] == b[f]).all(), f
