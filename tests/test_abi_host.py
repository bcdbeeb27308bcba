"""CPU-only checks of the C ABI library and the host driver: libsphg.so builds,
loads and exports every entry point include/sphg.h declares; the host-side
argument checks fail loudly; the driver reads the reference's configuration
keys and builds the reference's lattice (no GPU call is made)."""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

import oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "sphg.h")


@pytest.fixture(scope="module")
def built():
    import build as B
    B.build()
    return B


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:const\s+)?\w+\s*\*?\s*(sphg_\w+)\s*\(", text, flags=re.M)))


def test_library_exports_every_declared_function(built):
    names = declared_functions()
    assert len(names) >= 25, names
    lib = ctypes.CDLL(built.LIB)
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_version_and_default_options(built):
    import sphg as S
    assert "sm_103a" in S.lib().sphg_version().decode()
    o = S.options()
    assert (o.precision, o.track_ids, o.use_graph) == (S.PLAIN, 1, 1)


def test_host_argument_checks_fail_before_any_device_work(built):
    import sphg as S
    L = S.lib()
    h = ctypes.c_void_p()
    # null outputs / handles
    assert L.sphg_create(None, None, 10, ctypes.byref(h)) == S.INVALID_ARG
    assert L.sphg_step(None, 1, None) == S.INVALID_ARG
    assert L.sphg_preloop(None, None) == S.INVALID_ARG
    assert L.sphg_download(None, None, None, None, None, None, None, None, None, None) == S.INVALID_ARG
    assert L.sphg_step_headers(None, 1, None, None) == S.INVALID_ARG
    assert L.sphg_diagnostics_async(None, None, None) == S.INVALID_ARG
    # parameters the reference would accept silently and then misbehave on
    for bad in (dict(h=0.0), dict(h=-1.0), dict(dt=float("nan")), dict(hi=(0.0, 48.0)), dict(order=7)):
        p = S.params(**bad)
        assert L.sphg_create(ctypes.byref(p), None, 10, ctypes.byref(h)) == S.INVALID_ARG, bad
        assert L.sphg_last_error_string()
    o = S.options(precision=9)
    p = S.params()
    assert L.sphg_create(ctypes.byref(p), ctypes.byref(o), 10, ctypes.byref(h)) == S.INVALID_ARG
    o = S.options(tile_bits=4)  # tiles need Morton order; the default params are rowmajor
    assert L.sphg_create(ctypes.byref(p), ctypes.byref(o), 10, ctypes.byref(h)) == S.INVALID_ARG
    # launch shapes the autotuner may pick: threads per block 64/128/256, one or two particles per density thread
    for bad in (dict(block_threads=96), dict(block_threads=512), dict(cell_pairs=2), dict(cell_pairs=-1)):
        o = S.options(**bad)
        assert L.sphg_create(ctypes.byref(p), ctypes.byref(o), 10, ctypes.byref(h)) == S.INVALID_ARG, bad
    # the sorts keep 30-bit running counts in their look-back words
    sort = L.sphg_sort_pairs
    sort.argtypes = [ctypes.c_void_p] * 4 + [ctypes.c_int64, ctypes.c_int32, ctypes.c_void_p]
    assert sort(16, 16, 32, 32, 1 << 30, 22, None) == S.CAPACITY
    assert "2^30" in L.sphg_last_error_string().decode()


def _write_cfg(path, **kv):
    with open(path, "w") as f:
        for k, v in kv.items():
            f.write("%s = %s\n" % (k, v))


def _dry(built, cfg):
    r = subprocess.run([built.HOST_APP, cfg, "--dry-run"], capture_output=True, text=True, timeout=60)
    return r.returncode, r.stdout + r.stderr


@pytest.mark.parametrize("dom,lat", [((96, 48), (0.5, 0.5, 0.4, 0.8)), ((1.0, 1.0), (0.005, 0.005, 0.4, 0.8)),
                                     ((2.5, 1.3), (0.013, 0.011, 0.33, 0.71))])
def test_driver_lattice_matches_reference_lattice(built, tmp_path, dom, lat):
    cfg = str(tmp_path / "example.txt")
    _write_cfg(cfg, steps=5, dt=0.005, domain_x=dom[0], domain_y=dom[1], lattice_dx=lat[0],
               lattice_dy=lat[1], lattice_xvol=lat[2], lattice_yvol=lat[3], order="morton",
               compute_type="gb300", checkpoint_write_frequency=1)
    rc, out = _dry(built, cfg)
    assert rc == 0, out
    x, _ = O.lattice(dom[0], dom[1], lat[0], lat[1], lat[2], lat[3])
    n = int(re.search(r"\[LatticeCreator\] Total particles: (\d+)", out).group(1))
    assert n == len(x)


def test_driver_reference_parser_semantics(built, tmp_path):
    """Tabs and blanks around keys and values are trimmed; the first occurrence
    of a key wins; a missing key reads as 0 (core/utils/InputParser.cpp:10-52)."""
    cfg = str(tmp_path / "c.txt")
    with open(cfg, "w") as f:
        f.write("\tsteps\t=  7 \n steps = 99\ndomain_x=96\ndomain_y=48\nlattice_dx=0.5\nlattice_dy=0.5\n"
                "lattice_xvol=0.4\nlattice_yvol=0.8\norder=rowmajor\ncompute_type=sorted\n"
                "# comment line without equals sign\nH = 1.5\n")
    rc, out = _dry(built, cfg)
    assert rc == 0, out
    assert "[Configuration] steps=7" in out
    assert "H=1.5" in out
    assert "output frequency=0" in out and "no checkpoints" in out


@pytest.mark.parametrize("key,val,msg", [("order", "hilbert", "order must be"),
                                         ("compute_type", "cuda", "not served"),
                                         ("lattice_dx", "0", "must be positive")])
def test_driver_rejects_bad_configuration(built, tmp_path, key, val, msg):
    kv = dict(steps=5, dt=0.005, domain_x=96, domain_y=48, lattice_dx=0.5, lattice_dy=0.5,
              lattice_xvol=0.4, lattice_yvol=0.8, order="rowmajor", compute_type="gb300")
    kv[key] = val
    cfg = str(tmp_path / "c.txt")
    _write_cfg(cfg, **kv)
    rc, out = _dry(built, cfg)
    assert rc != 0 and msg in out


def test_driver_missing_file(built, tmp_path):
    rc, out = _dry(built, str(tmp_path / "nope.txt"))
    assert rc != 0 and "Cannot find configuration file" in out
