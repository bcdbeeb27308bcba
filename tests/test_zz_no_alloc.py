"""sphg_sort_pairs_noalloc -- the key/value radix sort for callers that cannot
allocate device memory when they sort (allocation-free graph capture,
fixed-budget allocators, hosts that forbid cudaMalloc).  Its scratch is a
fixed device array inside libsphg.so, so it sorts at most
SPHG_SORT_NOALLOC_MAX_PAIRS pairs.

Checked through the C ABI against the allocating entry point sphg_sort_pairs
on two calls in a row (the scratch keeps the first call's contents); the
result is integer data, so the comparison is exact.  This file is named to be
collected last.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MAX_PAIRS = 262144  # SPHG_SORT_NOALLOC_MAX_PAIRS in include/sphg.h


def _bind():
    import sphg
    L = sphg.lib()
    f = L.sphg_sort_pairs_noalloc
    f.argtypes = [ctypes.c_void_p] * 4 + [ctypes.c_int64, ctypes.c_int32, ctypes.c_void_p]
    f.restype = ctypes.c_int
    return sphg, L, f


def test_noalloc_sort_matches_allocating_sort_on_consecutive_calls():
    torch = pytest.importorskip("torch")
    sphg, L, noalloc = _bind()
    # (n, bits, seed, values given): multi-pass sorts through the ping-pong
    # buffers, a single-pass sort (bits <= 8), and the identity values (NULL)
    cases = [(200003, 22, 1, True), (MAX_PAIRS, 32, 2, True), (4097, 9, 3, True),
             (50001, 8, 4, True), (70001, 17, 5, False), (3000, 5, 6, False)]
    for n, bits, seed, with_vals in cases:
        rng = np.random.default_rng(seed)
        keys = rng.integers(0, 1 << bits, n, dtype=np.uint64).astype(np.uint32)
        keys[: n // 3] = keys[0]  # long runs of equal keys exercise stability
        vals = rng.permutation(n).astype(np.uint32) if with_vals else np.arange(n, dtype=np.uint32)
        ki = torch.from_numpy(keys.view(np.int32)).cuda()
        vi = torch.from_numpy(vals.view(np.int32)).cuda()
        vin = vi.data_ptr() if with_vals else None
        ko_ref = torch.empty_like(ki)
        vo_ref = torch.empty_like(vi)
        ko = torch.full_like(ki, -1)
        vo = torch.full_like(vi, -1)
        sphg.sort_pairs(ki.data_ptr(), vin or 0, ko_ref.data_ptr(), vo_ref.data_ptr(), n, bits)
        st = noalloc(ki.data_ptr(), vin, ko.data_ptr(), vo.data_ptr(), n, bits, None)
        assert st == 0, L.sphg_last_error_string().decode()
        torch.cuda.synchronize()
        assert torch.equal(ko, ko_ref) and torch.equal(vo, vo_ref)
        order = np.argsort(keys, kind="stable")
        assert (ko.cpu().numpy().view(np.uint32) == keys[order]).all()
        assert (vo.cpu().numpy().view(np.uint32) == vals[order]).all()


def test_noalloc_sort_rejects_sizes_above_its_scratch():
    torch = pytest.importorskip("torch")
    sphg, L, noalloc = _bind()
    buf = torch.zeros(16, dtype=torch.int32, device="cuda")
    p = buf.data_ptr()
    st = noalloc(p, p, p, p, MAX_PAIRS + 1, 22, None)
    assert st == sphg.CAPACITY
    assert str(MAX_PAIRS) in L.sphg_last_error_string().decode()
