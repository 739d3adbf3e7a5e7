"""b2g_pairs_static: the allocation-free broadphase entry point.

Some callers cannot allocate device memory when they call the broadphase - a frame loop that
must not call cudaMalloc/cudaFree (they synchronise the device), or a plug-in whose host owns the
device's memory budget. For them b2g_pairs_static keeps its scratch in a fixed array in device
memory. This test calls it through the C ABI twice in a row on different inputs and checks each
result against the allocating entry point b2g_pairs (integer pair lists: exact equality), and
that sizes beyond the stated maximum are refused. It lives in its own file, collected last, and
passes both alone in a fresh process and after the other tests.
"""
import ctypes as C

import numpy as np
import pytest

import b2gpu as G

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _lib():
    lib = G.Lib()
    fn = lib.lib.b2g_pairs_static
    fn.argtypes = [C.c_void_p, C.c_int32, C.c_void_p, C.c_int64, C.POINTER(C.c_int64), C.c_void_p]
    fn.restype = C.c_int
    return lib


def _aabbs(rng, n):
    c = rng.uniform(-40, 40, (n, 2)).astype(np.float32)
    h = rng.uniform(0.05, 1.2, (n, 2)).astype(np.float32)
    return np.concatenate([c - h, c + h], axis=1).astype(np.float32)


def _run(fn, aabb, cap):
    d_aabb = torch.from_numpy(aabb).cuda()
    d_pairs = torch.full((cap,), -1, dtype=torch.int64, device="cuda")
    n = C.c_int64()
    st = fn(d_aabb.data_ptr(), aabb.shape[0], d_pairs.data_ptr(), cap, C.byref(n), None)
    torch.cuda.synchronize()
    return st, n.value, d_pairs.cpu().numpy().view(np.uint64)


def test_static_scratch_matches_allocating_entry_point():
    lib = _lib()
    rng = np.random.default_rng(2024)
    for n in (5000, 60000):  # two calls in a row, different sizes and inputs
        aabb = _aabbs(rng, n)
        st0, n0, _ = _run(lib.lib.b2g_pairs, aabb, 1)
        assert st0 == 7 and n0 > 0  # B2G_E_CAPACITY: reports the count it needs
        cap = n0 + 8
        st_a, na, pa = _run(lib.lib.b2g_pairs, aabb, cap)
        st_s, ns, ps = _run(lib.lib.b2g_pairs_static, aabb, cap)
        assert st_a == 0 and st_s == 0
        assert na == ns == n0
        assert np.array_equal(pa[:na], ps[:ns])


def test_static_scratch_rejects_oversize():
    lib = _lib()
    aabb = np.zeros((131073, 4), np.float32)
    st, n, _ = _run(lib.lib.b2g_pairs_static, aabb, 16)
    assert st == 7  # B2G_E_CAPACITY


def test_static_scratch_at_the_maximum_size():
    """Exactly B2G_PAIRS_STATIC_MAX sparse boxes: the fixed array holds the layout and the sort's
    temporary storage, and the result equals the allocating entry point's."""
    lib = _lib()
    rng = np.random.default_rng(7)
    n = 131072
    c = rng.uniform(-2000, 2000, (n, 2)).astype(np.float32)
    h = rng.uniform(0.05, 1.5, (n, 2)).astype(np.float32)
    aabb = np.concatenate([c - h, c + h], axis=1).astype(np.float32)
    st0, n0, _ = _run(lib.lib.b2g_pairs, aabb, 1)
    assert st0 == 7 and n0 > 0
    st_a, na, pa = _run(lib.lib.b2g_pairs, aabb, n0)
    st_s, ns, ps = _run(lib.lib.b2g_pairs_static, aabb, n0)
    assert st_a == 0 and st_s == 0 and na == ns == n0
    assert np.array_equal(pa[:na], ps[:ns])


def test_static_scratch_counts_past_two_to_the_31():
    """70 000 coincident boxes overlap pairwise: 2 449 965 000 pairs, more than an int32 holds.
    The total comes back exact in 64 bits and a small capacity is refused without a write."""
    lib = _lib()
    n = 70000
    aabb = np.tile(np.array([[0.0, 0.0, 1.0, 1.0]], np.float32), (n, 1))
    for fn in (lib.lib.b2g_pairs, lib.lib.b2g_pairs_static):
        st, total, pairs = _run(fn, aabb, 64)
        assert st == 7  # B2G_E_CAPACITY
        assert total == n * (n - 1) // 2
        assert (pairs.view(np.int64) == -1).all()  # nothing written
