"""The parallel primitives through the C ABI, checked the way the reference's ParallelPrimitives
tests check theirs (test/OpenCL/ParallelPrimitives/main.cpp): each against a host implementation
at sizes up to 256k.  Bars: the radix sort is a STABLE sort of (key, value) pairs (keys and values
equal a host stable sort); the scan is EXCLUSIVE and reports the total; bound search lower/upper
match the reference's host loop (absent buckets untouched) and count = upper - lower; fill writes
exactly [offset, offset + n).  All integer results bit-exact."""
import ctypes as C

import numpy as np
import pytest

from bullet3_gb300 import capi

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
SIZES = [1, 2, 128, 1000, 65536 + 17, 262144]


def _dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def _ptr(t):
    return C.c_void_p(t.data_ptr())


@pytest.mark.parametrize("n", SIZES)
@pytest.mark.parametrize("bits", [8, 21, 32])
def test_radix_sort_is_stable_key_value_sort(n, bits):
    rng = np.random.Generator(np.random.PCG64(n + bits))
    keys = rng.integers(0, 2**32, n, dtype=np.uint64).astype(np.uint32)
    keys[: n // 3] = keys[n // 2: n // 2 + n // 3]  # many equal keys: stability matters
    vals = np.arange(n, dtype=np.uint32)
    kv = np.stack([keys, vals], 1).astype(np.uint32)
    t = _dev(kv.view(np.int32))
    capi.call("b3g_radix_sort32", C.c_int(0), _ptr(t), C.c_int(n), C.c_int(bits))
    got = t.cpu().numpy().view(np.uint32)
    mask = np.uint32(0xFFFFFFFF) if bits == 32 else np.uint32((1 << bits) - 1)
    order = np.argsort(keys & mask, kind="stable")  # the host LSD sort's order
    assert np.array_equal(got[:, 0], keys[order]) and np.array_equal(got[:, 1], vals[order])
    tk = _dev(keys.view(np.int32))
    capi.call("b3g_radix_sort32_keys", C.c_int(0), _ptr(tk), C.c_int(n), C.c_int(bits))
    assert np.array_equal(tk.cpu().numpy().view(np.uint32), keys[order])


@pytest.mark.parametrize("n", SIZES)
def test_prefix_scan_is_exclusive_with_total(n):
    rng = np.random.Generator(np.random.PCG64(n))
    src = rng.integers(0, 1000, n).astype(np.uint32)
    ts, td = _dev(src.view(np.int32)), torch.zeros(n, dtype=torch.int32, device="cuda")
    total = C.c_uint()
    capi.call("b3g_prefix_scan32", C.c_int(0), _ptr(ts), _ptr(td), C.c_int(n), C.byref(total))
    expect = np.concatenate([[0], np.cumsum(src, dtype=np.uint64)[:-1]]).astype(np.uint32)
    assert np.array_equal(td.cpu().numpy().view(np.uint32), expect)
    assert total.value == int(src.astype(np.uint64).sum())
    # in place, as the reference allows src == dst
    capi.call("b3g_prefix_scan32", C.c_int(0), _ptr(ts), _ptr(ts), C.c_int(n), C.byref(total))
    assert np.array_equal(ts.cpu().numpy().view(np.uint32), expect)


def _bound_host(keys, n_dst, upper):
    """The reference's executeHost loop (b3BoundSearchCL.cpp:133-187) over sorted keys."""
    dst = np.full(n_dst, 0xFFFFFFFF, np.uint32)
    n = len(keys)
    if not upper:
        for i in range(n):
            prev = -1 if i == 0 else keys[i - 1]
            if prev != keys[i]:
                dst[keys[i]] = i
    else:
        for i in range(1, n + 1):
            nxt = n_dst if i == n else keys[i]
            if keys[i - 1] != nxt:
                dst[keys[i - 1]] = i
    return dst


@pytest.mark.parametrize("n", [1, 128, 5000, 262144])
def test_bound_search_matches_host_loop(n):
    n_dst = 256
    rng = np.random.Generator(np.random.PCG64(7 + n))
    keys = np.sort(rng.integers(0, n_dst, n)).astype(np.int32)
    src = np.stack([keys, np.arange(n, dtype=np.int32)], 1)
    ts = _dev(src)
    res = {}
    for opt in (0, 1):
        td = torch.full((n_dst,), -1, dtype=torch.int32, device="cuda")
        capi.call("b3g_bound_search", C.c_int(0), _ptr(ts), C.c_int(n), _ptr(td), C.c_int(n_dst), C.c_int(opt))
        res[opt] = td.cpu().numpy().view(np.uint32)
        assert np.array_equal(res[opt], _bound_host(keys, n_dst, bool(opt)))
    for b in range(n_dst):  # every element between lower and upper carries the bucket's key
        if res[0][b] != 0xFFFFFFFF:
            assert (keys[res[0][b]:res[1][b]] == b).all()
    tc = torch.zeros(n_dst, dtype=torch.int32, device="cuda")
    capi.call("b3g_bound_search", C.c_int(0), _ptr(ts), C.c_int(n), _ptr(tc), C.c_int(n_dst), C.c_int(2))
    assert np.array_equal(tc.cpu().numpy(), np.bincount(keys, minlength=n_dst))


@pytest.mark.parametrize("n,offset", [(1, 0), (1000, 17), (262144 - 5, 5)])
def test_fill_writes_exactly_the_range(n, offset):
    t = torch.full((262144,), 7, dtype=torch.int32, device="cuda")
    capi.call("b3g_fill32", C.c_int(0), _ptr(t), C.c_int(-3), C.c_int(n), C.c_int(offset))
    got = t.cpu().numpy()
    assert (got[offset:offset + n] == -3).all()
    assert (got[:offset] == 7).all() and (got[offset + n:] == 7).all()


def test_invalid_arguments_are_rejected():
    with pytest.raises(capi.B3GError):
        capi.call("b3g_radix_sort32", C.c_int(0), C.c_void_p(None), C.c_int(10), C.c_int(32))
    with pytest.raises(capi.B3GError):
        capi.call("b3g_bound_search", C.c_int(0), C.c_void_p(None), C.c_int(0), C.c_void_p(None), C.c_int(0),
                  C.c_int(5))
