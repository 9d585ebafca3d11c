"""b3g_grid_pairs_noalloc: the grid broadphase with its scratch in a static device array.

Checked against the allocating entry point (b3g_calculate_overlapping_pairs + b3g_read_pairs) on
the same world AABBs, on two calls in a row with the bodies moved in between.  The file name
sorts last so the check also runs after every other GPU test in one process."""
import ctypes as C

import numpy as np
import pytest

from gpu_helpers import load, pairs_xy
from bullet3_gb300 import capi, scenes

MAX_AABBS, MAX_PAIRS, MAX_GRID = 65536, 262144, 64


def _call(*args):
    return capi.load().b3g_grid_pairs_noalloc(*args)


def test_noalloc_rejects_sizes_beyond_its_static_scratch():
    # argument checks run before any CUDA call, so this needs no GPU
    lib = capi.load()
    fake = C.c_void_p(256)
    cases = [(MAX_AABBS + 1, 1.0, 64, 1024), (16, 1.0, 64, MAX_PAIRS + 1), (16, 1.0, 128, 1024),
             (16, 1.0, 48, 1024), (16, 1.0, 2, 1024), (-1, 1.0, 64, 1024), (16, 1.0, 64, 0)]
    for n, cell, dim, cap in cases:
        st = _call(fake, C.c_int(n), C.c_float(cell), C.c_int(dim), fake, C.c_int(cap), fake, None)
        assert st == 3, (n, dim, cap)  # B3G_ERR_CAPACITY
        assert b"B3G_NOALLOC_MAX" in lib.b3g_last_error()
    st = _call(fake, C.c_int(16), C.c_float(0.0), C.c_int(64), fake, C.c_int(1024), fake, None)
    assert st == 1  # invalid argument: cell size
    st = _call(C.c_void_p(264), C.c_int(16), C.c_float(1.0), C.c_int(64), fake, C.c_int(1024), fake, None)
    assert st == 1  # invalid argument: AABBs not 16-byte aligned


@pytest.mark.gpu
def test_noalloc_pairs_match_allocating_entry_on_two_calls():
    torch = pytest.importorskip("torch")
    sc = scenes.mixed_scene(20000, extent=30.0, seed=7, plane=False)
    np_, bp, pl, shapes = load(sc, grid_dim=64, m_maxBroadphasePairs=400000)
    n = sc.num_bodies
    cap = 200000
    d_pairs = torch.full((cap, 4), 7, dtype=torch.int32, device="cuda")
    d_num = torch.full((1,), -5, dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    seen = []
    for call in range(2):
        pl.setupGpuAabbsFull()
        bp.calculateOverlappingPairs()
        pl.synchronize()
        ref = bp.getOverlappingPairsCPU()
        assert 1000 < len(ref) < cap
        st = _call(C.c_void_p(bp.getAabbBufferWS()), C.c_int(n), C.c_float(sc.cell), C.c_int(64),
                   C.c_void_p(d_pairs.data_ptr()), C.c_int(cap), C.c_void_p(d_num.data_ptr()), C.c_void_p(stream))
        assert st == 0, capi.load().b3g_last_error()
        torch.cuda.synchronize()
        num = int(d_num.item())
        got = d_pairs[:num].cpu().numpy()
        assert num == len(ref)
        assert np.array_equal(got[:, :2], pairs_xy(ref))
        assert (got[:, 2:] == -1).all()
        seen.append(pairs_xy(ref))
        # move the bodies: the second call sees different AABBs
        for _ in range(3):
            pl.stepSimulation(1 / 60)
        pl.synchronize()
    assert not np.array_equal(seen[0], seen[1])
    # overflow: the raw count is reported; max_pairs of the pairs (an unspecified subset) are written, sorted
    pl.setupGpuAabbsFull()
    bp.calculateOverlappingPairs()
    pl.synchronize()
    ref = pairs_xy(bp.getOverlappingPairsCPU())
    small = 1000
    st = _call(C.c_void_p(bp.getAabbBufferWS()), C.c_int(n), C.c_float(sc.cell), C.c_int(64),
               C.c_void_p(d_pairs.data_ptr()), C.c_int(small), C.c_void_p(d_num.data_ptr()), C.c_void_p(stream))
    assert st == 0
    torch.cuda.synchronize()
    assert int(d_num.item()) == len(ref)
    # a full buffer holds an arbitrary subset of the pairs, sorted
    got = d_pairs[:small, :2].cpu().numpy()
    key = got[:, 0].astype(np.int64) * (1 << 20) + got[:, 1]
    assert (np.diff(key) > 0).all()
    assert set(map(tuple, got.tolist())) <= set(map(tuple, ref.tolist()))
