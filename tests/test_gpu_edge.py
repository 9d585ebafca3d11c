"""Edge cases and failure detection on the GPU, none of which faults, traps or hangs the GPU:
capacity overflow reported through the status word, a grid-barrier wait cut short by a tiny spin
limit (the persistent kernel returns and reports B3G_FLAG_BARRIER_TIMEOUT), NaN detection,
degenerate worlds and the inclusive touching-AABB known answer."""
import numpy as np
import pytest

from gpu_helpers import load, pairs_xy, run_stages
from bullet3_gb300 import capi, scenes
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def test_pair_overflow_is_reported_and_clamped():
    sc = scenes.box_pile(6, 6, 6, spacing=1.0, base_y=0.45, seed=2)
    np_, bp, pl, shapes = load(sc, m_maxBroadphasePairs=100)
    run_stages(np_, bp, pl)
    assert pl.status() & capi.FLAG_PAIR_OVERFLOW
    assert bp.getNumOverlap() == 100


def test_barrier_timeout_returns_status_not_hang():
    sc = scenes.box_pile(6, 6, 6, spacing=1.0, base_y=0.45, seed=2)
    np_, bp, pl, shapes = load(sc, solver_mode=capi.SOLVER_PGS)
    # a spin limit of one poll makes every waiting block give up at its first barrier
    from bullet3_gb300.pipeline import b3Config  # noqa: F401
    cfg = np_.m_config.to_c()
    cfg.barrier_spin_limit = 1
    import ctypes as C
    h = C.c_void_p()
    capi.call("b3g_create", C.byref(cfg), C.c_int(0), C.byref(h))
    try:
        from bullet3_gb300.scenes import load_scene  # noqa: F401
        # register the same scene in the second world through the C ABI
        box = C.c_int()
        v = scenes.box_vertices(0.5, 0.5, 0.5)
        one = (C.c_float * 3)(1, 1, 1)
        capi.call("b3g_register_hull", h, capi.fptr(v), C.c_int(12), C.c_int(8), one, C.byref(box))
        plane = C.c_int()
        capi.call("b3g_register_plane", h, (C.c_float * 3)(0, 1, 0), C.c_float(0), C.byref(plane))
        out = C.c_int()
        capi.call("b3g_register_body", h, C.c_float(0), (C.c_float * 3)(0, 0, 0), (C.c_float * 4)(0, 0, 0, 1), plane,
                  C.c_int(0), C.byref(out))
        for i in range(64):
            p = (C.c_float * 3)(float(i % 4) * 0.98, 0.45 + float(i // 16) * 0.98, float((i // 4) % 4) * 0.98)
            capi.call("b3g_register_body", h, C.c_float(1), p, (C.c_float * 4)(0, 0, 0, 1), box, C.c_int(i),
                      C.byref(out))
        capi.call("b3g_write_all_to_gpu", h)
        capi.call("b3g_step", h, C.c_float(1 / 60))
        capi.call("b3g_synchronize", h)
        flags = C.c_uint()
        capi.call("b3g_status", h, C.byref(flags), C.c_int(1))
        assert flags.value & capi.FLAG_BARRIER_TIMEOUT
    finally:
        capi.load().b3g_destroy(h)
    # the context stays usable: the first world still steps normally
    pl.stepSimulation(1 / 60)
    pl.synchronize()
    assert pl.status() == 0


def test_nan_is_flagged():
    sc = scenes.box_pile(3, 3, 3, seed=0)
    np_, bp, pl, shapes = load(sc)
    b = np_.readbackAllBodiesToCpu()
    b["linVel"][5, 0] = np.nan
    np_.writeBodiesToGpu(b)
    pl.stepSimulation(1 / 60)
    pl.synchronize()
    assert pl.status() & capi.FLAG_NAN


def test_static_only_world_steps():
    sc = scenes.Scene(shapes=[{"type": "plane", "normal": (0, 1, 0), "constant": 0.0}],
                      body_shape=np.array([0], np.int32), mass=np.array([0.0], np.float32),
                      pos=np.zeros((1, 3), np.float32), orn=np.array([[0, 0, 0, 1]], np.float32))
    np_, bp, pl, shapes = load(sc)
    for _ in range(3):
        pl.stepSimulation(1 / 60)
    pl.synchronize()
    st = pl.stats()
    assert st.num_pairs == 0 and st.num_contacts == 0 and st.status == 0


def test_touching_aabbs_give_one_pair():
    # test/b3DynamicBvhBroadphase/main.cpp:40-69: AABBs [0,1]^3 and [1,2]^3 touch -> one pair
    sc = scenes.Scene(shapes=[{"type": "hull", "verts": scenes.box_vertices(0.5, 0.5, 0.5)}],
                      body_shape=np.array([0, 0], np.int32), mass=np.array([1.0, 1.0], np.float32),
                      pos=np.array([[0.5, 0.5, 0.5], [1.5, 1.5, 1.5]], np.float32),
                      orn=np.array([[0, 0, 0, 1], [0, 0, 0, 1]], np.float32))
    np_, bp, pl, shapes = load(sc, gravity=(0.0, 0.0, 0.0))
    run_stages(np_, bp, pl, solve=False)
    assert pairs_xy(bp.getOverlappingPairsCPU()).tolist() == [[0, 1]]


def test_sphere_sphere_and_plane_sphere_contacts():
    sc = scenes.Scene(shapes=[{"type": "plane", "normal": (0, 1, 0), "constant": 0.0},
                              {"type": "sphere", "radius": 0.5}, {"type": "sphere", "radius": 0.3}],
                      body_shape=np.array([0, 1, 2, 1], np.int32), mass=np.array([0, 1, 1, 1], np.float32),
                      pos=np.array([[0, 0, 0], [0, 0.45, 0], [0.7, 0.5, 0.1], [3, 2, 3]], np.float32),
                      orn=np.tile(np.array([0, 0, 0, 1], np.float32), (4, 1)))
    np_, bp, pl, shapes = load(sc)
    b = np_.readbackAllBodiesToCpu()
    run_stages(np_, bp, pl, solve=False)
    gc = np_.getContactsCPU()
    oc, _ = O.contacts(b, shapes, bp.getOverlappingPairsCPU())
    assert len(gc) == len(oc) >= 2
    np.testing.assert_array_equal(gc["normal"], oc["normal"])
    np.testing.assert_array_equal(gc["worldPosB"][:, 0], oc["worldPosB"][:, 0])


def test_free_fall_without_contacts():
    # bodies far apart and no plane: no pairs, no manifolds, an empty solve; the step is pure
    # integration, bit-identical to the oracle's integrateSingleTransform over the same state
    sc = scenes.box_pile(3, 3, 3, spacing=4.0, plane=False, seed=5)
    np_, bp, pl, shapes = load(sc, solver_mode=capi.SOLVER_PGS, use_cuda_graph=True)
    for _ in range(3):
        b = np_.readbackAllBodiesToCpu()
        pl.stepSimulation(1 / 60)
        pl.synchronize()
        st = pl.stats()
        assert st.num_pairs == 0 and st.num_contacts == 0 and pl.status() == 0
        ob = O.integrate(b)
        gb = np_.readbackAllBodiesToCpu()
        np.testing.assert_allclose(gb["pos"], ob["pos"], rtol=0, atol=0)
        np.testing.assert_allclose(gb["linVel"], ob["linVel"], rtol=0, atol=0)
