"""Ray casts (b3g_cast_rays) against the CPU restatement of the reference's ray kernels.

Bar: bit-exact -- every ray's hit fraction, hit body, hit point and normal equal the oracle's
brute force over all bodies in index order (the GPU walks the broadphase grid instead), on piles,
rotated mixed shapes, large static boxes, ignored bodies and independent scenes."""
import numpy as np
import pytest

from gpu_helpers import load
from bullet3_gb300 import capi, scenes
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _rays(rng, n, lo, hi, down=False, length=None):
    r = np.zeros(n, capi.RAY)
    f = rng.uniform(lo, hi, (n, 3)).astype(np.float32)
    if down:
        t = f.copy()
        f[:, 1] = hi[1] + 5.0
        t[:, 1] = -1.0
    else:
        d = rng.standard_normal((n, 3))
        d /= np.linalg.norm(d, axis=1, keepdims=True)
        t = (f + d * (length if length else rng.uniform(1.0, 40.0, (n, 1)))).astype(np.float32)
    r["from"][:, :3] = f
    r["to"][:, :3] = t
    return r


def _compare(pl, np_, shapes, rays, hits_in=None, body_scene=None):
    b = np_.readbackAllBodiesToCpu()
    g = pl.castRays(rays, hits_in)
    o = O.cast_rays(b, shapes, rays, hits_in, body_scene)
    assert np.array_equal(g["hitFraction"], o["hitFraction"])
    hit = o["hitFraction"] < 1.0
    assert np.array_equal(g["hitBody"][hit], o["hitBody"][hit])
    assert np.array_equal(g["hitPoint"][hit], o["hitPoint"][hit])
    assert np.array_equal(g["hitNormal"][hit], o["hitNormal"][hit])
    assert (g["hitBody"][~hit] == (-1 if hits_in is None else np.asarray(hits_in)["hitBody"][~hit])).all()
    return g, hit


def test_rays_onto_a_pile():
    sc = scenes.box_stack(16, 8, 16, seed=2)
    np_, bp, pl, shapes = load(sc, use_cuda_graph=True)
    for _ in range(10):
        pl.stepSimulation(1 / 60)
    pl.synchronize()
    rng = np.random.Generator(np.random.PCG64(1))
    rays = np.concatenate([_rays(rng, 2000, (-9, 0, -9), (9, 8, 9), down=True),
                           _rays(rng, 2000, (-9, 0, -9), (9, 8, 9))])
    g, hit = _compare(pl, np_, shapes, rays)
    assert hit[:2000].mean() > 0.5 and hit.sum() > 2000


def test_rays_through_rotated_mixed_shapes():
    sc = scenes.mixed_scene(4096, extent=24.0, seed=4)
    np_, bp, pl, shapes = load(sc, m_maxBroadphasePairs=400000)
    rng = np.random.Generator(np.random.PCG64(2))
    rays = np.concatenate([_rays(rng, 3000, (0, 0, 0), (24, 24, 24)),
                           _rays(rng, 500, (-5, -5, -5), (30, 30, 30), length=60.0)])
    g, hit = _compare(pl, np_, shapes, rays)
    kinds = np.array([s["type"] for s in sc.shapes])[sc.body_shape[g["hitBody"][hit]]]
    assert (kinds == "sphere").any() and (kinds == "hull").any()


def test_ignored_body_and_large_statics():
    sc = scenes.static_field(300, 1500, extent=40.0, seed=6)
    np_, bp, pl, shapes = load(sc, m_maxBroadphasePairs=200000)
    rng = np.random.Generator(np.random.PCG64(3))
    rays = _rays(rng, 1500, (0, 0, 0), (40, 8, 40), down=True)
    first, hit = _compare(pl, np_, shapes, rays)
    static = sc.mass == 0
    assert static[first["hitBody"][hit]].any() and (~static[first["hitBody"][hit]]).any()
    # the same rays ignoring the body each one hit first: they go on to the next body behind it
    again = np.zeros(len(rays), capi.RAYHIT)
    again["hitBody"] = -1
    again["hitResult2"] = np.where(hit, first["hitBody"], -1)
    g2, hit2 = _compare(pl, np_, shapes, rays, again)
    assert not (g2["hitBody"][hit2] == first["hitBody"][hit2]).any()
    assert (g2["hitFraction"][hit] >= first["hitFraction"][hit]).all()


def test_rays_see_only_their_scene():
    sc = scenes.batched_piles(24, seed=8, separate=True)
    np_, bp, pl, shapes = load(sc, use_cuda_graph=True)
    for _ in range(30):
        pl.stepSimulation(1 / 60)
    pl.synchronize()
    rng = np.random.Generator(np.random.PCG64(4))
    rays = _rays(rng, 2400, (-5, 0, -5), (5, 6, 5), down=True)
    rays["from"][:, 3] = np.repeat(np.arange(24), 100).astype(np.float32)
    g, hit = _compare(pl, np_, shapes, rays, body_scene=sc.scene_of)
    assert (sc.scene_of[g["hitBody"][hit]] == rays["from"][hit, 3].astype(int)).all()
    assert hit.mean() > 0.1  # small piles cover part of the ray footprint


def test_device_buffers_give_the_host_call_hits():
    torch = pytest.importorskip("torch")
    sc = scenes.box_stack(12, 6, 12, seed=5)
    np_, bp, pl, shapes = load(sc)
    rng = np.random.Generator(np.random.PCG64(9))
    rays = np.concatenate([_rays(rng, 3000, (-7, 0, -7), (7, 6, 7), down=True),
                           _rays(rng, 3000, (-7, 0, -7), (7, 6, 7))])
    host = pl.castRays(rays)
    d_rays = torch.from_numpy(rays.view(np.uint8)).cuda()
    h0 = np.zeros(len(rays), capi.RAYHIT)
    h0["hitBody"] = -1
    h0["hitResult2"] = -1
    d_hits = torch.from_numpy(h0.view(np.uint8)).cuda()
    torch.cuda.synchronize()
    pl.castRaysDevice(d_rays.data_ptr(), d_hits.data_ptr(), len(rays))
    pl.synchronize()
    dev = d_hits.cpu().numpy().view(capi.RAYHIT)
    assert np.array_equal(dev.view(np.uint8), host.view(np.uint8))


def test_rays_match_reference_host_twin():
    # the golden hits of the reference's own b3GpuRaycast::castRaysHost (rotated boxes and Gaussian
    # hulls on a plane, reference hull tables): same hit bodies and faces, fractions within the
    # tolerance the host twin's matrix transform allows; and bit for bit the oracle's
    from conftest import load_golden, shapes_from
    from gpu_helpers import scene_from_golden
    from test_oracle_golden import _ray_close
    g = load_golden("rays")
    sc = scene_from_golden(g)
    np_, bp, pl, shapes = load(sc)
    b = np_.readbackAllBodiesToCpu()
    assert np.array_equal(b["pos"], g["bodies"]["pos"]) and np.array_equal(b["quat"], g["bodies"]["quat"])
    hits = pl.castRays(g["rays"])
    hit = _ray_close(hits, g["hits"], g["rays"])
    assert hit.sum() > 1000
    o = O.cast_rays(b, shapes_from(g), g["rays"])
    assert np.array_equal(hits["hitFraction"], o["hitFraction"]) and np.array_equal(hits["hitBody"], o["hitBody"])
