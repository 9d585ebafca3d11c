"""Seeded synthetic scenes with the shapes, sizes and value distributions of the benchmark
configurations (numpy.random.Generator(PCG64(seed))).

  box_pile       unit boxes (8-vertex hulls, half extent 0.5, mass 1) on a lattice above a static
                 plane y=0; 10x10x10 spacing 1.1 jitter 0.01 (1,000 boxes) or 64x64x64 jitter 0.05
                 (262,144 boxes)
  mixed_scene    uniform positions in a cube, uniform random orientations; 50% boxes with half
                 extents U[0.2,0.6], 25% spheres r U[0.2,0.5], 25% hulls of 12-32 N(0, 0.4^2) points;
                 linear velocities N(0,1)
  batched_piles  many independent box/sphere piles, each on its own plane, body counts log-uniform
  compound_scene compounds of convex hulls (an L of two boxes, a dumbbell of two hulls and a box)
                 among boxes and hulls over a plane
  terrain_scene  boxes, hulls and compounds on a static concave height-field mesh

A Scene is plain numpy data; `load_scene` registers it through the reference-style API.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from . import capi


@dataclass
class Scene:
    shapes: list = field(default_factory=list)        # dicts: type hull/sphere/plane + parameters
    body_shape: np.ndarray = None                     # (N,) shape index per body
    mass: np.ndarray = None                           # (N,)
    pos: np.ndarray = None                            # (N,3)
    orn: np.ndarray = None                            # (N,4) x,y,z,w
    linvel: np.ndarray = None                         # (N,3) or None
    angvel: np.ndarray = None
    cell: float = 0.0                                 # grid cell size (0 = automatic)
    name: str = ""
    pairs_per_body: int = 0                           # pair capacity hint (0 = the library default)
    joints: list = field(default_factory=list)        # dicts: type p2p/fixed, a, b, pivot_a, pivot_b, rel, threshold

    @property
    def num_bodies(self) -> int:
        return len(self.mass)


def box_vertices(hx, hy, hz) -> np.ndarray:
    s = np.array([[x, y, z] for x in (-1, 1) for y in (-1, 1) for z in (-1, 1)], np.float32)
    return s * np.array([hx, hy, hz], np.float32)


def random_quaternions(rng, n) -> np.ndarray:
    q = rng.standard_normal((n, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    return q.astype(np.float32)


def batched_piles(n_scenes=4096, seed=0, min_bodies=8, max_bodies=256, spacing=1.1, base_y=0.6, jitter=0.01,
                  half=0.5, sphere_fraction=0.5, pitch=None, separate=False) -> Scene:
    """Many independent piles.  Body counts floor(exp(U(ln 8, ln 257))) clipped to [8, 256] (mean
    ~72); each pile is a jittered lattice (spacing 1.1, base 0.6, jitter 0.01, zero velocity, mass 1)
    of unit boxes and spheres of radius 0.5.

    separate=False: one shared plane y = 0, piles laid out on a square grid of scene cells far
    enough apart that no two interact; `scene_of` (per body: pile index, -1 for the plane) and
    `scene_offsets` (first body per pile).
    separate=True: independent scenes all at the origin, each with its own plane as its first
    body; `scene_first` (first body of each scene) is the offset table for setSceneOffsets and
    `scene_of` gives every body's scene."""
    rng = np.random.Generator(np.random.PCG64(seed))
    counts = np.clip(np.floor(np.exp(rng.uniform(np.log(min_bodies), np.log(max_bodies + 1), n_scenes))),
                     min_bodies, max_bodies).astype(int)
    side = int(np.ceil(np.sqrt(n_scenes)))
    foot = int(np.ceil(np.sqrt(max_bodies / 4.0)))  # lattice columns per side at 4 layers
    pitch = pitch if pitch else foot * spacing + 4.0
    sc = Scene(name=f"batched_{'scenes' if separate else 'piles'}_{n_scenes}")
    sc.shapes.append({"type": "plane", "normal": (0.0, 1.0, 0.0), "constant": 0.0})
    sc.shapes.append({"type": "hull", "verts": box_vertices(half, half, half)})
    sc.shapes.append({"type": "sphere", "radius": half})
    shapes, pos, scene_of, offsets, first = ([], [], [], [], []) if separate else ([0], [np.zeros(3)], [-1], [], [])
    for s, n in enumerate(counts):
        cx, cz = (0.0, 0.0) if separate else ((s % side) * pitch, (s // side) * pitch)
        if separate:
            first.append(len(shapes))
            shapes.append(0)
            pos.append(np.zeros(3))
            scene_of.append(s)
        cols = max(1, int(np.ceil(np.sqrt(n / 4.0))))
        layers = int(np.ceil(n / (cols * cols)))
        ii, kk, jj = np.meshgrid(np.arange(cols), np.arange(cols), np.arange(layers), indexing="ij")
        lat = np.stack([ii.ravel(), jj.ravel(), kk.ravel()], 1)
        lat = lat[np.lexsort((lat[:, 2], lat[:, 0], lat[:, 1]))][:n]  # bottom layers first
        p = np.stack([cx + (lat[:, 0] - (cols - 1) * 0.5) * spacing, base_y + lat[:, 1] * spacing,
                      cz + (lat[:, 2] - (cols - 1) * 0.5) * spacing], 1)
        p = p + rng.uniform(-jitter, jitter, p.shape)
        kind = np.where(rng.uniform(size=n) < sphere_fraction, 2, 1)
        offsets.append(len(shapes))
        shapes.extend(kind.tolist())
        pos.extend(list(p))
        scene_of.extend([s] * n)
    sc.body_shape = np.array(shapes, np.int32)
    sc.mass = np.where(sc.body_shape == 0, 0.0, 1.0).astype(np.float32)
    sc.pos = np.array(pos, np.float32)
    sc.orn = np.tile(np.array([0, 0, 0, 1], np.float32), (len(shapes), 1))
    sc.scene_of = np.array(scene_of, np.int32)
    sc.scene_offsets = np.array(offsets, np.int32)
    if separate:
        sc.scene_first = np.array(first, np.int32)
    return sc


def scene_part(sc: Scene, s: int) -> Scene:
    """Scene `s` of a separate-scenes batch as a world of its own (same shapes, bodies in order)."""
    first = sc.scene_first
    a = int(first[s])
    b = int(first[s + 1]) if s + 1 < len(first) else sc.num_bodies
    out = Scene(shapes=sc.shapes, body_shape=sc.body_shape[a:b].copy(), mass=sc.mass[a:b].copy(),
                pos=sc.pos[a:b].copy(), orn=sc.orn[a:b].copy(), cell=sc.cell, name=f"{sc.name}[{s}]")
    if sc.linvel is not None:
        out.linvel = sc.linvel[a:b].copy()
    return out


def box_pile(nx=10, ny=10, nz=10, spacing=1.1, base_y=0.6, jitter=0.01, half=0.5, mass=1.0, seed=0,
             plane=True) -> Scene:
    rng = np.random.Generator(np.random.PCG64(seed))
    sc = Scene(name=f"box_pile_{nx}x{ny}x{nz}")
    if plane:
        sc.shapes.append({"type": "plane", "normal": (0.0, 1.0, 0.0), "constant": 0.0})
    sc.shapes.append({"type": "hull", "verts": box_vertices(half, half, half)})
    box = len(sc.shapes) - 1
    ii, jj, kk = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    p = np.stack([ii.ravel() * spacing, base_y + jj.ravel() * spacing, kk.ravel() * spacing], axis=1)
    p = p - np.array([(nx - 1) * spacing * 0.5, 0.0, (nz - 1) * spacing * 0.5])
    p = p + rng.uniform(-jitter, jitter, p.shape)
    n = len(p)
    shapes = [box] * n
    masses = [mass] * n
    pos = list(p)
    if plane:
        shapes = [0] + shapes
        masses = [0.0] + masses
        pos = [np.zeros(3)] + pos
    sc.body_shape = np.array(shapes, np.int32)
    sc.mass = np.array(masses, np.float32)
    sc.pos = np.array(pos, np.float32)
    sc.orn = np.tile(np.array([0, 0, 0, 1], np.float32), (len(sc.mass), 1))
    return sc


def box_stack(nx=64, ny=64, nz=64, spacing=1.1, jitter=0.05, half=0.5, mass=1.0, seed=0, overlap=0.005) -> Scene:
    """Settled form of the box_pile lattice: every lattice column rests on the plane as a stack
    (each box `overlap` into the one below), lattice x/z positions with the same jitter."""
    rng = np.random.Generator(np.random.PCG64(seed))
    sc = Scene(name=f"box_stack_{nx}x{ny}x{nz}")
    sc.shapes.append({"type": "plane", "normal": (0.0, 1.0, 0.0), "constant": 0.0})
    sc.shapes.append({"type": "hull", "verts": box_vertices(half, half, half)})
    ii, jj, kk = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    p = np.stack([ii.ravel() * spacing, half - overlap + jj.ravel() * (2 * half - overlap), kk.ravel() * spacing], 1)
    p = p - np.array([(nx - 1) * spacing * 0.5, 0.0, (nz - 1) * spacing * 0.5])
    j = rng.uniform(-jitter, jitter, p.shape)
    j[:, 1] = 0.0
    p = p + j
    n = len(p)
    sc.body_shape = np.array([0] + [1] * n, np.int32)
    sc.mass = np.array([0.0] + [mass] * n, np.float32)
    sc.pos = np.vstack([np.zeros((1, 3)), p]).astype(np.float32)
    sc.orn = np.tile(np.array([0, 0, 0, 1], np.float32), (n + 1, 1))
    return sc


def mixed_scene(n=131072, extent=64.0, seed=0, velocity_sigma=1.0, plane=False, cell_factor=2.0) -> Scene:
    rng = np.random.Generator(np.random.PCG64(seed))
    sc = Scene(name=f"mixed_{n}")
    kinds = rng.permutation(np.repeat([0, 1, 2], [n // 2, n // 4, n - n // 2 - n // 4]))
    shapes, masses = [], []
    max_ext = 0.0
    if plane:
        sc.shapes.append({"type": "plane", "normal": (0.0, 1.0, 0.0), "constant": 0.0})
    for k in kinds:
        if k == 0:
            h = rng.uniform(0.2, 0.6, 3).astype(np.float32)
            sc.shapes.append({"type": "hull", "verts": box_vertices(*h)})
            max_ext = max(max_ext, 2 * float(h.max()))
        elif k == 1:
            r = float(rng.uniform(0.2, 0.5))
            sc.shapes.append({"type": "sphere", "radius": r})
            max_ext = max(max_ext, 2 * r)
        else:
            m = int(rng.integers(12, 33))
            pts = (rng.standard_normal((m, 3)) * 0.4).astype(np.float32)
            sc.shapes.append({"type": "hull", "verts": pts})
            max_ext = max(max_ext, float((pts.max(0) - pts.min(0)).max()))
        shapes.append(len(sc.shapes) - 1)
        masses.append(1.0)
    pos = rng.uniform(0.0, extent, (n, 3)).astype(np.float32)
    orn = random_quaternions(rng, n)
    vel = (rng.standard_normal((n, 3)) * velocity_sigma).astype(np.float32)
    if plane:
        shapes = [0] + shapes
        masses = [0.0] + masses
        pos = np.vstack([np.zeros((1, 3), np.float32), pos])
        orn = np.vstack([np.array([[0, 0, 0, 1]], np.float32), orn])
        vel = np.vstack([np.zeros((1, 3), np.float32), vel])
    sc.body_shape = np.array(shapes, np.int32)
    sc.mass = np.array(masses, np.float32)
    sc.pos = pos
    sc.orn = orn
    sc.linvel = vel
    sc.cell = cell_factor * max_ext
    return sc


def compound_scene(n=2048, extent=None, seed=0, plane=True, velocity_sigma=0.5, lattice=False) -> Scene:
    """Compounds of convex hulls among single hulls: an L of two boxes (0.5 x 0.25 x 0.25 and
    0.25 x 0.5 x 0.25 half extents), a dumbbell (two hulls of 20 N(0, 0.3^2) points at x = +-0.6
    around a 0.5 x 0.25 x 0.25 box), that box and that hull alone, in turn, over a plane y = 0.
    Uniform positions (x, z in [0, extent), y in [0, 1.5 + extent / 8)) with random orientations
    and N(0, velocity_sigma^2) velocities, or with lattice=True a jittered lattice spaced by the
    widest body's reach (random orientations, at rest, nothing overlapping) that settles into a
    pile."""
    rng = np.random.Generator(np.random.PCG64(seed))
    sc = Scene(name=f"compound_{n}")
    if plane:
        sc.shapes.append({"type": "plane", "normal": (0.0, 1.0, 0.0), "constant": 0.0})
    base = len(sc.shapes)
    gauss = (rng.standard_normal((20, 3)) * 0.3).astype(np.float32)
    sc.shapes += [{"type": "hull", "verts": box_vertices(0.5, 0.25, 0.25)},
                  {"type": "hull", "verts": box_vertices(0.25, 0.5, 0.25)},
                  {"type": "hull", "verts": gauss}]
    bx, by, gh = base, base + 1, base + 2
    q0 = (0.0, 0.0, 0.0, 1.0)
    sc.shapes.append({"type": "compound", "children": [(bx, (0.25, 0.0, 0.0), q0), (by, (0.0, 0.5, 0.0), q0)]})
    qa, qb = random_quaternions(rng, 2)
    sc.shapes.append({"type": "compound", "children": [(gh, (-0.6, 0.0, 0.0), tuple(qa)), (bx, (0.0, 0.0, 0.0), q0),
                                                        (gh, (0.6, 0.0, 0.0), tuple(qb))]})
    kinds = np.array([base + 3, base + 4, bx, gh], np.int32)[np.arange(n) % 4]
    # the widest body: the dumbbell, its hulls' farthest points 0.6 off the centre
    reach = 0.6 + float(np.linalg.norm(gauss, axis=1).max())
    if lattice:
        side = int(np.ceil(np.sqrt(n / 4)))
        i = np.arange(n)
        sp = 2.0 * reach + 0.1  # no two bodies and no body and the plane overlap at the start
        pos = np.stack([(i % side) * sp, reach + 0.1 + (i // (side * side)) * sp, ((i // side) % side) * sp], 1)
        pos = (pos + rng.uniform(-0.04, 0.04, (n, 3))).astype(np.float32)
        vel = np.zeros((n, 3), np.float32)
    else:
        extent = extent if extent is not None else float(np.sqrt(n) * 0.6)
        pos = np.stack([rng.uniform(0, extent, n), rng.uniform(0, 1.5 + extent / 8, n), rng.uniform(0, extent, n)],
                       1).astype(np.float32)
        vel = (rng.standard_normal((n, 3)) * velocity_sigma).astype(np.float32)
    orn = random_quaternions(rng, n)
    if plane:
        kinds = np.concatenate([[0], kinds]).astype(np.int32)
        pos = np.vstack([np.zeros((1, 3), np.float32), pos])
        orn = np.vstack([np.array([[0, 0, 0, 1]], np.float32), orn])
        vel = np.vstack([np.zeros((1, 3), np.float32), vel])
    sc.body_shape = kinds
    sc.mass = np.where(kinds == 0, 0.0, 1.0).astype(np.float32) if plane else np.ones(n, np.float32)
    sc.pos, sc.orn, sc.linvel = pos, orn, vel
    sc.cell = 2.0 * 2.0 * reach
    return sc


def terrain_mesh(grid=64, cell=1.0, amplitude=1.5, seed=0):
    """A height field as a triangle mesh: (grid + 1)^2 vertices (x, h, z), x and z multiples of cell,
    h a sum of two sines plus N(0, 0.05^2); two triangles per quad, row by row, wound so that their
    normals point up.  Returns (vertices (n, 3) float32, indices (3 t,) int32, height function)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    k = np.arange(grid + 1, dtype=np.float64) * cell
    X, Z = np.meshgrid(k, k, indexing="xy")  # row j (z), column i (x)

    def height(x, z):
        return amplitude * (np.sin(x * 0.35) * np.cos(z * 0.27) + 0.5 * np.sin(0.6 * x + 0.4 * z))

    H = height(X, Z) + rng.normal(0.0, 0.05, X.shape)
    verts = np.stack([X, H, Z], -1).reshape(-1, 3).astype(np.float32)
    idx = []
    w = grid + 1
    for j in range(grid):
        for i in range(grid):
            p00, p10, p01, p11 = j * w + i, j * w + i + 1, (j + 1) * w + i, (j + 1) * w + i + 1
            idx += [p00, p01, p10, p10, p01, p11]
    return verts, np.array(idx, np.int32), height


def terrain_scene(n=2048, grid=64, cell=1.0, seed=0, drop=False, velocity_sigma=0.3, spheres=True) -> Scene:
    """A static concave height-field mesh (terrain_mesh, body 0 at the identity pose) under boxes
    (half extents 0.5 x 0.25 x 0.25), 20-point Gaussian hulls, compounds (an L of two boxes, a
    dumbbell of two hulls around a box) and, with spheres, spheres of radius 0.3, in turn.  Either scattered just over the surface with
    random orientations and N(0, velocity_sigma^2) velocities (heights from 0.2 below the surface to
    0.6 above it, so that many touch it), or (drop=True) a lattice of them at rest, from 2 above
    the highest point, that falls onto it."""
    rng = np.random.Generator(np.random.PCG64(seed))
    sc = Scene(name=f"terrain_{n}")
    verts, idx, height = terrain_mesh(grid, cell, seed=seed)
    sc.shapes.append({"type": "mesh", "verts": verts, "indices": idx})
    gauss = (rng.standard_normal((20, 3)) * 0.3).astype(np.float32)
    sc.shapes += [{"type": "hull", "verts": box_vertices(0.5, 0.25, 0.25)},
                  {"type": "hull", "verts": box_vertices(0.25, 0.5, 0.25)},
                  {"type": "hull", "verts": gauss}]
    q0 = (0.0, 0.0, 0.0, 1.0)
    sc.shapes.append({"type": "compound", "children": [(1, (0.25, 0.0, 0.0), q0), (2, (0.0, 0.5, 0.0), q0)]})
    qa, qb = random_quaternions(rng, 2)
    sc.shapes.append({"type": "compound", "children": [(3, (-0.6, 0.0, 0.0), tuple(qa)), (1, (0.0, 0.0, 0.0), q0),
                                                        (3, (0.6, 0.0, 0.0), tuple(qb))]})
    kinds = [1, 3, 4, 5]
    if spheres:
        sc.shapes.append({"type": "sphere", "radius": 0.3})
        kinds.append(6)
    kinds = np.array(kinds, np.int32)[np.arange(n) % len(kinds)]
    reach = 0.6 + float(np.linalg.norm(gauss, axis=1).max())
    span = grid * cell
    if drop:
        sp = 2.0 * reach + 0.1  # nothing overlaps at the start
        side = max(1, min(int(np.ceil(np.sqrt(n / 3))), int((span - 2 * reach) // sp) + 1))
        i = np.arange(n)
        top = float(verts[:, 1].max()) + reach + 2.0
        pos = np.stack([reach + (i % side) * sp, top + (i // (side * side)) * (2.0 * reach + 0.1),
                        reach + ((i // side) % side) * sp], 1)
        pos = (pos + rng.uniform(-0.04, 0.04, (n, 3))).astype(np.float32)
        vel = np.zeros((n, 3), np.float32)
    else:
        x = rng.uniform(reach, span - reach, n)
        z = rng.uniform(reach, span - reach, n)
        pos = np.stack([x, height(x, z) + rng.uniform(-0.2, 0.6, n), z], 1).astype(np.float32)
        vel = (rng.standard_normal((n, 3)) * velocity_sigma).astype(np.float32)
    orn = random_quaternions(rng, n)
    sc.body_shape = np.concatenate([[0], kinds]).astype(np.int32)
    sc.mass = np.concatenate([[0.0], np.ones(n)]).astype(np.float32)
    sc.pos = np.vstack([np.zeros((1, 3), np.float32), pos])
    sc.orn = np.vstack([np.array([[0, 0, 0, 1]], np.float32), orn])
    sc.linvel = np.vstack([np.zeros((1, 3), np.float32), vel])
    sc.cell = 4.0 * reach
    return sc


def static_field(n_static=2000, n_dynamic=6000, extent=100.0, seed=0, plane=True, scenes=1) -> Scene:
    """Large finite static bodies with small dynamic ones among them: static boxes with half
    extents U[0.5, 6] (mass 0, random rotation about y) spread over an extent x extent area at
    heights U[0, 4], and dynamic boxes (half extents U[0.2, 0.5]) and spheres (r U[0.2, 0.5]) at
    heights U[0, 8] with N(0, 1) velocities, over a plane y = 0.  With scenes > 1 the bodies are
    split into that many independent scenes (each with its own plane), all in the same region;
    `scene_first` is the offset table."""
    rng = np.random.Generator(np.random.PCG64(seed))
    sc = Scene(name=f"static_field_{n_static}_{n_dynamic}")
    sc.shapes.append({"type": "plane", "normal": (0.0, 1.0, 0.0), "constant": 0.0})
    shapes, masses, pos, orn, vel, first = [], [], [], [], [], []
    per_s, per_d = n_static // scenes, n_dynamic // scenes
    for k in range(scenes):
        first.append(len(shapes))
        if plane:
            shapes.append(0)
            masses.append(0.0)
            pos.append(np.zeros(3))
            orn.append(np.array([0, 0, 0, 1.0]))
            vel.append(np.zeros(3))
        for _ in range(per_s):
            h = rng.uniform(0.5, 6.0, 3)
            sc.shapes.append({"type": "hull", "verts": box_vertices(*h)})
            shapes.append(len(sc.shapes) - 1)
            masses.append(0.0)
            pos.append(np.array([rng.uniform(0, extent), rng.uniform(0, 4), rng.uniform(0, extent)]))
            a = rng.uniform(0, np.pi)
            orn.append(np.array([0.0, np.sin(a / 2), 0.0, np.cos(a / 2)]))
            vel.append(np.zeros(3))
        for _ in range(per_d):
            if rng.uniform() < 0.5:
                sc.shapes.append({"type": "hull", "verts": box_vertices(*rng.uniform(0.2, 0.5, 3))})
            else:
                sc.shapes.append({"type": "sphere", "radius": float(rng.uniform(0.2, 0.5))})
            shapes.append(len(sc.shapes) - 1)
            masses.append(1.0)
            pos.append(np.array([rng.uniform(0, extent), rng.uniform(0, 8), rng.uniform(0, extent)]))
            orn.append(random_quaternions(rng, 1)[0])
            vel.append(rng.standard_normal(3))
    sc.body_shape = np.array(shapes, np.int32)
    sc.mass = np.array(masses, np.float32)
    sc.pos = np.array(pos, np.float32)
    sc.orn = np.array(orn, np.float32)
    sc.linvel = np.array(vel, np.float32)
    if scenes > 1:
        sc.scene_first = np.array(first, np.int32)
    return sc


def stress_container(n=1048576, width=128.0, depth=128.0, height=512.0, seed=0, cell_factor=2.0) -> Scene:
    """The collision-at-scale shape mix poured into a static container: 50% boxes (half extents
    U[0.2, 0.6]), 25% spheres (r U[0.2, 0.5]), 25% hulls of 12-32 N(0, 0.4^2) points, uniform random
    orientations, zero velocity, x in U[1, width-1], z in U[1, depth-1], y in U[0, height]; the
    container is five static planes (floor y = 0 and the walls x = 0, x = width, z = 0, z = depth,
    normals pointing inwards).  Grid cell = cell_factor x the largest AABB extent."""
    rng = np.random.Generator(np.random.PCG64(seed))
    sc = Scene(name=f"stress_{n}")
    walls = [((0.0, 1.0, 0.0), 0.0), ((1.0, 0.0, 0.0), 0.0), ((-1.0, 0.0, 0.0), -width), ((0.0, 0.0, 1.0), 0.0),
             ((0.0, 0.0, -1.0), -depth)]
    for nrm, c in walls:  # plane n . p = c
        sc.shapes.append({"type": "plane", "normal": nrm, "constant": c})
    kinds = rng.permutation(np.repeat([0, 1, 2], [n // 2, n // 4, n - n // 2 - n // 4]))
    shapes = list(range(len(walls)))
    max_ext = 0.0
    for k in kinds:
        if k == 0:
            h = rng.uniform(0.2, 0.6, 3).astype(np.float32)
            sc.shapes.append({"type": "hull", "verts": box_vertices(*h)})
            max_ext = max(max_ext, 2 * float(h.max()))
        elif k == 1:
            r = float(rng.uniform(0.2, 0.5))
            sc.shapes.append({"type": "sphere", "radius": r})
            max_ext = max(max_ext, 2 * r)
        else:
            pts = (rng.standard_normal((int(rng.integers(12, 33)), 3)) * 0.4).astype(np.float32)
            sc.shapes.append({"type": "hull", "verts": pts})
            max_ext = max(max_ext, float((pts.max(0) - pts.min(0)).max()))
        shapes.append(len(sc.shapes) - 1)
    pos = np.stack([rng.uniform(1.0, width - 1.0, n), rng.uniform(0.0, height, n), rng.uniform(1.0, depth - 1.0, n)], 1)
    nw = len(walls)
    sc.body_shape = np.array(shapes, np.int32)
    sc.mass = np.concatenate([np.zeros(nw), np.ones(n)]).astype(np.float32)
    sc.pos = np.vstack([np.zeros((nw, 3)), pos]).astype(np.float32)
    sc.orn = np.vstack([np.tile([0, 0, 0, 1.0], (nw, 1)), random_quaternions(rng, n)]).astype(np.float32)
    sc.cell = cell_factor * max_ext
    sc.pairs_per_body = 48  # the settled pour reaches ~24 overlapping AABBs per body
    return sc


def hanging_chains(n_chains=8, links=12, spacing=1.0, radius=0.2, seed=0, fixed_every=0, threshold=1e30,
                   anchor_index=0, ground=False, swing=1.0, random_orn=True, per_row=0) -> Scene:
    """Chains of spheres hanging from one static anchor box, neighbours joined by ball joints at
    the midpoint (every fixed_every-th joint a fixed joint holding the initial relative
    orientation).  The anchor is body `anchor_index` (0 or the last body).  Links start with
    random horizontal velocities of about `swing` m/s; chains are 3 apart (in a row along x, or
    in rows of `per_row` chains along z), links do not touch.
    random_orn=False starts every link unrotated (the fixed joints' target is then the identity,
    the case the reference's fixed-joint rows are built for: they drive wA - wB, the rate of the
    orientation error only while ornA ornB^-1 is near the identity)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    top = links * spacing + 2.0
    nb = n_chains * links + 1 + (1 if ground else 0)
    sc = Scene(name=f"chains{n_chains}x{links}")
    per_row = per_row if per_row > 0 else n_chains
    n_rows = (n_chains + per_row - 1) // per_row
    sc.shapes = [{"type": "hull", "verts": box_vertices(1.5 * per_row + 1.0, 0.1, 1.5 * n_rows)},
                 {"type": "sphere", "radius": radius}]
    if ground:
        sc.shapes.append({"type": "plane", "normal": (0.0, 1.0, 0.0), "constant": 0.0})
    shape = np.ones(nb, np.int32)
    mass = np.ones(nb, np.float32)
    pos = np.zeros((nb, 3), np.float32)
    orn = np.tile(np.array([0, 0, 0, 1], np.float32), (nb, 1))
    anchor = 0 if anchor_index == 0 else nb - 1 - (1 if ground else 0)
    dyn = [i for i in range(nb - (1 if ground else 0)) if i != anchor]
    shape[anchor], mass[anchor] = 0, 0.0
    pos[anchor] = (0.0, top, 0.0)
    if ground:
        shape[nb - 1], mass[nb - 1] = 2, 0.0
    if random_orn:
        orn[dyn] = random_quaternions(rng, len(dyn))
    lin = np.zeros((nb, 3), np.float32)
    dyn = np.asarray(dyn, np.int64)
    c = np.repeat(np.arange(n_chains), links)
    l = np.tile(np.arange(links), n_chains)
    pos[dyn, 0] = 3.0 * (c % per_row - (per_row - 1) / 2)
    pos[dyn, 1] = top - (l + 1) * spacing
    pos[dyn, 2] = 3.0 * (c // per_row - (n_rows - 1) / 2)
    u = rng.uniform(-swing, swing, (len(dyn), 2))
    lin[dyn, 0] = u[:, 0]
    lin[dyn, 2] = u[:, 1]
    # joint k joins link k to the link above it (the anchor for a chain's first link); pivots in
    # each body's own frame at the midpoint between the two centres
    a = np.where(l == 0, anchor, np.roll(dyn, 1))
    b = dyn
    mid = pos[b] + np.array([0.0, 0.5 * spacing, 0.0], np.float32)
    pa = _to_local_n(mid - pos[a], orn[a])
    pb = _to_local_n(mid - pos[b], orn[b])
    rel = _qmul_n(orn[a], _qconj_n(orn[b]))
    fixed = (l % fixed_every == fixed_every - 1) if fixed_every else np.zeros(len(dyn), bool)
    sc.joints = [{"type": "fixed" if fixed[k] else "p2p", "a": int(a[k]), "b": int(b[k]), "threshold": threshold,
                  "pivot_a": pa[k], "pivot_b": pb[k], "rel": rel[k]} for k in range(len(dyn))]
    sc.body_shape, sc.mass, sc.pos, sc.orn, sc.linvel = shape, mass, pos, orn, lin
    return sc


def welded_pairs(n_pairs=64, seed=0, twist=0.3, threshold=1e30) -> Scene:
    """Pairs of boxes far apart from each other, each pair joined by a fixed joint whose target
    relative orientation is the initial one turned by up to `twist` radians, with random spins."""
    rng = np.random.Generator(np.random.PCG64(seed))
    sc = Scene(name=f"welded{n_pairs}")
    sc.shapes = [{"type": "hull", "verts": box_vertices(0.4, 0.3, 0.2)}]
    nb = 2 * n_pairs
    pos = np.zeros((nb, 3), np.float32)
    g = int(np.ceil(np.sqrt(n_pairs)))
    orn = random_quaternions(rng, nb)
    for p in range(n_pairs):
        base = np.array([4.0 * (p % g), 10.0, 4.0 * (p // g)], np.float32)
        pos[2 * p] = base
        pos[2 * p + 1] = base + np.array([1.2, 0.0, 0.0], np.float32)
        axis = rng.standard_normal(3)
        axis /= np.linalg.norm(axis)
        ang = rng.uniform(-twist, twist)
        dq = np.array([*(np.sin(ang / 2) * axis), np.cos(ang / 2)], np.float32)
        mid = pos[2 * p] + np.array([0.6, 0.0, 0.0], np.float32)
        sc.joints.append({"type": "fixed", "a": 2 * p, "b": 2 * p + 1, "threshold": threshold,
                          "pivot_a": _to_local(mid - pos[2 * p], orn[2 * p]),
                          "pivot_b": _to_local(mid - pos[2 * p + 1], orn[2 * p + 1]),
                          "rel": _qmul(dq, _qmul(orn[2 * p], _qconj(orn[2 * p + 1])))})
    sc.body_shape = np.zeros(nb, np.int32)
    sc.mass = rng.uniform(0.5, 2.0, nb).astype(np.float32)
    sc.pos, sc.orn = pos, orn
    sc.linvel = rng.standard_normal((nb, 3)).astype(np.float32)
    sc.angvel = (2.0 * rng.standard_normal((nb, 3))).astype(np.float32)
    return sc


def _qconj_n(q):
    q = np.asarray(q, np.float64)
    return np.concatenate([-q[:, :3], q[:, 3:4]], 1)


def _qmul_n(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    v = np.cross(a[:, :3], b[:, :3]) + a[:, 3:4] * b[:, :3] + b[:, 3:4] * a[:, :3]
    w = a[:, 3] * b[:, 3] - np.einsum("ij,ij->i", a[:, :3], b[:, :3])
    return np.concatenate([v, w[:, None]], 1).astype(np.float32)


def _to_local_n(v, q):
    """Rows of v (world) in the frames of the rows of q: q^-1 v q."""
    v4 = np.concatenate([np.asarray(v, np.float64), np.zeros((len(v), 1))], 1)
    return _qmul_n(_qmul_n(_qconj_n(q), v4), q)[:, :3].astype(np.float32)


def _qconj(q):
    return np.array([-q[0], -q[1], -q[2], q[3]], np.float32)


def _qmul(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    v = np.cross(a[:3], b[:3]) + a[3] * b[:3] + b[3] * a[:3]
    return np.array([*v, a[3] * b[3] - np.dot(a[:3], b[:3])], np.float32)


def _to_local(v, q):
    """v (world) in the frame of orientation q: q^-1 v q."""
    r = _qmul(_qmul(_qconj(q), [*v, 0.0]), q)
    return r[:3].astype(np.float32)


def add_joints(pipeline, joints) -> list:
    """Registers joint dicts (as Scene.joints holds them) on a pipeline; returns their uids."""
    uids = []
    for j in joints:
        if j["type"] == "fixed":
            uids.append(pipeline.createFixedConstraint(j["a"], j["b"], j["pivot_a"], j["pivot_b"], j["rel"],
                                                       j["threshold"]))
        else:
            uids.append(pipeline.createPoint2PointConstraint(j["a"], j["b"], j["pivot_a"], j["pivot_b"],
                                                             j["threshold"]))
    return uids


def load_scene(scene: Scene, config=None, device: int = 0, upload: bool = True):
    """Register a Scene through the reference-style API; returns (narrowphase, broadphase, pipeline)."""
    from .pipeline import b3Config, b3GpuGridBroadphase, b3GpuNarrowPhase, b3GpuRigidBodyPipeline
    if config is None:
        config = b3Config()
    config.m_maxConvexBodies = max(config.m_maxConvexBodies, scene.num_bodies)
    config.m_maxConvexShapes = max(config.m_maxConvexShapes, len(scene.shapes))
    if scene.cell and not config.grid_cell_size:
        config.grid_cell_size = scene.cell
    if scene.pairs_per_body and not config.m_maxBroadphasePairs:
        config.m_maxBroadphasePairs = scene.pairs_per_body * scene.num_bodies
    np_ = b3GpuNarrowPhase(config, device)
    bp = b3GpuGridBroadphase()
    pl = b3GpuRigidBodyPipeline(np_, bp, None, config)
    col = []
    for s in scene.shapes:
        if s["type"] == "hull":
            c = np_.registerConvexHullShape(s["verts"])
        elif s["type"] == "sphere":
            c = np_.registerSphereShape(s["radius"])
        elif s["type"] == "plane":
            c = np_.registerPlaneShape(s["normal"], s["constant"])
        elif s["type"] == "hull_tables":
            c = np_.registerConvexHullShapeTables(s["verts"], s["planes"], s["face_counts"], s["indices"],
                                                  s["edges"])
        elif s["type"] == "compound":
            # children: (index of an earlier shape of the scene, position, orientation)
            c = np_.registerCompoundShape([(col[i], p, q) for i, p, q in s["children"]])
        elif s["type"] == "mesh":
            c = np_.registerConcaveMesh(s["verts"], s["indices"], s.get("scaling", (1.0, 1.0, 1.0)))
        else:
            raise ValueError(s["type"])
        if c < 0:
            raise RuntimeError(f"shape registration failed: {s['type']}")
        col.append(c)
    for i in range(scene.num_bodies):
        b = pl.registerPhysicsInstance(float(scene.mass[i]), scene.pos[i], scene.orn[i], col[scene.body_shape[i]], i)
        if b < 0:
            raise RuntimeError("body registration failed")
    if getattr(scene, "scene_first", None) is not None:
        pl.setSceneOffsets(scene.scene_first)
    if scene.joints:
        add_joints(pl, scene.joints)
    if upload:
        pl.writeAllInstancesToGpu()
        if scene.linvel is not None or scene.angvel is not None:
            bodies = np_.readbackAllBodiesToCpu()
            if scene.linvel is not None:
                bodies["linVel"][:, :3] = scene.linvel
            if scene.angvel is not None:
                bodies["angVel"][:, :3] = scene.angvel
            np_.writeBodiesToGpu(bodies)
    return np_, bp, pl


def registered_tables(narrowphase):
    """Host copies of the registered shape tables and bodies (no GPU needed)."""
    import ctypes as C
    h = narrowphase.world.handle
    counts = np.zeros(6, np.int32)
    capi.call("b3g_read_shape_tables", h, None, None, None, None, None, None, None, capi.iptr(counts))
    ncol, nh, nf, ni, nv, ne = (int(x) for x in counts)
    t = {
        "collidables": np.zeros(max(ncol, 1), capi.COLLIDABLE),
        "local_aabbs": np.zeros(max(ncol, 1), capi.AABB),
        "hulls": np.zeros(max(nh, 1), capi.HULL),
        "faces": np.zeros(max(nf, 1), capi.FACE),
        "indices": np.zeros(max(ni, 1), np.int32),
        "verts": np.zeros((max(nv, 1), 4), np.float32),
        "edges": np.zeros((max(ne, 1), 4), np.float32),
    }
    caps = np.array([max(ncol, 1), max(nh, 1), max(nf, 1), max(ni, 1), max(nv, 1), max(ne, 1)], np.int32)
    capi.call("b3g_read_shape_tables", h, capi.ptr(t["collidables"]), capi.ptr(t["hulls"]), capi.ptr(t["faces"]),
              capi.iptr(t["indices"]), capi.ptr(t["verts"]), capi.ptr(t["edges"]), capi.ptr(t["local_aabbs"]),
              capi.iptr(caps))
    nch = C.c_int()
    capi.call("b3g_read_child_shapes", h, None, C.c_int(0), C.byref(nch))
    t["children"] = np.zeros(max(nch.value, 1), capi.CHILD)
    if nch.value:
        capi.call("b3g_read_child_shapes", h, capi.ptr(t["children"]), C.c_int(nch.value), C.byref(nch))
    nb = narrowphase.getNumRigidBodies()
    bodies = np.zeros(nb, capi.BODY)
    inertias = np.zeros(nb, capi.INERTIA)
    capi.call("b3g_read_registered_bodies", h, capi.ptr(bodies), capi.ptr(inertias), C.c_int(nb))
    t["bodies"] = bodies
    t["inertias"] = inertias
    return t
