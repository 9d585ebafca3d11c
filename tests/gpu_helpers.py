"""Helpers shared by the GPU parity tests: load scenes/golden fixtures into a GPU world and run
the stages one by one through the C ABI."""
from __future__ import annotations

import numpy as np

from bullet3_gb300 import capi, scenes
from bullet3_gb300.pipeline import b3Config
from oracle import oracle as O


def scene_from_golden(d) -> scenes.Scene:
    """A Scene whose collidables reproduce the fixture's shape tables in the same order."""
    cols, hulls, faces = d["shape_collidables"], d["shape_hulls"], d["shape_faces"]
    idx, verts, edges = d["shape_indices"], d["shape_verts"], d["shape_edges"]
    sc = scenes.Scene(name="golden")
    for c in cols:
        t = int(c["shapeType"])
        if t == capi.SHAPE_PLANE:
            f = faces[c["shapeIndex"]]
            sc.shapes.append({"type": "plane", "normal": tuple(float(x) for x in f["plane"][:3]),
                              "constant": float(f["plane"][3])})
        elif t == capi.SHAPE_SPHERE:
            sc.shapes.append({"type": "sphere", "radius": float(c["radius"])})
        else:
            h = hulls[c["shapeIndex"]]
            v = verts[h["vertexOffset"]:h["vertexOffset"] + h["numVertices"], :3]
            fs = faces[h["faceOffset"]:h["faceOffset"] + h["numFaces"]]
            ix = np.concatenate([idx[f["indexOffset"]:f["indexOffset"] + f["numIndices"]] for f in fs])
            e = edges[h["uniqueEdgesOffset"]:h["uniqueEdgesOffset"] + h["numUniqueEdges"], :3]
            sc.shapes.append({"type": "hull_tables", "verts": v, "planes": fs["plane"], "face_counts": fs["numIndices"],
                              "indices": ix, "edges": e})
    b = d["bodies"]
    sc.body_shape = b["collidableIdx"].astype(np.int32)
    sc.mass = np.where(b["invMass"] != 0, 1.0 / np.where(b["invMass"] != 0, b["invMass"], 1), 0).astype(np.float32)
    sc.pos = b["pos"][:, :3].copy()
    sc.orn = b["quat"].copy()
    return sc


def load(scene, **cfg):
    c = b3Config(use_cuda_graph=False)
    for k, v in cfg.items():
        if not hasattr(c, k):  # a misspelt setting must not pass silently
            raise AttributeError(k)
        setattr(c, k, v)
    np_, bp, pl = scenes.load_scene(scene, c)
    shapes = O.Shapes.from_tables(scenes.registered_tables(np_))
    return np_, bp, pl, shapes


def pairs_xy(p):
    return np.stack([p["x"], p["y"]], 1)


def valid_points_equal(a, b):
    """Manifolds equal on their valid points (unused point slots carry no data)."""
    if len(a) != len(b):
        return False
    if not np.array_equal(a["normal"], b["normal"]):
        return False
    for f in ("bodyA", "bodyB", "frictionCmp", "restitutionCmp"):
        if not np.array_equal(a[f], b[f]):
            return False
    npts = a["normal"][:, 3].astype(int)
    valid = np.arange(4)[None, :] < npts[:, None]
    return np.array_equal(a["worldPosB"][valid], b["worldPosB"][valid])


def run_stages(np_, bp, pl, dt=1 / 60, solve=True):
    pl.setupGpuAabbsFull()
    bp.calculateOverlappingPairs()
    np_.computeContacts()
    if solve:
        pl.solveContacts(dt)
    pl.synchronize()
