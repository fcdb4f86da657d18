"""Ray queries of the oracle against the reference's own Scene::intersect /
intersectAny (CPU only): the two-level BVH (AccelerationStructure.h:94-156), the
object-space transform (Object.h:44-85), the watertight triangle test
(TriangleIndexed.h:75-177) and the shell-mapping discard (TriangleIndexed.h:221-256)
return the same hit distance, object, point and shading normal bit for bit on random
rays, on finite and infinite extents, and on rays aimed exactly at triangle vertices
and edge midpoints."""
import numpy as np
import pytest

from oracle.bindings import load_scene
from xitils_gb300 import scenes


def _have_reference():
    try:
        load_scene(scenes.cornell(8, 8, 1), "reference")
        return True
    except Exception:
        return False


pytestmark = pytest.mark.skipif(not _have_reference(), reason="reference checker not staged")

SCENES = {
    "cornell": lambda: scenes.cornell(8, 8, 1),
    "sandbox": lambda: scenes.simple_path_tracer_scene(8, 8, 1),
    "terrain": lambda: scenes.terrain(grid=33, width=8, height=8, spp=1, env_size=(16, 8)),
    "shell": lambda: scenes.shell_fabric(8, 8, 1, grid=8, tex_res=32, layers=4),
}


def _rays(desc, n, seed):
    """Random rays from inside the scene's bounds, plus rays from random origins aimed at
    vertices and edge midpoints of its meshes (world space)."""
    rng = np.random.default_rng(seed)
    pts = []
    for o in desc.objects:
        m = desc.meshes[o.mesh]
        M = np.asarray(o.transform.mat, np.float64).reshape(4, 4)
        P = np.c_[m.pos, np.ones(len(m.pos))] @ M.T
        P = P[:, :3] / P[:, 3:]
        tri = m.idx.reshape(-1, 3)
        take = tri[rng.integers(0, len(tri), min(len(tri), n // 8))]
        pts.append(P[take[:, 0]])
        pts.append(0.5 * (P[take[:, 0]] + P[take[:, 1]]))
    targets = np.concatenate(pts)
    lo, hi = targets.min(0), targets.max(0)
    pad = 0.25 * (hi - lo) + 1e-3
    org = rng.uniform(lo - pad, hi + pad, (n, 3))
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    k = min(len(targets), n // 2)
    aim = targets[rng.integers(0, len(targets), k)] - org[:k]
    d[:k] = aim / np.linalg.norm(aim, axis=1, keepdims=True)
    tmax = np.where(rng.uniform(size=n) < 0.5, np.inf, rng.uniform(0.05, 2.0, n) * np.linalg.norm(hi - lo + pad))
    return np.c_[org, d, tmax].astype(np.float32)


@pytest.mark.parametrize("name", list(SCENES))
def test_intersect_matches_reference(name):
    d = SCENES[name]()
    port, ref = load_scene(d, "port"), load_scene(d, "reference")
    rays = _rays(d, 20_000, seed=sum(map(ord, name)))
    a, b = port.intersect(rays), ref.intersect(rays)
    hit = a[1] >= 0
    assert 0.2 < hit.mean() < 1.0
    for x, y in zip(a, b):
        assert np.array_equal(x, y)
    assert np.array_equal(port.intersect_any(rays), ref.intersect_any(rays))
    assert np.array_equal(port.intersect_any(rays), hit.astype(np.int32))
