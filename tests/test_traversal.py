"""Closest-hit and any-hit queries of the GPU BVHs (both builders) against the
oracle's restatement of Scene::intersect / intersectAny on the reference's own
BVH (oracle/xgb_cpu.cpp).

Both sides run the same watertight triangle test in unfused FP32, so a ray that
finds the same triangle gets a bit-identical t. Where two triangles accept a ray
at (nearly) the same t -- a shared edge, or coplanar faces such as a box's
bottom on the floor -- the one the tree visits first wins; on these scenes that
is about 0.15 % of the rays, with the same count for every builder and layout."""
import numpy as np
import pytest

from oracle.bindings import load_scene as load_cpu
from xitils_gb300 import scenes

pytestmark = pytest.mark.gpu


def _rays(desc, n, seed):
    """Rays from random points of a box around the camera and the scene, with
    random directions, half of them with a finite tMax."""
    rng = np.random.default_rng(seed)
    lo, hi = desc.bounds() if hasattr(desc, "bounds") else (np.array([-1.0, -1.0, -1.0]), np.array([1.0, 1.0, 1.0]))
    o = rng.uniform(lo, hi, size=(n, 3))
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    t = np.where(rng.uniform(size=n) < 0.5, np.inf, rng.uniform(0.05, 2.0, size=n) * np.linalg.norm(hi - lo))
    return np.concatenate([o, d, t[:, None]], axis=1).astype(np.float32)


@pytest.fixture(scope="module")
def ctx():
    import __graft_entry__ as g
    g.build()
    from xitils_gb300 import api
    return api.Context(0)


@pytest.mark.parametrize("layout", ["binary", "wide8"])
@pytest.mark.parametrize("builder", ["ploc", "lbvh"])
@pytest.mark.parametrize("make", [
    lambda: scenes.cornell(8, 8, 1),
    lambda: scenes.terrain(grid=129, width=8, height=8, spp=1, env_size=(64, 32)),
    lambda: scenes.occluded_room(8, 8, 1, n_boxes=2000),
])
def test_queries_match_oracle(ctx, builder, layout, make):
    from xitils_gb300 import api
    desc = make()
    ctx.set_bvh_builder(builder)
    ctx.set_bvh_layout(layout)
    try:
        gpu = api.load_scene(ctx, desc)
    finally:
        ctx.set_bvh_builder("ploc")
        ctx.set_bvh_layout("binary")
    cpu = load_cpu(desc, "port")
    rays = _rays(desc, 20000, 7)
    hg, hc = gpu.scene.intersect(rays), cpu.trace(rays)
    hit = hc[:, 1] >= 0
    assert 0.05 < hit.mean() < 0.999
    assert np.array_equal(hg[:, 1] >= 0, hit)
    same = (hg[:, 1] == hc[:, 1]) & (hg[:, 2] == hc[:, 2])
    print(f"{desc.name} [{builder}, {layout}]: hits {hit.mean():.3f}, other triangle {np.sum(~same)}, "
          f"t differs {np.sum(hg[:, 0] != hc[:, 0])} (same triangle: {np.sum((hg[:, 0] != hc[:, 0]) & same)})")
    assert same.mean() >= 0.997
    assert np.array_equal(hg[same, 0], hc[same, 0])               # same triangle: same t, bit for bit
    np.testing.assert_allclose(hg[hit, 0], hc[hit, 0], rtol=1e-5, atol=1e-6)
    b0, b1 = hg[hit, 3], hg[hit, 4]
    assert np.all((b0 >= 0) & (b1 >= 0) & (b0 + b1 <= 1.0 + 1e-6))
    og, oc = gpu.scene.occluded(rays), cpu.occluded(rays)
    assert np.array_equal(og, oc)


@pytest.mark.parametrize("make,tol", [
    (lambda: scenes.terrain(grid=129, width=64, height=64, spp=4, env_size=(128, 64)), 1e-4),
    (lambda: scenes.cornell(48, 48, 4), 1e-4),
    # interpenetrating boxes with faces on the floor: coplanar ties (previous test)
    # send a few of the long room paths (RR only, no depth limit) elsewhere
    (lambda: scenes.occluded_room(48, 48, 4, n_boxes=2000), 2e-3),
])
def test_both_layouts_render_like_oracle(ctx, make, tol):
    """The wavefront's persistent traversal kernels over binary and 8-wide BVHs."""
    from oracle.bindings import relmse
    from xitils_gb300 import api
    desc = make()
    cpu = load_cpu(desc, "port").render_pcg(desc)
    errs = {}
    for layout in ("binary", "wide8"):
        ctx.set_bvh_layout(layout)
        try:
            b = api.load_scene(ctx, desc)
        finally:
            ctx.set_bvh_layout("binary")
        errs[layout] = relmse(api.render_desc(ctx, desc, builder=b), cpu)
    print(desc.name, errs)
    assert max(errs.values()) <= tol
