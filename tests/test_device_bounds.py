"""Device-side traversal bounds run out and come back.

The reference's traversal is recursive and unbounded (its only guard is
Utils.h:21-27's assertion macro); every traversal loop here is bounded. This
file makes each bound run out on ordinary scenes -- a step bound lowered to one
loop step, a stack bound lowered to one entry -- and checks that the render
returns the error status (XGB_DEVICE_TIMEOUT, XGB_QUEUE_OVERFLOW) with the
error bit in the statistics, that nothing faults or hangs (the loops end by
their own bound), and that the same scene on the same context then renders
correctly again (relMSE <= 1e-4 against the oracle) once the bounds are
restored. Every traversal kernel is covered: the one-instance kernel (terrain),
the flat kernel of a few instances (two terrain copies), the 8-wide kernel, the
general two-level kernel (more than 16 instances), the batch path and the ray
queries.
"""
import numpy as np
import pytest

from oracle.bindings import load_scene as load_cpu, relmse
from xitils_gb300 import scenes
from xitils_gb300.transform import scale, translate

pytestmark = pytest.mark.gpu
XGB_QUEUE_OVERFLOW = 4
XGB_DEVICE_TIMEOUT = 5
ERR_STACK, ERR_LOOP = 1, 4


@pytest.fixture(scope="module")
def api_mod():
    import __graft_entry__ as g
    g.build()
    from xitils_gb300 import api
    return api


def _terrain():
    return scenes.terrain(grid=65, width=48, height=40, spp=2, env_size=(128, 64))


def _two_terrains():
    d = _terrain()
    d.name = "two_terrains"
    d.add_object(0, d.objects[0].material, translate(0.0, -0.2, 0.9))
    return d


def _many_instances():
    """The terrain plus 17 small boxes: more than 16 instances."""
    d = _terrain()
    d.name = "terrain_boxes"
    cpos, cidx = scenes.unit_cube_mesh()
    cube = d.add_mesh(cpos, cidx)
    grey = d.diffuse([0.6, 0.6, 0.6])
    rng = np.random.default_rng(3)
    for k in range(17):
        x, z = rng.uniform(0.1, 0.9, 2)
        d.add_object(cube, grey, translate(float(x), 0.2, float(z)) * scale(0.04, 0.04, 0.04))
    return d


CASES = [
    ("single", _terrain, "binary"),
    ("flat", _two_terrains, "binary"),
    ("wide", _terrain, "wide8"),
    ("general", _many_instances, "binary"),
]


def _render(api, ctx, b, desc):
    rt = api.RenderTarget(ctx, desc.width, desc.height)
    rt.render(b.scene, desc.spp, desc.params)
    return rt.download()


@pytest.mark.parametrize("name,make,layout", CASES, ids=[c[0] for c in CASES])
@pytest.mark.parametrize("bound", ["steps", "stack"])
def test_bound_runs_out_then_renders(api_mod, name, make, layout, bound):
    api = api_mod
    ctx = api.Context(0)
    ctx.set_bvh_layout(layout)
    desc = make()
    b = api.load_scene(ctx, desc)
    if bound == "steps":
        b.scene.set_traversal_limits(max_steps=1)
        want_status, want_bit = XGB_DEVICE_TIMEOUT, ERR_LOOP
    else:
        b.scene.set_traversal_limits(max_stack=1)
        want_status, want_bit = XGB_QUEUE_OVERFLOW, ERR_STACK
    with pytest.raises(api.XgbError) as e:
        _render(api, ctx, b, desc)
    assert e.value.status == want_status, str(e.value)
    assert b.scene.stats()["error_flags"] & want_bit
    # the same scene on the same context, bounds restored: a correct render
    b.scene.set_traversal_limits(0, 0)
    gpu = _render(api, ctx, b, desc)
    assert b.scene.stats()["error_flags"] == 0
    cpu = load_cpu(desc, "port").render_pcg(desc)
    err = relmse(gpu, cpu)
    print(f"{name}/{layout}/{bound}: relMSE after restoring the bounds {err:.3e}")
    assert np.isfinite(gpu).all() and err <= 1e-4


def test_bounds_in_batches_and_queries(api_mod):
    api = api_mod
    ctx = api.Context(0)
    desc = _two_terrains()
    b = api.load_scene(ctx, desc)
    b.scene.set_traversal_limits(max_stack=1)
    rt = api.RenderTarget(ctx, desc.width, desc.height)
    with pytest.raises(api.XgbError) as e:
        api.render_batch(ctx, [(b.scene, rt, desc.params, 0, desc.spp)], queue_capacity=4096, iterations_per_sync=4)
    assert e.value.status == XGB_QUEUE_OVERFLOW
    rng = np.random.default_rng(5)
    o = np.tile([0.5, 0.6, -0.3], (256, 1)) + rng.uniform(-0.05, 0.05, (256, 3))
    d = np.tile([0.0, -0.5, 1.0], (256, 1)) + rng.uniform(-0.3, 0.3, (256, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    rays = np.concatenate([o, d, np.full((256, 1), np.inf)], axis=1).astype(np.float32)
    b.scene.set_traversal_limits(max_steps=1)
    with pytest.raises(api.XgbError) as e:
        b.scene.intersect(rays)
    assert e.value.status == XGB_DEVICE_TIMEOUT
    b.scene.set_traversal_limits(0, 0)
    hits = b.scene.intersect(rays)
    assert (hits[:, 1] >= 0).mean() > 0.5  # rays aimed down at the terrain hit it
    api.render_batch(ctx, [(b.scene, rt, desc.params, 0, desc.spp)], queue_capacity=4096, iterations_per_sync=4)
    assert api.batch_stats(ctx)["error_flags"] == 0


def test_limits_are_checked_on_the_host(api_mod):
    api = api_mod
    ctx = api.Context(0)
    b = api.load_scene(ctx, _terrain())
    for steps, stack in ((-1, 0), (0, -1), (0, 65)):
        with pytest.raises(api.XgbError) as e:
            b.scene.set_traversal_limits(steps, stack)
        assert e.value.status == 1


def test_tensor_core_inference_wait_runs_out(api_mod):
    """The learned proposal's tcgen05 inference waits on an mbarrier for its
    matrix operations; with the wait bound lowered to zero polls every wait gives
    up at once: the kernel records ERR_WAIT (bit 8), waits with the default bound
    for the operations it issued, frees its tensor memory and ends, and the call
    returns XGB_DEVICE_TIMEOUT -- for the host-row entry point (xgb_guide_infer)
    and for a guided render. With the bound restored, the same guide infers the
    same outputs as before and the same render succeeds on the same context."""
    api = api_mod
    ctx = api.Context(0)
    gd = api.Guide(ctx, seed=4)
    gd.set_bounds([0, 0, 0], [1, 1, 1])
    rng = np.random.default_rng(3)
    pos = rng.uniform(0, 1, (300, 3)).astype(np.float32)
    nrm = rng.normal(size=(300, 3)).astype(np.float32)
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    wo = rng.normal(size=(300, 3)).astype(np.float32)
    wo /= np.linalg.norm(wo, axis=1, keepdims=True)
    want = gd.infer(pos, nrm, wo)
    gd.set_wait_limit(0)
    with pytest.raises(api.XgbError) as e:
        gd.infer(pos, nrm, wo)
    assert e.value.status == XGB_DEVICE_TIMEOUT
    desc = scenes.occluded_room(32, 32, 2)
    b = api.load_scene(ctx, desc)
    b.scene.setGuide(gd, 0.5, train=False)
    rt = api.RenderTarget(ctx, desc.width, desc.height)
    with pytest.raises(api.XgbError) as e:
        rt.render(b.scene, desc.spp, desc.params)
    assert e.value.status == XGB_DEVICE_TIMEOUT
    assert b.scene.stats()["error_flags"] & 8
    gd.set_wait_limit()
    np.testing.assert_array_equal(gd.infer(pos, nrm, wo), want)
    rt.clear()
    rt.render(b.scene, desc.spp, desc.params)
    st = b.scene.stats()
    assert st["error_flags"] == 0 and st["paths"] == desc.n_paths
    assert np.isfinite(rt.download()).all()
    with pytest.raises(api.XgbError):
        gd.set_wait_limit(-1)
