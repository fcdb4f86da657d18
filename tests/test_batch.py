"""Batched rendering (xgb_render_batch): many scenes, films and sample ranges in
one wavefront. A job's film must equal what xgb_render adds for that job alone
(same per-(pixel, sample) streams; only the order of the FP32 film sums
differs, so the tolerance is 1e-5 relative), whatever the queue capacity,
iterations per check and CUDA-graph replay; one job is also checked against the
oracle."""
import numpy as np
import pytest

from xitils_gb300 import scenes
from xitils_gb300.scene import NAIVE, IntegratorParams

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def setup():
    import __graft_entry__ as g
    g.build()
    from xitils_gb300 import api
    ctx = api.Context(0)
    descs = [scenes.batch_scene(i, tris_range=(1_000, 30_000), resolutions=(32, 48, 64), spp=4) for i in range(5)]
    descs.append(scenes.cornell(40, 40, 4))
    descs.append(scenes.terrain(grid=65, width=48, height=32, spp=2, env_size=(128, 64)))
    builders = [api.load_scene(ctx, d) for d in descs]
    return api, ctx, descs, builders


def _single(api, ctx, d, b, params, begin, count):
    rt = api.RenderTarget(ctx, d.width, d.height)
    rt.render(b.scene, count, params, begin)
    return rt.download()


@pytest.mark.parametrize("cap,iters,graph", [(1024, 2, False), (4096, 8, True), (1 << 18, 4, True)])
def test_batch_films_equal_single_renders(setup, cap, iters, graph):
    api, ctx, descs, builders = setup
    jobs, targets, expect = [], [], []
    for k, (d, b) in enumerate(zip(descs, builders)):
        params = d.params if k != 2 else IntegratorParams(integrator=NAIVE, max_depth=6, rr_start=3, seed=9)
        begin = 3 * k
        rt = api.RenderTarget(ctx, d.width, d.height)
        jobs.append((b.scene, rt, params, begin, d.spp))
        targets.append(rt)
        expect.append(_single(api, ctx, d, b, params, begin, d.spp))
    api.render_batch(ctx, jobs, queue_capacity=cap, iterations_per_sync=iters, use_graph=graph)
    st = api.batch_stats(ctx)
    assert st["paths"] == sum(d.width * d.height * d.spp for d in descs)
    for d, rt, e in zip(descs, targets, expect):
        got = rt.download()
        assert np.isfinite(got).all()
        np.testing.assert_allclose(got, e, rtol=1e-5, atol=1e-5 * max(1.0, float(np.abs(e).max())), err_msg=d.name)
    # a second call of the same shape replays the cached graph: films add up
    api.render_batch(ctx, jobs, queue_capacity=cap, iterations_per_sync=iters, use_graph=graph)
    for d, rt, e in zip(descs, targets, expect):
        np.testing.assert_allclose(rt.download(), 2 * e, rtol=1e-5, atol=2e-5 * max(1.0, float(np.abs(e).max())))


def test_batch_job_matches_oracle(setup):
    from oracle.bindings import load_scene as load_cpu, relmse
    api, ctx, descs, builders = setup
    d, b = descs[5], builders[5]  # Cornell
    rt = api.RenderTarget(ctx, d.width, d.height)
    others = [(bb.scene, api.RenderTarget(ctx, dd.width, dd.height), dd.params, 0, dd.spp)
              for dd, bb in zip(descs[:3], builders[:3])]
    api.render_batch(ctx, others + [(b.scene, rt, d.params, 0, d.spp)], queue_capacity=2048, iterations_per_sync=6)
    cpu = load_cpu(d, "port").render_pcg(d)
    assert relmse(rt.download(), cpu) <= 1e-4


def test_autotune_picks_a_candidate_and_caches_it(setup):
    api, ctx, descs, builders = setup
    jobs = [(b.scene, api.RenderTarget(ctx, d.width, d.height), d.params, 0, d.spp) for d, b in zip(descs, builders)]
    opt = api.batch_autotune(ctx, jobs)
    assert opt["queue_capacity"] in tuple(1 << k for k in range(18, 24))
    assert opt["iterations_per_sync"] in (4, 8, 16)
    api.render_batch(ctx, jobs)  # zero options: the cached autotuned ones
    assert api.batch_stats(ctx)["paths"] == sum(d.width * d.height * d.spp for d in descs)
    for (_, rt, _, _, _), d in zip(jobs, descs):
        assert rt.download().sum() > 0


def test_batch_of_one_instance_scenes(setup):
    """A batch whose every job is one instance of a binary mesh BVH runs the
    one-instance traversal kernel with a per-ray mesh (k_trace_single over
    BatchScenes): terrains of three sizes and a transformed, textured-sky box,
    each film equal to its single render."""
    import math
    from xitils_gb300.scene import SKY_UNIFORM, SceneDesc
    from xitils_gb300.scenes import look_at, transformTRS, unit_cube_mesh
    api, ctx, _, _ = setup
    box = SceneDesc(name="one box", width=40, height=24, spp=4,
                    params=IntegratorParams(max_depth=5, rr_start=3, rr_prob=0.8, seed=5))
    cpos, cidx = unit_cube_mesh()
    box.add_object(box.add_mesh(cpos, cidx), box.metal(0.3, [0.9, 0.6, 0.3]),
                   transformTRS((0.1, -0.2, 0.3), (0.0, 35.0, 0.0), (0.8, 1.3, 0.6)))
    box.set_sky(SKY_UNIFORM, rgb=[0.8, 0.9, 1.0])
    box.set_camera(look_at((2.0, 1.5, -2.5), (0.0, 0.0, 0.0), (0, 1, 0)), 45.0 * math.pi / 180.0, 24 / 40)
    descs = [scenes.terrain(grid=g, width=w, height=h, spp=2, env_size=(64, 32))
             for g, w, h in ((17, 24, 16), (65, 48, 32), (129, 32, 32))] + [box]
    builders = [api.load_scene(ctx, d) for d in descs]
    jobs, expect = [], []
    for k, (d, b) in enumerate(zip(descs, builders)):
        rt = api.RenderTarget(ctx, d.width, d.height)
        jobs.append((b.scene, rt, d.params, 2 * k, d.spp))
        expect.append(_single(api, ctx, d, b, d.params, 2 * k, d.spp))
    api.render_batch(ctx, jobs, queue_capacity=4096, iterations_per_sync=4, use_graph=True)
    st = api.batch_stats(ctx)
    assert st["paths"] == sum(d.width * d.height * d.spp for d in descs) and st["error_flags"] == 0
    for d, (_, rt, _, _, _), e in zip(descs, jobs, expect):
        got = rt.download()
        assert np.isfinite(got).all() and got.sum() > 0
        np.testing.assert_allclose(got, e, rtol=1e-5, atol=1e-5 * max(1.0, float(np.abs(e).max())), err_msg=d.name)
