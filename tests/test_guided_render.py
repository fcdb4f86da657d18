"""Guided rendering through xgb_render: unbiased against the plain path tracer,
online training runs inside the wavefront, and the learned proposal lowers the
error on the occluded-light room at equal sample count."""
import numpy as np
import pytest

from xitils_gb300 import scenes

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def room():
    import __graft_entry__ as g
    g.build()
    from xitils_gb300 import api, guiding
    ctx = api.Context(0)
    desc = scenes.occluded_room(96, 96, 1)
    builder = api.load_scene(ctx, desc)
    ref = guiding.render_reference(ctx, builder, desc, 8192)
    return api, guiding, ctx, desc, builder, ref


def test_guided_is_unbiased_and_better_at_equal_spp(room):
    api, guiding, ctx, desc, builder, ref = room
    spp = 64
    plain = api.RenderTarget(ctx, desc.width, desc.height, fp64=True)
    builder.scene.setGuide(None)
    plain.render(builder.scene, spp, desc.params, 0)
    P = plain.download() / spp
    guide = api.Guide(ctx, seed=0)
    guide.set_training(1024)  # a 96x96 image yields a few thousand records per pass
    before = guide.params()
    builder.scene.setGuide(guide, 0.5, train=True, lr=1e-3)
    train = api.RenderTarget(ctx, desc.width, desc.height, fp64=True)
    for k in range(32):
        train.render(builder.scene, 1, desc.params, 1000 + k)
    after = guide.params()
    assert np.isfinite(after).all() and not np.array_equal(before, after)
    assert guide.steps() > 0
    builder.scene.setGuide(guide, 0.5, train=False)
    guided = api.RenderTarget(ctx, desc.width, desc.height, fp64=True)
    guided.render(builder.scene, spp, desc.params, 0)
    Gimg = guided.download() / spp
    builder.scene.setGuide(None)
    rp, rg = guiding.relmse(P, ref), guiding.relmse(Gimg, ref)
    print(f"relMSE plain {rp:.4e} guided {rg:.4e} means {P.mean():.5f} {Gimg.mean():.5f} {ref.mean():.5f}")
    assert np.isfinite(Gimg).all()
    assert abs(Gimg.mean() - ref.mean()) < 0.05 * ref.mean()
    assert rg < rp


def test_equal_time_harness_runs(room):
    api, guiding, ctx, desc, builder, ref = room
    out = guiding.equal_time_comparison(ctx, desc, time_s=1.0, reference=ref)
    print({k: v for k, v in out.items() if k != "images"})
    assert out["plain"]["spp"] > 0 and out["guided"]["spp"] > 0
    assert np.isfinite(out["guided"]["relmse"])


def test_guiding_leaves_normal_mapped_vertices_to_their_sampler(room):
    """Microfacet-normal-mapped vertices are not guided (their sampler's density is
    only approximated): with every surface normal-mapped, a guided render with
    a trained network draws the same paths as the plain one."""
    api, guiding, ctx, _, _, _ = room
    desc = scenes.mfnm_at_scale(32, 32, 4, grid=33, n_boxes=2, normal_res=64, env_size=(64, 32))
    b = api.load_scene(ctx, desc)
    plain = api.render_desc(ctx, desc, builder=b)
    guide = api.Guide(ctx, seed=1)
    b.scene.setGuide(guide, 0.5, train=False)
    guided = api.render_desc(ctx, desc, builder=b)
    b.scene.setGuide(None)
    np.testing.assert_allclose(guided, plain, rtol=1e-5, atol=1e-5)
