"""GPU path (libxgb.so through the C ABI) against the oracle on the same
scenes and the same per-(pixel, sample) PCG streams.

Tolerance (floating point): image relMSE <= 1e-4 with eps = 1e-2, the bar the
path tracer is held to. The shading arithmetic is unfused FP32 like the
reference's, and the sin / cos / pow that place sampled directions round
correctly, as the C library's do for all but ~1 % of arguments. Where paths
are chaotic (microfacet normal mapping's random walk, long glossy paths) the C
library's own misroundings are what is left: the oracle built with correctly
rounded functions (``port_cr255``) measures that envelope, and the GPU must
also match that oracle to 1e-8.
"""
import numpy as np
import pytest

from oracle.bindings import load_scene as load_cpu, relmse
from xitils_gb300 import scenes
from xitils_gb300.scene import NAIVE, IntegratorParams

pytestmark = pytest.mark.gpu
TOL = 1e-4


@pytest.fixture(scope="module")
def ctx():
    import __graft_entry__ as g
    g.build()
    from xitils_gb300 import api
    return api.Context(0)


CR_TOL = 1e-8  # GPU against the oracle with correctly rounded float functions


def _compare(ctx, desc, params=None, **kw):
    from xitils_gb300 import api
    P = params or desc.params
    gpu = api.render_desc(ctx, desc, params=P, **kw)
    cpu = load_cpu(desc, "port").render_pcg(desc, params=P, spp_begin=kw.get("spp_begin", 0),
                                            spp_count=kw.get("spp_count"))
    err = relmse(gpu, cpu)
    close = np.mean(np.abs(gpu - cpu) <= 1e-3 * (np.abs(cpu) + 1e-2))
    print(f"{desc.name}: relMSE {err:.3e}, pixels within 1e-3: {close:.4f}, means {gpu.mean():.5f} {cpu.mean():.5f}")
    assert np.isfinite(gpu).all()
    return gpu, cpu, err, close


@pytest.mark.parametrize("make,params", [
    (lambda: scenes.cornell(96, 96, 16), None),                                    # max depth 8, RR after 3
    (lambda: scenes.cornell(80, 64, 8), IntegratorParams()),                       # reference defaults
    (lambda: scenes.cornell(64, 64, 8), IntegratorParams(integrator=NAIVE)),
    (lambda: scenes.simple_path_tracer_scene(96, 96, 8), None),
])
def test_cornell_family(ctx, make, params):
    _, _, err, close = _compare(ctx, make(), params)
    assert err <= TOL
    assert close >= 0.98


def test_terrain_ggx_latlong(ctx):
    desc = scenes.terrain(grid=129, width=96, height=96, spp=8, env_size=(256, 128))
    _, _, err, close = _compare(ctx, desc)
    assert err <= TOL
    assert close >= 0.98


@pytest.mark.parametrize("sky", ["none", "uniform", "probe", "latlong"])
@pytest.mark.parametrize("only", [[], [1], [2], [3], [1, 2, 3]])
def test_material_zoo(ctx, sky, only):
    """Glossy, GlossyWithHighLight, SpecularReflection, SpecularFresnel under every sky."""
    desc = scenes.material_zoo(64, 64, 8, sky=sky, only=only)
    _, _, err, close = _compare(ctx, desc, IntegratorParams())
    assert err <= TOL
    assert close >= 0.98


def _against_cr_oracle(gpu, desc, params):
    """relMSE of the GPU image against the oracle whose float functions round correctly,
    and that oracle's own distance from the plain one (the C library's contribution)."""
    cpu = load_cpu(desc, "port").render_pcg(desc, params=params)
    cr = load_cpu(desc, "port_cr255").render_pcg(desc, params=params)
    err_cr, envelope = relmse(gpu, cr), relmse(cr, cpu)
    print(f"{desc.name}: relMSE vs correctly rounded oracle {err_cr:.3e}, C-library envelope {envelope:.3e}")
    return err_cr, envelope


@pytest.mark.parametrize("sky", ["none", "latlong"])
def test_microfacet_normal_mapping(ctx, sky):
    """Microfacet normal mapping with a normal map: its random walk turns a one-ulp
    difference in a sampled direction into a different walk (a one-ulp perturbation of
    every sin / cos / pow of the oracle moves this image by ~4e-3). With correctly
    rounded sampling functions the GPU is held to the path tracer's 1e-4 and to 1e-8
    against the correctly rounded oracle."""
    desc = scenes.material_zoo(64, 64, 8, sky=sky, only=[0])
    P = IntegratorParams()
    gpu, cpu, err, close = _compare(ctx, desc, P)
    assert err <= TOL
    assert close >= 0.98
    err_cr, _ = _against_cr_oracle(gpu, desc, P)
    assert err_cr <= CR_TOL


def test_sample_ranges_add_up_and_match_oracle(ctx):
    from xitils_gb300 import api
    desc = scenes.cornell(48, 48, 6)
    b = api.load_scene(ctx, desc)
    rt = api.RenderTarget(ctx, 48, 48)
    rt.render(b.scene, 3, desc.params, 0)
    rt.render(b.scene, 3, desc.params, 3)
    split = rt.download()
    cpu = load_cpu(desc, "port").render_pcg(desc)
    assert relmse(split, cpu) <= TOL


def test_fp64_film_and_clear(ctx):
    from xitils_gb300 import api
    desc = scenes.cornell(32, 32, 4)
    b = api.load_scene(ctx, desc)
    f32 = api.RenderTarget(ctx, 32, 32)
    f64 = api.RenderTarget(ctx, 32, 32, fp64=True)
    f32.render(b.scene, 4, desc.params)
    f64.render(b.scene, 4, desc.params)
    a, c = f32.download(), f64.download()
    np.testing.assert_allclose(a, c, rtol=1e-4, atol=1e-5)
    f64.clear()
    assert f64.download().sum() == 0.0


def test_small_queue_capacity_same_image(ctx):
    """A queue far smaller than the work forces many refills; the film must not change beyond summation order."""
    from xitils_gb300 import api
    desc = scenes.cornell(40, 40, 4)
    b = api.load_scene(ctx, desc)
    big = api.RenderTarget(ctx, 40, 40)
    big.render(b.scene, 4, desc.params)
    p = IntegratorParams(max_depth=8, rr_start=3)
    p.queue_capacity = 1024
    small = api.RenderTarget(ctx, 40, 40)
    small.render(b.scene, 4, p)
    np.testing.assert_allclose(small.download(), big.download(), rtol=1e-4, atol=1e-5)
    st = b.scene.stats()
    assert st["paths"] == 40 * 40 * 4 and st["error_flags"] == 0


@pytest.mark.parametrize("make,params,color_tol", [
    (lambda: scenes.cornell(64, 64, 4), IntegratorParams(), TOL),
    (lambda: scenes.cornell(48, 48, 4), IntegratorParams(integrator=NAIVE), TOL),
    # every material kind, microfacet normal mapping included
    (lambda: scenes.material_zoo(64, 64, 4, sky="latlong"), IntegratorParams(), TOL),
    (lambda: scenes.terrain(grid=65, width=48, height=48, spp=4, env_size=(128, 64)), IntegratorParams(), TOL),
])
def test_denoiser_aovs(ctx, make, params, color_tol):
    """First-hit albedo and normal sums (DenoisableRenderTarget) against the
    oracle: the first hit is the same triangle with the same barycentrics, so
    only the order of the per-pixel sums differs (FP32 atomics)."""
    from xitils_gb300 import api
    desc = make()
    rt = api.RenderTarget(ctx, desc.width, desc.height, aovs=True)
    b = api.load_scene(ctx, desc)
    rt.render(b.scene, desc.spp, params, 0)
    color, albedo, normal = rt.download(), rt.download_aov("albedo"), rt.download_aov("normal")
    c_cpu, a_cpu, n_cpu = load_cpu(desc, "port").render_pcg_aov(desc, params=params)
    np.testing.assert_allclose(albedo, a_cpu, rtol=1e-5, atol=1e-5)
    np.testing.assert_allclose(normal, n_cpu, rtol=1e-5, atol=1e-5)
    assert relmse(color, c_cpu) <= color_tol
    plain = api.render_desc(ctx, desc, params=params, builder=b)
    np.testing.assert_array_equal(np.isfinite(plain), True)
    assert relmse(plain, color) <= 1e-9  # enabling the AOV planes leaves the radiance alone
    rt.clear()
    assert not rt.download_aov("albedo").any() and not rt.download_aov("normal").any()


def test_mfnm_at_scale_small(ctx):
    """The normal-mapping-at-scale scene, scaled down: heightfield and boxes under
    MicrofacetNormalMapping over a textured GGX base, more than 16 instances (the
    general two-level traversal), environment plus quad lights, depth 12."""
    desc = scenes.mfnm_at_scale(64, 64, 8, grid=65, n_boxes=20, normal_res=64, env_size=(128, 64))
    gpu, cpu, err, close = _compare(ctx, desc)
    assert err <= TOL
    assert close >= 0.98
    err_cr, _ = _against_cr_oracle(gpu, desc, desc.params)
    assert err_cr <= CR_TOL


def test_tiled_path_order_same_image(ctx):
    """Camera paths in pixel blocks instead of scanline rows (xgb_ctx_set_path_order):
    every pixel keeps its own per-sample random streams, so the film equals the
    scanline film up to the order of the FP32 additions (bijective pixel mapping),
    for block sides that divide the film and ones that leave ragged edges."""
    from xitils_gb300 import api
    desc = scenes.cornell(50, 37, 4)
    b = api.load_scene(ctx, desc)
    base = api.RenderTarget(ctx, desc.width, desc.height)
    base.render(b.scene, desc.spp, desc.params)
    want = base.download()
    try:
        for tw, th in ((8, 4), (4, 8), (7, 3), (64, 64), (1, 1)):
            ctx.set_path_order(tw, th)
            rt = api.RenderTarget(ctx, desc.width, desc.height)
            rt.render(b.scene, desc.spp, desc.params)
            np.testing.assert_allclose(rt.download(), want, rtol=1e-5, atol=1e-6, err_msg=f"tile {tw}x{th}")
            assert b.scene.stats()["paths"] == desc.n_paths
    finally:
        ctx.set_path_order(0, 0)
    for tw, th in ((0, 4), (-1, -1), (257, 1)):
        with pytest.raises(api.XgbError):
            ctx.set_path_order(tw, th)


def test_sample_grouping_same_image(ctx):
    """Camera paths as runs of consecutive samples of one pixel
    (xgb_ctx_set_sample_grouping): every (pixel, sample) keeps its random stream,
    so the film equals the sample-pass order's up to the order of the FP32
    additions; group sizes that divide the call's samples, ones that leave a
    remainder, ones larger than the call, and a call that starts at sample 3."""
    from xitils_gb300 import api
    desc = scenes.cornell(40, 30, 6)
    b = api.load_scene(ctx, desc)
    for begin in (0, 3):
        ctx.set_sample_grouping(0)
        base = api.RenderTarget(ctx, desc.width, desc.height)
        base.render(b.scene, desc.spp, desc.params, begin)
        want = base.download()
        try:
            for g in (2, 3, 4, 8, 64):
                ctx.set_sample_grouping(g)
                rt = api.RenderTarget(ctx, desc.width, desc.height)
                rt.render(b.scene, desc.spp, desc.params, begin)
                np.testing.assert_allclose(rt.download(), want, rtol=1e-5, atol=1e-6, err_msg=f"group {g}, begin {begin}")
                st = b.scene.stats()
                assert st["paths"] == desc.n_paths and st["error_flags"] == 0
        finally:
            ctx.set_sample_grouping()
    cpu = load_cpu(desc, "port").render_pcg(desc)
    ctx.set_sample_grouping(4)
    try:
        gpu = api.render_desc(ctx, desc)
    finally:
        ctx.set_sample_grouping()
    assert relmse(gpu, cpu) <= TOL
    for g in (-1, 4097):
        with pytest.raises(api.XgbError):
            ctx.set_sample_grouping(g)
