"""Edge cases of the render call and the ray queries: ragged and tiny films, zero
samples, one-triangle meshes (a BVH that is a single leaf), degenerate
(zero-area) triangles, scenes with nothing to light them, query rays with a zero
extent or NaN components (no fault), and parameters the C ABI must refuse.
Images are compared with the oracle on the same per-(pixel, sample) streams."""
import ctypes as C
import math

import numpy as np
import pytest

from oracle.bindings import load_scene as load_cpu, relmse
from xitils_gb300 import scenes
from xitils_gb300.scene import IntegratorParams, SceneDesc
from xitils_gb300.transform import translate

pytestmark = pytest.mark.gpu
TOL = 1e-4


@pytest.fixture(scope="module")
def api_ctx():
    import __graft_entry__ as g
    g.build()
    from xitils_gb300 import api
    return api, api.Context(0)


def _parity(api, ctx, d, params=None):
    gpu = api.render_desc(ctx, d, params=params)
    cpu = load_cpu(d, "port").render_pcg(d, params=params)
    assert np.isfinite(gpu).all()
    assert relmse(gpu, cpu) <= TOL, relmse(gpu, cpu)
    return gpu


@pytest.mark.parametrize("w,h,spp", [(1, 1, 3), (33, 7, 2), (7, 33, 1), (97, 1, 2)])
def test_ragged_and_tiny_films(api_ctx, w, h, spp):
    api, ctx = api_ctx
    _parity(api, ctx, scenes.cornell(w, h, spp))


def test_zero_samples_leave_the_film_untouched(api_ctx):
    api, ctx = api_ctx
    d = scenes.cornell(16, 16, 1)
    b = api.load_scene(ctx, d)
    rt = api.RenderTarget(ctx, 16, 16)
    rt.render(b.scene, 0, d.params, 0)
    assert not rt.download().any()


def _single_triangle_scene(degenerate_extra: bool):
    s = SceneDesc(name="one_triangle", width=24, height=24, spp=4)
    grey = s.diffuse([0.6, 0.6, 0.6])
    tri = np.array([[-1, -1, 2], [1, -1, 2], [0, 1, 2]], np.float32)
    idx = [0, 1, 2]
    if degenerate_extra:  # a zero-area triangle (repeated vertex) and a collinear one
        tri = np.concatenate([tri, np.array([[0, 0, 1.5], [0, 0, 1.5], [0.5, 0.5, 1.5], [0, 0, 1], [1, 1, 1],
                                             [2, 2, 1]], np.float32)])
        idx += [3, 4, 5, 6, 7, 8]
    s.add_object(s.add_mesh(tri, idx), grey)
    s.set_sky(1, [1.0, 0.9, 0.8])
    s.set_camera(translate(0.0, 0.0, -1.0), 60.0 * math.pi / 180.0, 1.0)
    return s


@pytest.mark.parametrize("degenerate", [False, True])
def test_one_leaf_bvh_and_degenerate_triangles(api_ctx, degenerate):
    api, ctx = api_ctx
    img = _parity(api, ctx, _single_triangle_scene(degenerate), IntegratorParams(max_depth=4))
    assert img.max() > 0


def test_nothing_to_light_renders_black(api_ctx):
    api, ctx = api_ctx
    d = _single_triangle_scene(False)
    d.set_sky(0)
    img = _parity(api, ctx, d, IntegratorParams(max_depth=4))
    assert not img.any()


def test_query_rays_with_zero_or_nan_extent(api_ctx):
    api, ctx = api_ctx
    b = api.load_scene(ctx, _single_triangle_scene(False))
    rays = np.zeros((4, 7), np.float32)
    rays[:, 2] = -1.0
    rays[:, 5] = 1.0          # towards the triangle at z = 2
    rays[0, 6] = 10.0         # a normal ray: hits at t = 3
    rays[1, 6] = 0.0          # zero extent: the range test 0 < t <= tMax rejects every hit
    rays[2, 3:6] = np.nan     # NaN direction and NaN extent: the reference's comparisons are
    rays[3, 6] = np.nan       # false on NaN, so results are whatever they let through; no fault
    hits = b.scene.intersect(rays)
    assert abs(hits[0, 0] - 3.0) < 1e-5 and hits[0, 2] == 0
    assert hits[1, 2] == -1
    occ = b.scene.occluded(rays)
    assert occ[0] == 1 and occ[1] == 0
    assert hits.shape == (4, 5) and occ.shape == (4,)


def test_bad_parameters_are_refused(api_ctx):
    api, ctx = api_ctx
    d = scenes.cornell(8, 8, 1)
    b = api.load_scene(ctx, d)
    rt = api.RenderTarget(ctx, 8, 8)
    lib = ctx.lib
    for params in (api.IntegratorParamsC(0, 0, 0, 0.9, 0, 0),      # rr_start < 1
                   api.IntegratorParamsC(0, 0, 5, 1.0, 0, 0),      # no depth limit and no roulette
                   api.IntegratorParamsC(0, -1, 5, 0.9, 0, 0),     # negative depth
                   api.IntegratorParamsC(7, 0, 5, 0.9, 0, 0)):     # unknown integrator
        assert lib.xgb_render(b.scene.h, C.byref(params), rt.h, 0, 1, None) == 1  # XGB_INVALID_ARG
    bad_idx = np.array([0, 1, 5], np.int32)
    pos = np.zeros((3, 3), np.float32)
    h = C.c_void_p()
    assert lib.xgb_mesh_create(ctx.h, 3, pos.ctypes.data_as(C.POINTER(C.c_float)), None, None, None, None, 12, 8, 3,
                               bad_idx.ctypes.data_as(C.POINTER(C.c_int32)), C.byref(h)) == 1
    assert not rt.download().any()
