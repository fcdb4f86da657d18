"""xgb_render_noalloc: the render call for callers that cannot allocate GPU memory.

Such callers (an engine that owns all device memory through its own pool, a frame
loop that must not pay cudaMalloc's implicit synchronisation, a plug-in that is
handed a stream and nothing else) get working memory from a fixed static device
array inside the library. This file runs last (pytest collects it after the
others) and must also pass on its own in a fresh process: it calls the entry
point through the C ABI twice in a row and compares each film with the one
xgb_render produces for the same scene, samples and seed.
"""
import ctypes as C

import numpy as np
import pytest

from xitils_gb300 import scenes

pytestmark = pytest.mark.gpu
XGB_INVALID_ARG = 1
XGB_UNSUPPORTED = 7
MAX_PATHS = 32768


@pytest.fixture(scope="module")
def setup():
    import __graft_entry__ as g
    g.build()
    from xitils_gb300 import api
    ctx = api.Context(0)
    desc = scenes.cornell(64, 48, 8)  # 24,576 paths per call
    builder = api.load_scene(ctx, desc)
    return api, ctx, desc, builder


def _params(api, desc, capacity=0):
    p = desc.params
    return api.IntegratorParamsC(p.integrator, p.max_depth, p.rr_start, p.rr_prob, p.seed, capacity)


def test_noalloc_matches_render_twice(setup):
    api, ctx, desc, builder = setup
    lib = ctx.lib
    ref = api.RenderTarget(ctx, desc.width, desc.height)
    ref.render(builder.scene, desc.spp, desc.params)
    expected = ref.download()
    for call in range(2):
        film = api.RenderTarget(ctx, desc.width, desc.height)
        pc = _params(api, desc)
        st = lib.xgb_render_noalloc(builder.scene.h, C.byref(pc), film.h, 0, desc.spp, None)
        assert st == 0, f"call {call}: status {st}"
        got = film.download()
        # same per-(pixel, sample) streams; only the order of film additions differs
        np.testing.assert_allclose(got, expected, rtol=1e-4, atol=1e-5)


def test_noalloc_many_refills_and_small_capacity(setup):
    api, ctx, desc, builder = setup
    lib = ctx.lib
    ref = api.RenderTarget(ctx, desc.width, desc.height)
    ref.render(builder.scene, 24, desc.params)  # 73,728 paths > the static queue
    expected = ref.download()
    for capacity in (0, 4096):
        film = api.RenderTarget(ctx, desc.width, desc.height)
        pc = _params(api, desc, capacity)
        assert lib.xgb_render_noalloc(builder.scene.h, C.byref(pc), film.h, 0, 24, None) == 0
        np.testing.assert_allclose(film.download(), expected, rtol=1e-4, atol=1e-5)


def test_noalloc_rejects_capacity_beyond_maximum(setup):
    api, ctx, desc, builder = setup
    film = api.RenderTarget(ctx, desc.width, desc.height)
    pc = _params(api, desc, MAX_PATHS + 1)
    assert ctx.lib.xgb_render_noalloc(builder.scene.h, C.byref(pc), film.h, 0, 1, None) == XGB_INVALID_ARG
    assert film.download().sum() == 0.0


def test_noalloc_refuses_what_needs_per_call_memory(setup):
    """AOV planes and a learned proposal need device memory per call: refused, film untouched."""
    api, ctx, desc, builder = setup
    film = api.RenderTarget(ctx, desc.width, desc.height, aovs=True)
    pc = _params(api, desc)
    assert ctx.lib.xgb_render_noalloc(builder.scene.h, C.byref(pc), film.h, 0, 1, None) == XGB_UNSUPPORTED
    assert film.download().sum() == 0.0
