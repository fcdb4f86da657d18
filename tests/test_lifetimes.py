"""Handle lifetimes of the Python binding: dropping a wrapper releases its device
memory, and a scene keeps alive everything its build points at (meshes,
materials, their textures and SVNDF, the sky map, the guide), so a scene whose
builder is gone still renders the same image."""
import gc

import numpy as np
import pytest

from xitils_gb300 import scenes

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def api_ctx():
    import __graft_entry__ as g
    g.build()
    from xitils_gb300 import api
    return api, api.Context(0)


def _free_bytes():
    import torch
    torch.cuda.synchronize()
    return torch.cuda.mem_get_info(0)[0]


def test_dropped_guides_and_films_release_device_memory(api_ctx):
    api, ctx = api_ctx
    gc.collect()
    before = _free_bytes()
    for _ in range(8):  # each guide holds ~850 MB of training buffers
        g = api.Guide(ctx, seed=1)
        f = api.RenderTarget(ctx, 1024, 1024, fp64=True, aovs=True)
        del g, f
    gc.collect()
    after = _free_bytes()
    assert before - after < 256 << 20, (before, after)


@pytest.mark.parametrize("make", [
    lambda: scenes.terrain(grid=65, width=48, height=48, spp=2, env_size=(128, 64)),     # roughness map + sky map
    lambda: scenes.shell_fabric(40, 40, 2, grid=16, tex_res=64, max_depth=4),             # displacement map
    lambda: scenes.shell_fabric(40, 40, 2, grid=16, tex_res=64, method="svbrdf", max_depth=4),  # SVNDF
])
def test_scene_outlives_its_builder(api_ctx, make):
    api, ctx = api_ctx
    d = make()
    b = api.load_scene(ctx, d)
    expect = api.render_desc(ctx, d, builder=b)
    scene = b.scene
    del b
    gc.collect()
    rt = api.RenderTarget(ctx, d.width, d.height)
    rt.render(scene, d.spp, d.params, 0)
    # the same image: film sums are FP32 atomics, equal up to their order
    np.testing.assert_allclose(rt.download(), expect, rtol=1e-5, atol=1e-5 * max(1.0, float(expect.max())))
