"""Image output (xgb_film_tonemap, xgb_film_error_map, xgb_write_png) against
the CPU restatement in oracle/image_ref.py.

Tolerance: 8-bit values within one level (CUDA's powf and the host's may round
the last bit differently, which moves a truncated byte by one), and at least
99.9 % of the bytes identical; the PNG writer is exact."""
import os

import numpy as np
import pytest

from oracle import image_ref as I


def test_png_writer_round_trip(tmp_path):
    from xitils_gb300 import api
    rng = np.random.default_rng(0)
    for h, w in [(1, 1), (7, 13), (200, 120)]:  # the last image spans two stored deflate blocks
        img = rng.integers(0, 256, size=(h, w, 3), dtype=np.uint8)
        path = os.path.join(str(tmp_path), f"img_{h}x{w}.png")
        api.write_png(path, img)
        assert np.array_equal(I.read_png(path), img)


def test_restated_maps_on_known_values():
    # pow(1 * 0.3, 1 / 2.2) = 0.5785 -> 147; 0 -> 0; huge -> 255; negative -> NaN -> 0
    out = I.tonemap(np.array([[1.0, 0.0, 1e9, -1.0]], np.float32).reshape(1, 4, 1).repeat(3, axis=2))
    assert out[0, :, 0].tolist() == [147, 0, 255, 0]
    jet = I.error_map(np.zeros((1, 3, 3), np.float32), 1, np.array([[[0, 0, 0], [1, 1, 1], [9, 9, 9]]], np.float32), 1, 1.0)
    assert jet[0, 0].tolist() == [0, 0, 127]      # t = 0: dark blue
    assert jet[0, 2].tolist() == [127, 0, 0]      # t = 1: dark red
    mid = I.error_map(np.zeros((1, 1, 3), np.float32), 1, np.ones((1, 1, 3), np.float32), 1, 2.0)
    assert mid[0, 0].tolist() == [127, 255, 127]  # t = 0.5: green


@pytest.mark.gpu
def test_tonemap_and_error_map_match_restatement(tmp_path):
    import __graft_entry__ as g
    g.build()
    from xitils_gb300 import api, scenes
    ctx = api.Context(0)
    desc = scenes.cornell(96, 80, 8)
    b = api.load_scene(ctx, desc)
    a = api.RenderTarget(ctx, desc.width, desc.height)
    a.render(b.scene, 8, desc.params, 0)
    c = api.RenderTarget(ctx, desc.width, desc.height, fp64=True)
    c.render(b.scene, 4, desc.params, 100)
    img = a.tonemap(scale=1 / 8)
    ref = I.tonemap(a.download(), 1 / 8)
    diff = np.abs(img.astype(int) - ref.astype(int))
    assert diff.max() <= 1 and np.mean(diff == 0) >= 0.999
    err = a.error_map(c, 1 / 8, 1 / 4, 0.05)
    ref_err = I.error_map(a.download(), 1 / 8, c.download(), 1 / 4, 0.05)
    diff = np.abs(err.astype(int) - ref_err.astype(int))
    assert diff.max() <= 1 and np.mean(diff == 0) >= 0.999
    path = os.path.join(str(tmp_path), "cornell.png")
    api.write_png(path, img)
    assert np.array_equal(I.read_png(path), img)
