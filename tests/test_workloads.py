"""The synthetic workloads the benchmark measures, pinned to their stated sizes and
parameters (CPU only): the Cornell box (36 triangles, 512² × 16 spp, depth 8, RR after
3), the fBm terrain (2·1023² triangles, per-texel GGX roughness in [0.05, 0.5], a
1024 × 512 lat-long sky with a sun of peak ≈ 5e4, 1024² × 64 spp, depth 10), the
occluded room (10 × 4 × 10, 16,667 boxes = 200,026 triangles, reference integrator
defaults), the 64-scene batch (1e3–5e5 triangles, films of 128²–1024², 32 spp, depth 8,
1–4 quad lights) and the normal-mapping scene (3,999,564 triangles, 2048², depth 12)."""
import numpy as np
import pytest

from xitils_gb300 import scenes
from xitils_gb300.scene import EMISSION as MAT_EMISSION


def test_cornell():
    d = scenes.cornell(512, 512, 16)
    assert d.n_tris == 36
    assert (d.width, d.height, d.spp) == (512, 512, 16)
    assert (d.params.max_depth, d.params.rr_start, d.params.rr_prob) == (8, 3, 0.9)
    lights = [m for m in d.materials if m.kind == MAT_EMISSION]
    assert len(lights) == 1 and np.allclose(lights[0].f[:3], [17, 12, 4])


def test_terrain():
    d = scenes.terrain(grid=1024, width=1024, height=1024, spp=64, max_depth=10)
    assert d.n_tris == 2 * 1023 * 1023 == 2_093_058
    assert (d.width, d.height, d.spp, d.params.max_depth) == (1024, 1024, 64, 10)
    rough, env = (t.rgb for t in d.textures)
    assert rough.shape == (1023, 1023, 3) and 0.05 <= rough.min() and rough.max() <= 0.5
    assert env.shape == (512, 1024, 3) and 4e4 < env.max() <= 5e4 + 1


def test_occluded_room():
    d = scenes.occluded_room(1024, 1024, 4)
    assert d.n_tris == 16_667 * 12 + 10 * 2 + 2 == 200_026
    assert (d.params.max_depth, d.params.rr_start, d.params.rr_prob) == (0, 5, 0.9)
    lights = [m for m in d.materials if m.kind == MAT_EMISSION]
    assert len(lights) == 1 and np.allclose(lights[0].f[:3], 200.0)


def test_batch_scenes():
    descs = [scenes.batch_scene(i) for i in range(64)]
    tris = np.array([d.n_tris for d in descs])
    assert tris.min() >= 1_000 and tris.max() <= 500_000 + 4 * 2  # + the light quads
    assert {d.width for d in descs} <= set(scenes.BATCH_RESOLUTIONS)
    assert len({d.width for d in descs}) == 4  # every resolution occurs
    for d in descs:
        assert d.width == d.height and d.spp == 32 and d.params.max_depth == 8
        n_lights = sum(1 for o in d.objects if d.materials[o.material].kind == MAT_EMISSION)
        assert 1 <= n_lights <= 4


@pytest.mark.timeout(120)
def test_normal_mapping_at_scale():
    d = scenes.mfnm_at_scale()
    assert d.n_tris == 3_999_564
    assert (d.width, d.height, d.params.max_depth) == (2048, 2048, 12)
