"""Light sampling on the CPU checkers (CPU only): Scene::sampleSurface (Scene.h:40-47)
through Object::sampleSurface (Object.h:91-105), TriangleMesh::sampleSurface
(TriangleMesh.h:216-230) and TriangleIndexed::sampleSurface (TriangleIndexed.h:179-209).

Known answers: the oracle's draws (point, normal, area pdf) equal the reference's bit for
bit on the Cornell box and on a scene of two lights of different sizes, one of them
scaled and rotated (surfaceAreaScaling). Statistics: the pdf is the one of a uniform
choice of light, of triangle, then of a point -- 1 / (nLights nTris A_tri) -- while the
point itself is drawn from three uniforms normalised by their sum, which is not uniform
on the triangle (the reference quirk the GPU keeps): its barycentrics crowd the centroid.
"""
import math

import numpy as np
import pytest

from oracle.bindings import load_scene
from xitils_gb300 import scenes
from xitils_gb300.scene import SceneDesc
from xitils_gb300.transform import transformTRS, translate


def _have_reference():
    try:
        load_scene(scenes.cornell(8, 8, 1), "reference")
        return True
    except Exception:
        return False


HAVE_REF = _have_reference()


def two_lights():
    s = SceneDesc(name="two_lights", width=8, height=8, spp=1)
    grey = s.diffuse([0.5, 0.5, 0.5])
    floor = s.add_mesh(np.array([[-2, 0, -2], [2, 0, -2], [2, 0, 2], [-2, 0, 2]], np.float32), [0, 1, 2, 0, 2, 3])
    s.add_object(floor, grey)
    quad = s.add_mesh(np.array([[0, 0, 0], [1, 0, 0], [1, 0, 1], [0, 0, 1]], np.float32), [0, 2, 1, 0, 3, 2])
    tri = s.add_mesh(np.array([[0, 0, 0], [1, 0, 0], [0, 0, 2]], np.float32), [0, 2, 1])
    s.add_object(quad, s.emission([5, 5, 5]), translate(-0.5, 2.0, -0.5))
    s.add_object(tri, s.emission([1, 2, 3]), transformTRS((0.5, 1.5, 0.2), (30.0, 10.0, 0.0), (2.0, 1.0, 0.5)))
    s.set_camera(translate(0.0, 1.0, -4.0), 60.0 * math.pi / 180.0, 1.0)
    return s


@pytest.mark.skipif(not HAVE_REF, reason="reference checker not staged")
@pytest.mark.parametrize("make", [lambda: scenes.cornell(8, 8, 1), two_lights])
def test_light_samples_match_reference(make):
    d = make()
    a = load_scene(d, "port").light_sample(20_000, seed=9)
    b = load_scene(d, "reference").light_sample(20_000, seed=9)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)


def test_light_pdf_is_uniform_choice_of_light_triangle_and_point():
    d = two_lights()
    p, n, pdf = load_scene(d, "port").light_sample(20_000, seed=1)
    assert np.allclose(np.linalg.norm(n, axis=1), 1.0, atol=1e-5)
    upper = np.abs(p[:, 1] - 2.0) < 1e-5  # the quad at y = 2 (area 1, two triangles of 1/2); the other light is tilted
    assert 0.45 < upper.mean() < 0.55  # either light with probability 1/2
    assert np.allclose(pdf[upper], 1.0 / (2 * 2 * 0.5))
    # the triangle of area 1 in the plane y = 0, scaled by 2 in x and 0.5 in z (area
    # still 1) and rotated: pdf 1 / (2 lights x 1 triangle x area 1), up to rounding of
    # the area scaling
    lower = ~upper
    assert np.allclose(pdf[lower], 0.5, rtol=1e-6)


def test_barycentrics_crowd_the_centroid():
    s = SceneDesc(name="one_light", width=8, height=8, spp=1)
    tri = s.add_mesh(np.array([[0, 0, 0], [1, 0, 0], [0, 0, 1]], np.float32), [0, 2, 1])
    s.add_object(tri, s.emission([1, 1, 1]))
    s.set_camera(translate(0.0, 1.0, -2.0), 1.0, 1.0)
    p, _, pdf = load_scene(s, "port").light_sample(100_000, seed=2)
    assert np.allclose(pdf, 2.0)  # 1 / area
    # with p = b0 p0 + b1 p1 + (1 - b0 - b1) p2 = (b1, 0, 1 - b0 - b1) here
    b1 = p[:, 0].astype(np.float64)
    # uniform points on a triangle have E[b^2] = 1/6; three uniforms normalised by
    # their sum give a more concentrated distribution
    m2 = np.mean(b1 * b1)
    se = np.std(b1 * b1) / math.sqrt(len(b1))
    assert m2 < 1.0 / 6.0 - 20 * se, (m2, se)
    assert abs(b1.mean() - 1.0 / 3.0) < 5 * np.std(b1) / math.sqrt(len(b1))
