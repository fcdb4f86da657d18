"""The C++ host-side adapter (include/xgb_xitils.hpp): compiles with g++ against
the C ABI here, and on the GPU renders the same scene as the oracle."""
import math
import os
import subprocess

import numpy as np
import pytest

from xitils_gb300.scene import SKY_UNIFORM, IntegratorParams, SceneDesc
from xitils_gb300.transform import Transform

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "adapter_demo.cpp")


def compile_demo(out_dir):
    from xitils_gb300 import build
    lib = build.build()
    exe = os.path.join(out_dir, "adapter_demo")
    cmd = ["g++", "-std=c++17", "-O2", "-ffp-contract=off", f"-I{ROOT}/include", SRC, "-o", exe,
           f"-L{os.path.dirname(lib)}", "-lxgb", f"-Wl,-rpath,{os.path.dirname(lib)}"]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return exe


def scene_desc():
    W, H = 48, 40
    s = SceneDesc(name="cpp_demo", width=W, height=H, spp=8, params=IntegratorParams())
    grey = s.diffuse([0.7, 0.7, 0.7])
    metal = s.metal(0.3, [0.9, 0.8, 0.7])
    light = s.emission([10.0, 9.0, 8.0])
    q = np.array([0, 1, 2, 0, 2, 3], dtype=np.int32)
    s.add_object(s.add_mesh([[-1, 0, -1], [1, 0, -1], [1, 0, 1], [-1, 0, 1]], q), grey)
    s.add_object(s.add_mesh([[-.25, 1.5, -.25], [.25, 1.5, -.25], [.25, 1.5, .25], [-.25, 1.5, .25]], q), light)
    pos = np.array([[-0.5 if i & 1 else 0.5, -0.5 if i & 2 else 0.5, -0.5 if i & 4 else 0.5] for i in range(8)])
    idx = [0, 1, 2, 1, 3, 2, 2, 3, 6, 3, 7, 6, 0, 4, 1, 4, 5, 1, 0, 2, 6, 0, 6, 4, 1, 5, 3, 5, 7, 3, 4, 6, 5, 6, 7, 5]
    F = np.float32
    c = F(math.cos(F(30.0) * F(3.14159265) / F(180.0)))
    sn = F(math.sin(F(30.0) * F(3.14159265) / F(180.0)))
    m = np.array([[c * F(.4), 0, sn * F(.4), 0], [0, .4, 0, .3], [-sn * F(.4), 0, c * F(.4), 0], [0, 0, 0, 1]], F)
    mi = np.array([[c / F(.4), 0, -sn / F(.4), 0], [0, F(1) / F(.4), 0, F(-.3) / F(.4)],
                   [sn / F(.4), 0, c / F(.4), 0], [0, 0, 0, 1]], F)
    s.add_object(s.add_mesh(pos, idx), metal, Transform(m, mi))
    cam = Transform(np.array([[1, 0, 0, 0], [0, 1, 0, .6], [0, 0, 1, -2.5], [0, 0, 0, 1]], F),
                    np.array([[1, 0, 0, 0], [0, 1, 0, -.6], [0, 0, 1, 2.5], [0, 0, 0, 1]], F))
    s.set_camera(cam, 0.8, H / W)
    s.set_sky(SKY_UNIFORM, rgb=[0.1, 0.12, 0.15])
    return s


def test_adapter_compiles(tmp_path):
    assert os.path.exists(compile_demo(str(tmp_path)))


@pytest.mark.gpu
def test_adapter_renders_like_oracle(tmp_path):
    from oracle.bindings import load_scene, relmse
    exe = compile_demo(str(tmp_path))
    out = os.path.join(str(tmp_path), "film.bin")
    r = subprocess.run([exe, out], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    desc = scene_desc()
    planes = np.fromfile(out, dtype=np.float32).reshape(3, desc.height, desc.width, 3)
    film, albedo, normal = planes
    ref, ref_albedo, ref_normal = load_scene(desc, "port").render_pcg_aov(desc)
    assert np.isfinite(film).all()
    assert relmse(film, ref) <= 1e-4
    np.testing.assert_allclose(albedo, ref_albedo, rtol=1e-5, atol=1e-5)
    np.testing.assert_allclose(normal, ref_normal, rtol=1e-5, atol=1e-5)
