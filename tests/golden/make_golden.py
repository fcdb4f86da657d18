"""Generate the golden fixtures in tests/golden from the reference's own code.

Runs the reference headers (oracle/_ref/libxref.so, built by
oracle/build_ref.py from the reference checkout) on small seeded scenes with
per-(pixel, sample) PCG streams and stores
  reference_films.npz   the radiance films;
  reference_aov_vmf.npz the DenoisableRenderTargetPixel sums (color, first-hit
                        albedo and normal, RenderTarget.h:131-145) of the same
                        kind of scenes, and the reference's 8-lobe vMF EM fit
                        (VonMisesFisherDistribution<8>::approximateBySEM) of a
                        checker-masked hemisphere sample set built the way
                        Sandbox/VonMisesFisherDistribution/Main.cpp:71-82 builds
                        its set (numpy seeded draws here), with the fitted
                        mixture's pdf at random directions; and the SVNDF fit
                        (the displacement sandbox's downsampling with
                        VonMisesFisherDistribution<4>::approximateBySEM per
                        low texel) of a plain-weave height map.
Usage: python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle.bindings import load_scene  # noqa: E402
from xitils_gb300 import scenes  # noqa: E402
from xitils_gb300.scene import NAIVE, IntegratorParams  # noqa: E402

CASES = {
    "cornell_48x48x4": (lambda: scenes.cornell(48, 48, 4), IntegratorParams()),
    "cornell_naive_32x32x4": (lambda: scenes.cornell(32, 32, 4), IntegratorParams(integrator=NAIVE)),
    "simple_path_tracer_48x48x4": (lambda: scenes.simple_path_tracer_scene(48, 48, 4), IntegratorParams()),
    "terrain_g65_40x40x2": (lambda: scenes.terrain(grid=65, width=40, height=40, spp=2, env_size=(128, 64)),
                            IntegratorParams()),
    "shell_fabric_g24_40x40x2": (lambda: scenes.shell_fabric(40, 40, 2, grid=24, tex_res=64), IntegratorParams()),
    "shell_svbrdf_g20_40x40x2": (lambda: scenes.shell_fabric(40, 40, 2, grid=20, tex_res=64, method="svbrdf"),
                                 IntegratorParams()),
}


AOV_CASES = {
    "cornell_40x40x3": (lambda: scenes.cornell(40, 40, 3), IntegratorParams()),
    "cornell_naive_32x32x3": (lambda: scenes.cornell(32, 32, 3), IntegratorParams(integrator=NAIVE)),
    "zoo_latlong_40x40x2": (lambda: scenes.material_zoo(40, 40, 2, sky="latlong"), IntegratorParams()),
    "terrain_g65_32x32x2": (lambda: scenes.terrain(grid=65, width=32, height=32, spp=2, env_size=(128, 64)),
                            IntegratorParams()),
    "shell_fabric_g24_32x32x2": (lambda: scenes.shell_fabric(32, 32, 2, grid=24, tex_res=64), IntegratorParams()),
}


def checker_hemisphere_samples(n=10000, seed=0):
    """Directions on the +z hemisphere kept with probability 1 on the checker
    cells of (theta = asin z) x (phi = atan2(y, x) + pi) in 4 x 8 bins, else 0."""
    rng = np.random.default_rng(seed)
    out = []
    while len(out) < n:
        z = rng.uniform(0.0, 1.0)
        phi0 = rng.uniform(0.0, 2 * np.pi)
        r = np.sqrt(max(0.0, 1.0 - z * z))
        v = np.array([r * np.cos(phi0), r * np.sin(phi0), z], np.float32)
        theta = np.arcsin(v[2])
        phi = np.arctan2(v[1], v[0]) + np.pi
        p = 1.0 if (int(theta / np.pi * 4) + int(phi / (2 * np.pi) * 8)) % 2 == 0 else 0.0
        if rng.uniform() < p:
            out.append(v)
    return np.stack(out).astype(np.float32)


def vmf_fixture():
    import ctypes as C
    from oracle.bindings import CpuChecker
    lib = CpuChecker("reference").lib
    fp = C.POINTER(C.c_float)
    samples = checker_hemisphere_samples()
    enc = np.zeros(39, np.float32)
    assert lib.xref_vmf8_fit(samples.ctypes.data_as(fp), C.c_int(len(samples)), C.c_uint32(0), enc.ctypes.data_as(fp)) == 0
    rng = np.random.default_rng(1)
    dirs = rng.normal(size=(2000, 3))
    dirs = (dirs / np.linalg.norm(dirs, axis=1, keepdims=True)).astype(np.float32)
    pdf = np.zeros(len(dirs), np.float32)
    lib.xref_vmf8_eval(enc.ctypes.data_as(fp), C.c_int(len(dirs)), dirs.ctypes.data_as(fp), pdf.ctypes.data_as(fp))
    spdf = np.zeros(len(samples), np.float32)
    lib.xref_vmf8_eval(enc.ctypes.data_as(fp), C.c_int(len(samples)), samples.ctypes.data_as(fp),
                       spdf.ctypes.data_as(fp))
    return {"vmf_samples": samples, "vmf_encoded": enc, "vmf_dirs": dirs, "vmf_pdf": pdf, "vmf_sample_pdf": spdf}


def main():
    out = {}
    for name, (make, params) in CASES.items():
        desc = make()
        ref = load_scene(desc, "reference")
        out[name] = ref.render_pcg(desc, params=params)
        print(name, float(out[name].mean()))
    np.savez_compressed(os.path.join(HERE, "reference_films.npz"), **out)
    aov = {}
    for name, (make, params) in AOV_CASES.items():
        desc = make()
        film, albedo, normal = load_scene(desc, "reference").render_pcg_aov(desc, params=params)
        aov[name + "_color"], aov[name + "_albedo"], aov[name + "_normal"] = film, albedo, normal
        print(name, float(film.mean()), float(albedo.mean()), float(normal.mean()))
    aov.update(vmf_fixture())
    # SVNDF fit (per-texel 4-lobe EM) of the plain-weave map, wrap addressing, rate 8, seed 7
    from oracle.bindings import CpuChecker
    aov["svndf_low"], aov["svndf_lobes"] = CpuChecker("reference").svndf_fit(scenes.weave_displacement(64), 0.05, 8, 7,
                                                                             False)
    print("vmf log-likelihood", float(np.mean(np.log(aov["vmf_sample_pdf"]))))
    np.savez_compressed(os.path.join(HERE, "reference_aov_vmf.npz"), **aov)


if __name__ == "__main__":
    main()
