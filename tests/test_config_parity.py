"""GPU against the oracle on the benchmark workloads at their own sizes.

The other parity files use small films and scaled-down scenes. Here every
workload the benchmark measures is checked at the size it is measured on:

* the Cornell box exactly as timed: 512 x 512 film, 16 spp, max depth 8,
  Russian roulette after depth 3 (36 triangles);
* the full terrain the headline is timed on: 1024 x 1024 grid (2,093,058
  triangles, the default GPU-built PLOC tree, whose depth the 64-entry stacks
  must hold), lat-long environment 1024 x 512, max depth 10, at a 512 x 512
  film and 4 spp;
* the batch workload's largest scenes in one batch call: a 500,000-triangle
  scene on a 1024 x 1024 film (the 24-bit pixel field of batched paths at its
  largest film), the two largest of the 64 benchmark scenes (369,802 and
  363,680 triangles) and a 1024 x 1024 benchmark scene, 2 spp each;
* the occluded room (200,026 triangles) at 128 x 128 x 4 with the reference's
  own defaults (no depth limit, Russian roulette after 5 at 0.9);
* normal mapping at scale (3,999,564 triangles, 2048^2 normal map) on its
  2048^2 film and the shell-mapped fabric (2,080,812 triangles, 1024^2
  displacement map) on its 1024^2 film, 2 spp, a 160 x 160 crop on the oracle.

Tolerance (floating point, the bar of the whole path): relMSE <= 1e-4 with
eps = 1e-2 and at least 98 % of pixel channels within 1e-3 relative; no device
error bit. The oracle runs on all host cores. The room's paths (14 diffuse
segments on average among 200k interpenetrating boxes) are long enough that the
C library's own misrounded sinf / cosf (about 1 % of the azimuths the
diffuse sampler draws) send a few paths elsewhere: the oracle built with
correctly rounded functions differs from the plain oracle by relMSE ~1.3e-4
there. The normal-mapping random walk draws several azimuths per facet bounce,
and on its crop the envelope is relMSE ~9e-2 (99.5 % of the channels within
1e-3). For these scenes the GPU must match that correctly rounded oracle to
1e-8, and the plain one to 1e-4 or 1.5 times that envelope, whichever is larger.
"""
import numpy as np
import pytest

from oracle.bindings import load_scene as load_cpu, relmse
from xitils_gb300 import scenes
from xitils_gb300.scene import IntegratorParams

pytestmark = pytest.mark.gpu
TOL = 1e-4


@pytest.fixture(scope="module")
def api_ctx():
    import __graft_entry__ as g
    g.build()
    from xitils_gb300 import api
    return api, api.Context(0)


def _close(gpu, cpu):
    return float(np.mean(np.abs(gpu - cpu) <= 1e-3 * (np.abs(cpu) + 1e-2)))


def _check(name, gpu, cpu, stats):
    err, close = relmse(gpu, cpu), _close(gpu, cpu)
    print(f"{name}: relMSE {err:.3e}, within 1e-3: {close:.4f}, means {gpu.mean():.6f} {cpu.mean():.6f}, "
          f"error_flags {stats.get('error_flags')}")
    assert np.isfinite(gpu).all()
    assert stats["error_flags"] == 0
    assert err <= TOL
    assert close >= 0.98


def _render_and_check(api, ctx, desc, params=None):
    P = params or desc.params
    b = api.load_scene(ctx, desc)
    rt = api.RenderTarget(ctx, desc.width, desc.height)
    rt.render(b.scene, desc.spp, P)
    gpu = rt.download()
    st = b.scene.stats()
    assert st["paths"] == desc.width * desc.height * desc.spp
    cpu = load_cpu(desc, "port").render_pcg(desc, params=P)
    _check(desc.name, gpu, cpu, st)


def test_cornell_as_benchmarked(api_ctx):
    """512 x 512 x 16, max depth 8, RR after 3: exactly the Cornell benchmark line."""
    api, ctx = api_ctx
    desc = scenes.cornell(512, 512, 16)
    assert (desc.params.max_depth, desc.params.rr_start) == (8, 3) and desc.n_tris == 36
    _render_and_check(api, ctx, desc)


def test_full_terrain(api_ctx):
    """The 2,093,058-triangle terrain of the headline at 512 x 512 x 4, depth 10."""
    api, ctx = api_ctx
    desc = scenes.terrain(grid=1024, width=512, height=512, spp=4)
    assert desc.n_tris == 2_093_058
    _render_and_check(api, ctx, desc)


def test_full_terrain_reference_defaults(api_ctx):
    """The same terrain with the reference's own integrator defaults (no depth limit)."""
    api, ctx = api_ctx
    desc = scenes.terrain(grid=1024, width=256, height=256, spp=4)
    _render_and_check(api, ctx, desc, IntegratorParams(seed=desc.params.seed))


def test_occluded_room_reference_defaults(api_ctx):
    api, ctx = api_ctx
    desc = scenes.occluded_room(128, 128, 4)
    assert desc.params.max_depth == 0 and desc.n_tris > 200_000
    b = api.load_scene(ctx, desc)
    rt = api.RenderTarget(ctx, desc.width, desc.height)
    rt.render(b.scene, desc.spp, desc.params)
    gpu = rt.download()
    assert b.scene.stats()["error_flags"] == 0
    cpu = load_cpu(desc, "port").render_pcg(desc)
    cr = load_cpu(desc, "port_cr255").render_pcg(desc)
    err, err_cr, envelope = relmse(gpu, cpu), relmse(gpu, cr), relmse(cr, cpu)
    print(f"occluded room: relMSE {err:.3e} (within 1e-3: {_close(gpu, cpu):.4f}), against the correctly "
          f"rounded oracle {err_cr:.3e}, C-library envelope {envelope:.3e}")
    assert np.isfinite(gpu).all()
    assert err_cr <= 1e-8
    assert err <= max(TOL, 1.5 * envelope)
    assert _close(gpu, cpu) >= 0.98


def test_batch_with_largest_jobs(api_ctx):
    """One batch call holding a 500k-triangle 1024^2 job next to the benchmark's
    largest scenes; every job's film against the oracle."""
    api, ctx = api_ctx
    descs = [
        scenes.batch_scene(100, tris_range=(500_000, 500_000), resolutions=(1024,), spp=2),
        scenes.batch_scene(45, spp=2),  # 369,802 triangles, 128^2
        scenes.batch_scene(63, spp=2),  # 363,680 triangles, 512^2
        scenes.batch_scene(18, spp=2),  # 1024^2
    ]
    assert descs[0].n_tris >= 499_000 and descs[0].width == 1024
    builders = [api.load_scene(ctx, d) for d in descs]
    films = [api.RenderTarget(ctx, d.width, d.height) for d in descs]
    jobs = [(b.scene, f, d.params, 0, d.spp) for d, b, f in zip(descs, builders, films)]
    api.render_batch(ctx, jobs)
    st = api.batch_stats(ctx)
    assert st["paths"] == sum(d.n_paths for d in descs)
    for d, f in zip(descs, films):
        cpu = load_cpu(d, "port").render_pcg(d)
        _check(f"{d.name} ({d.n_tris} tris, {d.width}^2)", f.download(), cpu, st)


def _crop_check(api, ctx, desc, rect):
    """The whole film on the GPU, a crop of it on the oracle (render_pcg's pixel
    rectangle draws the same per-(pixel, sample) streams as the full film), gated
    like the room: the correctly rounded oracle to 1e-8, the plain one to 1e-4 or
    1.5 times the C-library envelope, whichever is larger."""
    b = api.load_scene(ctx, desc)
    rt = api.RenderTarget(ctx, desc.width, desc.height)
    rt.render(b.scene, desc.spp, desc.params)
    gpu = rt.download()
    st = b.scene.stats()
    x0, y0, x1, y1 = rect
    g = gpu[y0:y1, x0:x1]
    cpu = load_cpu(desc, "port").render_pcg(desc, rect=rect)[y0:y1, x0:x1]
    cr = load_cpu(desc, "port_cr255").render_pcg(desc, rect=rect)[y0:y1, x0:x1]
    err, err_cr, envelope = relmse(g, cpu), relmse(g, cr), relmse(cr, cpu)
    print(f"{desc.name} ({desc.n_tris} tris, {desc.width}^2, crop {x1 - x0}x{y1 - y0}): relMSE {err:.3e} "
          f"(within 1e-3: {_close(g, cpu):.4f}), against the correctly rounded oracle {err_cr:.3e}, "
          f"C-library envelope {envelope:.3e}, error_flags {st.get('error_flags')}")
    assert np.isfinite(g).all()
    assert st["error_flags"] == 0
    assert err_cr <= 1e-8
    assert err <= max(TOL, 1.5 * envelope)
    assert _close(g, cpu) >= 0.98


def test_normal_mapping_at_scale_full_size(api_ctx):
    """The normal-mapping-at-scale workload as benchmarked: 3,999,564 triangles
    (fBm heightfield and 64 instanced boxes under MicrofacetNormalMapping over a
    textured GGX base), the 2048^2 normal map, environment plus two quad lights,
    depth 12, on the 2048^2 film at 2 spp; the oracle renders a 160 x 160 crop."""
    api, ctx = api_ctx
    desc = scenes.mfnm_at_scale(2048, 2048, 2)
    assert desc.n_tris > 3_900_000
    _crop_check(api, ctx, desc, (944, 944, 1104, 1104))


def test_shell_fabric_full_size(api_ctx):
    """The shell-mapping workload as benchmarked: a 256^2 cloth grid x 16 layers
    (2,080,812 triangles), the 1024^2 weave displacement map, reference defaults,
    on the 1024^2 film at 2 spp; the oracle renders a 160 x 160 crop."""
    api, ctx = api_ctx
    desc = scenes.shell_fabric(1024, 1024, 2, grid=256, layers=16, tex_res=1024)
    assert desc.n_tris > 2_000_000
    _crop_check(api, ctx, desc, (432, 432, 592, 592))
