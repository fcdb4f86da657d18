"""SVNDF and MultiLobeSVBRDF: the displacement prefiltering sandbox's naive method
(Sandbox/PrefilteringForRenderingDisplacementMappedSurfaces/Main.cpp:361-517).

CPU: the oracle against the reference's own code -- VonMisesFisherDistribution<4>
sampling, the per-texel EM fit (approximateBySEM) of the downsampled normal
distribution, and a MultiLobeSVBRDF render -- bit for bit, live where the reference
is staged and through golden fixtures it generated. GPU: the fit against the oracle
(lobes within float tolerance, the EM running on CUDA's expf / powf) and the render
against the oracle with the same lobes on both sides (relMSE <= 1e-4, short paths and
the reference's unlimited depth).
"""
import os

import numpy as np
import pytest

from oracle.bindings import CpuChecker, load_scene as load_cpu, relmse
from xitils_gb300 import scenes
from xitils_gb300.scene import IntegratorParams

TOL = 1e-4
GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "reference_aov_vmf.npz")
LOBES = np.array([[0, 0, 1, 20, 0.4], [0.6, 0, 0.8, 5, 0.3], [0, 0.6, 0.8, 0, 0.2], [0.3, 0.3, 0.9, 100, 0.1]],
                 np.float32)


def _ref():
    try:
        return CpuChecker("reference")
    except Exception:
        return None


REF = _ref()
needs_ref = pytest.mark.skipif(REF is None, reason="reference checker not staged")


def weave(res=64):
    return scenes.weave_displacement(res)


# ------------------------------------------------------------------ CPU side --
@needs_ref
def test_vmf4_sampling_matches_reference():
    a = CpuChecker("port").vmf4_sample(LOBES, 4000, 3)
    b = REF.vmf4_sample(LOBES, 4000, 3)
    assert np.array_equal(a, b)
    assert np.allclose(np.linalg.norm(a, axis=1), 1.0, atol=1e-5)


@needs_ref
@pytest.mark.parametrize("clamp,rate,shape", [(True, 8, (64, 64)), (False, 8, (64, 64)), (False, 4, (40, 56)),
                                              (True, 5, (37, 29))])
def test_svndf_fit_matches_reference(clamp, rate, shape):
    rgb = weave(max(shape))[: shape[0], : shape[1]]
    la, pa = CpuChecker("port").svndf_fit(rgb, 0.05, rate, 7, clamp)
    lb, pb = REF.svndf_fit(rgb, 0.05, rate, 7, clamp)
    assert la.shape == ((shape[0] + rate - 1) // rate, (shape[1] + rate - 1) // rate)
    assert np.array_equal(la, lb)
    assert np.array_equal(pa, pb)


def test_svndf_fit_matches_golden():
    g = np.load(GOLDEN)
    low, lobes = CpuChecker("port").svndf_fit(weave(64), 0.05, 8, 7, False)
    assert np.array_equal(low, g["svndf_low"])
    assert np.array_equal(lobes, g["svndf_lobes"])


def test_svndf_fit_is_a_distribution():
    low, lobes = CpuChecker("port").svndf_fit(weave(64), 0.05, 8, 7, False)
    mu, kappa, alpha = lobes[..., :3], lobes[..., 3], lobes[..., 4]
    assert np.allclose(np.linalg.norm(mu, axis=-1), 1.0, atol=1e-5)
    assert np.all((kappa >= 0) & (kappa <= 1000))
    assert np.allclose(alpha.sum(-1), 1.0, atol=1e-5)
    assert np.all(mu[..., 2] > 0.5)  # normals of a gentle height map point up
    assert 0.0 < low.min() and low.max() <= 1.0


@needs_ref
@pytest.mark.parametrize("seed", [5, 6])
def test_svbrdf_render_matches_reference(seed):
    d = scenes.shell_fabric(32, 32, 2, grid=16, tex_res=64, method="svbrdf", seed=seed)
    a = load_cpu(d, "port").render_pcg(d, params=IntegratorParams(seed=seed))
    b = load_cpu(d, "reference").render_pcg(d, params=IntegratorParams(seed=seed))
    assert np.array_equal(a, b)


def test_svbrdf_render_matches_golden():
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "reference_films.npz"))
    d = scenes.shell_fabric(40, 40, 2, grid=20, tex_res=64, method="svbrdf")
    assert np.array_equal(load_cpu(d, "port").render_pcg(d, params=IntegratorParams()), g["shell_svbrdf_g20_40x40x2"])


def test_svbrdf_differs_from_the_shells_alone():
    """The SVNDF perturbation is live: the same low-resolution shells under the plain base
    material render differently."""
    d = scenes.shell_fabric(32, 32, 4, grid=16, tex_res=64, method="svbrdf")
    plain = scenes.shell_fabric(32, 32, 4, grid=16, tex_res=64, method="svbrdf")
    cloth = plain.objects[-1]
    cloth.material = plain.materials[cloth.material].base
    a = load_cpu(d, "port").render_pcg(d)
    b = load_cpu(plain, "port").render_pcg(plain)
    assert np.abs(a - b).mean() > 0.02 * b.mean()


# ------------------------------------------------------------------ GPU side --
@pytest.fixture(scope="module")
def api_ctx():
    import __graft_entry__ as g
    g.build()
    from xitils_gb300 import api
    return api, api.Context(0)


def _texels_close(a, b, tol=1e-3):
    err = np.abs(a - b) / (np.abs(b) + 1e-3)
    return np.mean(err.reshape(err.shape[0], err.shape[1], -1).max(-1) < tol)


def _block_log_likelihood(rgb, lobes, scale, rate, clamp):
    """Mean log-likelihood of each low texel's block normals under its fitted mixture
    (numpy FP64 restatement of the fit's inputs and of vMF(), VonMisesFisherDistribution.h:205-211)."""
    h = rgb[..., 0].astype(np.float64)
    H, W = h.shape
    xs, ys = np.arange(W), np.arange(H)
    if clamp:
        xp, xm, yp, ym = np.minimum(xs + 1, W - 1), np.maximum(xs - 1, 0), np.minimum(ys + 1, H - 1), np.maximum(ys - 1, 0)
    else:
        xp, xm, yp, ym = (xs + 1) % W, (xs - 1) % W, (ys + 1) % H, (ys - 1) % H
    du = (h[:, xp] - h[:, xm]) * 0.5 * W
    dv = (h[yp, :] - h[ym, :]) * 0.5 * H
    n = np.stack([-du * scale, -dv * scale, np.ones_like(h)], -1)
    n /= np.linalg.norm(n, axis=-1, keepdims=True)
    out = np.zeros(lobes.shape[:2])
    for py in range(lobes.shape[0]):
        for px in range(lobes.shape[1]):
            blk = n[py * rate:(py + 1) * rate, px * rate:(px + 1) * rate].reshape(-1, 3)
            L = lobes[py, px].astype(np.float64)
            k = np.maximum(L[:, 3], 1e-9)
            pdf = (L[:, 4] * k / (2 * np.pi * (1 - np.exp(-2 * k))) * np.exp(k * (blk @ L[:, :3].T - 1))).sum(-1)
            out[py, px] = np.mean(np.log(np.maximum(pdf, 1e-30)))
    return out


@pytest.mark.gpu
@pytest.mark.parametrize("clamp,rate,res", [(False, 8, 256), (True, 4, 96), (False, 5, 77)])
def test_gpu_fit_matches_oracle(api_ctx, clamp, rate, res):
    """The reference's EM stops on a signed difference of successive fits, which makes
    the result sensitive to the last ulp of expf / powf (a one-ulp perturbation of the
    oracle's own functions moves ~15 % of the texels' lobes by more than 1e-3). The GPU
    fit uses correctly rounded exp / pow / asin / sin / cos: it must equal the fit of
    the oracle whose functions round correctly on all texels but a few, and agree with
    the plain oracle on as many texels as that correctly rounded fit does (the C
    library's misroundings decide the rest), with the same mean log-likelihood."""
    api, ctx = api_ctx
    rgb = weave(res)
    tex = api.Texture(ctx, rgb, warpClamp=clamp)
    sv = api.Svndf(ctx, tex, 0.05, rate, 7)
    _, lobes_cpu = CpuChecker("port").svndf_fit(rgb, 0.05, rate, 7, clamp)
    _, lobes_cr = CpuChecker("port_cr255").svndf_fit(rgb, 0.05, rate, 7, clamp)
    lobes = sv.lobes()
    assert lobes.shape == lobes_cpu.shape
    assert np.isfinite(lobes).all()
    assert np.allclose(lobes[..., 4].sum(-1), 1.0, atol=1e-5)
    gpu_cr, gpu_close, cr_close = (_texels_close(lobes, lobes_cr), _texels_close(lobes, lobes_cpu),
                                   _texels_close(lobes_cr, lobes_cpu))
    ll_gpu = _block_log_likelihood(rgb, lobes, 0.05, rate, clamp).mean()
    ll_cpu = _block_log_likelihood(rgb, lobes_cpu, 0.05, rate, clamp).mean()
    print(f"svndf rate {rate}: texels within 1e-3: GPU~correctly rounded oracle {gpu_cr:.4f}, GPU~oracle "
          f"{gpu_close:.4f}, correctly rounded~oracle {cr_close:.4f}; mean log-likelihood GPU {ll_gpu:.5f} "
          f"oracle {ll_cpu:.5f}")
    assert gpu_cr >= 0.995
    assert gpu_close >= cr_close - 0.005
    assert abs(ll_gpu - ll_cpu) <= 0.01 * abs(ll_cpu)


@pytest.mark.gpu
def test_gpu_fit_rejects_bad_rate(api_ctx):
    api, ctx = api_ctx
    tex = api.Texture(ctx, weave(32))
    for rate in (0, 17):
        with pytest.raises(RuntimeError):
            api.Svndf(ctx, tex, 0.05, rate, 0)


def _gpu_vs_oracle(api, ctx, d):
    """Both sides render with the oracle's SVNDF fit (its lobes uploaded into the GPU's
    SVNDF), so that the comparison covers the render, not the fit's ulp sensitivity."""
    b = api.load_scene(ctx, d)
    src, scale, rate, seed = next(t.svndf for t in d.textures if t.svndf is not None)
    _, lobes = CpuChecker("port").svndf_fit(d.textures[src].rgb, scale, rate, seed, d.textures[src].clamp)
    b.svndfs[0].set_lobes(lobes)
    gpu = api.render_desc(ctx, d, builder=b)
    cpu = load_cpu(d, "port").render_pcg(d)
    err = relmse(gpu, cpu)
    close = np.mean(np.abs(gpu - cpu) <= 1e-3 * (np.abs(cpu) + 1e-2))
    print(f"{d.name} svbrdf: relMSE {err:.3e}, close {close:.4f}")
    assert np.isfinite(gpu).all()
    return gpu, cpu, err, close


@pytest.mark.gpu
def test_gpu_render_matches_oracle_short_paths(api_ctx):
    """Up to 3 segments: the SVNDF draws (texel choice, lobe, disk, W) happen at every
    bounce and every NEE, with CUDA's powf / logf / cosf; relMSE <= 1e-4."""
    api, ctx = api_ctx
    d = scenes.shell_fabric(64, 64, 8, grid=32, tex_res=128, method="svbrdf", max_depth=3)
    _, _, err, close = _gpu_vs_oracle(api, ctx, d)
    assert err <= TOL
    assert close >= 0.98


@pytest.mark.gpu
def test_gpu_render_matches_oracle_reference_defaults(api_ctx):
    """No depth limit: with the same lobes on both sides the SVNDF draws keep the
    paths together (measured relMSE ~5e-8)."""
    api, ctx = api_ctx
    d = scenes.shell_fabric(64, 64, 8, grid=32, tex_res=128, method="svbrdf")
    gpu, cpu, err, close = _gpu_vs_oracle(api, ctx, d)
    assert err <= TOL
    assert close >= 0.99
