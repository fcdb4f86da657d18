"""Equal-time comparison of neural-guided and plain NEE+MIS rendering.

Protocol: a converged reference image is rendered with the plain path tracer
(FP64 film), then each method renders progressive passes for the same GPU time
budget T. The guided run trains the network online during the first
``train_fraction`` of T and renders with the frozen network for the rest; every
pass of both runs is kept (guided passes are unbiased at any network state,
because the BSDF remains a sampling strategy of the one-sample MIS). The score
is relMSE = mean((I - R)^2 / (R^2 + 1e-2)) against the reference.

The reference is finite too: it is rendered as two independent halves A and B,
and relMSE(A, B) / 4 estimates its own relMSE, which adds to both arms' scores;
the result reports the raw ratio and the ratio with that estimate taken off.
"""
from __future__ import annotations

import time
from typing import Optional

import numpy as np

from . import api
from .scene import IntegratorParams, SceneDesc


def relmse(img: np.ndarray, ref: np.ndarray, eps: float = 1e-2) -> float:
    img = np.asarray(img, np.float64)
    ref = np.asarray(ref, np.float64)
    return float(np.mean((img - ref) ** 2 / (ref ** 2 + eps)))


def luminance_breakdown(plain: np.ndarray, guided: np.ndarray, ref: np.ndarray,
                        quantiles=(0.0, 0.5, 0.9, 0.99, 1.0), eps: float = 1e-2) -> list:
    """relMSE and MSE of both arms over pixel groups of the reference's luminance
    (Rec. 709 weights): the dark half, the next 40 %, the next 9 % and the
    brightest 1 % of the pixels, with each group's share of the whole image's MSE."""
    lum = ref @ np.array([0.2126, 0.7152, 0.0722])
    edges = np.quantile(lum, quantiles)
    out = []
    se_p = ((plain - ref) ** 2).mean(-1)
    se_g = ((guided - ref) ** 2).mean(-1)
    rel_p = ((plain - ref) ** 2 / (ref ** 2 + eps)).mean(-1)
    rel_g = ((guided - ref) ** 2 / (ref ** 2 + eps)).mean(-1)
    for k in range(len(quantiles) - 1):
        lo, hi = edges[k], edges[k + 1]
        m = (lum >= lo) & ((lum < hi) if k < len(quantiles) - 2 else (lum <= hi))
        if not m.any():
            continue
        out.append({"quantiles": [quantiles[k], quantiles[k + 1]], "luminance": [float(lo), float(hi)],
                    "pixels": int(m.sum()),
                    "relmse_plain": float(rel_p[m].mean()), "relmse_guided": float(rel_g[m].mean()),
                    "mse_plain": float(se_p[m].mean()), "mse_guided": float(se_g[m].mean()),
                    "mse_share_plain": float(se_p[m].sum() / max(se_p.sum(), 1e-300)),
                    "mse_share_guided": float(se_g[m].sum() / max(se_g.sum(), 1e-300))})
    return out


def render_reference(ctx: api.Context, builder: api.GpuSceneBuilder, desc: SceneDesc, spp: int,
                     chunk: int = 256, seed_offset: int = 1 << 20) -> np.ndarray:
    """Plain path tracer, FP64 film, sample indices disjoint from the compared runs."""
    rt = api.RenderTarget(ctx, desc.width, desc.height, fp64=True)
    builder.scene.setGuide(None)
    done = 0
    while done < spp:
        n = min(chunk, spp - done)
        rt.render(builder.scene, n, desc.params, seed_offset + done)
        done += n
    return rt.download() / spp


def _timed_passes(ctx, builder, desc, time_s, pass_spp, params, on_pass=None, sample_base=0):
    """Progressive passes until time_s has passed; on_pass(elapsed) may return
    the sample count of the next pass (else pass_spp)."""
    rt = api.RenderTarget(ctx, desc.width, desc.height, fp64=True)
    spp = 0
    ctx.synchronize()
    t0 = time.perf_counter()
    while True:
        elapsed = time.perf_counter() - t0
        if elapsed >= time_s:
            break
        n = (on_pass(elapsed) if on_pass else None) or pass_spp
        rt.render(builder.scene, n, params, sample_base + spp)
        spp += n
    img = rt.download() / max(spp, 1)
    return img, spp, time.perf_counter() - t0


def _warm_up(ctx, builder, desc, params, pass_spp):
    """One untimed pass (buffer allocation, first launches) before an arm is timed."""
    rt = api.RenderTarget(ctx, desc.width, desc.height, fp64=True)
    rt.render(builder.scene, pass_spp, params, 1 << 30)
    rt.download()


def reference_halves(ctx: api.Context, builder, desc: SceneDesc, spp: int, chunk: int = 64):
    """Plain-path reference as two independent halves: (mean, estimated relMSE of the mean)."""
    a = render_reference(ctx, builder, desc, spp // 2, chunk=chunk, seed_offset=1 << 20)
    b = render_reference(ctx, builder, desc, spp // 2, chunk=chunk, seed_offset=(1 << 20) + (1 << 24))
    ref = 0.5 * (a + b)
    noise = float(np.mean((a - b) ** 2 / (ref ** 2 + 1e-2))) / 4.0
    return ref, noise


def equal_time_comparison(ctx: api.Context, desc: SceneDesc, time_s: float = 4.0, train_fraction: float = 0.25,
                          reference_spp: int = 16384, pass_spp: int = 1, bsdf_fraction: float = 0.5,
                          lr: float = 1e-3, reference: Optional[np.ndarray] = None, seed: int = 0,
                          batch_rows: int = 8192, builder=None, train_pass_spp: int = 1,
                          reference_noise: Optional[float] = None, max_steps_per_call: int = 512) -> dict:
    """Both arms are warmed up by one untimed pass; the guided arm's clock
    includes its network inference and every training step. Training passes
    take train_pass_spp samples (one network update per pass), the rest pass_spp."""
    builder = builder if builder is not None else api.load_scene(ctx, desc)
    params = desc.params
    if reference is None:
        reference, reference_noise = reference_halves(ctx, builder, desc, reference_spp)
    ref = reference
    builder.scene.setGuide(None)
    _warm_up(ctx, builder, desc, params, pass_spp)
    plain, plain_spp, plain_t = _timed_passes(ctx, builder, desc, time_s, pass_spp, params)
    warm = api.Guide(ctx, seed=seed + 1)  # allocations and first launches of the guided path, then discarded
    builder.scene.setGuide(warm, bsdf_fraction, train=True, lr=lr)
    _warm_up(ctx, builder, desc, params, pass_spp)
    guide = api.Guide(ctx, seed=seed)
    guide.set_training(batch_rows, max_steps_per_call)
    state = {"training": True}
    builder.scene.setGuide(guide, bsdf_fraction, train=True, lr=lr)

    def on_pass(elapsed):
        if state["training"] and elapsed >= train_fraction * time_s:
            builder.scene.setGuide(guide, bsdf_fraction, train=False)
            state["training"] = False
        return train_pass_spp if state["training"] else pass_spp

    guided, guided_spp, guided_t = _timed_passes(ctx, builder, desc, time_s, pass_spp, params, on_pass)
    # share of the network in a guided render: one profiled training pass and one
    # profiled pass with the frozen network, after the timed arms
    share = {}
    rt = api.RenderTarget(ctx, desc.width, desc.height, fp64=True)
    builder.scene.set_profiling(True)
    for what, train, n in (("training_pass", True, train_pass_spp), ("frozen_pass", False, pass_spp)):
        builder.scene.setGuide(guide, bsdf_fraction, train=train, lr=lr)
        rt.render(builder.scene, n, params, 1 << 29)
        st = builder.scene.stats()
        wave = sum(st["kernel_ms"])
        total = wave + st["guide_infer_ms"] + st["guide_train_ms"]
        share[what] = {"spp": n, "wavefront_ms": wave, "inference_ms": st["guide_infer_ms"],
                       "training_ms": st["guide_train_ms"], "train_steps": st["guide_train_steps"],
                       "network_share": (st["guide_infer_ms"] + st["guide_train_ms"]) / total if total > 0 else None}
    builder.scene.set_profiling(False)
    builder.scene.setGuide(None)
    rp, rg = relmse(plain, ref), relmse(guided, ref)
    corrected = None
    if reference_noise is not None and rg - reference_noise > 0:
        corrected = (rp - reference_noise) / (rg - reference_noise)
    return {
        "time_s": time_s, "train_fraction": train_fraction, "bsdf_fraction": bsdf_fraction,
        "pass_spp": pass_spp, "train_pass_spp": train_pass_spp, "learning_rate": lr, "batch_rows": batch_rows,
        "max_steps_per_call": max_steps_per_call,
        "reference_relmse_estimate": reference_noise,
        "relmse_ratio_reference_noise_removed": corrected,
        "plain": {"spp": plain_spp, "seconds": plain_t, "relmse": rp, "mse": float(np.mean((plain - ref) ** 2))},
        "guided": {"spp": guided_spp, "seconds": guided_t, "relmse": rg, "mse": float(np.mean((guided - ref) ** 2)),
                   "train_steps": guide.steps()},
        "relmse_ratio_plain_over_guided": rp / rg if rg > 0 else None,
        "by_reference_luminance": luminance_breakdown(plain, guided, ref),
        "network_time_share": share,
        "images": (plain, guided, ref),
    }
