#!/usr/bin/env python
"""Throughput benchmark of the GPU path tracer (Mpaths/s) on the terrain workload.

Workload (one step = one render call of the whole film):
  fBm heightfield terrain, 1024 x 1024 vertex grid (2,093,058 triangles), GGX
  conductor with per-texel roughness U[0.05, 0.5], procedural 1024 x 512 lat-long
  HDR environment (sky gradient + kappa=2000 sun of peak 5e4), 1024 x 1024 film,
  64 samples per pixel, max depth 10, plain NEE + BSDF MIS path tracer.
  Inputs are seeded synthetic data; the BVH + triangles (~0.3 GB) exceed L2.

Arms:
  default           : libxgb.so through its C ABI (ctypes), device-timed with CUDA
                      events on the render stream; e2e = the same call with the film
                      downloaded to pinned host memory every step.
  --impl reference  : the reference's own CPU path tracer (oracle/_ref: Xitils
                      headers, RenderTarget::render with per-tile samplers, OpenMP on
                      all host cores) on a bounded sample of the same scene.

Guided section (rank 0, after the throughput measurement; --no-guided skips it):
  relMSE at equal GPU time of the neural-guided path against the plain NEE+MIS
  path on the occluded-light room (10 x 4 x 10 room, 16,667 seeded boxes =
  200,026 triangles, 0.5 x 0.5 light of radiance 200 behind a wall with a
  1.0 x 0.2 gap; reference defaults: no depth limit, Russian roulette after 5 at
  0.9), --guided-res square film (default 1024 x 1024, the configuration's),
  --guided-seconds per arm, training during the first 25 % of the guided arm's
  time (Adam, lr 1e-3, one-sample MIS with BSDF fraction 0.5), against a
  --guided-ref-spp plain reference rendered as two halves (FP64 films) whose own
  relMSE estimate is reported beside the ratio; also MSE, a breakdown of both
  over the reference's luminance and the network's share of guided render time.

Multi-GPU (torchrun, N > 1): replicas -- every rank renders its own disjoint
sample range of the same film (weak scaling, no data-path collective); the
timing is the max over ranks.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

L2_BYTES = 129 * 1024 * 1024
# Algorithmic bytes of one closest-hit ray in the extension kernel: ray origin +
# direction read (2 x 16 B), hit record written (16 B + 4 B instance id).
EXTEND_BYTES_PER_RAY = 52
# BVH traffic per visit (reported against L2, not HBM): 64 B node, 48 B triangle.
NODE_BYTES, TRI_BYTES = 64, 48
# DRAM bytes per extension ray of k_trace_single: dram__bytes_read.sum +
# dram__bytes_write.sum summed over the 24 closest-hit launches of one terrain
# render (6.98 GB for 119,571,102 rays, camera paths in runs of 64 samples of a
# pixel), from a one-pass ncu capture; scaled to the average launch for
# roofline.traffic.
EXTEND_DRAM_BYTES_PER_RAY = 58.4


def wavefront_bytes(paths: int, ext: int, shadow: int) -> int:
    """Algorithmic queue bytes of the whole wavefront, from the record sizes of the
    path, hit and shadow queues: generate writes a 56 B path per camera path; extend
    reads the 32 B ray and writes a 20 B hit; shade reads the 56 B path and the hit,
    writes a 56 B path per continuing path (extension rays - paths) and a 56 B
    shadow record per shadow ray, of which the shadow kernel reads 48 B. Film
    atomics, texture and BVH reads are data-dependent and not counted."""
    return 56 * paths + (52 + 76) * ext + 56 * (ext - paths) + (56 + 48) * shadow


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=20)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="xgb", choices=["xgb", "reference"])
    p.add_argument("--workload", default="terrain",
                   choices=["terrain", "cornell", "room", "shell", "svbrdf", "batch", "mfnm"])
    p.add_argument("--shell-grid", type=int, default=256)
    p.add_argument("--mfnm-res", type=int, default=2048)
    p.add_argument("--mfnm-ref-spp", type=int, default=2048)
    p.add_argument("--batch-scenes", type=int, default=64)
    p.add_argument("--grid", type=int, default=1024)
    p.add_argument("--res", type=int, default=None)
    p.add_argument("--spp", type=int, default=None)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--cpu-sample-res", type=int, default=1024)
    p.add_argument("--cpu-sample-spp", type=int, default=4)
    p.add_argument("--no-guided", action="store_true")
    p.add_argument("--no-extras", action="store_true",
                   help="skip the Cornell, small-batch and reference-defaults measurements after the main line")
    p.add_argument("--guided-res", type=int, default=1024)
    p.add_argument("--guided-seconds", type=float, default=15.0)
    p.add_argument("--guided-ref-spp", type=int, default=4096)
    p.add_argument("--guided-pass-spp", type=int, default=16)
    p.add_argument("--guided-train-pass-spp", type=int, default=4)
    p.add_argument("--guided-max-steps", type=int, default=512)
    return p.parse_args()


SINGLE_KERNEL = "k_trace_single (closest-hit traversal of a one-instance scene, binary BVH, persistent)"
FLAT_KERNEL = "k_trace_flat2 (closest-hit traversal of a scene of <= 16 instances, binary BVHs, persistent)"


def make_workload(args):
    """(scene, label, meta): meta names the data, the extension kernel the scene
    runs and how the timed steps relate to L2."""
    from xitils_gb300 import scenes
    big = "inputs larger than L2 (BVH + triangles exceed 129 MB)"
    if args.workload == "terrain":
        res = args.res or 1024
        spp = args.spp or 64
        desc = scenes.terrain(grid=args.grid, width=res, height=res, spp=spp, max_depth=10)
        label = (f"terrain {args.grid}x{args.grid} grid ({desc.n_tris} tris), {res}x{res} film, {spp} spp, "
                 f"max depth 10, GGX per-texel roughness, lat-long env 1024x512")
        meta = {"data": "synthetic (seeded fBm terrain, procedural lat-long environment)", "kernel": SINGLE_KERNEL,
                "l2": big}
    elif args.workload in ("shell", "svbrdf"):
        res = args.res or 1024
        spp = args.spp or 16
        grid = args.shell_grid
        desc = scenes.shell_fabric(res, res, spp, grid=grid, layers=16, tex_res=1024, method=args.workload)
        how = ("1024^2 weave displacement map" if args.workload == "shell" else
               "1024^2 weave displacement map downsampled 8x with a 4-lobe vMF SVNDF per low texel, "
               "MultiLobeSVBRDF over the base material")
        label = (f"shell-mapped fabric: {grid}x{grid} cloth grid x 16 layers ({desc.n_tris} tris), {how}, "
                 f"Cornell-style room, {res}x{res} film, {spp} spp, reference defaults "
                 f"(no depth limit, RR after 5 at 0.9)")
        meta = {"data": "synthetic (seeded cloth patch, procedural plain-weave displacement map)",
                "kernel": "k_trace_flat2 (closest-hit traversal of <= 16 instances with the shell-mapping discard, persistent)",
                "l2": big}
    elif args.workload == "room":
        res = args.res or 1024
        spp = args.spp or 4
        desc = scenes.occluded_room(res, res, spp)
        label = (f"occluded room ({desc.n_tris} tris: 16,667 random boxes in a 10x4x10 room, light behind a slit), "
                 f"{res}x{res} film, {spp} spp, reference defaults (no depth limit, RR after 5 at 0.9)")
        meta = {"data": "synthetic (seeded random boxes)", "kernel": FLAT_KERNEL,
                "l2": "the scene (BVH + triangles, about 23 MB) fits in L2; path queues of 2^23 paths stream through HBM"}
    else:
        res = args.res or 512
        spp = args.spp or 16
        desc = scenes.cornell(res, res, spp)
        label = f"cornell 36 tris, {res}x{res} film, {spp} spp, max depth 8, RR after depth 3"
        meta = {"data": "synthetic (the Cornell box of the workload description)", "kernel": FLAT_KERNEL,
                "l2": "the scene fits in L2 (36 triangles); path queues of 2^23 paths stream through HBM"}
    return desc, label, meta


def arm_config(label, meta, world):
    """The `config` object of both arms' lines (the reference arm runs a bounded
    sample of this workload and says so outside `config`)."""
    return {"workload": label, "parallelism": f"replicas x{world} (disjoint sample ranges)", "l2": meta["l2"],
            "queue_capacity": 1 << 23}


class ClockSampler:
    """nvidia-smi sampling of SM clock and throttle reasons during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.path = None

    def __enter__(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.path or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        rows = [r.split(",") for r in open(self.path).read().strip().splitlines() if r.strip()]
        os.unlink(self.path)
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1]))
                mx = float(r[2])
                for k, nm in enumerate(names):
                    if r[5 + k].strip() == "Active":
                        reasons.add(nm)
            except Exception:
                continue
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def cpu_reference_sample(desc, res, spp, nthreads, chk=None):
    """The reference's own RenderTarget::render (oracle/_ref) on res x res x spp of
    the same scene; where the reference checker is not built, the oracle port
    (the CPU restatement, OpenMP over pixel rows). Returns (Mpaths/s, seconds, kind)."""
    import copy

    from oracle.bindings import CpuChecker
    if chk is None:
        try:
            chk = CpuChecker("reference")
            desc.emit(chk)
        except Exception:
            chk = None
    if chk is not None and chk.kind == "reference":
        film, sec = chk.render_stock(res, res, spp, nthreads=nthreads)
        return res * res * spp / sec / 1e6, sec, "reference"
    d = copy.copy(desc)
    d.width, d.height = res, res
    port = CpuChecker("port")
    d.emit(port)
    t0 = time.perf_counter()
    port.render_pcg(d, spp_count=spp, nthreads=nthreads)
    sec = time.perf_counter() - t0
    return res * res * spp / sec / 1e6, sec, "port"


def svndf_fit_timing(api, ctx, desc):
    """GPU SVNDF fit of the workload's displacement map (xgb_svndf_create, one warp per
    low texel) against the same fit on the host: the oracle's restatement on all
    cores (OpenMP over texels, as the reference's precomputation runs)."""
    from oracle.bindings import CpuChecker
    src, scale, rate, seed = next(t.svndf for t in desc.textures if t.svndf is not None)
    rgb = desc.textures[src].rgb
    tex = api.Texture(ctx, rgb, warpClamp=desc.textures[src].clamp)
    api.Svndf(ctx, tex, scale, rate, seed)  # first call: module load
    times = []
    for _ in range(3):
        ctx.synchronize()
        t0 = time.perf_counter()
        api.Svndf(ctx, tex, scale, rate, seed)  # synchronises before returning
        times.append(time.perf_counter() - t0)
    t0 = time.perf_counter()
    CpuChecker("port").svndf_fit(rgb, scale, rate, seed, desc.textures[src].clamp)
    cpu_s = time.perf_counter() - t0
    h, w = rgb.shape[:2]
    return {"map": f"{w}x{h}", "rate": rate, "low_texels": ((w + rate - 1) // rate) * ((h + rate - 1) // rate),
            "gpu_ms": 1e3 * min(times), "cpu_ms": 1e3 * cpu_s, "cpu_cores": os.cpu_count(),
            "cpu_kind": "oracle restatement of the reference's fit, OpenMP over texels"}


def peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        return {}


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    desc, label, meta = make_workload(args)
    res, spp = args.cpu_sample_res, 1
    nthreads = os.cpu_count() or 1
    from oracle.bindings import CpuChecker
    try:
        chk = CpuChecker("reference")
        desc.emit(chk)
    except Exception:
        chk = None  # reference headers not staged here: the oracle port stands in
    kind = "reference"
    for _ in range(args.warmup):
        cpu_reference_sample(desc, res, spp, nthreads, chk)
    times = []
    for _ in range(args.steps):
        _, sec, kind = cpu_reference_sample(desc, res, spp, nthreads, chk)
        times.append(sec)
    total = sum(times)
    value = res * res * spp * args.steps / total / 1e6
    out = {
        "impl": "reference", "metric": "Mpaths/s", "value": value, "unit": "Mpaths/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": meta["data"],
        "config": arm_config(label, meta, 1),
        "sample_per_step": f"{res}x{res} film x {spp} spp of the same scene and camera",
        "integrator": ("the reference's StandardPathTracer with its own constants (no depth limit, RR after "
                       "length 5 at 0.9); the GPU line's reference_defaults entry times the GPU with the same"),
        "cpu_baseline": {"value": value, "unit": "Mpaths/s", "cores": nthreads, "kind": kind,
                         "sample": f"{res}x{res}x{spp} per step, {args.steps} steps"},
        "e2e": {"value": value, "unit": "Mpaths/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out))
    return 0


def guided_equal_time(ctx, args):
    """relMSE of neural-guided vs plain rendering at equal GPU time (occluded room)."""
    from xitils_gb300 import api, guiding, scenes

    res = args.guided_res
    desc = scenes.occluded_room(res, res, 1)
    t0 = time.perf_counter()
    builder = api.load_scene(ctx, desc)
    ref, noise = guiding.reference_halves(ctx, builder, desc, args.guided_ref_spp)
    t_ref = time.perf_counter() - t0
    out = guiding.equal_time_comparison(ctx, desc, time_s=args.guided_seconds, reference=ref, reference_noise=noise,
                                        builder=builder, pass_spp=args.guided_pass_spp,
                                        train_pass_spp=args.guided_train_pass_spp,
                                        max_steps_per_call=args.guided_max_steps)
    out.pop("images")
    out["workload"] = (f"occluded room ({desc.n_tris} triangles), {res}x{res} film, reference defaults "
                       f"(no depth limit, RR after 5 at 0.9)")
    out["reference_spp"] = args.guided_ref_spp
    out["reference_seconds"] = t_ref
    out["relmse_eps"] = 1e-2
    return out


def batch_measure(ctx, n_scenes, steps, warmup):
    """The first `n_scenes` scenes of the batch workload (seeded soups / heightfields
    of 1k-500k triangles, films of 128^2-1024^2, 32 spp, max depth 8, 1-4 quad
    lights) rendered by one xgb_render_batch call per step with autotuned queue
    size and graph replay, against the same jobs rendered one xgb_render call
    after another. Returns the measurement as a dict."""
    import ctypes as C

    import torch

    from xitils_gb300 import api, scenes

    descs = [scenes.batch_scene(i) for i in range(n_scenes)]
    builders = [api.load_scene(ctx, d) for d in descs]
    targets = [api.RenderTarget(ctx, d.width, d.height) for d in descs]
    paths = sum(d.width * d.height * d.spp for d in descs)

    def jobs(step):
        return [(b.scene, t, d.params, step * d.spp, d.spp) for d, b, t in zip(descs, builders, targets)]

    t0 = time.perf_counter()
    tuned = api.batch_autotune(ctx, jobs(0))
    t_tune = time.perf_counter() - t0
    for k in range(warmup):
        api.render_batch(ctx, jobs(k))
    ctx.synchronize()
    with ClockSampler(0) as clocks:
        t0 = time.perf_counter()
        for k in range(steps):
            api.render_batch(ctx, jobs(warmup + k))
        ctx.synchronize()
        t_batch = time.perf_counter() - t0
    st = api.batch_stats(ctx)
    # end to end: the same call plus every job's film downloaded to pinned host memory each step
    hosts = [torch.empty((d.height, d.width, 3), dtype=torch.float32, pin_memory=True).numpy() for d in descs]
    ctx.synchronize()
    t0 = time.perf_counter()
    for k in range(steps):
        api.render_batch(ctx, jobs(warmup + steps + k))
        for t, h in zip(targets, hosts):
            t.download(h)
    t_e2e = time.perf_counter() - t0
    # the same jobs one render call after another
    for d, b, t in zip(descs, builders, targets):
        t.render(b.scene, d.spp, d.params, 0)
    ctx.synchronize()
    t0 = time.perf_counter()
    for k in range(steps):
        for d, b, t in zip(descs, builders, targets):
            t.render(b.scene, d.spp, d.params, (warmup + k) * d.spp)
    ctx.synchronize()
    t_seq = time.perf_counter() - t0
    return {
        "metric": "Mpaths/s", "value": paths * steps / t_batch / 1e6, "unit": "Mpaths/s", "n_gpus": 1,
        "steps": steps, "warmup": warmup, "ms_per_step": 1e3 * t_batch / steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded triangle soups and fBm heightfields)",
        "config": {"workload": f"{len(descs)}-scene batch, {sum(d.n_tris for d in descs)} triangles in all, "
                               f"{paths} paths per step (32 spp each), one xgb_render_batch call per step",
                   "autotuned": tuned, "autotune_seconds": t_tune},
        "sequential": {"value": paths * steps / t_seq / 1e6, "unit": "Mpaths/s",
                       "ms_per_step": 1e3 * t_seq / steps, "how": "one xgb_render call per scene"},
        "e2e": {"value": paths * steps / t_e2e / 1e6, "unit": "Mpaths/s",
                "h2d_bytes_per_step": len(descs) * C.sizeof(api.BatchJobC),
                "d2h_bytes_per_step": sum(d.width * d.height * 12 for d in descs)},
        "gpu_launches": st["kernel_launches"] * steps,
        "clocks": clocks.summary(),
        "render_stats": st,
        "timing": "host wall clock around the calls, synchronised (each call ends with a device sync)",
    }


def run_batch(args):
    """The batch workload as the main line (--workload batch)."""
    from xitils_gb300 import api

    out = batch_measure(api.Context(0), args.batch_scenes, args.steps, args.warmup)
    out["cpu_baseline"] = None
    print(json.dumps(out))
    return 0


def render_measure(ctx, desc, params, steps, warmup, builder=None):
    """Device time (CUDA events on the render stream) and end-to-end time (the
    same call plus a film download to pinned host memory) of `steps` render calls
    of `desc` after `warmup` untimed ones; every call renders new samples."""
    import ctypes as C

    import torch

    from xitils_gb300 import api

    b = builder or api.load_scene(ctx, desc)
    W, H, spp = desc.width, desc.height, desc.spp
    rt = api.RenderTarget(ctx, W, H)
    stream = torch.cuda.Stream()
    sptr = C.c_void_p(stream.cuda_stream)
    for k in range(warmup):
        rt.render(b.scene, spp, params, k * spp, stream=sptr)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for k in range(steps):
        rt.render(b.scene, spp, params, (warmup + k) * spp, stream=sptr)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    err = b.scene.stats(stream=sptr)["error_flags"]
    host = torch.empty((H, W, 3), dtype=torch.float32, pin_memory=True).numpy()
    t0 = time.perf_counter()
    for k in range(steps):
        rt.render(b.scene, spp, params, (warmup + steps + k) * spp, stream=sptr)
        rt.download(host, stream=sptr)
    t_e2e = time.perf_counter() - t0
    paths = W * H * spp * steps
    return {"value": paths / (ms / 1e3) / 1e6, "unit": "Mpaths/s", "ms_per_step": ms / steps, "steps": steps,
            "warmup": warmup,
            "e2e": {"value": paths / t_e2e / 1e6, "unit": "Mpaths/s",
                    "h2d_bytes_per_step": C.sizeof(api.IntegratorParamsC), "d2h_bytes_per_step": W * H * 12},
            "error_flags": err}


def run_mfnm(args):
    """Microfacet normal mapping at scale (4.0 M triangles, 2048^2 normal map,
    environment + 2 quad lights, depth 12): plain throughput, then neural-guided
    vs plain relMSE at equal GPU time, the time being that of 256 spp of the plain
    path, against a --mfnm-ref-spp plain reference rendered as two halves."""
    from xitils_gb300 import api, guiding, scenes

    ctx = api.Context(0)
    res = args.mfnm_res
    desc = scenes.mfnm_at_scale(res, res, 1)
    builder = api.load_scene(ctx, desc)
    rt = api.RenderTarget(ctx, res, res)
    spp_step = 16
    for k in range(args.warmup):
        rt.render(builder.scene, spp_step, desc.params, k * spp_step)
    ctx.synchronize()
    with ClockSampler(0) as clocks:
        t0 = time.perf_counter()
        for k in range(args.steps):
            rt.render(builder.scene, spp_step, desc.params, (args.warmup + k) * spp_step)
        ctx.synchronize()
        dt = time.perf_counter() - t0
    st = builder.scene.stats()
    mpaths = res * res * spp_step * args.steps / dt / 1e6
    t256 = res * res * 256 / (mpaths * 1e6)
    t0 = time.perf_counter()
    ref, noise = guiding.reference_halves(ctx, builder, desc, args.mfnm_ref_spp, chunk=16)
    t_ref = time.perf_counter() - t0
    cmp = guiding.equal_time_comparison(ctx, desc, time_s=t256, reference=ref, reference_noise=noise, builder=builder,
                                        pass_spp=4, train_pass_spp=1)
    cmp.pop("images")
    out = {
        "metric": "Mpaths/s", "value": mpaths, "unit": "Mpaths/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * dt / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded fBm heightfield, boxes, procedural maps)",
        "config": {"workload": f"microfacet normal mapping at scale, {desc.n_tris} triangles, {res}x{res} film, "
                               f"{spp_step} spp per step, depth 12, GGX base with the horizon fix"},
        "render_stats": st, "clocks": clocks.summary(),
        "timing": "host wall clock around synchronised render calls",
        "guided_equal_time": dict(cmp, time_budget="256 spp of the plain path", reference_spp=args.mfnm_ref_spp,
                                  reference_seconds=t_ref),
    }
    print(json.dumps(out))
    return 0


def run_xgb(args):
    import ctypes as C

    import numpy as np
    import torch

    from xitils_gb300 import api

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    desc, label, meta = make_workload(args)
    ctx = api.Context(local)
    builder = api.load_scene(ctx, desc)
    svndf_fit = svndf_fit_timing(api, ctx, desc) if args.workload == "svbrdf" and rank == 0 else None
    scene = builder.scene
    W, H, spp = desc.width, desc.height, desc.spp
    rt = api.RenderTarget(ctx, W, H)
    stream = torch.cuda.Stream(device=local)
    sptr = C.c_void_p(stream.cuda_stream)
    params = desc.params
    step_paths = W * H * spp
    sample_base = rank * spp * (args.warmup + 3 * args.steps + 1)

    def render(k):
        rt.render(scene, spp, params, sample_base + k * spp, stream=sptr)

    for k in range(args.warmup):
        render(k)
    torch.cuda.synchronize()
    with ClockSampler(local) as clocks:
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for k in range(args.steps):
            render(args.warmup + k)
        e1.record(stream)
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
    ms = e0.elapsed_time(e1)
    ms_t = torch.tensor([ms], dtype=torch.float64, device=f"cuda:{local}")
    if dist:
        dist.all_reduce(ms_t, op=dist.ReduceOp.MAX)
    ms_max = float(ms_t.item())
    value = world * step_paths * args.steps / (ms_max / 1e3) / 1e6
    clk = clocks.summary()

    # profiled pass (not timed above): CUDA events around every kernel on the
    # render stream, plus BVH work counters, for the per-kernel roofline
    scene.set_profiling(True)
    stats = []
    for k in range(max(1, min(args.steps, 5))):
        render(args.warmup + args.steps + k)
        stats.append(scene.stats(stream=sptr))
    scene.set_profiling(False)

    # end to end through the C ABI: render call + film download to pinned host memory every step
    host = torch.empty((H, W, 3), dtype=torch.float32, pin_memory=True)
    host_np = host.numpy()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    t0 = time.perf_counter()
    for k in range(args.steps):
        render(args.warmup + 2 * args.steps + k)
        rt.download(host_np, stream=sptr)
    t1 = time.perf_counter()
    e2e_s = torch.tensor([t1 - t0], dtype=torch.float64, device=f"cuda:{local}")
    if dist:
        dist.all_reduce(e2e_s, op=dist.ReduceOp.MAX)
    e2e = world * step_paths * args.steps / float(e2e_s.item()) / 1e6

    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return 0

    agg = {k: sum(s[k] for s in stats) for k in ("paths", "extension_rays", "shadow_rays", "iterations",
                                                   "kernel_launches", "node_visits", "tri_tests")}
    agg["error_flags"] = 0
    for s_ in stats:
        agg["error_flags"] |= s_["error_flags"]
    stage_ms = [sum(s["kernel_ms"][j] for s in stats) for j in range(5)]
    stage_launch = [sum(s["stage_launches"][j] for s in stats) for j in range(5)]
    pk = peaks()
    hbm = pk.get("hbm_gbs")
    ext_ms = stage_ms[2]
    ext_launches = max(stage_launch[2], 1)
    achieved = EXTEND_BYTES_PER_RAY * agg["extension_rays"] / (ext_ms / 1e3) / 1e9 if ext_ms > 0 else None
    roofline = {
        "kernel": meta["kernel"],
        "bound": "hbm",
        "achieved": achieved,
        "peak": hbm if hbm else 6800.0,
        "peak_source": "measured (MEASURED_PEAKS.json hbm_gbs)" if hbm else "fallback 6.8 TB/s",
        "unit": "GB/s",
        "frac": (achieved / (hbm or 6800.0)) if achieved else None,
        # the DRAM bytes per ray come from the terrain's ncu capture; other workloads have none
        "traffic": (EXTEND_DRAM_BYTES_PER_RAY * agg["extension_rays"] / ext_launches
                    if args.workload == "terrain" else None),
        "traffic_source": ("ncu dram__bytes_read.sum + dram__bytes_write.sum per ray of a terrain extension launch "
                           "x rays per launch" if args.workload == "terrain" else "no ncu capture of this workload"),
        "algorithmic_bytes_per_launch": EXTEND_BYTES_PER_RAY * agg["extension_rays"] / ext_launches,
        "avg_launch_ms": ext_ms / ext_launches,
        "bvh_l2_gbs": ((NODE_BYTES * agg["node_visits"] + TRI_BYTES * agg["tri_tests"]) / (ext_ms / 1e3) / 1e9
                       if ext_ms > 0 else None),
        "nodes_per_ray": agg["node_visits"] / max(agg["extension_rays"], 1),
        "tris_per_ray": agg["tri_tests"] / max(agg["extension_rays"], 1),
    }
    total_ms = sum(stage_ms)
    wf_bytes = wavefront_bytes(agg["paths"], agg["extension_rays"], agg["shadow_rays"])
    wf_achieved = wf_bytes / (total_ms / 1e3) / 1e9 if total_ms > 0 else None
    wavefront = {
        "what": "queue records of all five stages (generate, extend, shade, shadow) over the summed stage time",
        "bound": "hbm", "unit": "GB/s", "achieved": wf_achieved, "peak": hbm if hbm else 6800.0,
        "frac": (wf_achieved / (hbm or 6800.0)) if wf_achieved else None,
        "bytes_per_path": wf_bytes / max(agg["paths"], 1),
    }
    cpu = None
    if not args.no_cpu_baseline:
        try:
            n = os.cpu_count() or 1
            v, sec, kind = cpu_reference_sample(desc, args.cpu_sample_res, args.cpu_sample_spp, n)
            how = ("reference RenderTarget::render + StandardPathTracer" if kind == "reference"
                   else "oracle port (CPU restatement), per-pixel PCG streams")
            cpu = {"value": v, "unit": "Mpaths/s", "cores": n, "kind": kind,
                   "sample": f"{args.cpu_sample_res}x{args.cpu_sample_res} film x {args.cpu_sample_spp} spp of the "
                             f"same scene ({sec:.1f} s), {how}"}
        except Exception as e:
            cpu = {"value": None, "unit": "Mpaths/s", "cores": os.cpu_count(), "kind": "reference",
                   "sample": f"unavailable: {e}"}
    extras = {}
    if not args.no_extras and world == 1:
        from xitils_gb300 import scenes
        from xitils_gb300.scene import IntegratorParams
        if args.workload == "terrain":
            m = render_measure(ctx, desc, IntegratorParams(seed=desc.params.seed), args.steps, 3, builder=builder)
            m["config"] = dict(arm_config(label.replace("max depth 10", "reference integrator defaults"), meta, 1),
                               integrator="no depth limit, RR after length 5 at 0.9 (the reference arm's settings)")
            extras["reference_defaults"] = m
        c1 = scenes.cornell(512, 512, 16)
        m = render_measure(ctx, c1, c1.params, args.steps, 3)
        m["config"] = {"workload": "cornell 36 tris, 512x512 film, 16 spp, max depth 8, RR after depth 3"}
        extras["cornell"] = m
        extras["batch"] = batch_measure(ctx, 16, 3, 1)
    guided = None
    if not args.no_guided and world == 1:
        try:
            guided = guided_equal_time(ctx, args)
        except Exception as e:  # reported, not hidden: the line still carries the throughput
            guided = {"unavailable": f"{type(e).__name__}: {e}"}
    total_rays = agg["extension_rays"] + agg["shadow_rays"]
    out = {
        "metric": "Mpaths/s", "value": value, "unit": "Mpaths/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32",
        "data": meta["data"],
        "config": arm_config(label, meta, world),
        "e2e": {"value": e2e, "unit": "Mpaths/s", "h2d_bytes_per_step": C.sizeof(api.IntegratorParamsC),
                "d2h_bytes_per_step": W * H * 12},
        "gpu_launches": agg["kernel_launches"] // len(stats) * args.steps,
        "mrays_per_s": total_rays / len(stats) * args.steps * world / (ms_max / 1e3) / 1e6,
        "roofline": roofline,
        "wavefront_roofline": wavefront,
        "cpu_baseline": cpu,
        "clocks": clk,
        "stage_ms": {"plan": stage_ms[0], "generate": stage_ms[1], "extend": stage_ms[2], "shade": stage_ms[3],
                     "shadow": stage_ms[4]},
        "render_stats": agg,
        "guided_equal_time": guided,
    }
    out.update(extras)
    if svndf_fit is not None:
        out["svndf_fit"] = svndf_fit
    print(json.dumps(out))
    if dist:
        dist.destroy_process_group()
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "batch":
        return run_batch(args)
    if args.workload == "mfnm":
        return run_mfnm(args)
    return run_xgb(args)


if __name__ == "__main__":
    sys.exit(main())
