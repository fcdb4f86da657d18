"""Seeded synthetic scenes for the benchmark workloads.

No external asset is used: every mesh, texture and environment map is generated
here from a fixed seed, with the sizes and value distributions of the workloads
(Cornell box, fBm heightfield terrain, batched random scenes, occluded-light
room, microfacet-normal-mapped terrain). Scenes are built through the same
construction calls a Xitils program makes (``SceneDesc`` records them).
"""
from __future__ import annotations

import math

import numpy as np

from .scene import (DIFFUSE, EMISSION, METAL, MF_NORMALMAP, SKY_LATLONG, SKY_UNIFORM, IntegratorParams, SceneDesc)
from .transform import Transform, transformTRS, translate

F = np.float32


# ------------------------------------------------------------------ helpers --
def _normalize32(v):
    v = np.asarray(v, dtype=F)
    l2 = F(F(v[0] * v[0] + v[1] * v[1]) + F(v[2] * v[2]))
    inv = F(F(1) / F(np.sqrt(l2)))
    return (v * inv).astype(F)


def _cross64(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return np.array([a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]], dtype=F)


def look_at(pos, look, up) -> Transform:
    """lookAt (Transform.h:344-368): columns right / newUp / dir, translation pos;
    like the reference, the stored inverse is the transpose."""
    pos = np.asarray(pos, dtype=F)
    d = _normalize32(np.asarray(look, dtype=F) - pos)
    right = _normalize32(_cross64(_normalize32(up), d))
    new_up = _cross64(d, right)
    m = np.zeros((4, 4), dtype=F)
    m[:3, 0], m[:3, 1], m[:3, 2], m[:3, 3] = right, new_up, d, pos
    m[3, 3] = 1
    return Transform.from_matrix(m)


def unit_cube_mesh():
    """The reference's Cube (TriangleMesh.h:369-397): corners at +-0.5."""
    pos = np.array([[-0.5 if i & 1 else 0.5, -0.5 if i & 2 else 0.5, -0.5 if i & 4 else 0.5] for i in range(8)], dtype=F)
    idx = np.array([0, 1, 2, 1, 3, 2, 2, 3, 6, 3, 7, 6, 0, 4, 1, 4, 5, 1, 0, 2, 6, 0, 6, 4,
                    1, 5, 3, 5, 7, 3, 4, 6, 5, 6, 7, 5], dtype=np.int32)
    return pos, idx


def quad(p0, p1, p2, p3):
    """Two triangles (p0,p1,p2), (p0,p2,p3); geometric normal = cross(p1-p0, p2-p0)."""
    return np.array([p0, p1, p2, p3], dtype=F), np.array([0, 1, 2, 0, 2, 3], dtype=np.int32)


# ---------------------------------------------------------------- Cornell box --
def cornell(width: int = 512, height: int = 512, spp: int = 16, max_depth: int = 8, rr_start: int = 3,
            seed: int = 0) -> SceneDesc:
    """Cornell box: unit box [0,1]^3 of 5 quads (Lambert 0.75 grey, left wall
    (0.63,0.065,0.05), right wall (0.14,0.45,0.09)), a 0.3x0.6x0.3 box rotated 15
    degrees and a 0.3x0.3x0.3 box rotated -18 degrees, a 0.25x0.25 light quad at
    y=0.999 facing -y with radiance (17,12,4). 36 triangles."""
    s = SceneDesc(name="cornell", width=width, height=height, spp=spp,
                  params=IntegratorParams(max_depth=max_depth, rr_start=rr_start, rr_prob=0.9, seed=seed))
    grey = s.diffuse([0.75, 0.75, 0.75])
    red = s.diffuse([0.63, 0.065, 0.05])
    green = s.diffuse([0.14, 0.45, 0.09])
    light = s.emission([17.0, 12.0, 4.0])
    walls = [
        (quad([0, 0, 0], [1, 0, 0], [1, 0, 1], [0, 0, 1]), grey),    # floor
        (quad([0, 1, 0], [0, 1, 1], [1, 1, 1], [1, 1, 0]), grey),    # ceiling
        (quad([0, 0, 1], [1, 0, 1], [1, 1, 1], [0, 1, 1]), grey),    # back
        (quad([0, 0, 0], [0, 0, 1], [0, 1, 1], [0, 1, 0]), red),     # left (x = 0)
        (quad([1, 0, 0], [1, 1, 0], [1, 1, 1], [1, 0, 1]), green),   # right (x = 1)
    ]
    for (pos, idx), mat in walls:
        s.add_object(s.add_mesh(pos, idx), mat)
    lo, hi, y = 0.375, 0.625, 0.999
    pos, idx = quad([lo, y, lo], [hi, y, lo], [hi, y, hi], [lo, y, hi])  # normal -y
    s.add_object(s.add_mesh(pos, idx), light)
    cpos, cidx = unit_cube_mesh()
    cube = s.add_mesh(cpos, cidx)
    s.add_object(cube, grey, transformTRS((0.33, 0.3, 0.62), (0, 15, 0), (0.3, 0.6, 0.3)))
    s.add_object(cube, grey, transformTRS((0.67, 0.15, 0.33), (0, -18, 0), (0.3, 0.3, 0.3)))
    s.set_camera(translate(0.5, 0.5, -1.3), 40.0 * math.pi / 180.0, height / width)
    return s


# ------------------------------------------------------------------ terrain --
def fbm_heights(n: int, seed: int, octaves: int = 6, amplitude: float = 0.15, lacunarity: float = 2.0,
                gain: float = 0.5, base_cells: int = 4) -> np.ndarray:
    """Value-noise fBm on an n x n vertex grid over [0,1]^2 (float32)."""
    rng = np.random.default_rng(seed)
    x = np.linspace(0.0, 1.0, n, dtype=np.float64)
    h = np.zeros((n, n), dtype=np.float64)
    amp, cells, norm = 1.0, base_cells, 0.0
    for _ in range(octaves):
        lattice = rng.random((cells + 2, cells + 2))
        g = x * cells
        i0 = np.floor(g).astype(np.int64)
        t = g - i0
        t = t * t * (3 - 2 * t)
        i1 = i0 + 1
        a = lattice[np.ix_(i0, i0)]
        b = lattice[np.ix_(i0, i1)]
        c = lattice[np.ix_(i1, i0)]
        d = lattice[np.ix_(i1, i1)]
        tz, tx = t[:, None], t[None, :]
        h += amp * ((a * (1 - tx) + b * tx) * (1 - tz) + (c * (1 - tx) + d * tx) * tz)
        norm += amp
        amp *= gain
        cells = int(cells * lacunarity)
    return (amplitude * h / norm).astype(F)


def heightfield_mesh(heights: np.ndarray, extent: float = 1.0):
    n = heights.shape[0]
    g = np.linspace(0.0, extent, n, dtype=F)
    xx, zz = np.meshgrid(g, g)
    pos = np.stack([xx, heights, zz], axis=-1).reshape(-1, 3).astype(F)
    u = np.linspace(0.0, 1.0, n, dtype=F)
    uu, vv = np.meshgrid(u, u)
    uv = np.stack([uu, vv], axis=-1).reshape(-1, 2).astype(F)
    i = np.arange(n - 1, dtype=np.int64)
    r, c = np.meshgrid(i, i, indexing="ij")
    v00 = (r * n + c).ravel()
    v01, v10, v11 = v00 + 1, v00 + n, v00 + n + 1
    idx = np.stack([v00, v10, v11, v00, v11, v01], axis=-1).reshape(-1).astype(np.int32)
    return pos, uv, idx


def latlong_sky(width: int = 1024, height: int = 512, sun_dir=(0.45, 0.55, -0.35), kappa: float = 2000.0,
                peak: float = 5.0e4) -> np.ndarray:
    """Procedural HDR lat-long map: sky gradient plus a sun lobe
    peak * exp(kappa * (mu . w - 1)). Texel (i, j) looks along the direction with
    u = atan2(x, -z) / 2pi + 1/2, v = acos(y) / pi (the lat-long lookup)."""
    u = (np.arange(width) + 0.5) / width
    v = (np.arange(height) + 0.5) / height
    phi = (u - 0.5) * 2 * np.pi
    theta = v * np.pi
    st, ct = np.sin(theta)[:, None], np.cos(theta)[:, None]
    x = st * np.sin(phi)[None, :]
    y = np.broadcast_to(ct, (height, width))
    z = -st * np.cos(phi)[None, :]
    up = np.clip(y, 0.0, 1.0)[..., None]
    horizon = np.array([0.95, 0.9, 0.85])
    zenith = np.array([0.25, 0.45, 0.95])
    ground = np.array([0.18, 0.15, 0.12])
    sky = np.where(y[..., None] >= 0.0, horizon * (1 - np.sqrt(up)) + zenith * np.sqrt(up), ground)
    mu = np.asarray(sun_dir, dtype=np.float64)
    mu = mu / np.linalg.norm(mu)
    cosw = x * mu[0] + y * mu[1] + z * mu[2]
    sun = peak * np.exp(kappa * (cosw - 1.0))
    rgb = sky + sun[..., None] * np.array([1.0, 0.92, 0.8])
    return rgb.astype(F)


def terrain(grid: int = 1024, width: int = 1024, height: int = 1024, spp: int = 64, max_depth: int = 10,
            seed: int = 7, env_size=(1024, 512)) -> SceneDesc:
    """Displacement-heightfield terrain: grid x grid vertices (2*(grid-1)^2
    triangles) with seeded 6-octave fBm heights (amplitude 0.15, lacunarity 2,
    gain 0.5), a GGX conductor whose roughness is uniform per texel in
    [0.05, 0.5], lit by a procedural lat-long HDR environment (sky gradient plus
    a kappa=2000 sun lobe of peak radiance 5e4)."""
    s = SceneDesc(name="terrain", width=width, height=height, spp=spp,
                  params=IntegratorParams(max_depth=max_depth, rr_start=5, rr_prob=0.9, seed=seed))
    h = fbm_heights(grid, seed)
    pos, uv, idx = heightfield_mesh(h)
    rng = np.random.default_rng(seed + 1)
    cells = max(grid - 1, 1)
    rough = rng.uniform(0.05, 0.5, size=(cells, cells)).astype(F)
    rough_tex = s.add_texture(np.repeat(rough[..., None], 3, axis=2), clamp=True, filter=False)
    env = s.add_texture(latlong_sky(*env_size), clamp=True, filter=True)
    mat = s.metal(0.3, [0.95, 0.64, 0.54], rough_tex=rough_tex)
    s.add_object(s.add_mesh(pos, idx, uv=uv), mat)
    s.set_sky(SKY_LATLONG, tex=env)
    s.set_camera(look_at((0.5, 0.42, -0.25), (0.5, 0.02, 0.55), (0, 1, 0)), 50.0 * math.pi / 180.0, height / width)
    return s


def simple_path_tracer_scene(width: int = 128, height: int = 128, spp: int = 4) -> SceneDesc:
    """The reference's SimplePathTracer sandbox scene (Sandbox/SimplePathTracer/
    Main.cpp:66-114) with the Cinder teapot (unavailable) replaced by a Metal(0.3)
    unit cube scaled 1.2 and rotated 15 degrees; reference integrator defaults."""
    s = SceneDesc(name="simple_path_tracer", width=width, height=height, spp=spp, params=IntegratorParams())
    white = s.diffuse([0.8, 0.8, 0.8])
    red = s.diffuse([0.8, 0.1, 0.1])
    green = s.diffuse([0.1, 0.8, 0.1])
    light = s.emission([8.0, 8.0, 7.6])
    metal = s.metal(0.3, [0.9, 0.9, 0.9])
    cpos, cidx = unit_cube_mesh()
    cube = s.add_mesh(cpos, cidx)
    ppos = np.array([[-0.5 if i & 1 else 0.5, -0.5 if i & 2 else 0.5, 0.0] for i in range(4)], dtype=F)
    plane = s.add_mesh(ppos, np.array([0, 2, 1, 1, 2, 3], dtype=np.int32))  # TriangleMesh.h:399-423
    s.add_object(cube, white, transformTRS((0, 0, 0), (0, 0, 0), (4, 0.01, 4)))
    s.add_object(cube, green, transformTRS((2, 2, 0), (0, 0, 0), (0.01, 4, 4)))
    s.add_object(cube, red, transformTRS((-2, 2, 0), (0, 0, 0), (0.01, 4, 4)))
    s.add_object(cube, white, transformTRS((0, 2, 2), (0, 0, 0), (4, 4, 0.01)))
    s.add_object(cube, white, transformTRS((0, 4, 0), (0, 0, 0), (4, 0.01, 4)))
    s.add_object(plane, light, transformTRS((0, 4.0 - 0.01, 0), (-90, 0, 0), (2.0, 2.0, 2.0)))
    s.add_object(cube, metal, transformTRS((0, 0.6, 0), (0, 15, 0), (1.2, 1.2, 1.2)))
    s.set_camera(translate(0, 2.0, -5), 60.0 * math.pi / 180.0, height / width)
    return s


def material_zoo(width: int = 64, height: int = 64, spp: int = 8, sky: str = "none", seed: int = 3,
                 only=None) -> SceneDesc:
    """The SimplePathTracer room plus tangent-space cubes covering every material
    kind: Glossy, GlossyClamped under MicrofacetNormalMapping with a normal map,
    GlossyWithHighLight, SpecularReflection, SpecularFresnel. ``sky`` is one of
    none / uniform / probe / latlong."""
    from .scene import (GLOSSY, GLOSSY_CLAMPED, GLOSSY_HIGHLIGHT, SKY_PROBE, SPECULAR_FRESNEL,
                        SPECULAR_REFLECTION, MaterialDesc)
    s = simple_path_tracer_scene(width, height, spp)
    s.name = f"material_zoo_{sky}"
    rng = np.random.default_rng(seed)
    nm = s.add_texture(np.clip(rng.normal([0.5, 0.5, 1.0], [0.15, 0.15, 0.05], (32, 32, 3)), 0, 1).astype(F))
    s.materials[4] = MaterialDesc(GLOSSY, [0.7, 0.6, 0.5, 40.0])
    base = s.add_material(GLOSSY_CLAMPED, [0.8, 0.8, 0.8, 30.0])
    mf = s.add_material(MF_NORMALMAP, [], base=base, normalmap=nm)
    gh = s.add_material(GLOSSY_HIGHLIGHT, [0.5, 0.5, 0.5, 1, 1, 1, 5.0, 200.0, 0.3])
    spec = s.add_material(SPECULAR_REFLECTION, [])
    fres = s.add_material(SPECULAR_FRESNEL, [1.5])
    cpos, cidx = unit_cube_mesh()
    uv = cpos[:, :2] + 0.5
    nrm = cpos / np.linalg.norm(cpos, axis=1, keepdims=True)
    tan = np.tile([1.0, 0.0, 0.0], (8, 1))
    bit = np.tile([0.0, 1.0, 0.0], (8, 1))
    cm = s.add_mesh(cpos, cidx, uv=uv, nrm=nrm, tan=tan, bit=bit)
    s.add_object(cm, mf, transformTRS((-1.0, 0.7, -0.5), (10, 30, 0), (0.8, 0.8, 0.8)))
    s.add_object(cm, gh, transformTRS((1.2, 0.5, -0.8), (0, -20, 5), (0.6, 0.6, 0.6)))
    s.add_object(cm, spec, transformTRS((1.0, 1.6, 0.5), (0, 40, 0), (0.5, 0.5, 0.5)))
    s.add_object(cm, fres, transformTRS((-1.2, 1.8, 0.2), (20, 10, 0), (0.5, 0.5, 0.5)))
    if sky == "uniform":
        s.set_sky(SKY_UNIFORM, rgb=[0.2, 0.3, 0.4])
    elif sky == "probe":
        s.set_sky(SKY_PROBE, tex=s.add_texture(rng.random((64, 64, 3)).astype(F)))
    elif sky == "latlong":
        s.set_sky(SKY_LATLONG, tex=s.add_texture(latlong_sky(128, 64)))
    if only is not None:  # keep the room plus the listed zoo cubes: 0 mfnm, 1 highlight, 2 mirror, 3 fresnel
        s.objects = s.objects[:7] + [s.objects[7 + k] for k in only]
    return s


def box_mesh(centers, sizes, angles):
    """Axis-aligned boxes (the reference Cube's corner order and triangles) scaled
    per box, rotated about y and translated, merged into one vertex/index array."""
    cpos, cidx = unit_cube_mesh()
    n = len(centers)
    c, s = np.cos(angles), np.sin(angles)
    local = cpos[None, :, :] * sizes[:, None, :]
    x = local[:, :, 0] * c[:, None] + local[:, :, 2] * s[:, None]
    z = -local[:, :, 0] * s[:, None] + local[:, :, 2] * c[:, None]
    pos = np.stack([x, local[:, :, 1], z], axis=2) + centers[:, None, :]
    idx = (cidx[None, :] + 8 * np.arange(n)[:, None]).reshape(-1)
    return pos.reshape(-1, 3).astype(F), idx.astype(np.int32)


def occluded_room(width: int = 1024, height: int = 1024, spp: int = 4, n_boxes: int = 16667, seed: int = 11,
                  max_depth: int = 0) -> SceneDesc:
    """Occluded-light interior: a 10 x 4 x 10 room whose only light, a 0.5 x 0.5
    quad of radiance 200, sits behind a partition wall at x = 8.5 and shines into
    the room through a 1.0 x 0.2 slit; ~200k triangles of seeded random boxes
    (edge lengths U[0.1, 1]) resting on the floor clutter the main room, so paths
    are indirect-dominated."""
    s = SceneDesc(name="occluded_room", width=width, height=height, spp=spp,
                  params=IntegratorParams(max_depth=max_depth, rr_start=5, rr_prob=0.9, seed=seed))
    rng = np.random.default_rng(seed)
    grey = s.diffuse([0.7, 0.7, 0.7])
    light = s.emission([200.0, 200.0, 200.0])
    # room shell (quads facing inward; Diffuse shading is two-sided anyway)
    X, Y, Z, WX = 10.0, 4.0, 10.0, 8.5
    shell = [quad([0, 0, 0], [X, 0, 0], [X, 0, Z], [0, 0, Z]), quad([0, Y, 0], [0, Y, Z], [X, Y, Z], [X, Y, 0]),
             quad([0, 0, 0], [0, 0, Z], [0, Y, Z], [0, Y, 0]), quad([X, 0, 0], [X, Y, 0], [X, Y, Z], [X, 0, Z]),
             quad([0, 0, 0], [0, Y, 0], [X, Y, 0], [X, 0, 0]), quad([0, 0, Z], [X, 0, Z], [X, Y, Z], [0, Y, Z])]
    # partition wall at x = WX with a slit y in [1.9, 2.1], z in [4.5, 5.5]: four panels
    gy0, gy1, gz0, gz1 = 1.9, 2.1, 4.5, 5.5
    panels = [quad([WX, 0, 0], [WX, gy0, 0], [WX, gy0, Z], [WX, 0, Z]),
              quad([WX, gy1, 0], [WX, Y, 0], [WX, Y, Z], [WX, gy1, Z]),
              quad([WX, gy0, 0], [WX, gy1, 0], [WX, gy1, gz0], [WX, gy0, gz0]),
              quad([WX, gy0, gz1], [WX, gy1, gz1], [WX, gy1, Z], [WX, gy0, Z])]
    sizes = rng.uniform(0.1, 1.0, (n_boxes, 3))
    centers = np.stack([rng.uniform(0.3, WX - 0.3, n_boxes), np.zeros(n_boxes), rng.uniform(0.3, Z - 0.3, n_boxes)], 1)
    centers[:, 1] = sizes[:, 1] / 2  # resting on the floor: a clutter layer at most 1 m deep
    bpos, bidx = box_mesh(centers, sizes, rng.uniform(0, np.pi, n_boxes))
    parts = shell + panels + [(bpos, bidx)]
    pos_all, idx_all, off = [], [], 0
    for pos, idx in parts:
        pos_all.append(np.asarray(pos, F))
        idx_all.append(np.asarray(idx, np.int32) + off)
        off += len(pos)
    s.add_object(s.add_mesh(np.concatenate(pos_all), np.concatenate(idx_all)), grey)
    lz, ly, h = 5.0, 2.0, 0.25
    lx = 9.9  # light quad facing -x (toward the slit)
    pos, idx = quad([lx, ly - h, lz - h], [lx, ly - h, lz + h], [lx, ly + h, lz + h], [lx, ly + h, lz - h])
    s.add_object(s.add_mesh(pos, idx), light)
    s.set_camera(look_at((1.2, 2.6, 1.0), (6.0, 1.6, 6.5), (0, 1, 0)), 70.0 * math.pi / 180.0, height / width)
    return s


# ------------------------------------------------------------ batched scenes --
BATCH_RESOLUTIONS = (128, 256, 512, 1024)


def batch_scene(index: int, seed: int = 21, tris_range=(1_000, 500_000), resolutions=BATCH_RESOLUTIONS,
                spp: int = 32, max_depth: int = 8) -> SceneDesc:
    """One scene of the batched-rendering workload: a seeded random triangle soup
    or fBm heightfield in the unit box with a triangle count log-uniform in
    ``tris_range``, split between a Lambert and a GGX (roughness U[0.02, 0.8])
    material, lit by 1-4 quad lights (radiance U[1, 50]) facing down from above
    it; square film from ``resolutions``, ``spp`` samples, max depth 8."""
    rng = np.random.default_rng(seed * 1009 + index)
    n_tris = int(round(math.exp(rng.uniform(math.log(tris_range[0]), math.log(tris_range[1])))))
    res = int(rng.choice(resolutions))
    s = SceneDesc(name=f"batch{index}", width=res, height=res, spp=spp,
                  params=IntegratorParams(max_depth=max_depth, rr_start=5, rr_prob=0.9, seed=index))
    lambert = s.diffuse(rng.uniform(0.2, 0.85, 3))
    ggx = s.metal(float(rng.uniform(0.02, 0.8)), rng.uniform(0.4, 0.95, 3))
    if rng.uniform() < 0.5:  # triangle soup: two halves, one per material
        centers = rng.uniform(0.05, 0.95, (n_tris, 3))
        centers[:, 1] *= 0.6
        size = 1.6 * n_tris ** (-1.0 / 3.0)
        offs = rng.normal(scale=size, size=(n_tris, 3, 3))
        pos = (centers[:, None, :] + offs).reshape(-1, 3).astype(F)
        half = n_tris // 2
        for lo, hi, mat in ((0, half, lambert), (half, n_tris, ggx)):
            if hi > lo:
                idx = np.arange(3 * lo, 3 * hi, dtype=np.int32) - 3 * lo
                s.add_object(s.add_mesh(pos[3 * lo:3 * hi], idx), mat)
    else:  # heightfield: the grid whose triangle count is closest, ground Lambert, a GGX copy raised above it
        g = max(2, int(round(math.sqrt(n_tris / 2.0))) + 1)
        heights = fbm_heights(g, int(rng.integers(1 << 30)))
        hp, huv, hidx = heightfield_mesh(heights)
        s.add_object(s.add_mesh(hp, hidx, uv=huv), lambert if rng.uniform() < 0.5 else ggx)
    n_lights = int(rng.integers(1, 5))
    for k in range(n_lights):
        cx, cz = rng.uniform(0.2, 0.8, 2)
        w = float(rng.uniform(0.05, 0.2))
        y = float(rng.uniform(0.9, 1.3))
        pos, idx = quad([cx - w, y, cz - w], [cx + w, y, cz - w], [cx + w, y, cz + w], [cx - w, y, cz + w])  # normal -y
        s.add_object(s.add_mesh(pos, idx), s.emission([float(rng.uniform(1.0, 50.0))] * 3))
    s.set_camera(look_at((0.5, 1.1, -0.9), (0.5, 0.2, 0.5), (0.0, 1.0, 0.0)), 50.0 * math.pi / 180.0, 1.0)
    return s


# ------------------------------------------------ normal mapping at scale --
def fbm_normal_map(res: int, seed: int, slope: float = 1.5) -> np.ndarray:
    """Tangent-space normal map [res, res, 3] in [0, 1] from the gradients of a
    seeded fBm height field: n = normalize(-slope * dh/du, -slope * dh/dv, 1),
    stored as n * 0.5 + 0.5 (r = tangent, g = bitangent, b = normal, the
    reference's decoding n = rgb * 2 - 1, Object.h:58-68)."""
    h = fbm_heights(res, seed, amplitude=1.0).astype(np.float64)
    gv, gu = np.gradient(h)  # rows follow v, columns follow u
    n = np.stack([-slope * gu * res / 16.0, -slope * gv * res / 16.0, np.ones_like(h)], axis=-1)
    n /= np.linalg.norm(n, axis=-1, keepdims=True)
    return (n * 0.5 + 0.5).astype(F)


def heightfield_frames(heights: np.ndarray, extent: float = 1.0):
    """Per-vertex normal, tangent (along +x = +u) and bitangent (along +z = +v) of
    a heightfield from central differences."""
    n = heights.shape[0]
    h = heights.astype(np.float64)
    step = extent / max(n - 1, 1)
    dz, dx = np.gradient(h, step)  # axis 0 = z (rows), axis 1 = x
    t = np.stack([np.ones_like(h), dx, np.zeros_like(h)], axis=-1)
    b = np.stack([np.zeros_like(h), dz, np.ones_like(h)], axis=-1)
    t /= np.linalg.norm(t, axis=-1, keepdims=True)
    b /= np.linalg.norm(b, axis=-1, keepdims=True)
    nrm = np.cross(b, t)
    nrm /= np.linalg.norm(nrm, axis=-1, keepdims=True)
    f = lambda a: a.reshape(-1, 3).astype(F)
    return f(nrm), f(t), f(b)


def mfnm_at_scale(width: int = 2048, height: int = 2048, spp: int = 256, grid: int = 1415, n_boxes: int = 64,
                  normal_res: int = 2048, seed: int = 17, max_depth: int = 12, env_size=(1024, 512)) -> SceneDesc:
    """Microfacet-based normal mapping at scale: a seeded fBm heightfield of
    grid x grid vertices (2 (grid - 1)^2 triangles; 3,998,792 at 1415) and
    n_boxes instanced boxes, all under MicrofacetNormalMapping (same-material
    tangent facets) over a GGX conductor (with the below-horizon fix) whose
    roughness is uniform per texel in [0.1, 0.4], with a normal_res^2 normal map from fBm gradients (slope scale
    1.5); lit by the procedural lat-long environment plus 2 quad lights.
    Reference Russian roulette (after 5 at 0.9) and max depth 12."""
    # 2^21 paths in flight: the normal-mapping walk re-reads the 2048^2 normal map at
    # every facet bounce, and a smaller queue streams less past it through L2
    # (95 against 91 Mpaths/s with the default 2^23)
    s = SceneDesc(name="mfnm_at_scale", width=width, height=height, spp=spp,
                  params=IntegratorParams(max_depth=max_depth, rr_start=5, rr_prob=0.9, seed=seed,
                                          queue_capacity=1 << 21))
    rng = np.random.default_rng(seed)
    h = fbm_heights(grid, seed)
    pos, uv, idx = heightfield_mesh(h)
    nrm, tan, bit = heightfield_frames(h)
    nm = s.add_texture(fbm_normal_map(normal_res, seed + 1), clamp=False, filter=True)
    cells = 256
    rough = rng.uniform(0.1, 0.4, size=(cells, cells)).astype(F)
    rough_tex = s.add_texture(np.repeat(rough[..., None], 3, axis=2), clamp=False, filter=False)
    # the reference's Metal returns NaN inside the normal-mapping random walk
    # (below-horizon facet configurations): the opt-in horizon fix keeps it finite
    base = s.metal(0.25, [0.95, 0.93, 0.88], rough_tex=rough_tex, horizon_fix=True)
    mf = s.add_material(MF_NORMALMAP, [], base=base, normalmap=nm)
    s.add_object(s.add_mesh(pos, idx, uv=uv * 8.0, nrm=nrm, tan=tan, bit=bit), mf)
    cpos, cidx = unit_cube_mesh()
    cuv = cpos[:, :2] + 0.5
    cnrm = cpos / np.linalg.norm(cpos, axis=1, keepdims=True)
    cube = s.add_mesh(cpos, cidx, uv=cuv, nrm=cnrm, tan=np.tile([1.0, 0.0, 0.0], (8, 1)),
                      bit=np.tile([0.0, 1.0, 0.0], (8, 1)))
    for _ in range(n_boxes):
        x, z = rng.uniform(0.05, 0.95, 2)
        size = float(rng.uniform(0.02, 0.08))
        y = float(h[int(z * (grid - 1)), int(x * (grid - 1))]) + 0.5 * size
        s.add_object(cube, mf, transformTRS((x, y, z), (0.0, float(rng.uniform(0, 90)), 0.0), (size, size, size)))
    for k in range(2):
        cx, cz = (0.3, 0.35) if k == 0 else (0.7, 0.6)
        w, y = 0.06, 0.45
        lp, li = quad([cx - w, y, cz - w], [cx + w, y, cz - w], [cx + w, y, cz + w], [cx - w, y, cz + w])  # normal -y
        s.add_object(s.add_mesh(lp, li), s.emission([30.0, 27.0, 22.0]))
    s.set_sky(SKY_LATLONG, tex=s.add_texture(latlong_sky(*env_size), clamp=True, filter=True))
    s.set_camera(look_at((0.5, 0.42, -0.25), (0.5, 0.02, 0.55), (0, 1, 0)), 50.0 * math.pi / 180.0, height / width)
    s.fixes = 2  # samples the normal-mapping walk still turns non-finite (0/0 facet weights) are dropped
    return s


# ------------------------------------------------------- shell-mapped fabric --
def weave_displacement(res: int = 256, threads: int = 8) -> np.ndarray:
    """Plain-weave height map [res, res, 3] in [0, 1]: warp threads along v and
    weft threads along u with round cross-sections, each passing over and under
    the crossing threads in turn (r = g = b = height)."""
    x = (np.arange(res, dtype=np.float64) + 0.5) / res * threads
    X, Y = np.meshgrid(x, x)  # X follows u (columns), Y follows v (rows)
    cx = np.abs(np.mod(X, 1.0) - 0.5) * 2.0
    cy = np.abs(np.mod(Y, 1.0) - 0.5) * 2.0
    warp = np.sqrt(np.clip(1.0 - cx * cx, 0.0, 1.0)) * (0.55 + 0.45 * np.sin(np.pi * (Y + np.floor(X))))
    weft = np.sqrt(np.clip(1.0 - cy * cy, 0.0, 1.0)) * (0.55 - 0.45 * np.sin(np.pi * (X + np.floor(Y))))
    h = np.clip(np.maximum(warp, weft), 0.0, 1.0)
    return np.repeat(h[..., None], 3, axis=2).astype(F)


def shell_fabric(width: int = 512, height: int = 512, spp: int = 16, grid: int = 96, layers: int = 16,
                 disp_scale: float = 0.012, tiling: float = 6.0, tex_res: int = 256, max_depth: int = 0,
                 seed: int = 5, method: str = "shell", rate: int = 8) -> SceneDesc:
    """Displacement-mapped fabric by shell mapping, after the reference's
    displacement sandbox (a cloth under GlossyWithHighLight((0.8, 0.2, 0.2), 1, 2,
    10, 0.05) with 16 shell layers in a Cornell-style room lit from the ceiling):
    a draped grid x grid cloth patch whose texcoords tile a plain-weave height map
    `tiling` times, layers copies up to disp_scale along the normals, inside a
    unit room with a 0.4 x 0.4 ceiling light. Reference integrator defaults
    (no depth limit, Russian roulette after 5 at 0.9) unless max_depth is set.

    method = "svbrdf" is the sandbox's naive prefiltering (MethodModeMultiLobeSVBRDF):
    the displacement map is downsampled by `rate` with a 4-lobe vMF SVNDF fitted per
    low texel, the shells follow the low-resolution map and the material is
    MultiLobeSVBRDF(base, low map, scale, SVNDF)."""
    from .scene import GLOSSY_HIGHLIGHT
    s = SceneDesc(name="shell_fabric", width=width, height=height, spp=spp,
                  params=IntegratorParams(max_depth=max_depth, rr_start=5, rr_prob=0.9, seed=seed))
    white = s.diffuse([0.6, 0.6, 0.6])
    red = s.diffuse([0.8, 0.1, 0.1])
    green = s.diffuse([0.1, 0.8, 0.1])
    walls = [
        (quad([0, 0, 0], [1, 0, 0], [1, 0, 1], [0, 0, 1]), white),   # floor
        (quad([0, 1, 0], [0, 1, 1], [1, 1, 1], [1, 1, 0]), white),   # ceiling
        (quad([0, 0, 1], [1, 0, 1], [1, 1, 1], [0, 1, 1]), white),   # back
        (quad([0, 0, 0], [0, 0, 1], [0, 1, 1], [0, 1, 0]), red),     # left
        (quad([1, 0, 0], [1, 1, 0], [1, 1, 1], [1, 0, 1]), green),   # right
    ]
    for (pos, idx), mat in walls:
        s.add_object(s.add_mesh(pos, idx), mat)
    lo, hi, y = 0.3, 0.7, 0.999
    lp, li = quad([lo, y, lo], [hi, y, lo], [hi, y, hi], [lo, y, hi])  # normal -y
    s.add_object(s.add_mesh(lp, li), s.emission([8.0, 8.0, 7.6]))
    # draped cloth: gentle folds over [0.1, 0.9]^2 at y ~ 0.1
    g = np.linspace(0.0, 1.0, grid, dtype=np.float64)
    xx, zz = np.meshgrid(g, g)
    hts = 0.06 * np.sin(2.5 * np.pi * xx + 0.7) * np.cos(1.5 * np.pi * zz) + 0.1
    heights = hts.astype(F)
    pos, uv, idx = heightfield_mesh(heights)
    pos = pos.copy()
    pos[:, 0] = 0.1 + 0.8 * pos[:, 0]
    pos[:, 2] = 0.1 + 0.8 * pos[:, 2]
    nrm, tan, bit = heightfield_frames(heights * F(1.0 / 0.8), extent=1.0)
    disp = s.add_texture(weave_displacement(tex_res), clamp=False, filter=True)
    base = s.add_material(GLOSSY_HIGHLIGHT, [0.8, 0.2, 0.2, 1.0, 1.0, 1.0, 2.0, 10.0, 0.05])
    if method == "svbrdf":
        from .scene import MULTILOBE_SVBRDF
        svndf, low = s.add_svndf(disp, disp_scale, rate, seed)
        cloth = s.add_mesh_shell(pos, idx, uv * F(tiling), nrm, tan, bit, low, disp_scale, layers)
        s.add_object(cloth, s.add_material(MULTILOBE_SVBRDF, [], base=base, tex=svndf))
    else:
        cloth = s.add_mesh_shell(pos, idx, uv * F(tiling), nrm, tan, bit, disp, disp_scale, layers)
        s.add_object(cloth, base)
    s.set_camera(look_at((0.5, 0.55, -0.35), (0.5, 0.08, 0.5), (0, 1, 0)), 40.0 * math.pi / 180.0, height / width)
    return s
