"""Backend-neutral scene description.

A ``SceneDesc`` records what a Xitils program passes to the reference's
construction API -- ``TriangleMesh::setGeometry`` (TriangleMesh.h:151-161),
``Object(shape, material, transform)`` (Object.h:32-34), the material
constructors (Material.h), ``Scene::addObject`` (Scene.h:17-22), the camera and
the sky -- as plain numpy arrays, and replays it into any backend that exposes
the same calls: the GPU library (``xitils_gb300.api``) or, in tests, the CPU
checkers.
"""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import Optional

import numpy as np

from .transform import Transform

# Material kinds (same numbering as the C ABI's xgb_material_kind).
DIFFUSE, METAL, GLOSSY, GLOSSY_HIGHLIGHT, GLOSSY_CLAMPED, EMISSION = 0, 1, 2, 3, 4, 5
SPECULAR_REFLECTION, SPECULAR_REFRACTION, SPECULAR_FRESNEL, MF_NORMALMAP = 6, 7, 8, 9
MULTILOBE_SVBRDF = 10  # base material + SVNDF (the displacement sandbox's MultiLobeSVBRDF)
# Sky kinds.
SKY_NONE, SKY_UNIFORM, SKY_PROBE, SKY_LATLONG = 0, 1, 2, 3
# Integrators.
STANDARD, NAIVE = 0, 1


@dataclass
class TextureDesc:
    rgb: Optional[np.ndarray]  # float32 [h, w, 3]; None for the low-resolution texture of an SVNDF
    clamp: bool = True
    filter: bool = True
    svndf: Optional[tuple] = None  # (source texture, displacement scale, rate, seed) of a derived texture


@dataclass
class MeshDesc:
    pos: np.ndarray  # float32 [nV, 3]
    idx: np.ndarray  # int32 [nIdx]
    uv: Optional[np.ndarray] = None
    nrm: Optional[np.ndarray] = None
    tan: Optional[np.ndarray] = None
    bit: Optional[np.ndarray] = None
    shell: Optional[tuple] = None  # (displacement texture, scale, layers): shell-mapped mesh

    @property
    def n_tris(self) -> int:
        return int(self.idx.size // 3) * (self.shell[2] if self.shell else 1)


@dataclass
class MaterialDesc:
    kind: int
    f: list
    base: int = -1
    tex: int = -1
    normalmap: int = -1


@dataclass
class ObjectDesc:
    mesh: int
    material: int
    transform: Transform


@dataclass
class IntegratorParams:
    """Integrator settings. Reference defaults: no depth limit, Russian roulette
    when pathLength > 5 with survival 0.9 (PathTracer.h:253-257)."""
    integrator: int = STANDARD
    max_depth: int = 0
    rr_start: int = 5
    rr_prob: float = 0.9
    seed: int = 0
    queue_capacity: int = 0


@dataclass
class SceneDesc:
    name: str = "scene"
    textures: list = field(default_factory=list)
    meshes: list = field(default_factory=list)
    materials: list = field(default_factory=list)
    objects: list = field(default_factory=list)
    camera: tuple = None  # (Transform, fov_radians, aspect)
    sky: tuple = (SKY_NONE, None, -1)
    width: int = 64
    height: int = 64
    spp: int = 1
    params: IntegratorParams = field(default_factory=IntegratorParams)
    fixes: int = 0  # opt-in quirk fixes of the render (2 = drop non-finite contributions)
    svndf_count: int = 0

    # -- construction -----------------------------------------------------
    def add_texture(self, rgb: np.ndarray, clamp: bool = True, filter: bool = True) -> int:
        rgb = np.ascontiguousarray(rgb, dtype=np.float32)
        assert rgb.ndim == 3 and rgb.shape[2] == 3
        self.textures.append(TextureDesc(rgb, clamp, filter))
        return len(self.textures) - 1

    def add_mesh(self, pos, idx, uv=None, nrm=None, tan=None, bit=None) -> int:
        c = lambda a, k: None if a is None else np.ascontiguousarray(np.asarray(a, dtype=np.float32).reshape(-1, k))
        m = MeshDesc(c(pos, 3), np.ascontiguousarray(np.asarray(idx, dtype=np.int32).reshape(-1)),
                     c(uv, 2), c(nrm, 3), c(tan, 3), c(bit, 3))
        self.meshes.append(m)
        return len(self.meshes) - 1

    def add_mesh_shell(self, pos, idx, uv, nrm, tan, bit, displacement: int, scale: float, layers: int) -> int:
        """Shell-mapped mesh (TriangleMesh::setGeometryWithShellMapping): `layers`
        copies offset along the normals up to `scale`, texture `displacement`'s
        red channel deciding which copy is hit."""
        i = self.add_mesh(pos, idx, uv, nrm, tan, bit)
        m = self.meshes[i]
        assert all(a is not None for a in (m.uv, m.nrm, m.tan, m.bit)), "shell mapping needs every attribute"
        m.shell = (int(displacement), float(scale), int(layers))
        return i

    def add_svndf(self, displacement: int, scale: float, rate: int = 8, seed: int = 0):
        """SVNDF of a displacement texture (the displacement sandbox's
        downsampleDisplacementTexture): per rate x rate block a 4-lobe vMF fit of the
        block's normals and the block's mean height. Returns (svndf id, id of the
        low-resolution height texture, which is added to the textures)."""
        src = self.textures[displacement]
        self.textures.append(TextureDesc(None, src.clamp, True, (int(displacement), float(scale), int(rate), int(seed))))
        self.svndf_count += 1
        return self.svndf_count - 1, len(self.textures) - 1

    def add_material(self, kind: int, f=(), base: int = -1, tex: int = -1, normalmap: int = -1) -> int:
        self.materials.append(MaterialDesc(kind, [float(x) for x in f], base, tex, normalmap))
        return len(self.materials) - 1

    def diffuse(self, albedo, tex: int = -1, normalmap: int = -1) -> int:
        return self.add_material(DIFFUSE, albedo, tex=tex, normalmap=normalmap)

    def metal(self, roughness: float, f0, rough_tex: int = -1, normalmap: int = -1, horizon_fix: bool = False) -> int:
        """Metal (GGX conductor); horizon_fix = the opt-in below-horizon fix
        (XGB_FIX_METAL_HORIZON), which the reference does not have."""
        f = [roughness, *f0] + ([1.0] if horizon_fix else [])
        return self.add_material(METAL, f, tex=rough_tex, normalmap=normalmap)

    def emission(self, power) -> int:
        return self.add_material(EMISSION, power)

    def add_object(self, mesh: int, material: int, transform: Optional[Transform] = None) -> int:
        self.objects.append(ObjectDesc(mesh, material, transform or Transform.identity()))
        return len(self.objects) - 1

    def set_camera(self, c2w: Transform, fov: float, aspect: float) -> None:
        self.camera = (c2w, float(fov), float(aspect))

    def set_sky(self, kind: int, rgb=None, tex: int = -1) -> None:
        self.sky = (kind, None if rgb is None else [float(x) for x in rgb], tex)

    # -- facts ---------------------------------------------------------------
    @property
    def n_tris(self) -> int:
        return sum(self.meshes[o.mesh].n_tris for o in self.objects)

    @property
    def n_paths(self) -> int:
        return self.width * self.height * self.spp

    def bounds(self):
        """World-space box (lo, hi) of every object's vertices (float64)."""
        lo, hi = np.full(3, np.inf), np.full(3, -np.inf)
        for o in self.objects:
            mesh = self.meshes[o.mesh]
            p = mesh.pos.astype(np.float64)
            if mesh.shell:  # the top layer too
                p = np.concatenate([p, p + mesh.shell[1] * mesh.nrm.astype(np.float64)])
            m = np.asarray(o.transform.mat, np.float64).reshape(4, 4)
            w = p @ m[:3, :3].T + m[:3, 3]
            lo, hi = np.minimum(lo, w.min(axis=0)), np.maximum(hi, w.max(axis=0))
        return lo, hi

    # -- replay ----------------------------------------------------------------
    def emit(self, backend):
        """Replay into a backend exposing add_texture / add_mesh / add_material /
        add_object / set_camera / set_sky / build (see xitils_gb300.api.Scene and
        the CPU checker bindings)."""
        for t in self.textures:
            if t.svndf is not None:
                backend.add_svndf(*t.svndf)
            else:
                backend.add_texture(t.rgb, t.clamp, t.filter)
        for m in self.meshes:
            if m.shell:
                backend.add_mesh_shell(m.pos, m.idx, m.uv, m.nrm, m.tan, m.bit, *m.shell)
            else:
                backend.add_mesh(m.pos, m.idx, m.uv, m.nrm, m.tan, m.bit)
        for mt in self.materials:
            backend.add_material(mt.kind, mt.f, mt.base, mt.tex, mt.normalmap)
        for o in self.objects:
            backend.add_object(o.mesh, o.material, o.transform.mat, o.transform.matInv)
        c2w, fov, aspect = self.camera
        backend.set_camera(c2w.mat, c2w.matInv, fov, aspect)
        kind, rgb, tex = self.sky
        backend.set_sky(kind, rgb, tex)
        if self.fixes:
            backend.set_fixes(self.fixes)
        backend.build()
        return backend
