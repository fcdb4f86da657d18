"""Python binding of the C ABI (include/xgb.h) over ctypes.

The classes mirror the reference's construction API so that a Xitils program
reads the same: ``TriangleMesh.setGeometry``, ``Object(mesh, material,
transform)``, ``Scene.addObject / buildAccelerationStructure``,
``PinholeCamera``, the material classes, ``RenderTarget.render``. Everything
runs on the GPU through libxgb.so; there is no CPU fallback -- constructing a
``Context`` without the built library or without a CUDA device raises.
"""
from __future__ import annotations

import ctypes as C
import os
from typing import Optional

import numpy as np

from .scene import (DIFFUSE, EMISSION, GLOSSY, GLOSSY_CLAMPED, GLOSSY_HIGHLIGHT, METAL, MF_NORMALMAP, MULTILOBE_SVBRDF,
                    NAIVE, SKY_LATLONG, SKY_NONE, SKY_PROBE, SKY_UNIFORM, SPECULAR_FRESNEL, SPECULAR_REFLECTION,
                    SPECULAR_REFRACTION, STANDARD, IntegratorParams)
from .transform import Transform

LIB_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "libxgb.so")

STATUS = {0: "OK", 1: "INVALID_ARG", 2: "OOM", 3: "CUDA_ERROR", 4: "QUEUE_OVERFLOW", 5: "DEVICE_TIMEOUT",
          6: "NOT_BUILT", 7: "UNSUPPORTED"}


class XgbError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS.get(status, status)}: {message}")
        self.status = status


class IntegratorParamsC(C.Structure):
    _fields_ = [("integrator", C.c_int), ("max_depth", C.c_int), ("rr_start", C.c_int), ("rr_prob", C.c_float),
                ("seed", C.c_uint32), ("queue_capacity", C.c_int)]


class BatchJobC(C.Structure):
    _fields_ = [("scene", C.c_void_p), ("film", C.c_void_p), ("params", IntegratorParamsC), ("spp_begin", C.c_uint32),
                ("spp_count", C.c_uint32)]


class BatchOptionsC(C.Structure):
    _fields_ = [("queue_capacity", C.c_int), ("iterations_per_sync", C.c_int), ("use_graph", C.c_int)]


class RenderStatsC(C.Structure):
    _fields_ = [("paths", C.c_uint64), ("extension_rays", C.c_uint64), ("shadow_rays", C.c_uint64),
                ("iterations", C.c_uint64), ("kernel_launches", C.c_uint64), ("node_visits", C.c_uint64),
                ("tri_tests", C.c_uint64), ("error_flags", C.c_uint32), ("profiled", C.c_uint32),
                ("kernel_ms", C.c_double * 5), ("stage_launches", C.c_uint64 * 5),
                ("guide_train_steps", C.c_uint64), ("guide_infer_ms", C.c_double), ("guide_train_ms", C.c_double)]


_lib = None
P = C.c_void_p
FP = C.POINTER(C.c_float)


def load_library(path: str = LIB_PATH) -> C.CDLL:
    """Loads libxgb.so; raises if it has not been built (no fallback)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise FileNotFoundError(f"{path} is missing: run __graft_entry__.build() (python -m xitils_gb300.build)")
    lib = C.CDLL(path)
    sig = {
        "xgb_ctx_create": [C.c_int, C.POINTER(P)],
        "xgb_ctx_destroy": [P],
        "xgb_ctx_synchronize": [P, P],
        "xgb_ctx_set_bvh_builder": [P, C.c_int],
        "xgb_ctx_set_bvh_layout": [P, C.c_int],
        "xgb_ctx_set_path_order": [P, C.c_int, C.c_int],
        "xgb_ctx_set_sample_grouping": [P, C.c_int],
        "xgb_scene_intersect": [P, C.c_int, FP, FP, P],
        "xgb_scene_occluded": [P, C.c_int, FP, C.POINTER(C.c_int32), P],
        "xgb_film_enable_aovs": [P],
        "xgb_film_tonemap": [P, C.c_float, C.c_float, C.c_float, C.POINTER(C.c_uint8), P],
        "xgb_film_error_map": [P, C.c_float, P, C.c_float, C.c_float, C.POINTER(C.c_uint8), P],
        "xgb_write_png": [C.c_char_p, C.c_int, C.c_int, C.POINTER(C.c_uint8)],
        "xgb_film_download_aov": [P, C.c_int, FP, C.c_int, P],
        "xgb_texture_create": [P, C.c_int, C.c_int, C.c_int, FP, C.c_int, C.c_int, C.POINTER(P)],
        "xgb_texture_destroy": [P],
        "xgb_mesh_create": [P, C.c_int, FP, FP, FP, FP, FP, C.c_int, C.c_int, C.c_int, C.POINTER(C.c_int32), C.POINTER(P)],
        "xgb_mesh_create_shell": [P, C.c_int, FP, FP, FP, FP, FP, C.c_int, C.c_int, C.c_int, C.POINTER(C.c_int32), P,
                                  C.c_float, C.c_int, C.POINTER(P)],
        "xgb_svndf_create": [P, P, C.c_float, C.c_int, C.c_uint32, C.POINTER(P), C.POINTER(P)],
        "xgb_svndf_destroy": [P],
        "xgb_svndf_size": [P, C.POINTER(C.c_int), C.POINTER(C.c_int)],
        "xgb_svndf_get_lobes": [P, FP],
        "xgb_svndf_set_lobes": [P, FP],
        "xgb_material_multilobe_svbrdf": [P, P, P, C.POINTER(P)],
        "xgb_mesh_destroy": [P],
        "xgb_mesh_triangle_count": [P, C.POINTER(C.c_int)],
        "xgb_material_diffuse": [P, FP, P, C.POINTER(P)],
        "xgb_material_metal": [P, C.c_float, FP, P, C.POINTER(P)],
        "xgb_material_glossy": [P, FP, C.c_float, C.POINTER(P)],
        "xgb_material_glossy_highlight": [P, FP, FP, C.c_float, C.c_float, C.c_float, C.POINTER(P)],
        "xgb_material_glossy_clamped": [P, FP, C.c_float, C.POINTER(P)],
        "xgb_material_emission": [P, FP, C.POINTER(P)],
        "xgb_material_specular_reflection": [P, C.POINTER(P)],
        "xgb_material_specular_refraction": [P, C.c_float, C.POINTER(P)],
        "xgb_material_specular_fresnel": [P, C.c_float, C.POINTER(P)],
        "xgb_material_mf_normalmap": [P, P, C.POINTER(P)],
        "xgb_material_set_normalmap": [P, P],
        "xgb_material_set_fixes": [P, C.c_uint32],
        "xgb_scene_set_fixes": [P, C.c_uint32],
        "xgb_material_destroy": [P],
        "xgb_scene_create": [P, C.POINTER(P)],
        "xgb_scene_destroy": [P],
        "xgb_scene_add_object": [P, P, P, FP, FP],
        "xgb_scene_set_camera_pinhole": [P, FP, FP, C.c_float, C.c_float],
        "xgb_scene_set_sky_none": [P],
        "xgb_scene_set_sky_uniform": [P, FP],
        "xgb_scene_set_sky_probe": [P, P],
        "xgb_scene_set_sky_latlong": [P, P],
        "xgb_scene_build": [P, P],
        "xgb_film_create": [P, C.c_int, C.c_int, C.c_int, C.POINTER(P)],
        "xgb_film_destroy": [P],
        "xgb_film_clear": [P, P],
        "xgb_film_download": [P, FP, C.c_int, P],
        "xgb_film_device_pointer": [P, C.POINTER(P), C.POINTER(C.c_int)],
        "xgb_render": [P, C.POINTER(IntegratorParamsC), P, C.c_uint32, C.c_uint32, P],
        "xgb_render_stats_get": [P, C.POINTER(RenderStatsC), P],
        "xgb_render_batch": [C.POINTER(BatchJobC), C.c_int, C.POINTER(BatchOptionsC), P],
        "xgb_batch_autotune": [C.POINTER(BatchJobC), C.c_int, P, C.POINTER(BatchOptionsC)],
        "xgb_batch_stats_get": [P, C.POINTER(RenderStatsC)],
        "xgb_scene_set_profiling": [P, C.c_int],
        "xgb_scene_set_traversal_limits": [P, C.c_int, C.c_int],
        "xgb_render_noalloc": [P, C.POINTER(IntegratorParamsC), P, C.c_uint32, C.c_uint32, P],
        "xgb_guide_create": [P, C.c_uint32, C.POINTER(P)],
        "xgb_guide_destroy": [P],
        "xgb_guide_param_count": [C.POINTER(C.c_size_t)],
        "xgb_guide_get_params": [P, FP, C.c_size_t],
        "xgb_guide_set_params": [P, FP, C.c_size_t],
        "xgb_guide_get_grads": [P, FP, C.c_size_t],
        "xgb_guide_set_bounds": [P, FP, FP],
        "xgb_guide_infer": [P, C.c_int, FP, FP, FP, FP],
        "xgb_guide_sample": [P, C.c_int, FP, FP, FP, C.c_uint32, FP, FP],
        "xgb_guide_train_batch": [P, C.c_int, FP, FP, FP, FP, FP, FP, C.c_float, FP],
        "xgb_guide_set_training": [P, C.c_int, C.c_int, C.c_int],
        "xgb_guide_set_wait_limit": [P, C.c_int],
        "xgb_guide_train_steps": [P, C.POINTER(C.c_uint64)],
        "xgb_scene_set_guide": [P, P, C.c_float, C.c_int, C.c_float],
    }
    for name, args in sig.items():
        f = getattr(lib, name)
        f.argtypes = args
        f.restype = C.c_int
    lib.xgb_get_last_error.argtypes = [P]
    lib.xgb_get_last_error.restype = C.c_char_p
    lib.xgb_version.restype = C.c_char_p
    lib.xgb_integrator_params_default.argtypes = [C.POINTER(IntegratorParamsC)]
    lib.xgb_integrator_params_default.restype = None
    _lib = lib
    return lib


def _f32(a, n=None) -> np.ndarray:
    a = np.ascontiguousarray(np.asarray(a, dtype=np.float32))
    if n is not None:
        assert a.size == n
    return a


def _fp(a: Optional[np.ndarray]):
    return None if a is None else a.ctypes.data_as(FP)


class Context:
    """One GPU (xgb_ctx_create)."""

    def __init__(self, device: int = 0):
        self.lib = load_library()
        h = P()
        st = self.lib.xgb_ctx_create(device, C.byref(h))
        if st != 0:
            raise XgbError(st, f"xgb_ctx_create({device}) failed (no CUDA device?)")
        self.h = h
        self._keep = []

    def check(self, st: int, what: str = ""):
        if st != 0:
            msg = self.lib.xgb_get_last_error(self.h).decode()
            raise XgbError(st, f"{what}: {msg}")

    BVH_BUILDERS = {"ploc": 0, "lbvh": 1}

    def set_bvh_builder(self, name: str):
        """BVH builder for meshes created afterwards: "ploc" (default) or "lbvh"."""
        self.check(self.lib.xgb_ctx_set_bvh_builder(self.h, self.BVH_BUILDERS[name]), "set_bvh_builder")

    BVH_LAYOUTS = {"binary": 0, "wide8": 1}

    def set_bvh_layout(self, name: str):
        """Node layout of the BVH of meshes created afterwards: "binary" (default) or "wide8"."""
        self.check(self.lib.xgb_ctx_set_bvh_layout(self.h, self.BVH_LAYOUTS[name]), "set_bvh_layout")

    def set_path_order(self, tile_w: int = 0, tile_h: int = 0):
        """Camera paths in tile_w x tile_h pixel blocks (0, 0 = scanline rows); speed only."""
        self.check(self.lib.xgb_ctx_set_path_order(self.h, int(tile_w), int(tile_h)), "set_path_order")

    def set_sample_grouping(self, samples: int = 64):
        """Camera paths as runs of `samples` consecutive samples of one pixel (the
        default 64; 0 = one sample pass over the film after the other); speed only."""
        self.check(self.lib.xgb_ctx_set_sample_grouping(self.h, int(samples)), "set_sample_grouping")

    def synchronize(self, stream=None):
        self.check(self.lib.xgb_ctx_synchronize(self.h, stream), "synchronize")

    def close(self):
        if getattr(self, "h", None):
            self.lib.xgb_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _release(obj, destroy: str) -> None:
    """Destroys obj's handle while its context is alive. Every wrapper keeps Python
    references to the handles its handle points at (a scene to its meshes, materials,
    textures and guide; a material to its textures, base and SVNDF; a shell-mapped
    mesh to its displacement map), so nothing the library still reads is freed; the
    library's destroy calls free device memory with cudaFree, which waits for the
    device's work in flight."""
    h = getattr(obj, "h", None)
    ctx = getattr(obj, "ctx", None)
    if h and ctx is not None and getattr(ctx, "h", None):
        try:
            getattr(ctx.lib, destroy)(h)
        except Exception:
            pass
    obj.h = None


class Texture:
    """xitils::Texture built from float RGB texels [h, w, 3] (Texture.h:25-32)."""

    def __init__(self, ctx: Context, rgb: np.ndarray, warpClamp: bool = True, filter: bool = True):
        rgb = _f32(rgb)
        h, w, ch = rgb.shape
        self.ctx = ctx
        self.h = P()
        ctx.check(ctx.lib.xgb_texture_create(ctx.h, w, h, ch, _fp(rgb), int(warpClamp), int(filter), C.byref(self.h)),
                  "Texture")

    def __del__(self):
        _release(self, "xgb_texture_destroy")


class Svndf:
    """SVNDF of a displacement texture fitted on the GPU (the displacement sandbox's
    downsampleDisplacementTexture + SVNDF); ``low`` is the low-resolution height
    texture it produces."""

    def __init__(self, ctx: Context, displacement: Texture, displacementScale: float, rate: int = 8, seed: int = 0):
        self.ctx = ctx
        self.h = P()
        low = P()
        ctx.check(ctx.lib.xgb_svndf_create(ctx.h, displacement.h, C.c_float(displacementScale), int(rate),
                                           C.c_uint32(seed), C.byref(self.h), C.byref(low)), "Svndf")
        self.low = Texture.__new__(Texture)
        self.low.ctx, self.low.h = ctx, low
        w, h = C.c_int(), C.c_int()
        ctx.check(ctx.lib.xgb_svndf_size(self.h, C.byref(w), C.byref(h)), "Svndf.size")
        self.width, self.height = w.value, h.value

    def lobes(self) -> np.ndarray:
        """Fitted mixtures [height, width, 4, 5] = mu.xyz, kappa, alpha."""
        out = np.zeros((self.height, self.width, 4, 5), np.float32)
        self.ctx.check(self.ctx.lib.xgb_svndf_get_lobes(self.h, _fp(out)), "Svndf.lobes")
        return out

    def set_lobes(self, lobes: np.ndarray):
        lobes = _f32(lobes).reshape(self.height, self.width, 4, 5)
        self.ctx.check(self.ctx.lib.xgb_svndf_set_lobes(self.h, _fp(lobes)), "Svndf.set_lobes")

    def __del__(self):
        _release(self, "xgb_svndf_destroy")


class TriangleMesh:
    """xitils::TriangleMesh; setGeometry copies the arrays and builds its BVH on the GPU."""

    def __init__(self, ctx: Context):
        self.ctx = ctx
        self.h = None
        self.n_tris = 0

    def setGeometry(self, positions, texCoords=None, normals=None, tangents=None, bitangents=None, indices=None):
        pos = _f32(positions).reshape(-1, 3)
        arr = lambda a, k: None if a is None else _f32(a).reshape(-1, k)
        uv, n, t, b = arr(texCoords, 2), arr(normals, 3), arr(tangents, 3), arr(bitangents, 3)
        idx = np.ascontiguousarray(np.asarray(indices, dtype=np.int32).reshape(-1))
        self.h = P()
        ctx = self.ctx
        ctx.check(ctx.lib.xgb_mesh_create(ctx.h, pos.shape[0], _fp(pos), _fp(uv), _fp(n), _fp(t), _fp(b), 12, 8,
                                          idx.size, idx.ctypes.data_as(C.POINTER(C.c_int32)), C.byref(self.h)),
                  "TriangleMesh.setGeometry")
        self.n_tris = idx.size // 3
        return self

    def setGeometryWithShellMapping(self, positions, texCoords, normals, tangents, bitangents, indices,
                                    displacement: "Texture", displacementScale: float, layerNum: int):
        """TriangleMesh::setGeometryWithShellMapping (TriangleMesh.h:163-177):
        layerNum copies offset along the normals, hits discarded below the
        displacement's height; every attribute array is required."""
        pos = _f32(positions).reshape(-1, 3)
        uv, n, t, b = (_f32(a).reshape(-1, k) for a, k in ((texCoords, 2), (normals, 3), (tangents, 3),
                                                           (bitangents, 3)))
        idx = np.ascontiguousarray(np.asarray(indices, dtype=np.int32).reshape(-1))
        self.h = P()
        self.displacement = displacement  # the library keeps a reference to the texture's device data
        ctx = self.ctx
        ctx.check(ctx.lib.xgb_mesh_create_shell(ctx.h, pos.shape[0], _fp(pos), _fp(uv), _fp(n), _fp(t), _fp(b), 12, 8,
                                                idx.size, idx.ctypes.data_as(C.POINTER(C.c_int32)), displacement.h,
                                                C.c_float(displacementScale), int(layerNum), C.byref(self.h)),
                  "TriangleMesh.setGeometryWithShellMapping")
        self.n_tris = idx.size // 3 * int(layerNum)
        return self

    def __del__(self):
        _release(self, "xgb_mesh_destroy")


class Material:
    def __init__(self, ctx: Context, maker, *args):
        self.ctx = ctx
        self.h = P()
        ctx.check(maker(ctx.h, *args, C.byref(self.h)), type(self).__name__)
        self.normalmap = None

    def set_normalmap(self, tex: Optional[Texture]):
        self.normalmap = tex
        self.ctx.check(self.ctx.lib.xgb_material_set_normalmap(self.h, tex.h if tex else None), "normalmap")

    def __del__(self):
        _release(self, "xgb_material_destroy")


class Diffuse(Material):
    def __init__(self, ctx, albedo, texture: Optional[Texture] = None):
        a = _f32(albedo, 3)
        super().__init__(ctx, ctx.lib.xgb_material_diffuse, _fp(a), texture.h if texture else None)
        self.texture = texture


class Metal(Material):
    def __init__(self, ctx, roughness, f0, roughness_texture: Optional[Texture] = None):
        f = _f32(f0, 3)
        super().__init__(ctx, ctx.lib.xgb_material_metal, C.c_float(roughness), _fp(f),
                         roughness_texture.h if roughness_texture else None)
        self.roughness_texture = roughness_texture


class Glossy(Material):
    def __init__(self, ctx, albedo, sharpness):
        super().__init__(ctx, ctx.lib.xgb_material_glossy, _fp(_f32(albedo, 3)), C.c_float(sharpness))


class GlossyWithHighLight(Material):
    def __init__(self, ctx, albedo, highlight, sharpness, sharpnessHighLight, highlightRate):
        super().__init__(ctx, ctx.lib.xgb_material_glossy_highlight, _fp(_f32(albedo, 3)), _fp(_f32(highlight, 3)),
                         C.c_float(sharpness), C.c_float(sharpnessHighLight), C.c_float(highlightRate))


class GlossyClamped(Material):
    def __init__(self, ctx, albedo, sharpness):
        super().__init__(ctx, ctx.lib.xgb_material_glossy_clamped, _fp(_f32(albedo, 3)), C.c_float(sharpness))


class Emission(Material):
    def __init__(self, ctx, power):
        super().__init__(ctx, ctx.lib.xgb_material_emission, _fp(_f32(power, 3)))


class SpecularReflection(Material):
    def __init__(self, ctx):
        super().__init__(ctx, ctx.lib.xgb_material_specular_reflection)


class SpecularRefraction(Material):
    def __init__(self, ctx, index=1.0):
        super().__init__(ctx, ctx.lib.xgb_material_specular_refraction, C.c_float(index))


class SpecularFresnel(Material):
    def __init__(self, ctx, index=1.0):
        super().__init__(ctx, ctx.lib.xgb_material_specular_fresnel, C.c_float(index))


class MicrofacetNormalMapping(Material):
    def __init__(self, ctx, base: Material):
        super().__init__(ctx, ctx.lib.xgb_material_mf_normalmap, base.h)
        self.base = base


class MultiLobeSVBRDF(Material):
    """MultiLobeSVBRDF(base, lowDisplacement, scale, svndf) of the displacement sandbox."""

    def __init__(self, ctx, base: Material, svndf: Svndf):
        super().__init__(ctx, ctx.lib.xgb_material_multilobe_svbrdf, base.h, svndf.h)
        self.base, self.svndf = base, svndf


class PinholeCamera:
    def __init__(self, cameraToWorld: Transform, fov: float, aspectRatio: float):
        self.cameraToWorld, self.fov, self.aspectRatio = cameraToWorld, float(fov), float(aspectRatio)


class Object:
    def __init__(self, shape: TriangleMesh, material: Material, objectToWorld: Optional[Transform] = None):
        self.shape, self.material = shape, material
        self.objectToWorld = objectToWorld or Transform.identity()


class Scene:
    """xitils::Scene: objects, camera and sky; buildAccelerationStructure uploads it."""

    def __init__(self, ctx: Context):
        self.ctx = ctx
        self.h = P()
        ctx.check(ctx.lib.xgb_scene_create(ctx.h, C.byref(self.h)), "Scene")
        self.objects = []
        self.camera = None
        self.skySphere = None
        self._keep = []

    def addObject(self, obj: Object):
        m = _f32(obj.objectToWorld.mat, 16)
        mi = _f32(obj.objectToWorld.matInv, 16)
        self.ctx.check(self.ctx.lib.xgb_scene_add_object(self.h, obj.shape.h, obj.material.h, _fp(m), _fp(mi)),
                       "addObject")
        self.objects.append(obj)

    def setCamera(self, cam: PinholeCamera):
        m = _f32(cam.cameraToWorld.mat, 16)
        mi = _f32(cam.cameraToWorld.matInv, 16)
        self.ctx.check(self.ctx.lib.xgb_scene_set_camera_pinhole(self.h, _fp(m), _fp(mi), cam.fov, cam.aspectRatio),
                       "camera")
        self.camera = cam

    def setSky(self, kind: int, rgb=None, tex: Optional[Texture] = None):
        lib = self.ctx.lib
        if kind == SKY_NONE:
            st = lib.xgb_scene_set_sky_none(self.h)
        elif kind == SKY_UNIFORM:
            st = lib.xgb_scene_set_sky_uniform(self.h, _fp(_f32(rgb, 3)))
        elif kind == SKY_PROBE:
            st = lib.xgb_scene_set_sky_probe(self.h, tex.h)
        elif kind == SKY_LATLONG:
            st = lib.xgb_scene_set_sky_latlong(self.h, tex.h)
        else:
            raise ValueError(kind)
        self.ctx.check(st, "sky")
        self.skySphere = (kind, rgb, tex)

    def buildAccelerationStructure(self, stream=None):
        self.ctx.check(self.ctx.lib.xgb_scene_build(self.h, stream), "buildAccelerationStructure")

    def __del__(self):
        _release(self, "xgb_scene_destroy")

    def setGuide(self, guide, bsdf_fraction: float = 0.5, train: bool = False, lr: float = 1e-3):
        self.ctx.check(self.ctx.lib.xgb_scene_set_guide(self.h, guide.h if guide else None, C.c_float(bsdf_fraction),
                                                        int(train), C.c_float(lr)), "setGuide")
        self._guide = guide

    def intersect(self, rays, stream=None) -> np.ndarray:
        """Closest hits of float32 [n, 7] rays (o, d, tMax) -> [n, 5] (t, object, triangle, b0, b1)."""
        rays = np.ascontiguousarray(rays, dtype=np.float32).reshape(-1, 7)
        hits = np.zeros((rays.shape[0], 5), np.float32)
        self.ctx.check(self.ctx.lib.xgb_scene_intersect(self.h, rays.shape[0], _fp(rays), _fp(hits), stream),
                       "intersect")
        return hits

    def occluded(self, rays, stream=None) -> np.ndarray:
        rays = np.ascontiguousarray(rays, dtype=np.float32).reshape(-1, 7)
        out = np.zeros(rays.shape[0], np.int32)
        self.ctx.check(self.ctx.lib.xgb_scene_occluded(self.h, rays.shape[0], _fp(rays),
                                                       out.ctypes.data_as(C.POINTER(C.c_int32)), stream), "occluded")
        return out

    def set_profiling(self, enable: bool = True):
        self.ctx.check(self.ctx.lib.xgb_scene_set_profiling(self.h, int(enable)), "set_profiling")

    def set_traversal_limits(self, max_steps: int = 0, max_stack: int = 0):
        """Device-side traversal bounds (0 = default: 2^22 steps, 64 stack entries)."""
        self.ctx.check(self.ctx.lib.xgb_scene_set_traversal_limits(self.h, int(max_steps), int(max_stack)),
                       "set_traversal_limits")

    def stats(self, stream=None) -> dict:
        s = RenderStatsC()
        self.ctx.check(self.ctx.lib.xgb_render_stats_get(self.h, C.byref(s), stream), "stats")
        out = {}
        for k, _ in RenderStatsC._fields_:
            v = getattr(s, k)
            if k in ("kernel_ms", "stage_launches"):
                out[k] = list(v)
            else:
                out[k] = float(v) if k.endswith("_ms") else int(v)
        return out


class RenderTarget:
    """Per-pixel radiance sums on the GPU (RenderTarget<Vector3f>); with
    ``aovs=True`` also the first-hit albedo and normal sums of a
    DenoisableRenderTarget (RenderTarget.h:131-145)."""

    AOV = {"albedo": 0, "normal": 1}

    def __init__(self, ctx: Context, width: int, height: int, fp64: bool = False, aovs: bool = False):
        self.ctx, self.width, self.height = ctx, width, height
        self.h = P()
        ctx.check(ctx.lib.xgb_film_create(ctx.h, width, height, int(fp64), C.byref(self.h)), "RenderTarget")
        if aovs:
            ctx.check(ctx.lib.xgb_film_enable_aovs(self.h), "enable_aovs")

    def __del__(self):
        _release(self, "xgb_film_destroy")

    def tonemap(self, scale: float = 1.0, exposure: float = 0.3, gamma: float = 2.2, stream=None) -> np.ndarray:
        """8-bit display image [H, W, 3] (RTCamp8's mapping; scale = 1 / spp)."""
        out = np.empty((self.height, self.width, 3), np.uint8)
        self.ctx.check(self.ctx.lib.xgb_film_tonemap(self.h, C.c_float(scale), C.c_float(exposure), C.c_float(gamma),
                                                     out.ctypes.data_as(C.POINTER(C.c_uint8)), stream), "tonemap")
        return out

    def error_map(self, other: "RenderTarget", scale: float, other_scale: float, max_value: float,
                  stream=None) -> np.ndarray:
        """Jet-coloured squared luminance difference against another film [H, W, 3] uint8."""
        out = np.empty((self.height, self.width, 3), np.uint8)
        self.ctx.check(self.ctx.lib.xgb_film_error_map(self.h, C.c_float(scale), other.h, C.c_float(other_scale),
                                                       C.c_float(max_value), out.ctypes.data_as(C.POINTER(C.c_uint8)),
                                                       stream), "error_map")
        return out

    def download_aov(self, which: str, out: Optional[np.ndarray] = None, stream=None) -> np.ndarray:
        if out is None:
            out = np.empty((self.height, self.width, 3), dtype=np.float32)
        assert out.dtype == np.float32 and out.flags.c_contiguous and out.size == self.width * self.height * 3
        self.ctx.check(self.ctx.lib.xgb_film_download_aov(self.h, self.AOV[which], _fp(out), 12, stream), "download_aov")
        return out

    def clear(self, stream=None):
        self.ctx.check(self.ctx.lib.xgb_film_clear(self.h, stream), "clear")

    def render(self, scene: Scene, sampleNum: int, params: Optional[IntegratorParams] = None, sampleBegin: int = 0,
               stream=None):
        p = params or IntegratorParams()
        pc = IntegratorParamsC(p.integrator, p.max_depth, p.rr_start, p.rr_prob, p.seed, getattr(p, "queue_capacity", 0))
        self.ctx.check(self.ctx.lib.xgb_render(scene.h, C.byref(pc), self.h, sampleBegin, sampleNum, stream), "render")

    def download(self, out: Optional[np.ndarray] = None, stream=None) -> np.ndarray:
        if out is None:
            out = np.empty((self.height, self.width, 3), dtype=np.float32)
        assert out.dtype == np.float32 and out.flags.c_contiguous and out.size == self.width * self.height * 3
        self.ctx.check(self.ctx.lib.xgb_film_download(self.h, _fp(out), 12, stream), "download")
        return out

    def device_pointer(self):
        p = P()
        f = C.c_int()
        self.ctx.check(self.ctx.lib.xgb_film_device_pointer(self.h, C.byref(p), C.byref(f)), "device_pointer")
        return p.value, bool(f.value)


def _batch_jobs(jobs):
    arr = (BatchJobC * len(jobs))()
    for k, (scene, target, params, spp_begin, spp_count) in enumerate(jobs):
        p = params or IntegratorParams()
        arr[k].scene = scene.h.value
        arr[k].film = target.h.value
        arr[k].params = IntegratorParamsC(p.integrator, p.max_depth, p.rr_start, p.rr_prob, p.seed,
                                          getattr(p, "queue_capacity", 0))
        arr[k].spp_begin = spp_begin
        arr[k].spp_count = spp_count
    return arr


def render_batch(ctx: Context, jobs, queue_capacity: int = 0, iterations_per_sync: int = 0, use_graph: bool = True,
                 stream=None) -> None:
    """xgb_render_batch: jobs = [(Scene, RenderTarget, IntegratorParams, spp_begin, spp_count), ...];
    zero options are autotuned (cached per batch shape)."""
    arr = _batch_jobs(jobs)
    opt = BatchOptionsC(queue_capacity, iterations_per_sync, int(use_graph))
    ctx.check(ctx.lib.xgb_render_batch(arr, len(jobs), C.byref(opt), stream), "render_batch")


def batch_autotune(ctx: Context, jobs, stream=None) -> dict:
    arr = _batch_jobs(jobs)
    out = BatchOptionsC()
    ctx.check(ctx.lib.xgb_batch_autotune(arr, len(jobs), stream, C.byref(out)), "batch_autotune")
    return {"queue_capacity": out.queue_capacity, "iterations_per_sync": out.iterations_per_sync,
            "use_graph": bool(out.use_graph)}


def batch_stats(ctx: Context) -> dict:
    s = RenderStatsC()
    ctx.check(ctx.lib.xgb_batch_stats_get(ctx.h, C.byref(s)), "batch_stats")
    out = {}
    for k, _ in RenderStatsC._fields_:
        v = getattr(s, k)
        out[k] = list(v) if k in ("kernel_ms", "stage_launches") else (float(v) if k.endswith("_ms") else int(v))
    return out


def write_png(path: str, rgb: np.ndarray) -> None:
    """8-bit RGB PNG (xgb_write_png)."""
    lib = load_library()
    rgb = np.ascontiguousarray(rgb, dtype=np.uint8)
    h, w = rgb.shape[:2]
    st = lib.xgb_write_png(path.encode(), w, h, rgb.ctypes.data_as(C.POINTER(C.c_uint8)))
    if st != 0:
        raise XgbError(st, f"write_png({path}) failed")


class Guide:
    """The learned directional proposal (xgb_guide_*): an MLP predicting an
    8-lobe vMF mixture, trained with Adam on BF16 tensor cores."""

    N_OUT = 40

    def __init__(self, ctx: Context, seed: int = 0):
        self.ctx = ctx
        self.h = P()
        ctx.check(ctx.lib.xgb_guide_create(ctx.h, seed, C.byref(self.h)), "Guide")
        n = C.c_size_t()
        ctx.lib.xgb_guide_param_count(C.byref(n))
        self.n_params = n.value

    def __del__(self):
        _release(self, "xgb_guide_destroy")

    def params(self) -> np.ndarray:
        out = np.empty(self.n_params, np.float32)
        self.ctx.check(self.ctx.lib.xgb_guide_get_params(self.h, _fp(out), out.size), "get_params")
        return out

    def set_params(self, p):
        p = _f32(p, self.n_params)
        self.ctx.check(self.ctx.lib.xgb_guide_set_params(self.h, _fp(p), p.size), "set_params")

    def grads(self) -> np.ndarray:
        out = np.empty(self.n_params, np.float32)
        self.ctx.check(self.ctx.lib.xgb_guide_get_grads(self.h, _fp(out), out.size), "get_grads")
        return out

    def set_bounds(self, lo, hi):
        self.ctx.check(self.ctx.lib.xgb_guide_set_bounds(self.h, _fp(_f32(lo, 3)), _fp(_f32(hi, 3))), "set_bounds")

    def infer(self, pos, nrm, wo) -> np.ndarray:
        pos, nrm, wo = (_f32(a).reshape(-1, 3) for a in (pos, nrm, wo))
        out = np.empty((pos.shape[0], self.N_OUT), np.float32)
        self.ctx.check(self.ctx.lib.xgb_guide_infer(self.h, pos.shape[0], _fp(pos), _fp(nrm), _fp(wo), _fp(out)),
                       "infer")
        return out

    def sample(self, pos, nrm, wo, seed: int = 0):
        pos, nrm, wo = (_f32(a).reshape(-1, 3) for a in (pos, nrm, wo))
        n = pos.shape[0]
        dirs = np.empty((n, 3), np.float32)
        pdf = np.empty(n, np.float32)
        self.ctx.check(self.ctx.lib.xgb_guide_sample(self.h, n, _fp(pos), _fp(nrm), _fp(wo), seed, _fp(dirs), _fp(pdf)),
                       "sample")
        return dirs, pdf

    def set_wait_limit(self, polls: int = 1 << 22):
        """Polls of each tensor-core inference wait before it gives up (tests: 0)."""
        self.ctx.check(self.ctx.lib.xgb_guide_set_wait_limit(self.h, int(polls)), "set_wait_limit")

    def set_training(self, batch_rows: int = 8192, max_steps_per_call: int = 512, product: bool = True):
        self.ctx.check(self.ctx.lib.xgb_guide_set_training(self.h, batch_rows, max_steps_per_call, int(product)),
                       "set_training")

    def steps(self) -> int:
        n = C.c_uint64()
        self.ctx.check(self.ctx.lib.xgb_guide_train_steps(self.h, C.byref(n)), "train_steps")
        return n.value

    def train_batch(self, pos, nrm, wo, wi, pdf, radiance, lr: float) -> float:
        arrs = [_f32(a).reshape(-1, 3) for a in (pos, nrm, wo, wi)]
        pdf, radiance = _f32(pdf), _f32(radiance)
        loss = np.zeros(1, np.float32)
        self.ctx.check(self.ctx.lib.xgb_guide_train_batch(self.h, arrs[0].shape[0], *[_fp(a) for a in arrs], _fp(pdf),
                                                          _fp(radiance), C.c_float(lr), _fp(loss)), "train_batch")
        return float(loss[0])


class GpuSceneBuilder:
    """Backend for ``SceneDesc.emit``: replays a recorded scene into the GPU library."""

    KIND_MAKERS = {DIFFUSE, METAL, GLOSSY, GLOSSY_HIGHLIGHT, GLOSSY_CLAMPED, EMISSION, SPECULAR_REFLECTION,
                   SPECULAR_REFRACTION, SPECULAR_FRESNEL, MF_NORMALMAP, MULTILOBE_SVBRDF}

    def __init__(self, ctx: Context):
        self.ctx = ctx
        self.scene = Scene(ctx)
        self.textures, self.meshes, self.materials, self.svndfs = [], [], [], []

    def add_svndf(self, tex, scale, rate, seed):
        sv = Svndf(self.ctx, self.textures[tex], scale, rate, seed)
        self.svndfs.append(sv)
        self.textures.append(sv.low)
        return len(self.svndfs) - 1, len(self.textures) - 1

    def add_texture(self, rgb, clamp=True, filter=True):
        self.textures.append(Texture(self.ctx, rgb, clamp, filter))
        return len(self.textures) - 1

    def add_mesh(self, pos, idx, uv=None, nrm=None, tan=None, bit=None):
        self.meshes.append(TriangleMesh(self.ctx).setGeometry(pos, uv, nrm, tan, bit, idx))
        return len(self.meshes) - 1

    def add_mesh_shell(self, pos, idx, uv, nrm, tan, bit, tex, scale, layers):
        self.meshes.append(TriangleMesh(self.ctx).setGeometryWithShellMapping(pos, uv, nrm, tan, bit, idx,
                                                                             self.textures[tex], scale, layers))
        return len(self.meshes) - 1

    def add_material(self, kind, f, base=-1, tex=-1, normalmap=-1):
        ctx = self.ctx
        t = self.textures[tex] if tex >= 0 else None
        if kind == DIFFUSE:
            m = Diffuse(ctx, f[:3], t)
        elif kind == METAL:
            m = Metal(ctx, f[0], f[1:4], t)
            if len(f) > 4 and f[4]:
                ctx.check(ctx.lib.xgb_material_set_fixes(m.h, int(f[4])), "set_fixes")
        elif kind == GLOSSY:
            m = Glossy(ctx, f[:3], f[3])
        elif kind == GLOSSY_HIGHLIGHT:
            m = GlossyWithHighLight(ctx, f[:3], f[3:6], f[6], f[7], f[8])
        elif kind == GLOSSY_CLAMPED:
            m = GlossyClamped(ctx, f[:3], f[3])
        elif kind == EMISSION:
            m = Emission(ctx, f[:3])
        elif kind == SPECULAR_REFLECTION:
            m = SpecularReflection(ctx)
        elif kind == SPECULAR_REFRACTION:
            m = SpecularRefraction(ctx, f[0])
        elif kind == SPECULAR_FRESNEL:
            m = SpecularFresnel(ctx, f[0])
        elif kind == MF_NORMALMAP:
            m = MicrofacetNormalMapping(ctx, self.materials[base])
        elif kind == MULTILOBE_SVBRDF:
            m = MultiLobeSVBRDF(ctx, self.materials[base], self.svndfs[tex])
        else:
            raise ValueError(kind)
        if normalmap >= 0:
            m.set_normalmap(self.textures[normalmap])
        self.materials.append(m)
        return len(self.materials) - 1

    def add_object(self, mesh, material, mat, matInv):
        self.scene.addObject(Object(self.meshes[mesh], self.materials[material], Transform(np.asarray(mat, np.float32),
                                                                                         np.asarray(matInv, np.float32))))

    def set_camera(self, c2w, c2wInv, fov, aspect):
        self.scene.setCamera(PinholeCamera(Transform(np.asarray(c2w, np.float32), np.asarray(c2wInv, np.float32)),
                                           fov, aspect))

    def set_sky(self, kind, rgb, tex):
        self.scene.setSky(kind, rgb, self.textures[tex] if tex >= 0 else None)

    def set_fixes(self, fixes):
        self.ctx.check(self.ctx.lib.xgb_scene_set_fixes(self.scene.h, fixes), "set_fixes")

    def build(self):
        self.scene.buildAccelerationStructure()


def load_scene(ctx: Context, desc) -> GpuSceneBuilder:
    return desc.emit(GpuSceneBuilder(ctx))


def render_desc(ctx: Context, desc, spp_begin: int = 0, spp_count: Optional[int] = None, params=None,
                builder: Optional[GpuSceneBuilder] = None) -> np.ndarray:
    """Builds (or reuses) a scene and renders it; returns float32 [H, W, 3] sums."""
    b = builder or load_scene(ctx, desc)
    rt = RenderTarget(ctx, desc.width, desc.height)
    rt.render(b.scene, desc.spp if spp_count is None else spp_count, params or desc.params, spp_begin)
    return rt.download()
