"""ctypes bindings for the CPU checkers (test infrastructure only).

``CpuChecker("port")`` loads oracle/liboracle.so (the project's restatement,
prefix ``xcpu_``); ``CpuChecker("reference")`` loads oracle/_ref/libxref.so
(the reference's own headers, prefix ``xref_``). Both expose the scene API of
oracle/scene_api.h. Only tests/, __graft_entry__.smoke() and bench.py's CPU
legs use this module.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_LIBS = {}


def _fptr(a):
    if a is None:
        return None
    a = np.ascontiguousarray(a, dtype=np.float32)
    return a, a.ctypes.data_as(C.POINTER(C.c_float))


class CpuChecker:
    def __init__(self, kind: str = "port"):
        from . import build_ref
        if kind == "port":
            path, prefix = build_ref.build_oracle(), "xcpu_"
        elif kind == "port_ulp":
            path, prefix = build_ref.build_oracle_perturbed(), "xcpu_"
        elif kind.startswith("port_cr"):
            path, prefix = build_ref.build_oracle_cr(int(kind[len("port_cr"):])), "xcpu_"
        elif kind == "reference":
            path, prefix = build_ref.build_ref(), "xref_"
            if path is None:
                raise FileNotFoundError("reference checker unavailable (no staged reference sources)")
        else:
            raise ValueError(kind)
        if path not in _LIBS:
            _LIBS[path] = C.CDLL(path)
        self.lib = _LIBS[path]
        self.kind = kind
        self.p = prefix
        fn = lambda n: getattr(self.lib, prefix + n)
        self._new = fn("scene_new"); self._new.restype = C.c_void_p
        self._free = fn("scene_free"); self._free.argtypes = [C.c_void_p]
        self.h = self._new()
        self._keep = []

    def __del__(self):
        try:
            if self.h:
                self._free(self.h)
        except Exception:
            pass

    def _call(self, name, *args):
        f = getattr(self.lib, self.p + name)
        return f(C.c_void_p(self.h), *args)

    # -- scene API (same calls as xitils_gb300.scene.SceneDesc.emit expects) --
    def add_texture(self, rgb, clamp=True, filter=True):
        rgb = np.ascontiguousarray(rgb, dtype=np.float32)
        self._keep.append(rgb)
        h, w = rgb.shape[:2]
        r = self._call("add_texture", C.c_int(w), C.c_int(h), rgb.ctypes.data_as(C.POINTER(C.c_float)),
                       C.c_int(int(clamp)), C.c_int(int(filter)))
        assert r >= 0
        return r

    def add_mesh(self, pos, idx, uv=None, nrm=None, tan=None, bit=None):
        arrs = [_fptr(a) for a in (pos, uv, nrm, tan, bit)]
        idx = np.ascontiguousarray(idx, dtype=np.int32)
        self._keep.extend([a[0] for a in arrs if a] + [idx])
        ptr = lambda a: a[1] if a else None
        r = self._call("add_mesh", C.c_int(len(pos)), ptr(arrs[0]), ptr(arrs[1]), ptr(arrs[2]), ptr(arrs[3]),
                       ptr(arrs[4]), C.c_int(idx.size), idx.ctypes.data_as(C.POINTER(C.c_int32)))
        assert r >= 0, "add_mesh failed"
        return r

    def add_svndf(self, tex, scale, rate, seed):
        """SVNDF of texture `tex` (the displacement sandbox's downsampleDisplacementTexture);
        returns (svndf id, id of the low-resolution height texture it appends)."""
        low = C.c_int(-1)
        r = self._call("add_svndf", C.c_int(tex), C.c_float(scale), C.c_int(rate), C.c_uint32(seed), C.byref(low))
        assert r >= 0, "add_svndf failed"
        return r, low.value

    def svndf_fit(self, rgb, scale, rate, seed, clamp=True):
        """Stand-alone fit: (low red channel [h', w'], lobes [h', w', 4, 5] = mu.xyz, kappa, alpha)."""
        rgb = np.ascontiguousarray(rgb, dtype=np.float32)
        h, w = rgb.shape[:2]
        lh, lw = (h + rate - 1) // rate, (w + rate - 1) // rate
        low = np.zeros((lh, lw), np.float32)
        lobes = np.zeros((lh, lw, 4, 5), np.float32)
        fp = lambda a: a.ctypes.data_as(C.POINTER(C.c_float))
        r = getattr(self.lib, self.p + "svndf_fit")(fp(rgb), C.c_int(w), C.c_int(h), C.c_int(int(clamp)),
                                                    C.c_float(scale), C.c_int(rate), C.c_uint32(seed), fp(low),
                                                    fp(lobes))
        assert r == 0
        return low, lobes

    def vmf4_sample(self, lobes, n, seed):
        lobes = np.ascontiguousarray(lobes, dtype=np.float32).reshape(4, 5)
        dirs = np.zeros((n, 3), np.float32)
        fp = lambda a: a.ctypes.data_as(C.POINTER(C.c_float))
        assert getattr(self.lib, self.p + "vmf4_sample_pcg")(fp(lobes), C.c_int(n), C.c_uint32(seed), fp(dirs)) == 0
        return dirs

    def add_mesh_shell(self, pos, idx, uv, nrm, tan, bit, tex, scale, layers):
        arrs = [_fptr(a) for a in (pos, uv, nrm, tan, bit)]
        idx = np.ascontiguousarray(idx, dtype=np.int32)
        self._keep.extend([a[0] for a in arrs] + [idx])
        r = self._call("add_mesh_shell", C.c_int(len(pos)), *[a[1] for a in arrs], C.c_int(idx.size),
                       idx.ctypes.data_as(C.POINTER(C.c_int32)), C.c_int(tex), C.c_float(scale), C.c_int(layers))
        assert r >= 0, "add_mesh_shell failed"
        return r

    def add_material(self, kind, f, base=-1, tex=-1, normalmap=-1):
        fa = np.zeros(16, dtype=np.float32)
        fa[:len(f)] = f
        r = self._call("add_material", C.c_int(kind), fa.ctypes.data_as(C.POINTER(C.c_float)), C.c_int(base),
                       C.c_int(tex), C.c_int(normalmap))
        assert r >= 0, "add_material failed"
        return r

    def bsdf_sample(self, material, wo, n, seed=0):
        """n draws of the material's evalAndSample at the flat shading point of
        scene_api.h: (wi [n, 3], weight [n, 3], pdf [n]); draw k on stream (k, 0, seed)."""
        wo = np.ascontiguousarray(wo, dtype=np.float32).reshape(3)
        out = np.zeros((n, 7), np.float32)
        fp = lambda a: a.ctypes.data_as(C.POINTER(C.c_float))
        r = self._call("bsdf_sample_pcg", C.c_int(material), fp(wo), C.c_int(n), C.c_uint32(seed), fp(out))
        assert r == 0, r
        return out[:, :3], out[:, 3:6], out[:, 6]

    def bsdf_eval(self, material, wo, wi, seed=0):
        """getPDF and bsdfCos of the material for each direction wi [n, 3]: (pdf [n], f [n, 3])."""
        wo = np.ascontiguousarray(wo, dtype=np.float32).reshape(3)
        wi = np.ascontiguousarray(wi, dtype=np.float32).reshape(-1, 3)
        out = np.zeros((len(wi), 4), np.float32)
        fp = lambda a: a.ctypes.data_as(C.POINTER(C.c_float))
        r = self._call("bsdf_eval_pcg", C.c_int(material), fp(wo), C.c_int(len(wi)), fp(wi), C.c_uint32(seed), fp(out))
        assert r == 0, r
        return out[:, 0], out[:, 1:]

    def light_sample(self, n, seed=0):
        """n draws of Scene::sampleSurface on a built scene: (p [n, 3], n [n, 3], pdf [n]);
        draw k on stream (k, 2, seed)."""
        out = np.zeros((n, 7), np.float32)
        r = self._call("light_sample_pcg", C.c_int(n), C.c_uint32(seed), out.ctypes.data_as(C.POINTER(C.c_float)))
        assert r == 0, r
        return out[:, :3], out[:, 3:6], out[:, 6]

    def intersect(self, rays):
        """Scene::intersect of float32 [n, 7] rays (o, d, tMax) -> (t [n], object [n], p [n, 3],
        shading normal [n, 3]); object -1 on a miss."""
        rays = np.ascontiguousarray(rays, dtype=np.float32)
        out = np.zeros((rays.shape[0], 8), np.float32)
        r = self._call("intersect", C.c_int(rays.shape[0]), rays.ctypes.data_as(C.POINTER(C.c_float)),
                       out.ctypes.data_as(C.POINTER(C.c_float)))
        assert r == 0, r
        return out[:, 0], out[:, 1].astype(np.int32), out[:, 2:5], out[:, 5:8]

    def intersect_any(self, rays):
        rays = np.ascontiguousarray(rays, dtype=np.float32)
        out = np.zeros(rays.shape[0], np.int32)
        r = self._call("intersect_any", C.c_int(rays.shape[0]), rays.ctypes.data_as(C.POINTER(C.c_float)),
                       out.ctypes.data_as(C.POINTER(C.c_int32)))
        assert r == 0, r
        return out

    def add_object(self, mesh, material, mat, matInv):
        m = np.ascontiguousarray(mat, dtype=np.float32)
        mi = np.ascontiguousarray(matInv, dtype=np.float32)
        r = self._call("add_object", C.c_int(mesh), C.c_int(material), m.ctypes.data_as(C.POINTER(C.c_float)),
                       mi.ctypes.data_as(C.POINTER(C.c_float)))
        assert r >= 0
        return r

    def set_camera(self, c2w, c2wInv, fov, aspect):
        m = np.ascontiguousarray(c2w, dtype=np.float32)
        mi = np.ascontiguousarray(c2wInv, dtype=np.float32)
        return self._call("set_camera", m.ctypes.data_as(C.POINTER(C.c_float)), mi.ctypes.data_as(C.POINTER(C.c_float)),
                          C.c_float(fov), C.c_float(aspect))

    def set_sky(self, kind, rgb, tex):
        a = np.zeros(3, dtype=np.float32) if rgb is None else np.asarray(rgb, dtype=np.float32)
        r = self._call("set_sky", C.c_int(kind), a.ctypes.data_as(C.POINTER(C.c_float)), C.c_int(tex))
        assert r == 0
        return r

    def set_fixes(self, fixes):
        assert self._call("set_fixes", C.c_int(fixes)) == 0, "set_fixes refused"

    def build(self):
        assert self._call("build") == 0

    # -- rendering ---------------------------------------------------------------
    def render_pcg(self, desc, spp_begin=0, spp_count=None, rect=None, nthreads=0, params=None):
        """Per-(pixel, sample) PCG render; returns float32 [H, W, 3] radiance sums."""
        P = params or desc.params
        W, H = desc.width, desc.height
        x0, y0, x1, y1 = rect or (0, 0, W, H)
        film = np.zeros((H, W, 3), dtype=np.float32)
        n = desc.spp if spp_count is None else spp_count
        r = self._call("render_pcg", C.c_int(W), C.c_int(H), C.c_uint32(spp_begin), C.c_uint32(n), C.c_uint32(P.seed),
                       C.c_int(P.integrator), C.c_int(P.max_depth), C.c_int(P.rr_start), C.c_float(P.rr_prob),
                       C.c_int(x0), C.c_int(y0), C.c_int(x1), C.c_int(y1),
                       film.ctypes.data_as(C.POINTER(C.c_float)), C.c_int(nthreads))
        if r != 0:
            raise RuntimeError(f"{self.kind} render_pcg failed ({r})")
        return film

    def render_pcg_aov(self, desc, spp_begin=0, spp_count=None, rect=None, nthreads=0, params=None):
        """render_pcg plus the first-hit albedo and normal sums (DenoisableRenderTargetPixel).
        Returns (film [H, W, 3], albedo [H, W, 3], normal [H, W, 3])."""
        P = params or desc.params
        W, H = desc.width, desc.height
        x0, y0, x1, y1 = rect or (0, 0, W, H)
        film = np.zeros((H, W, 3), dtype=np.float32)
        aov = np.zeros((H, W, 6), dtype=np.float32)
        n = desc.spp if spp_count is None else spp_count
        r = self._call("render_pcg_aov", C.c_int(W), C.c_int(H), C.c_uint32(spp_begin), C.c_uint32(n),
                       C.c_uint32(P.seed), C.c_int(P.integrator), C.c_int(P.max_depth), C.c_int(P.rr_start),
                       C.c_float(P.rr_prob), C.c_int(x0), C.c_int(y0), C.c_int(x1), C.c_int(y1),
                       film.ctypes.data_as(C.POINTER(C.c_float)), aov.ctypes.data_as(C.POINTER(C.c_float)),
                       C.c_int(nthreads))
        if r != 0:
            raise RuntimeError(f"{self.kind} render_pcg_aov failed ({r})")
        return film, aov[..., :3].copy(), aov[..., 3:].copy()

    def render_stock(self, W, H, spp, integrator=0, nthreads=0):
        """The reference's own RenderTarget::render (per-tile MT samplers). Returns (film, seconds)."""
        assert self.kind == "reference"
        f = self.lib.xref_render_stock
        f.restype = C.c_double
        film = np.zeros((H, W, 3), dtype=np.float32)
        t = f(C.c_void_p(self.h), C.c_int(W), C.c_int(H), C.c_int(spp), C.c_int(integrator),
              film.ctypes.data_as(C.POINTER(C.c_float)), C.c_int(nthreads))
        return film, float(t)

    def trace(self, rays):
        """Closest hits of float32 [n, 7] rays (o, d, tMax) -> float32 [n, 5] (t, object, tri, -, -)."""
        assert self.kind.startswith("port")
        rays = np.ascontiguousarray(rays, dtype=np.float32)
        hits = np.zeros((rays.shape[0], 5), dtype=np.float32)
        r = self.lib.xcpu_trace(C.c_void_p(self.h), C.c_int(rays.shape[0]), rays.ctypes.data_as(C.POINTER(C.c_float)),
                                hits.ctypes.data_as(C.POINTER(C.c_float)))
        assert r == 0
        return hits

    def occluded(self, rays):
        assert self.kind.startswith("port")
        rays = np.ascontiguousarray(rays, dtype=np.float32)
        out = np.zeros(rays.shape[0], dtype=np.int32)
        r = self.lib.xcpu_occluded(C.c_void_p(self.h), C.c_int(rays.shape[0]), rays.ctypes.data_as(C.POINTER(C.c_float)),
                                   out.ctypes.data_as(C.POINTER(C.c_int32)))
        assert r == 0
        return out


def load_scene(desc, kind: str = "port") -> CpuChecker:
    chk = CpuChecker(kind)
    desc.emit(chk)
    return chk


def relmse(img: np.ndarray, ref: np.ndarray, eps: float = 1e-2) -> float:
    """mean over pixels and channels of (I - R)^2 / (R^2 + eps)."""
    img = np.asarray(img, dtype=np.float64)
    ref = np.asarray(ref, dtype=np.float64)
    return float(np.mean((img - ref) ** 2 / (ref ** 2 + eps)))
