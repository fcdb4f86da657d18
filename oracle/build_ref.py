"""Build recipe for the CPU checkers (test infrastructure only).

Two libraries come out of this recipe:

* ``oracle/liboracle.so`` from ``oracle/xgb_cpu.cpp`` -- the project's own CPU
  restatement of the reference path tracer (the oracle).
* ``oracle/_ref/libxref.so`` from ``oracle/ref_harness.cpp`` compiled against
  the reference's own headers.

The reference does not compile with g++ as it stands (its CMake build targets
MSVC), so ``stage_reference()`` copies the headers it needs from the reference
checkout into ``oracle/_ref/src`` and applies two mechanical fixes there:

1. ``Include/Xitils/Vector.h`` spells ``simdpp::load_u<V::_T_SIMD>`` without
   ``typename`` inside templates (Vector.h:619-678); the copy adds it.
2. The never-instantiated ``_inRange`` template contains the statement
   ``_T_SIMD = simdpp::load_u<_T_SIMD>(&v);`` (Vector.h:695), which assigns to a
   type and is a syntax error for g++; the copy drops that one line.

It also extracts the sandbox-only materials ``GlossyClamped`` and
``MicrofacetNormalMapping`` (Sandbox/MicrofacetBasedNormalMapping/Main.cpp,
from ``enum _MethodMode`` up to ``struct MyFrameData``) into
``oracle/_ref/src/mfnm_extract.h`` unchanged, and from the displacement
prefiltering sandbox (Sandbox/PrefilteringForRenderingDisplacementMappedSurfaces/
Main.cpp) the ``VMFLobeNum`` constant and the classes ``SVNDF`` and
``MultiLobeSVBRDF`` into ``oracle/_ref/src/svndf_extract.h``, unchanged. glm, libsimdpp, Cinder and stb are
empty submodules in the reference checkout; ``oracle/shim`` stands in for them.

``oracle/_ref`` is git-ignored (no reference source enters history) but it is
copied to the GPU machine with the rest of the working tree, where the
reference checkout is absent: there ``build()`` finds the staged sources and
compiles them again for that machine's architecture.
"""
from __future__ import annotations

import os
import re
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REF_OUT = os.path.join(HERE, "_ref")
REF_SRC = os.path.join(REF_OUT, "src")
ORACLE_SO = os.path.join(HERE, "liboracle.so")
ORACLE_PERTURBED_SO = os.path.join(HERE, "liboracle_ulp.so")
REF_SO = os.path.join(REF_OUT, "libxref.so")

# The reference checkout: XGB_REFERENCE_ROOT, else a sibling directory of the
# repository named "reference".
REFERENCE_ROOT = os.environ.get("XGB_REFERENCE_ROOT",
                                os.path.normpath(os.path.join(HERE, os.pardir, os.pardir, "reference")))
HEADERS = [
    "AccelerationStructure.h", "Bounds.h", "Camera.h", "Geometry.h", "Interaction.h", "Material.h",
    "Matrix.h", "Object.h", "PathTracer.h", "Ray.h", "RenderTarget.h", "Sampler.h", "Scene.h",
    "Shape.h", "SkySphere.h", "Texture.h", "Transform.h", "TriangleIndexed.h", "TriangleMesh.h",
    "Utils.h", "Vector.h", "VonMisesFisherDistribution.h",
]
MFNM_SANDBOX = os.path.join("Sandbox", "MicrofacetBasedNormalMapping", "Main.cpp")
PREFILTER_SANDBOX = os.path.join("Sandbox", "PrefilteringForRenderingDisplacementMappedSurfaces", "Main.cpp")

CXXFLAGS = ["-O2", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off", "-w"]


def _read(path: str) -> str:
    with open(path, "r", encoding="utf-8-sig", errors="replace") as f:
        return f.read()


def _write(path: str, text: str) -> None:
    os.makedirs(os.path.dirname(path), exist_ok=True)
    with open(path, "w", encoding="utf-8") as f:
        f.write(text)


def stage_reference(root: str = REFERENCE_ROOT) -> bool:
    """Copy + patch the reference headers into oracle/_ref/src. Returns False
    when the reference checkout is not present (e.g. on the GPU machine)."""
    inc = os.path.join(root, "Include", "Xitils")
    if not os.path.isdir(inc):
        return False
    dst = os.path.join(REF_SRC, "Xitils")
    os.makedirs(dst, exist_ok=True)
    for h in HEADERS:
        text = _read(os.path.join(inc, h))
        if h == "Vector.h":
            text = text.replace("<V::_T_SIMD>", "<typename V::_T_SIMD>")
            text, n = re.subn(r"^\s*_T_SIMD = simdpp::load_u<_T_SIMD>\(&v\);\s*$\n", "", text, flags=re.M)
            if n != 1:
                raise RuntimeError("Vector.h patch did not apply (expected one dead statement)")
        _write(os.path.join(dst, h), text)
    main = _read(os.path.join(root, MFNM_SANDBOX))
    start = main.index("enum _MethodMode")
    end = main.index("struct MyFrameData")
    _write(os.path.join(REF_SRC, "mfnm_extract.h"),
           "// Extracted by oracle/build_ref.py from " + MFNM_SANDBOX.replace(os.sep, "/") + "\n#pragma once\n"
           + main[start:end])
    pre = _read(os.path.join(root, PREFILTER_SANDBOX))
    lobes = re.search(r"^const int VMFLobeNum = \d+;$", pre, flags=re.M)
    if lobes is None:
        raise RuntimeError("VMFLobeNum not found in the prefiltering sandbox")
    svndf = pre[pre.index("class SVNDF {"):pre.index("std::shared_ptr<Texture> downsampleDisplacementTexture")]
    svbrdf = pre[pre.index("class MultiLobeSVBRDF : public Material {"):pre.index("class PrefilteredDisplaceMapping")]
    _write(os.path.join(REF_SRC, "svndf_extract.h"),
           "// Extracted by oracle/build_ref.py from " + PREFILTER_SANDBOX.replace(os.sep, "/") + "\n#pragma once\n"
           + lobes.group(0) + "\n\n" + svndf + "\n" + svbrdf)
    return True


def _compile(src: str, out: str, includes: list[str], std: str, defines: tuple = ()) -> None:
    cmd = ["g++", f"-std={std}"] + CXXFLAGS + [f"-D{d}" for d in defines] + [f"-I{i}" for i in includes] + [src, "-o", out]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("compile failed: " + " ".join(cmd) + "\n" + res.stderr[-4000:])


def build_oracle(force: bool = False) -> str:
    src = os.path.join(HERE, "xgb_cpu.cpp")
    deps = [src, os.path.join(HERE, "scene_api.h")]
    if force or not os.path.exists(ORACLE_SO) or any(os.path.getmtime(d) > os.path.getmtime(ORACLE_SO) for d in deps):
        _compile(src, ORACLE_SO, [HERE], "c++17")
    return ORACLE_SO


def build_oracle_perturbed(force: bool = False) -> str:
    """The oracle with cosf / sinf / powf moved by one ulp: a sensitivity probe
    used by tests to show how far last-ulp libm differences move an image."""
    src = os.path.join(HERE, "xgb_cpu.cpp")
    if force or not os.path.exists(ORACLE_PERTURBED_SO) or os.path.getmtime(src) > os.path.getmtime(ORACLE_PERTURBED_SO):
        _compile(src, ORACLE_PERTURBED_SO, [HERE], "c++17", ("XGB_ORACLE_ULP_PERTURB",))
    return ORACLE_PERTURBED_SO


def build_oracle_cr(mask: int, force: bool = False) -> str:
    """The oracle with the float functions of `mask` correctly rounded (1 sinf,
    2 cosf, 4 powf, 8 expf, 16 logf, 32 asinf, 64 acosf, 128 atan2f; computed in
    long double): a diagnostic that measures what the C library's misrounded
    results contribute to an image."""
    src = os.path.join(HERE, "xgb_cpu.cpp")
    out = os.path.join(HERE, f"liboracle_cr{mask}.so")
    if force or not os.path.exists(out) or os.path.getmtime(src) > os.path.getmtime(out):
        _compile(src, out, [HERE], "c++17", (f"XGB_ORACLE_CR={mask}",))
    return out


def build_ref(force: bool = False) -> str | None:
    """Build oracle/_ref/libxref.so when staged sources exist. Returns the path
    or None when neither the reference checkout nor a staged copy is present."""
    staged_now = stage_reference()
    if not os.path.isdir(os.path.join(REF_SRC, "Xitils")):
        return None
    src = os.path.join(HERE, "ref_harness.cpp")
    deps = [src, os.path.join(HERE, "scene_api.h"), os.path.join(REF_SRC, "mfnm_extract.h"),
            os.path.join(REF_SRC, "svndf_extract.h")]
    if force or staged_now or not os.path.exists(REF_SO) or any(
            os.path.getmtime(d) > os.path.getmtime(REF_SO) for d in deps):
        _compile(src, REF_SO, [os.path.join(HERE, "shim"), REF_SRC, HERE], "c++20")
    return REF_SO


def main() -> int:
    print(build_oracle(force="--force" in sys.argv))
    print(build_ref(force="--force" in sys.argv))
    return 0


if __name__ == "__main__":
    sys.exit(main())
