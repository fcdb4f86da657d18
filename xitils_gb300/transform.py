"""Transforms with the semantics of Xitils' ``Transform`` (Include/Xitils/Transform.h).

A transform is a pair of row-major float32 4x4 matrices ``(mat, matInv)``
(``m[r][c]``, the ``Matrix4x4`` layout, Matrix.h:8-12). The helpers reproduce
the reference's float32 arithmetic exactly -- products summed left to right as
in ``Matrix4x4::operator*`` (Matrix.h:184-192), ``matInv`` of a composition as
``t.matInv * matInv`` (Transform.h:52-54), rotation inverses as transposes
(Transform.h:32-45) -- so that the same matrices reach the GPU path and both
CPU checkers bit for bit.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

F = np.float32
TO_RAD = F(F(math.pi) / F(180.0))  # Utils.h:34


def _matmul(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    """Matrix4x4::operator* (Matrix.h:184-192): ((a0*b0 + a1*b1) + a2*b2) + a3*b3 in float32."""
    out = np.zeros((4, 4), dtype=F)
    for r in range(4):
        for c in range(4):
            acc = F(a[r, 0] * b[0, c])
            acc = F(acc + F(a[r, 1] * b[1, c]))
            acc = F(acc + F(a[r, 2] * b[2, c]))
            acc = F(acc + F(a[r, 3] * b[3, c]))
            out[r, c] = acc
    return out


@dataclass
class Transform:
    mat: np.ndarray
    matInv: np.ndarray

    @staticmethod
    def identity() -> "Transform":
        return Transform(np.eye(4, dtype=F), np.eye(4, dtype=F))

    @staticmethod
    def from_matrix(m: np.ndarray) -> "Transform":
        """Transform(const Matrix4x4&) (Transform.h:22-25): the inverse is the transpose."""
        m = np.asarray(m, dtype=F)
        return Transform(m.copy(), m.T.copy())

    def __mul__(self, t: "Transform") -> "Transform":
        return Transform(_matmul(self.mat, t.mat), _matmul(t.matInv, self.matInv))

    def inverse(self) -> "Transform":
        return Transform(self.matInv.copy(), self.mat.copy())

    def point(self, v) -> np.ndarray:
        """Transform::operator()(Vector3f) (Transform.h:61-72), float32."""
        m = self.mat
        v = np.asarray(v, dtype=F)
        r = []
        for i in range(4):
            acc = F(m[i, 0] * v[0])
            acc = F(acc + F(m[i, 1] * v[1]))
            acc = F(acc + F(m[i, 2] * v[2]))
            acc = F(acc + m[i, 3])
            r.append(acc)
        if r[3] == F(1):
            return np.array(r[:3], dtype=F)
        inv = F(F(1) / r[3])
        return np.array([F(r[0] * inv), F(r[1] * inv), F(r[2] * inv)], dtype=F)


def translate(x: float, y: float, z: float) -> Transform:  # Transform.h:227-241
    m = np.eye(4, dtype=F)
    mi = np.eye(4, dtype=F)
    m[0, 3], m[1, 3], m[2, 3] = F(x), F(y), F(z)
    mi[0, 3], mi[1, 3], mi[2, 3] = -F(x), -F(y), -F(z)
    return Transform(m, mi)


def scale(x: float, y: float, z: float) -> Transform:  # Transform.h:247-261
    m = np.diag(np.array([x, y, z, 1], dtype=F)).astype(F)
    mi = np.diag(np.array([F(1) / F(x), F(1) / F(y), F(1) / F(z), 1], dtype=F)).astype(F)
    return Transform(m, mi)


def _sincos(theta_deg: float):
    rad = F(F(theta_deg) * TO_RAD)
    # std::sin / std::cos of a float (Transform.h:269-270) are the float overloads.
    return F(np.sin(rad, dtype=F)), F(np.cos(rad, dtype=F))


def rotateX(theta: float) -> Transform:  # Transform.h:267-277
    s, c = _sincos(theta)
    return Transform.from_matrix(np.array([[1, 0, 0, 0], [0, c, -s, 0], [0, s, c, 0], [0, 0, 0, 1]], dtype=F))


def rotateY(theta: float) -> Transform:  # Transform.h:279-289
    s, c = _sincos(theta)
    return Transform.from_matrix(np.array([[c, 0, s, 0], [0, 1, 0, 0], [-s, 0, c, 0], [0, 0, 0, 1]], dtype=F))


def rotateZ(theta: float) -> Transform:  # Transform.h:291-301
    s, c = _sincos(theta)
    return Transform.from_matrix(np.array([[c, -s, 0, 0], [s, c, 0, 0], [0, 0, 1, 0], [0, 0, 0, 1]], dtype=F))


def rotateYXZ(x: float, y: float, z: float) -> Transform:  # Transform.h:303-308
    return rotateY(y) * rotateX(x) * rotateZ(z)


def transformTRS(t, r, s) -> Transform:  # Transform.h:370-374
    return translate(*t) * rotateYXZ(*r) * scale(*s)
