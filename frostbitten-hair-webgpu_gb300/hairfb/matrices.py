"""4x4 matrix helpers with the conventions of wgpu-matrix@2.9.0.

The reference builds every matrix on the host with wgpu-matrix
(src/utils/matrices.ts:5-36, src/camera.ts:107-111) and uploads it in the
uniform blocks; the kernels only consume the bytes.  Matrices here are
column-major float32 arrays of 16 (like wgpu-matrix's Float32Array); the
arithmetic runs in float64 and is stored as float32, as JavaScript numbers
written into a Float32Array are.
"""
from __future__ import annotations

import math

import numpy as np


def _f32(a) -> np.ndarray:
    return np.asarray(a, dtype=np.float64).astype(np.float32)


def identity() -> np.ndarray:
    return np.eye(4, dtype=np.float32).reshape(16)


def to_rows(m: np.ndarray) -> np.ndarray:
    """Column-major 16-array -> 4x4 row-major float64 matrix."""
    return np.asarray(m, dtype=np.float64).reshape(4, 4).T


def from_rows(r: np.ndarray) -> np.ndarray:
    return _f32(np.asarray(r, dtype=np.float64).T.reshape(16))


def multiply(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    """mat4.multiply(a, b) = a * b"""
    return from_rows(to_rows(a) @ to_rows(b))


def invert(m: np.ndarray) -> np.ndarray:
    return from_rows(np.linalg.inv(to_rows(m)))


def perspective(fovy_rad: float, aspect: float, near: float, far: float) -> np.ndarray:
    """mat4.perspective: WebGPU clip space, z in [0, 1]."""
    f = math.tan(math.pi * 0.5 - 0.5 * fovy_rad)
    d = np.zeros(16, dtype=np.float64)
    d[0] = f / aspect
    d[5] = f
    d[11] = -1.0
    range_inv = 1.0 / (near - far)
    d[10] = far * range_inv
    d[14] = far * near * range_inv
    return _f32(d)


def ortho(left, right, bottom, top, near, far) -> np.ndarray:
    """mat4.ortho: WebGPU clip space, z in [0, 1]."""
    d = np.zeros(16, dtype=np.float64)
    d[0] = 2.0 / (right - left)
    d[5] = 2.0 / (top - bottom)
    d[10] = 1.0 / (near - far)
    d[12] = (right + left) / (left - right)
    d[13] = (top + bottom) / (bottom - top)
    d[14] = near / (near - far)
    d[15] = 1.0
    return _f32(d)


def look_at(eye, target, up=(0.0, 1.0, 0.0)) -> np.ndarray:
    """mat4.lookAt -> view matrix (camera looks down -z)."""
    eye = np.asarray(eye, dtype=np.float64)
    z = eye - np.asarray(target, dtype=np.float64)
    z /= np.linalg.norm(z)
    x = np.cross(np.asarray(up, dtype=np.float64), z)
    x /= np.linalg.norm(x)
    y = np.cross(z, x)
    y /= np.linalg.norm(y)
    d = np.array([x[0], y[0], z[0], 0.0,
                  x[1], y[1], z[1], 0.0,
                  x[2], y[2], z[2], 0.0,
                  -x @ eye, -y @ eye, -z @ eye, 1.0])
    return _f32(d)


def translation(v) -> np.ndarray:
    d = np.eye(4).reshape(16)
    d[12:15] = np.asarray(v, dtype=np.float64)[:3]
    return _f32(d)


def scale(m: np.ndarray, s) -> np.ndarray:
    return multiply(m, _f32(np.diag([s[0], s[1], s[2], 1.0]).reshape(16)))


def transform_point(m: np.ndarray, p) -> np.ndarray:
    """vec4.transformMat4 of (p, 1)."""
    v = np.array([p[0], p[1], p[2], 1.0], dtype=np.float64)
    return _f32(to_rows(m) @ v)


def spherical_to_cartesian(phi: float, theta: float, degrees: bool = True) -> np.ndarray:
    """sphericalToCartesian, src/utils/index.ts:60-76"""
    if degrees:
        phi, theta = math.radians(phi), math.radians(theta)
    return np.array([math.cos(phi) * math.sin(theta), math.cos(theta),
                     math.sin(phi) * math.sin(theta)], dtype=np.float64)
