"""Host-side builders of the static per-hair buffers.

Restates ``createHairObject`` (src/scene/loadScene.ts:94-148) and the buffer
builders it calls.  The reference computes these in JavaScript (float64)
through wgpu-matrix, storing every vector in a Float32Array; the same
float64-compute / float32-store rounding is kept here so the bytes match.
"""
from __future__ import annotations

import dataclasses

import numpy as np


@dataclasses.dataclass
class HairAsset:
    """TfxFileData (src/scene/hair/tfxFileLoader.ts:33-37): positions are
    ``array<vec4f>`` (xyz + w = isMovable), strand-major."""
    strands: int
    points_per_strand: int
    positions: np.ndarray  # (strands * points, 4) float32


def bounding_box(positions: np.ndarray):
    """calcBoundingBox(positions, 4), src/utils/bounds.ts:69-76"""
    p = positions[:, :3]
    return p.min(axis=0).astype(np.float32), p.max(axis=0).astype(np.float32)


def bounding_sphere(bmin, bmax):
    """calcBoundingSphere, src/utils/bounds.ts:101-108 (vec3.midpoint, vec3.distance)."""
    a = np.asarray(bmin, np.float64)
    b = np.asarray(bmax, np.float64)
    center = (a + 0.5 * (b - a)).astype(np.float32)
    radius = float(np.sqrt(np.sum((b - center.astype(np.float64)) ** 2)))
    return center, np.float32(radius)


def scale_bounding_box(bmin, bmax, scale: float):
    """scaleBoundingBox, src/utils/bounds.ts:120-133 (GridData bounds, gridData.ts:34-38)."""
    a = np.asarray(bmin, np.float64)
    b = np.asarray(bmax, np.float64)
    center = (a + 0.5 * (b - a)).astype(np.float32).astype(np.float64)
    v = (b - center).astype(np.float32).astype(np.float64)
    sv = (v * scale).astype(np.float32).astype(np.float64)
    return (center - sv).astype(np.float32), (center + sv).astype(np.float32)


def hair_data_bytes(strands: int, points: int, sphere_center, sphere_radius) -> bytes:
    """createHairDataBuffer, src/scene/hair/hairDataBuffer.ts:26-47:
    struct HairData { boundingSphere: vec4f, strandsCount: u32, pointsPerStrand: u32 }"""
    b = np.zeros(8, dtype=np.uint32)
    b.view(np.float32)[0:3] = np.asarray(sphere_center, np.float32)
    b.view(np.float32)[3] = np.float32(sphere_radius)
    b[4] = strands
    b[5] = points
    return b.tobytes()


def tangents(asset: HairAsset) -> np.ndarray:
    """createHairTangentsBuffer, src/scene/hair/hairTangentsBuffer.ts:35-76.
    Static tangents from the initial positions; tip copies the previous; w = 0."""
    S, P = asset.strands, asset.points_per_strand
    pos = asset.positions[:, :3].reshape(S, P, 3).astype(np.float64)
    k = np.arange(P)
    k = np.where(k == P - 1, P - 2, k)
    d = (pos[:, k + 1, :] - pos[:, k, :]).astype(np.float32).astype(np.float64)  # vec3.subtract -> f32
    ln = np.sqrt(np.sum(d * d, axis=-1, keepdims=True))
    with np.errstate(invalid="ignore", divide="ignore"):
        t = np.where(ln > 0.00001, d / ln, 0.0)  # vec3.normalize
    out = np.zeros((S, P, 4), dtype=np.float32)
    out[..., :3] = t.astype(np.float32)
    return out.reshape(S * P, 4)


def segment_lengths(asset: HairAsset) -> np.ndarray:
    """createHairSegmentLengthsBuffer, src/scene/hair/hairSegmentLengthsBuffer.ts:26-55."""
    S, P = asset.strands, asset.points_per_strand
    pos = asset.positions[:, :3].reshape(S, P, 3).astype(np.float64)
    out = np.zeros((S, P), dtype=np.float64)
    out[:, :-1] = np.sqrt(np.sum((pos[:, 1:] - pos[:, :-1]) ** 2, axis=-1))
    out[:, -1] = out[:, -2]
    return out.astype(np.float32).reshape(S * P)


def initial_shading(strands: int, shading_points: int) -> np.ndarray:
    """createHairShadingBuffer, src/scene/hair/hairShadingBuffer.ts:49-76:
    red at the root, green at the tip."""
    p = np.arange(shading_points, dtype=np.float64) / (shading_points - 1)
    g = np.stack([1.0 - p, p, np.zeros_like(p), np.ones_like(p)], axis=-1).astype(np.float32)
    return np.tile(g, (strands, 1))


@dataclasses.dataclass
class HairBuffers:
    """Every static host array of one hair object, in the reference layouts."""
    asset: HairAsset
    tangents: np.ndarray
    segment_lengths: np.ndarray
    bbox: tuple
    sphere_center: np.ndarray
    sphere_radius: np.float32
    hair_data: bytes


def build_hair_buffers(asset: HairAsset) -> HairBuffers:
    bmin, bmax = bounding_box(asset.positions)
    c, r = bounding_sphere(bmin, bmax)
    return HairBuffers(
        asset=asset,
        tangents=tangents(asset),
        segment_lengths=segment_lengths(asset),
        bbox=(bmin, bmax),
        sphere_center=c,
        sphere_radius=r,
        hair_data=hair_data_bytes(asset.strands, asset.points_per_strand, c, r),
    )


def rendered_strand_count(strands: int, lod_percent: float = 100.0) -> int:
    """HairObject.getRenderedStrandCount, src/scene/hair/hairObject.ts:52-57"""
    pct = min(max(lod_percent, 0.0), 100.0)
    return int(min(max(int(np.ceil(strands * pct / 100.0)), 0), strands))
