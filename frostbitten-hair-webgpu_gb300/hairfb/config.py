"""Compile-time constants of the hair passes (the reference's global CONFIG).

Mirrors the fields of ``CONFIG.hairRender`` / ``CONFIG.hairSimulation`` that
the reference splices into its WGSL at pipeline creation
(src/constants.ts:86-349, src/passes/swHair/shaderImpl/tileUtils.wgsl.ts:5-6,
src/passes/swHair/hairFinePass.wgsl.ts:43, src/scene/hair/hairShadingBuffer.ts:24,
src/passes/simulation/grids/grids.wgsl.ts:7).

``HfbConfig`` is the ctypes twin of ``struct HfbConfig`` in include/hairfb.h;
the byte layout is the C-ABI contract.
"""
from __future__ import annotations

import ctypes
import dataclasses
import math


class HfbConfig(ctypes.Structure):
    """``struct HfbConfig`` (include/hairfb.h), 64 bytes."""

    _fields_ = [
        ("tileSize", ctypes.c_uint32),
        ("tileDepthBins", ctypes.c_uint32),
        ("slicesPerPixel", ctypes.c_uint32),
        ("shadingPoints", ctypes.c_uint32),
        ("gridDims", ctypes.c_uint32),
        ("sortBuckets", ctypes.c_uint32),
        ("sortBucketSize", ctypes.c_uint32),
        ("avgSegmentsPerTile", ctypes.c_uint32),
        ("avgFragmentsPerSlice", ctypes.c_uint32),
        ("invalidTilesPerSegmentThreshold", ctypes.c_uint32),
        ("processorCount", ctypes.c_uint32),
        ("alphaQuadratic", ctypes.c_uint32),
        ("alphaMultiplier", ctypes.c_float),
        ("cameraNear", ctypes.c_float),
        ("cameraFar", ctypes.c_float),
        ("reserved", ctypes.c_uint32),
    ]


assert ctypes.sizeof(HfbConfig) == 64


@dataclasses.dataclass
class HairConfig:
    """Pass constants. Defaults are the reference's CONFIG values."""

    tile_size: int = 8                        # hairRender.tileSize
    tile_depth_bins: int = 32                 # hairRender.tileDepthBins
    slices_per_pixel: int = 8                 # hairRender.slicesPerPixel
    shading_points: int = 64                  # hairRender.shadingPoints
    grid_dims: int = 64                       # hairSimulation.physicsForcesGrid.dims
    sort_buckets: int = 64                    # hairRender.sortBuckets
    sort_bucket_size: int = 16                # hairRender.sortBucketSize
    avg_segments_per_tile: int = 128          # hairRender.avgSegmentsPerTile
    avg_fragments_per_slice: int = 16         # hairRender.avgFragmentsPerSlice
    invalid_tiles_per_segment_threshold: int = 128
    processor_count: int = 512                # hairRender.processorCount
    alpha_quadratic: bool = False             # hairRender.alphaQuadratic
    alpha_multiplier: float = 1.1             # hairRender.alphaMultipler
    camera_near: float = 0.01                 # camera.projection.near
    camera_far: float = 100.0                 # camera.projection.far

    def to_c(self) -> HfbConfig:
        return HfbConfig(
            self.tile_size, self.tile_depth_bins, self.slices_per_pixel,
            self.shading_points, self.grid_dims, self.sort_buckets,
            self.sort_bucket_size, self.avg_segments_per_tile,
            self.avg_fragments_per_slice, self.invalid_tiles_per_segment_threshold,
            self.processor_count, 1 if self.alpha_quadratic else 0,
            self.alpha_multiplier, self.camera_near, self.camera_far, 0)

    # --- derived sizes (src/passes/swHair/shared/*.ts) -------------------
    def tile_count(self, width: int, height: int) -> tuple[int, int]:
        """getTileCount, src/passes/swHair/shared/utils.ts:4-10"""
        return (-(-width // self.tile_size), -(-height // self.tile_size))

    def max_drawn_segments(self, width: int, height: int) -> int:
        """getLengthOfHairTileSegmentsBuffer, hairTileSegmentsBuffer.ts:81-87"""
        tx, ty = self.tile_count(width, height)
        return 1 + int(math.ceil(tx * ty * self.avg_segments_per_tile))

    def slice_data_per_processor(self) -> int:
        """SLICE_DATA_PER_PROCESSOR_COUNT, hairSlicesDataBuffer.ts:16-20"""
        return (self.avg_fragments_per_slice * self.slices_per_pixel
                * self.tile_size * self.tile_size)


@dataclasses.dataclass
class SimulationParams:
    """Runtime simulation settings (CONFIG.hairSimulation, constants.ts:267-340)."""

    delta_time: float = 1.0 / 30.0
    gravity: float = 0.03
    friction: float = 0.3
    volume_preservation: float = 0.00003
    collision_sphere: tuple = (-0.18, 1.56, 0.06, 0.06)
    constraint_iterations: int = 7
    stiffness_length: float = 1.0
    stiffness_global: float = 0.2
    global_extent: float = 0.1
    global_fade: float = 0.75
    stiffness_local: float = 0.3
    stiffness_collisions: float = 1.0
    stiffness_sdf: float = 1.0
    wind_dir_phi: float = 18.0
    wind_dir_theta: float = 91.0
    wind_strength: float = 0.0
    wind_strength_lull: float = 0.75
    wind_strength_frequency: float = 1.8
    wind_strength_jitter: float = 0.7
    wind_phase_offset: float = 0.45
    wind_collision_trace_offset: float = 1.5
    sdf_distance_offset: float = -0.0015
    grid_scale: float = 2.0
