"""The reference's per-pass operator interface over libhairfb.so.

Each class mirrors one pass of src/passes (constructor, onViewportResize,
cmdClearBeforeRender, cmd<Work>) and forwards to its ``hfb_*`` entry point.
Device buffers are torch CUDA tensors in the reference layouts; uniform
blocks are the raw bytes of ``hairfb.uniforms`` (what the reference writes
with queue.writeBuffer).  ``Renderer`` runs the passes in the order of
src/renderer.ts:171-295.
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import hair_object as HO
from .config import HairConfig
from .formats import SdfVolume
from .lib import Context, HfbHairData, HfbPresentItem, HfbRasterBuffers, byref, ptr, strand_grid_order


def _dev(a, dtype=None) -> torch.Tensor:
    t = torch.as_tensor(np.ascontiguousarray(a))
    if dtype is not None:
        t = t.to(dtype)
    return t.cuda()


def _ub(b: bytes):
    """Host pointer to a uniform block (kept alive by the caller's bytes)."""
    return ctypes.cast(ctypes.c_char_p(b), ctypes.c_void_p)


# ---------------------------------------------------------------------------
# scene objects (src/scene/hair/hairObject.ts, src/scene/sdfCollider,
# src/passes/simulation/grids/gridData.ts)
# ---------------------------------------------------------------------------

class HairObject:
    """GPU buffers of one hair object; tick-tock positions
    (src/scene/hair/hairObject.ts:29-155)."""

    def __init__(self, buffers: HO.HairBuffers, shading_points: int, upload=None, grid_order=None):
        """upload: host array -> device tensor (default: a blocking copy);
        grid_order: the asset's strand_grid_order, if already known."""
        up = upload or _dev
        a = buffers.asset
        self.buffers = buffers
        self.strands_count = a.strands
        self.points_per_strand = a.points_per_strand
        self.initial = up(a.positions)
        self.positions_0 = self.initial.clone()
        self.positions_1 = self.initial.clone()
        self.tangents = up(buffers.tangents)
        self.segment_lengths = up(buffers.segment_lengths)
        self.shading = up(HO.initial_shading(a.strands, shading_points))
        # the order the grid splat visits the strands in (neighbouring roots together)
        if grid_order is None:
            grid_order = strand_grid_order(a.positions, a.strands, a.points_per_strand).view(np.int32)
        self.grid_order = up(grid_order)
        self.hair_data = HfbHairData()
        for i in range(3):
            self.hair_data.boundingSphere[i] = float(buffers.sphere_center[i])
        self.hair_data.boundingSphere[3] = float(buffers.sphere_radius)
        self.hair_data.strandsCount = a.strands
        self.hair_data.pointsPerStrand = a.points_per_strand
        self._current = 0
        self.lod_render_percent = 100.0

    @property
    def positions(self) -> torch.Tensor:  # bindPointsPositions
        return self.positions_0 if self._current == 0 else self.positions_1

    @property
    def positions_prev(self) -> torch.Tensor:  # bindPointsPositions_PREV
        return self.positions_1 if self._current == 0 else self.positions_0

    def swap_position_buffers_after_sim_integration(self) -> None:
        self._current = 1 - self._current

    def reset_simulation(self) -> None:
        """resetSimulation, hairObject.ts:75-91"""
        self.positions_0.copy_(self.initial)
        self.positions_1.copy_(self.initial)

    def rendered_strand_count(self) -> int:
        return HO.rendered_strand_count(self.strands_count, self.lod_render_percent)


class SdfCollider:
    def __init__(self, vol: SdfVolume, upload=None):
        self.dims = int(vol.dims)
        self.bounds = (np.asarray(vol.bounds_min, np.float32), np.asarray(vol.bounds_max, np.float32))
        self.texture = (upload or _dev)(vol.distances)


class PhysicsGrids:
    """The two physics grids of GridData (gridData.ts:34-62)."""

    def __init__(self, dims: int):
        n = dims * dims * dims
        self.dims = dims
        self.density_velocity = torch.zeros((n, 4), dtype=torch.int32, device="cuda")
        self.density_grad_wind = torch.zeros((n, 4), dtype=torch.float32, device="cuda")

    def clear(self) -> None:
        self.density_velocity.zero_()
        self.density_grad_wind.zero_()


# ---------------------------------------------------------------------------
# simulation passes
# ---------------------------------------------------------------------------

class GridPreSimPass:
    """src/passes/simulation/gridPreSimPass.ts"""
    NAME = "GridPreSimPass"

    def __init__(self, ctx: Context):
        self.ctx = ctx

    def cmd_update_grids_before_sim(self, sim_uniforms: bytes, grids: PhysicsGrids, sdf: SdfCollider):
        self.ctx.call("hfb_grid_pre_sim", _ub(sim_uniforms), ptr(grids.density_velocity),
                      ptr(grids.density_grad_wind), ptr(sdf.texture), sdf.dims)


class HairSimIntegrationPass:
    """src/passes/simulation/hairSimIntegrationPass.ts"""
    NAME = "HairSimIntegrationPass"

    def __init__(self, ctx: Context):
        self.ctx = ctx

    def cmd_simulate_hair_positions(self, sim_uniforms: bytes, hair: HairObject, grids: PhysicsGrids,
                                    sdf: SdfCollider):
        self.ctx.call("hfb_sim_integrate", _ub(sim_uniforms), byref(hair.hair_data),
                      ptr(hair.positions_prev), ptr(hair.positions), ptr(hair.initial),
                      ptr(hair.segment_lengths), ptr(grids.density_velocity),
                      ptr(grids.density_grad_wind), ptr(sdf.texture), sdf.dims)
        hair.swap_position_buffers_after_sim_integration()  # hairSimIntegrationPass.ts:59


class GridPostSimPass:
    """src/passes/simulation/gridPostSimPass.ts"""
    NAME = "GridPostSimPass"

    def __init__(self, ctx: Context):
        self.ctx = ctx

    def cmd_update_grids_after_sim(self, sim_uniforms: bytes, hair: HairObject, grids: PhysicsGrids):
        self.ctx.call("hfb_grid_post_sim_ordered", _ub(sim_uniforms), byref(hair.hair_data),
                      ptr(hair.positions_prev), ptr(hair.positions), ptr(grids.density_velocity),
                      ptr(hair.grid_order))


# ---------------------------------------------------------------------------
# shading + raster passes
# ---------------------------------------------------------------------------

class HairShadingPass:
    """src/passes/hairShadingPass/hairShadingPass.ts"""
    NAME = "HairShadingPass"

    def __init__(self, ctx: Context):
        self.ctx = ctx

    def cmd_compute_shading_points(self, uniforms: bytes, hair: HairObject, depth: torch.Tensor,
                                   ao: torch.Tensor | None = None, ao_size=(0, 0),
                                   shadow_map: torch.Tensor | None = None, shadow_size: int = 0):
        self.ctx.call("hfb_shading", _ub(uniforms), byref(hair.hair_data), ptr(hair.positions),
                      ptr(hair.tangents), ptr(depth), ptr(ao), ao_size[0], ao_size[1],
                      ptr(shadow_map), shadow_size, ptr(hair.shading))


class RasterBuffers:
    """The viewport-sized buffers the three raster passes share (PassCtx)."""

    def __init__(self, ctx: Context, width: int, height: int, max_drawn: int | None = None,
                 pooled: bool = False):
        """max_drawn: the segment pool's size in records (None: the config's
        1 + tiles * avgSegmentsPerTile).  pooled: carve the buffers out of one
        tensor from torch's caching allocator on the current stream instead
        of hfb_raster_buffers_alloc_sized's cudaMalloc calls, so that making
        and dropping them never waits for the device (cudaFree does); a
        server admitting and retiring sessions while frames run uses it."""
        self.ctx = ctx
        self.rb = HfbRasterBuffers()
        self._block = None
        if pooled:
            self._alloc_pooled(width, height, max_drawn)
        elif max_drawn is None:
            ctx.call("hfb_raster_buffers_alloc", width, height, byref(self.rb))
        else:
            ctx.call("hfb_raster_buffers_alloc_sized", width, height, int(max_drawn), byref(self.rb))
        self.width, self.height = width, height

    def _alloc_pooled(self, width: int, height: int, max_drawn: int | None) -> None:
        c = self.ctx.cfg
        tiles = (-(-width // c.tileSize)) * (-(-height // c.tileSize))
        md = 1 + tiles * c.avgSegmentsPerTile if max_drawn is None else int(max_drawn)
        scratch = int(self.ctx.lib.hfb_raster_scratch_bytes_for(byref(c), width, height, md))
        sizes = [tiles * c.tileDepthBins * 16, 4 + md * 8, tiles * 4, c.sortBuckets * 8, (4 + tiles) * 4,
                 16 + width * height * 16, scratch]
        offs, total = [], 0
        for n in sizes:  # every buffer 256-byte aligned
            offs.append(total)
            total += (n + 255) // 256 * 256
        # zeroed: the cleared state of hfb_raster_buffers_alloc_sized
        self._block = torch.zeros(total, dtype=torch.uint8, device="cuda")
        base = self._block.data_ptr()
        rb = self.rb
        rb.width, rb.height, rb.maxDrawnSegments = width, height, md
        (rb.tiles, rb.tileSegments, rb.segmentCountPerTile, rb.sortBuckets, rb.tileList, rb.rasterizerResult,
         rb.scratch) = [base + o for o in offs]
        rb.scratchBytes = scratch

    @property
    def nbytes(self) -> int:
        """Device bytes of a pooled set (0 for the library's allocations)."""
        return 0 if self._block is None else self._block.numel()

    @property
    def max_drawn_segments(self) -> int:
        return int(self.rb.maxDrawnSegments)

    def close(self):
        if self._block is not None:
            self._block = None  # back to torch's cache; the caller ensured no frame still uses it
            self.rb = HfbRasterBuffers()
        elif self.rb.tiles:
            self.ctx.call("hfb_raster_buffers_free", byref(self.rb))

    # ---- readback helpers (numpy copies of the reference-layout buffers) ----
    def _download(self, addr, count, dtype):
        out = np.empty(count, dtype=dtype)
        self.ctx.call("hfb_buffer_download", out.ctypes.data, addr, out.nbytes)
        return out

    def tile_count(self):
        c = self.ctx.cfg
        return (-(-self.width // c.tileSize)) * (-(-self.height // c.tileSize))

    def read_tiles(self):
        T = self.tile_count()
        return self._download(self.rb.tiles, T * self.ctx.cfg.tileDepthBins * 4, np.uint32).reshape(-1, 4)

    def read_tile_segments(self):
        return self._download(self.rb.tileSegments, 1 + 2 * self.max_drawn_segments, np.uint32)

    def read_segment_counts(self):
        return self._download(self.rb.segmentCountPerTile, self.tile_count(), np.uint32)

    def read_sort_buckets(self):
        return self._download(self.rb.sortBuckets, 2 * self.ctx.cfg.sortBuckets, np.uint32)

    def read_tile_list(self):
        return self._download(self.rb.tileList, 4 + self.tile_count(), np.uint32)

    def read_result(self):
        return self._download(self.rb.rasterizerResult, 4 + 4 * self.width * self.height, np.float32)

    def result_tensor(self) -> torch.Tensor:
        """Zero-copy view of the pixels is not exposed by torch for raw
        pointers; copy through the C-ABI instead."""
        return torch.from_numpy(self.read_result()[4:].reshape(self.height, self.width, 4))


class HairTilesPass:
    """src/passes/swHair/hairTilesPass.ts"""
    NAME = "HairTilesPass"

    def __init__(self, ctx: Context):
        self.ctx = ctx

    def cmd_draw_hair_to_tiles(self, uniforms: bytes, hair: HairObject, depth: torch.Tensor,
                               rb: RasterBuffers):
        self.ctx.call("hfb_tiles_pass", _ub(uniforms), byref(hair.hair_data), ptr(hair.positions),
                      ptr(hair.tangents), ptr(depth), hair.rendered_strand_count(), byref(rb.rb))


class HairTileSortPass:
    """src/passes/swHair/hairTileSortPass.ts"""
    NAME = "HairTileSortPass"

    def __init__(self, ctx: Context):
        self.ctx = ctx

    def cmd_sort_hair_tiles(self, rb: RasterBuffers):
        self.ctx.call("hfb_tile_sort", byref(rb.rb))


class HairFinePass:
    """src/passes/swHair/hairFinePass.ts"""
    NAME = "HairFinePass"

    def __init__(self, ctx: Context):
        self.ctx = ctx

    def cmd_rasterize_slices_hair(self, uniforms: bytes, hair: HairObject, depth: torch.Tensor,
                                  rb: RasterBuffers):
        self.ctx.call("hfb_fine_pass", _ub(uniforms), byref(hair.hair_data), ptr(hair.positions),
                      ptr(hair.tangents), ptr(hair.shading), ptr(depth), byref(rb.rb))


class HwHairPass:
    """src/passes/hwHair/hwHairPass.ts: the depth it draws (cmdDrawHair's depth
    attachment), which the shading pass reads."""
    NAME = "HwHairPass"

    def __init__(self, ctx: Context):
        self.ctx = ctx

    def cmd_draw_hair_depth(self, uniforms: bytes, hair: HairObject, scene_depth: torch.Tensor,
                            hair_depth: torch.Tensor, rb: RasterBuffers):
        """hair_depth = scene_depth with the hair's triangles drawn over it
        (depth test 'less')."""
        self.ctx.call("hfb_hair_depth", _ub(uniforms), byref(hair.hair_data), ptr(hair.positions),
                      ptr(hair.tangents), hair.rendered_strand_count(), ptr(scene_depth), ptr(hair_depth),
                      byref(rb.rb))

    def cmd_draw_hair_normals(self, uniforms: bytes, hair: HairObject, hair_depth: torch.Tensor,
                              normals: torch.Tensor, rb: RasterBuffers, winner: torch.Tensor | None = None):
        """The pass's normal output: normals ((H*W, 2) float32, in/out) gets
        the hair's octahedron-encoded tangent where the hair is in front in
        hair_depth (as cmd_draw_hair_depth left it)."""
        if winner is None:
            winner = torch.empty(rb.width * rb.height, dtype=torch.int32, device="cuda")
        self.ctx.call("hfb_hair_normals", _ub(uniforms), byref(hair.hair_data), ptr(hair.positions),
                      ptr(hair.tangents), hair.rendered_strand_count(), ptr(hair_depth), ptr(normals), ptr(winner),
                      byref(rb.rb))


class PresentPass:
    """src/passes/hairCombine/hairCombinePass.ts + src/passes/presentPass/
    presentPass.ts (final display mode): the frame's 8-bit image."""
    NAME = "PresentPass"

    def __init__(self, ctx: Context):
        self.ctx = ctx

    def cmd_draw(self, uniforms: bytes, rb: RasterBuffers, scene_color: torch.Tensor | None = None,
                 out: torch.Tensor | None = None) -> torch.Tensor:
        """The fine pass's result over scene_color ((H, W, 4) float32, row 0
        at the top; None = black), tone mapped: (H, W, 4) uint8, row 0 at
        the top."""
        if out is None:
            out = torch.empty((rb.height, rb.width, 4), dtype=torch.uint8, device="cuda")
        self.ctx.call("hfb_present", _ub(uniforms), byref(rb.rb), ptr(scene_color), ptr(out))
        return out

    def cmd_draw_batch(self, items) -> None:
        """cmd_draw for every (uniforms, rb, scene_color or None, out) of
        items, out given: one launch per 64 images (hfb_present_batch), each
        image as cmd_draw makes it."""
        arr = (HfbPresentItem * len(items))()
        keep = []  # the uniform blocks' host pointers stay valid through the call
        for k, (uniforms, rb, scene_color, out) in enumerate(items):
            ub = _ub(uniforms)
            keep.append((uniforms, ub))
            arr[k] = HfbPresentItem(ub.value, ctypes.addressof(rb.rb), ptr(scene_color), ptr(out))
        self.ctx.call("hfb_present_batch", arr, len(items))


class AoPass:
    """src/passes/aoPass/aoPass.ts: GTAO from the depth and the normals."""
    NAME = "AoPass"

    def __init__(self, ctx: Context):
        self.ctx = ctx

    def cmd_calc_ao(self, uniforms: bytes, depth: torch.Tensor, normals: torch.Tensor, width: int, height: int,
                    scale: float = 0.5) -> torch.Tensor:
        """(ceil(height*scale), ceil(width*scale)) float32 AO (r16float
        values), for hfb_shading's ao input."""
        import math
        out = torch.empty((math.ceil(height * scale), math.ceil(width * scale)), dtype=torch.float32, device="cuda")
        self.ctx.call("hfb_gtao", _ub(uniforms), ptr(depth), ptr(normals), ctypes.c_float(scale), ptr(out))
        return out


def clear_before_render(ctx: Context, rb: RasterBuffers):
    """cmdClearBeforeRender of the tiles, fine and sort passes."""
    ctx.call("hfb_clear_before_render", byref(rb.rb))
