"""Frame orchestration of the hair hot path (src/renderer.ts:145-295).

    simulateHair           GridPreSimPass -> HairSimIntegrationPass (+ swap)
                           -> GridPostSimPass                  (:212-240)
    cmdDrawScene           clear -> HairTilesPass -> HairTileSortPass
                           -> HairFinePass                      (:263-277)
    updateResources...     HairShadingPass (used by the next frame)  (:285-295)

The mesh pass, hardware hair pass, AO and shadow maps of the reference are
outside this path: their outputs come in as buffers (the scene depth used
by the tiles / fine depth tests, the depth-with-hair used by the shading
attenuation, AO and shadow map textures).
"""
from __future__ import annotations

import ctypes

import torch

from . import synthetic, uniforms as UN
from .config import HairConfig
from .lib import Context, HfbInstance, ptr
from .passes import (GridPostSimPass, GridPreSimPass, HairFinePass, HairObject, HairShadingPass,
                     HairSimIntegrationPass, HairTileSortPass, HairTilesPass, HwHairPass, PhysicsGrids,
                     PresentPass, RasterBuffers, SdfCollider, AoPass, clear_before_render)


class Renderer:
    """One hair instance rendered frame by frame through libhairfb.so."""

    def __init__(self, inst: synthetic.Instance, device: int = -1, ctx: Context | None = None,
                 max_drawn: int | None = None, hair_depth: bool = False, ao: bool = False,
                 pooled: bool = False, upload=None, grid_order=None):
        """max_drawn: this instance's segment pool in records (None: the
        config's 1 + tiles * avgSegmentsPerTile).  hair_depth: draw the hair's
        depth over the scene depth after the fine pass (HwHairPass) and shade
        with it, as the reference does; otherwise the shading reads the scene
        depth.  ao (with hair_depth): also the hair's normals and GTAO
        (AoPass) after it, which the shading then reads, as the reference's
        updateResourcesForNextFrame does (renderer.ts:286-296); the scene's
        normals are the reference's clear value, 0 (no mesh pass here).
        These run in the pass-by-pass frames (frame()); hfb_frame and
        hfb_frame_batch take the AO as an input instead.  pooled: the raster
        buffers come from torch's caching allocator (RasterBuffers).  upload:
        host array -> device tensor for the static data (default: blocking
        copies); grid_order: the asset's strand order for the grid splat."""
        self.inst = inst
        self.cfg: HairConfig = inst.cfg
        self.ctx = ctx or Context(inst.cfg.to_c(), device)
        self.max_drawn = max_drawn
        self.hair = HairObject(inst.hair, inst.cfg.shading_points, upload, grid_order)
        self.sdf = SdfCollider(inst.sdf, upload)
        self.grids = PhysicsGrids(inst.cfg.grid_dims)
        self.rb = RasterBuffers(self.ctx, inst.width, inst.height, max_drawn, pooled=pooled)
        self.scene_depth = upload(inst.scene_depth) if upload else torch.as_tensor(inst.scene_depth).cuda()
        # depth buffer with hair drawn, for the shading attenuation; before the
        # first frame draws the hair it holds the scene alone
        self.hair_depth = self.scene_depth.clone() if hair_depth else None
        self.shading_depth = self.hair_depth if hair_depth else self.scene_depth
        assert hair_depth or not ao, "AO needs the hair depth"
        n = inst.width * inst.height
        self.normals = torch.zeros((n, 2), dtype=torch.float32, device="cuda") if ao else None
        self.winner = torch.empty(n, dtype=torch.int32, device="cuda") if ao else None
        self.ao = None
        self.grid_pre = GridPreSimPass(self.ctx)
        self.integrate = HairSimIntegrationPass(self.ctx)
        self.grid_post = GridPostSimPass(self.ctx)
        self.shading = HairShadingPass(self.ctx)
        self.tiles = HairTilesPass(self.ctx)
        self.sort = HairTileSortPass(self.ctx)
        self.fine = HairFinePass(self.ctx)
        self.hw_hair = HwHairPass(self.ctx)
        self.frame_idx = 0
        self.uniforms = UN.pack_render_uniforms(inst.scene, inst.cfg, max_drawn)
        self._inst = self._inst_uniforms = self._inst_rb = None  # cached HfbInstance (instance())

    def use_config(self, cfg: HairConfig, ctx: Context) -> None:
        """Re-targets the renderer to other pass constants (a context of
        that config): new uniforms, and new raster buffers unless their
        sizes (tile size, depth bins, segment pool) are unchanged; the
        simulation state and the hair stay resident.  The grid size must not
        change."""
        assert cfg.grid_dims == self.cfg.grid_dims and cfg.shading_points == self.cfg.shading_points
        same_buffers = (cfg.tile_size, cfg.tile_depth_bins, cfg.sort_buckets) == \
            (self.cfg.tile_size, self.cfg.tile_depth_bins, self.cfg.sort_buckets) and \
            (self.max_drawn is not None or cfg.avg_segments_per_tile == self.cfg.avg_segments_per_tile)
        old = self.rb
        self.cfg = cfg
        self.ctx = ctx
        if not same_buffers:
            self.rb = RasterBuffers(ctx, self.inst.width, self.inst.height, self.max_drawn)
        else:
            self.rb.ctx = ctx
        for p in (self.grid_pre, self.integrate, self.grid_post, self.shading, self.tiles, self.sort, self.fine,
                  self.hw_hair):
            p.ctx = ctx
        self.uniforms = UN.pack_render_uniforms(self.inst.scene, cfg, self.max_drawn)
        if not same_buffers:
            old.close()

    def sim_uniforms(self, frame_idx: int) -> bytes:
        i = self.inst
        return UN.pack_sim_uniforms(i.sim, i.scene.model_matrix, i.scene.sdf_bounds, i.scene.grid_bounds,
                                    frame_idx, wind_dir=i.wind_dir, wind_strength=i.wind_strength(frame_idx))

    def before_first_frame(self) -> None:
        """beforeFirstFrame, renderer.ts:145-169: initial density grid and
        the first shading."""
        su = self.sim_uniforms(0)
        self.grid_post.cmd_update_grids_after_sim(su, self.hair, self.grids)
        self._resources_for_next_frame()

    def simulate(self) -> None:
        su = self.sim_uniforms(self.frame_idx)
        self.grid_pre.cmd_update_grids_before_sim(su, self.grids, self.sdf)
        self.integrate.cmd_simulate_hair_positions(su, self.hair, self.grids, self.sdf)
        self.grid_post.cmd_update_grids_after_sim(su, self.hair, self.grids)

    def draw(self) -> None:
        clear_before_render(self.ctx, self.rb)
        self.tiles.cmd_draw_hair_to_tiles(self.uniforms, self.hair, self.scene_depth, self.rb)
        self.sort.cmd_sort_hair_tiles(self.rb)
        self.fine.cmd_rasterize_slices_hair(self.uniforms, self.hair, self.scene_depth, self.rb)
        self._resources_for_next_frame()

    def _resources_for_next_frame(self) -> None:
        """updateResourcesForNextFrame, renderer.ts:286-296: hwHair (depth,
        and normals when AO is on), AO, then the shading."""
        if self.hair_depth is not None:
            self.hw_hair.cmd_draw_hair_depth(self.uniforms, self.hair, self.scene_depth, self.hair_depth, self.rb)
        if self.normals is not None:
            self.normals.zero_()  # CONFIG.clearNormals
            self.hw_hair.cmd_draw_hair_normals(self.uniforms, self.hair, self.hair_depth, self.normals, self.rb,
                                               self.winner)
            self.ao = AoPass(self.ctx).cmd_calc_ao(self.uniforms, self.hair_depth, self.normals,
                                                   self.inst.width, self.inst.height)
            self.shading.cmd_compute_shading_points(self.uniforms, self.hair, self.shading_depth, self.ao,
                                                    (self.ao.shape[1], self.ao.shape[0]))
            return
        self.shading.cmd_compute_shading_points(self.uniforms, self.hair, self.shading_depth)

    def image(self, scene_color: torch.Tensor | None = None) -> torch.Tensor:
        """The last frame composited over scene_color and presented
        (HairCombinePass + PresentPass): (H, W, 4) uint8 on the device, row
        0 at the top; formats.write_png makes a PNG of it."""
        return PresentPass(self.ctx).cmd_draw(self.uniforms, self.rb, scene_color)

    def frame(self) -> None:
        """cmdRender, renderer.ts:171-210 (hair passes only), pass by pass."""
        self.simulate()
        self.draw()
        self.frame_idx += 1

    # ---- whole frames through hfb_frame / hfb_frame_batch ----
    def instance(self) -> HfbInstance:
        """This frame's HfbInstance.  The uniform blocks it points to live on
        the renderer: the render block as packed, the simulation block packed
        once and patched per frame (frameIdx, wind strength)."""
        i = self.inst
        if self._inst is None or self._inst_uniforms is not self.uniforms or self._inst_rb is not self.rb:
            self._u_buf = ctypes.create_string_buffer(self.uniforms, len(self.uniforms))
            su = self.sim_uniforms(self.frame_idx)
            self._su_buf = ctypes.create_string_buffer(su, len(su))
            h = self.hair
            inst = HfbInstance()
            inst.uniforms = ctypes.addressof(self._u_buf)
            inst.simUniforms = ctypes.addressof(self._su_buf)
            inst.hair = h.hair_data
            inst.positions[0] = ptr(h.positions_0)
            inst.positions[1] = ptr(h.positions_1)
            inst.positionsInitial = ptr(h.initial)
            inst.tangents = ptr(h.tangents)
            inst.segmentLengths = ptr(h.segment_lengths)
            inst.densityVelocity = ptr(self.grids.density_velocity)
            inst.densityGradWind = ptr(self.grids.density_grad_wind)
            inst.sdf = ptr(self.sdf.texture)
            inst.sdfDims = self.sdf.dims
            inst.shading = ptr(h.shading)
            inst.sceneDepth = ptr(self.scene_depth)
            inst.shadingDepth = ptr(self.shading_depth)
            inst.raster = self.rb.rb
            inst.hairDepth = ptr(self.hair_depth) if self.hair_depth is not None else None
            inst.gridOrder = ptr(h.grid_order)
            self._inst, self._inst_uniforms, self._inst_rb = inst, self.uniforms, self.rb
        else:
            UN.patch_sim_uniforms(self._su_buf, self.frame_idx, i.wind_strength(self.frame_idx))
        self._inst.current = self.hair._current
        self._inst.strandsToRender = self.hair.rendered_strand_count()
        return self._inst

    def after_native_frame(self, inst: HfbInstance) -> None:
        self.hair._current = inst.current
        self.frame_idx += 1

    def frame_native(self) -> None:
        """One frame through hfb_frame (the same passes, one C call)."""
        inst = self.instance()
        self.ctx.call("hfb_frame", ctypes.byref(inst))
        self.after_native_frame(inst)


class BatchRenderer:
    """Many hair instances, one hfb_frame_batch call per frame.  Every
    renderer must share the batch's context (its config applies to all)."""

    def __init__(self, renderers: list[Renderer]):
        assert renderers, "empty batch"
        self.ctx = renderers[0].ctx
        assert all(r.ctx is self.ctx for r in renderers), "a batch shares one context"
        self.renderers = renderers
        self._arr = None

    def before_first_frame(self) -> None:
        for r in self.renderers:
            r.before_first_frame()

    def frame(self) -> None:
        n = len(self.renderers)
        if self._arr is None or len(self._arr) != n:
            self._arr = (HfbInstance * n)()
        arr = self._arr
        for k, r in enumerate(self.renderers):
            arr[k] = r.instance()
        self.ctx.call("hfb_frame_batch", arr, n)
        for r, inst in zip(self.renderers, arr):
            r.after_native_frame(inst)


class SplitBatchRenderer:
    """Instance groups that carry their own pass constants: each group is a
    BatchRenderer on its own context (and stream), the groups' batched
    frames run side by side, and the caller's stream waits for all of them.
    Results are those of each instance rendered alone with its group's
    constants."""

    def __init__(self, groups: list[list[Renderer]], stream: torch.cuda.Stream):
        self.batches = [BatchRenderer(g) for g in groups if g]
        self.stream = stream
        self.renderers = [r for b in self.batches for r in b.renderers]

    def frame(self) -> None:
        start = torch.cuda.Event()
        start.record(self.stream)
        for b in self.batches:
            s = b.ctx.stream_obj
            s.wait_event(start)
            b.frame()
            done = torch.cuda.Event()
            done.record(s)
            self.stream.wait_event(done)
