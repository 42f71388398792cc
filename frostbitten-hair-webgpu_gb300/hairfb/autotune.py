"""Autotuner of batched frames: picks the pass constants a batch runs with.

The search runs in stages, each timed on the batch itself with
``hfb_frame_batch`` (CUDA events, after warm-up frames), keeping the fastest
candidate that drops no (segment, tile) record -- a dropped record would
change the image, so such a candidate is not an equal-accuracy choice:

1. tile size x depth bins (CONFIG.hairRender.tileSize / tileDepthBins);
2. slices per pixel (slicesPerPixel, src/constants.ts:251) at the winner;
3. the fine pass's persistent CTA count (processorCount, src/constants.ts:255,
   dispatched at src/passes/swHair/hairFinePass.ts:85): one full wave of
   resident CTAs, or the reference's 512;
4. instance groups that carry their own constants: the batch split by
   viewport size (the largest viewports apart from the rest), each part
   tuned through stages 1-3 on its own context and stream, the parts'
   frames running side by side;
5. for a single part, the number of instance groups that run side by side
   (``hfb_ctx_set_batch_groups``) and the pipelined frame.

The segment pool is sized per tile area (``avg_segments_per_tile`` scales
with the tile's pixel count), as the reference sizes it per tile.  Every
candidate renders exactly what the reference renders with the same
constants; the tuner only chooses among them.
"""
from __future__ import annotations

import dataclasses
import itertools
import time

import torch

from .config import HairConfig
from .lib import Context
from .renderer import BatchRenderer, Renderer, SplitBatchRenderer

TILE_SIZES = (8, 16, 32)
DEPTH_BINS = (4, 8, 16, 32)
SLICES = (2, 4, 8)
PROCESSOR_COUNTS = (0, 512)  # 0: one full wave of resident CTAs; 512: the reference's processorCount
GROUPS = (1, 2, 3, 4)
MIN_GAIN = 0.03  # a candidate must beat the current choice by this fraction
MIN_GAIN_PIPELINE = 0.10


@dataclasses.dataclass
class Trial:
    tile_size: int
    depth_bins: int
    processor_count: int
    ms: float
    dropped: int
    groups: int = 1  # 0: the pipelined frame
    slices: int = 4
    part: str = "all"

    def as_dict(self):
        return dataclasses.asdict(self)


@dataclasses.dataclass
class Tuned:
    """The tuner's choice: one config for all instances, or one per part."""
    parts: list            # [(name, HairConfig, Context, [Renderer])]
    batch: object          # BatchRenderer or SplitBatchRenderer
    trials: list
    groups: int = 1
    pipelined: bool = False

    @property
    def cfg(self) -> HairConfig:
        return self.parts[0][1]

    @property
    def ctxs(self) -> list:
        return [p[2] for p in self.parts]

    def describe(self) -> dict:
        def one(c: HairConfig):
            return {"tile_size": c.tile_size, "depth_bins": c.tile_depth_bins, "slices": c.slices_per_pixel,
                    "processor_count": c.processor_count, "avg_segments_per_tile": c.avg_segments_per_tile}
        d = {"parts": {name: dict(one(c), instances=len(rs)) for name, c, _, rs in self.parts},
             "groups": self.groups, "pipelined": self.pipelined}
        if len(self.parts) == 1:
            d.update(one(self.parts[0][1]))
        return d


def candidate_config(base: HairConfig, tile_size: int, depth_bins: int, processor_count: int = 0,
                     slices: int | None = None) -> HairConfig:
    scale = (tile_size / base.tile_size) ** 2
    return dataclasses.replace(base, tile_size=tile_size, tile_depth_bins=depth_bins,
                               processor_count=processor_count,
                               slices_per_pixel=base.slices_per_pixel if slices is None else slices,
                               avg_segments_per_tile=max(16, int(round(base.avg_segments_per_tile * scale))))


def time_batch(renderers: list[Renderer], ctx: Context, stream, frames: int, warmup: int) -> tuple[float, int]:
    """Mean ms per batched frame, and the records dropped meanwhile."""
    batch = BatchRenderer(renderers)
    return time_frames(batch, [ctx], stream, frames, warmup)


def time_frames(batch, ctxs, stream, frames: int, warmup: int) -> tuple[float, int]:
    for _ in range(warmup):
        batch.frame()
    torch.cuda.synchronize()
    d0 = sum(c.counters()["tileRecordsDropped"] for c in ctxs)
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    t0.record(stream)
    for _ in range(frames):
        batch.frame()
    t1.record(stream)
    torch.cuda.synchronize()
    return t0.elapsed_time(t1) / frames, sum(c.counters()["tileRecordsDropped"] for c in ctxs) - d0


def _tune_config(renderers, base: HairConfig, device, stream, tile_sizes, depth_bins, slices, processor_counts,
                 frames, warmup, deadline, part, trials):
    """Stages 1-3 for one set of renderers; leaves them on the winner's
    context and returns (its ms per frame, its HairConfig, its Context)."""
    ctxs: list[Context] = []
    best = None  # (ms, cfg, ctx)

    def run(cfg):
        ctx = Context(cfg.to_c(), device)
        ctxs.append(ctx)
        ctx.set_stream(stream)
        for r in renderers:  # frees the previous candidate's raster buffers (if their sizes change)
            r.use_config(cfg, ctx)
        ms, dropped = time_batch(renderers, ctx, stream, frames, warmup)
        trials.append(Trial(cfg.tile_size, cfg.tile_depth_bins, cfg.processor_count, ms, dropped,
                            slices=cfg.slices_per_pixel, part=part))
        return ms, dropped, ctx

    # 1. tile size x depth bins; the base constants are kept unless a candidate is clearly faster
    at_base = None
    for ts, b in itertools.product(tile_sizes, depth_bins):
        if ctxs and time.perf_counter() > deadline:
            break
        cfg = candidate_config(base, ts, b)
        ms, dropped, ctx = run(cfg)
        if dropped == 0 and (best is None or ms < best[0]):
            best = (ms, cfg, ctx)
        if dropped == 0 and (ts, b) == (base.tile_size, base.tile_depth_bins):
            at_base = (ms, cfg, ctx)
    if best is None:
        raise RuntimeError("no candidate rendered without dropping records")
    if at_base is not None and best[0] > at_base[0] * (1.0 - MIN_GAIN):
        best = at_base
    # 2. slices, 3. persistent CTA count, each kept only when clearly faster
    for field, values in (("slices_per_pixel", slices), ("processor_count", processor_counts)):
        cur = best
        for v in values:
            if getattr(cur[1], field) == v or time.perf_counter() > deadline:
                continue
            cfg = dataclasses.replace(cur[1], **{field: v})
            ms, dropped, ctx = run(cfg)
            if dropped == 0 and ms < best[0] * (1.0 - MIN_GAIN):
                best = (ms, cfg, ctx)
    _, cfg, ctx = best
    for r in renderers:
        r.use_config(cfg, ctx)
    torch.cuda.synchronize()
    for c in ctxs:
        if c is not ctx:
            c.close()
    return best[0], cfg, ctx


def tune(renderers: list[Renderer], base: HairConfig, device: int, stream=None, tile_sizes=TILE_SIZES,
         depth_bins=DEPTH_BINS, frames: int = 3, warmup: int = 2, budget_s: float = 120.0, groups=GROUPS,
         slices=SLICES, processor_counts=PROCESSOR_COUNTS, split: bool = True) -> Tuned:
    """Runs the stages on the batch; leaves the renderers on the chosen
    contexts.  Returns a Tuned (its `batch` renders the chosen frame)."""
    stream = stream or torch.cuda.current_stream()
    trials: list[Trial] = []
    t_start = time.perf_counter()
    deadline = t_start + budget_s
    ms1, cfg, ctx = _tune_config(renderers, base, device, stream, tile_sizes, depth_bins, slices,
                                 processor_counts, frames, warmup, deadline, "all", trials)
    single = Tuned([("all", cfg, ctx, list(renderers))], BatchRenderer(renderers), trials)

    # 4. parts by viewport size, each with its own constants and stream
    areas = sorted({r.inst.width * r.inst.height for r in renderers})
    if split and len(areas) > 1 and time.perf_counter() < deadline:
        big = [r for r in renderers if r.inst.width * r.inst.height == areas[-1]]
        small = [r for r in renderers if r.inst.width * r.inst.height != areas[-1]]
        parts = []
        for name, rs in (("largest viewports", big), ("smaller viewports", small)):
            s = torch.cuda.Stream()
            _, c, x = _tune_config(rs, base, device, s, tile_sizes, depth_bins, slices, processor_counts, frames,
                                   warmup, deadline + budget_s / 2, name, trials)
            parts.append((name, c, x, rs))
        sb = SplitBatchRenderer([p[3] for p in parts], stream)
        ms2, dropped = time_frames(sb, [p[2] for p in parts], stream, frames, warmup)
        trials.append(Trial(0, 0, 0, ms2, dropped, part="split by viewport"))
        if dropped == 0 and ms2 < ms1 * (1.0 - MIN_GAIN):
            ctx.close()
            return Tuned(parts, sb, trials)
        for _, _, x, rs in parts:  # back to the single choice
            for r in rs:
                r.use_config(cfg, ctx)
        torch.cuda.synchronize()
        for _, _, x, _ in parts:
            x.close()

    # 5. instance groups side by side, then the pipelined frame
    best_g = (ms1, 1)
    for g in groups:
        if g == 1 or g > len(renderers):
            continue
        ctx.set_batch_groups(g)
        ms, dropped = time_batch(renderers, ctx, stream, frames, warmup)
        trials.append(Trial(cfg.tile_size, cfg.tile_depth_bins, cfg.processor_count, ms, dropped, g,
                            slices=cfg.slices_per_pixel))
        if dropped == 0 and ms < best_g[0] * (1.0 - MIN_GAIN):
            best_g = (ms, g)
    ctx.set_batch_groups(best_g[1])
    single.groups = best_g[1]
    ctx.set_batch_pipeline(True)
    ms, dropped = time_batch(renderers, ctx, stream, frames, warmup)
    trials.append(Trial(cfg.tile_size, cfg.tile_depth_bins, cfg.processor_count, ms, dropped, 0,
                        slices=cfg.slices_per_pixel))
    # it trades a frame's latency for throughput: kept only for a large gain
    if dropped == 0 and ms < best_g[0] * (1.0 - MIN_GAIN_PIPELINE):
        single.pipelined = True
    else:
        ctx.set_batch_pipeline(False)
    return single
