"""Autotuner of batched frames: picks the pass constants a batch runs with.

The candidates are tile size x depth bins, then the number of instance
groups that run side by side (``hfb_ctx_set_batch_groups``); each is timed
on the batch itself with ``hfb_frame_batch`` (CUDA events, after
warm-up frames), and the fastest candidate that drops no (segment, tile)
record wins -- a dropped record would change the image, so such a
candidate is not an equal-accuracy choice.  The segment pool is sized per
tile area (``avg_segments_per_tile`` scales with the tile's pixel count),
as the reference sizes it per tile.  Every candidate renders exactly what
the reference renders with the same constants; the tuner only chooses
among them.
"""
from __future__ import annotations

import dataclasses
import itertools
import time

import torch

from .config import HairConfig
from .lib import Context
from .renderer import BatchRenderer, Renderer

TILE_SIZES = (8, 16, 32)
DEPTH_BINS = (4, 8, 16, 32)
GROUPS = (1, 2, 3, 4)
MIN_GAIN = 0.03  # a candidate must beat the base (or one group) by this fraction
MIN_GAIN_PIPELINE = 0.10


@dataclasses.dataclass
class Trial:
    tile_size: int
    depth_bins: int
    processor_count: int
    ms: float
    dropped: int
    groups: int = 1  # 0: the pipelined frame

    def as_dict(self):
        return dataclasses.asdict(self)


def candidate_config(base: HairConfig, tile_size: int, depth_bins: int, processor_count: int = 0) -> HairConfig:
    scale = (tile_size / base.tile_size) ** 2
    return dataclasses.replace(base, tile_size=tile_size, tile_depth_bins=depth_bins,
                               processor_count=processor_count,
                               avg_segments_per_tile=max(16, int(round(base.avg_segments_per_tile * scale))))


def time_batch(renderers: list[Renderer], ctx: Context, stream, frames: int, warmup: int) -> tuple[float, int]:
    """Mean ms per batched frame, and the records dropped meanwhile."""
    batch = BatchRenderer(renderers)
    for _ in range(warmup):
        batch.frame()
    torch.cuda.synchronize()
    d0 = ctx.counters()["tileRecordsDropped"]
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    t0.record(stream)
    for _ in range(frames):
        batch.frame()
    t1.record(stream)
    torch.cuda.synchronize()
    return t0.elapsed_time(t1) / frames, ctx.counters()["tileRecordsDropped"] - d0


def tune(renderers: list[Renderer], base: HairConfig, device: int, stream=None, tile_sizes=TILE_SIZES,
         depth_bins=DEPTH_BINS, frames: int = 3, warmup: int = 2, budget_s: float = 120.0, groups=GROUPS):
    """Times every candidate on the batch, then the instance groups on the
    winner; leaves the renderers on the winner's context, set to the best
    group count.  Returns (best HairConfig, its Context, trials)."""
    trials: list[Trial] = []
    ctxs: list[Context] = []
    best = at_base = None
    t_start = time.perf_counter()
    for ts, b in itertools.product(tile_sizes, depth_bins):
        if ctxs and time.perf_counter() - t_start > budget_s:
            break
        cfg = candidate_config(base, ts, b)
        ctx = Context(cfg.to_c(), device)
        ctxs.append(ctx)
        if stream is not None:
            ctx.set_stream(stream)
        for r in renderers:  # frees the previous candidate's raster buffers
            r.use_config(cfg, ctx)
        ms, dropped = time_batch(renderers, ctx, stream or torch.cuda.current_stream(), frames, warmup)
        trials.append(Trial(ts, b, cfg.processor_count, ms, dropped))
        if dropped == 0 and (best is None or ms < best[0]):
            best = (ms, cfg, ctx)
        if dropped == 0 and (ts, b) == (base.tile_size, base.tile_depth_bins):
            at_base = (ms, cfg, ctx)
    if best is None:
        raise RuntimeError("no candidate rendered without dropping records")
    # a candidate replaces the base constants only when it is clearly faster
    # (frame-to-frame timing noise is ~1-2 %)
    if at_base is not None and best[0] > at_base[0] * (1.0 - MIN_GAIN):
        best = at_base
    _, cfg, ctx = best
    for r in renderers:
        r.use_config(cfg, ctx)
    torch.cuda.synchronize()
    for c in ctxs:
        if c is not ctx:
            c.close()
    # then the number of instance groups that run side by side
    best_g = (best[0], 1)
    for g in groups:
        if g == 1 or g > len(renderers):
            continue
        ctx.set_batch_groups(g)
        ms, dropped = time_batch(renderers, ctx, stream or torch.cuda.current_stream(), frames, warmup)
        trials.append(Trial(cfg.tile_size, cfg.tile_depth_bins, cfg.processor_count, ms, dropped, g))
        if dropped == 0 and ms < best_g[0] * (1.0 - MIN_GAIN):
            best_g = (ms, g)
    ctx.set_batch_groups(best_g[1])
    # then the pipelined frame (the simulation beside the previous raster passes)
    ctx.set_batch_pipeline(True)
    ms, dropped = time_batch(renderers, ctx, stream or torch.cuda.current_stream(), frames, warmup)
    trials.append(Trial(cfg.tile_size, cfg.tile_depth_bins, cfg.processor_count, ms, dropped, 0))
    # it trades a frame's latency for throughput: kept only for a large gain
    if not (dropped == 0 and ms < best_g[0] * (1.0 - MIN_GAIN_PIPELINE)):
        ctx.set_batch_pipeline(False)
    return cfg, ctx, trials
