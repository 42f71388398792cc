"""Serving many hair sessions on one GPU: admission under a device-memory
budget and continuous batching of their frames through hfb_frame_batch.

The reference renders one hair object per frame for one viewer.  A server
runs many such sessions at once: each session is one hair instance with its
own camera, viewport and simulation state, rendering a fixed number of
frames.  Sessions arrive over time; the server

- admits a waiting session (first come, first served) as soon as its device
  memory fits in what the budget leaves, and allocates its buffers then;
- runs ticks: every tick renders the next frame of every admitted session
  in one hfb_frame_batch call (sessions join and leave between ticks:
  continuous batching), and waits for it;
- retires a session after its last frame and frees its memory.

A session's frames are exactly those it would render alone (the batched
kernels run each instance's own arithmetic); `tests/test_serve.py` checks
that against hfb_frame.
"""
from __future__ import annotations

import collections
import ctypes
import dataclasses
import math
import time

import numpy as np
import torch

from . import synthetic
from .config import HairConfig
from .lib import Context
from .renderer import BatchRenderer, Renderer


@dataclasses.dataclass
class SessionSpec:
    """One viewer's hair instance and how many frames it renders."""
    sid: int
    arrival_s: float
    strands: int
    points: int
    width: int
    height: int
    frames: int
    seed: int


def poisson_sessions(seed: int = 0, count: int = 256, rate_hz: float = 2000.0, frames: int = 600,
                     strands=(500, 50000), points: int = 32, side=(256, 2048)) -> list[SessionSpec]:
    """Sessions arriving as a Poisson process of rate `rate_hz`: strand counts
    log-uniform in `strands`, square viewports whose pixel count is
    log-uniform in [side[0]^2, side[1]^2] (sides rounded to 16 px)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    t = 0.0
    out = []
    for sid in range(count):
        t += float(rng.exponential(1.0 / rate_hz))
        s = int(round(math.exp(rng.uniform(math.log(strands[0]), math.log(strands[1])))))
        px = math.exp(rng.uniform(math.log(side[0] ** 2), math.log(side[1] ** 2)))
        w = max(16, int(round(math.sqrt(px) / 16.0)) * 16)
        out.append(SessionSpec(sid, t, s, points, w, w, frames, int(rng.integers(1 << 31))))
    return out


def snap(specs: list[SessionSpec], strand_levels: int = 8, side_levels: int = 8,
         strands=(500, 50000), side=(256, 2048)) -> list[SessionSpec]:
    """The specs with strand counts and viewport sides rounded (in log space)
    to a few levels, so that a handful of host-generated assets and depth
    images serve every session (SessionFactory)."""
    sl = np.unique(np.round(np.exp(np.linspace(math.log(strands[0]), math.log(strands[1]), strand_levels))))
    wl = np.unique(np.round(np.exp(np.linspace(math.log(side[0]), math.log(side[1]), side_levels)) / 16.0) * 16)

    def near(levels, v):
        return int(levels[int(np.argmin(np.abs(np.log(levels) - math.log(v))))])
    return [dataclasses.replace(sp, strands=near(sl, sp.strands), width=near(wl, sp.width),
                                height=near(wl, sp.height)) for sp in specs]


class SessionFactory:
    """Session instances built from shared host assets: one hair asset per
    strand count and one scene depth image per (asset, viewport), generated
    once (`prepare`) and reused by every session that asks for them.  Each
    session still gets its own device buffers and simulation state."""

    def __init__(self, cfg: HairConfig, seed: int = 0):
        self.cfg = cfg
        self.seed = seed
        self.assets: dict = {}
        self.depths: dict = {}

    def _asset(self, strands: int, points: int) -> synthetic.Instance:
        key = (strands, points)
        if key not in self.assets:
            rng = np.random.Generator(np.random.PCG64((self.seed, strands, points)))
            c = self.cfg
            self.assets[key] = synthetic.make_instance(
                rng, strands=strands, points=points, width=16, height=16, tile_size=c.tile_size,
                depth_bins=c.tile_depth_bins, slices=c.slices_per_pixel, shading_points=c.shading_points,
                grid_dims=c.grid_dims, avg_segments_per_tile=c.avg_segments_per_tile)
        return self.assets[key]

    def __call__(self, spec: SessionSpec) -> synthetic.Instance:
        base = self._asset(spec.strands, spec.points)
        key = (spec.strands, spec.points, spec.width, spec.height)
        if key not in self.depths:
            self.depths[key] = synthetic.sphere_depth(spec.width, spec.height, base.scene.camera, base.head_center,
                                                      base.head_radius * 0.98)
        scene = dataclasses.replace(base.scene, width=spec.width, height=spec.height)
        return dataclasses.replace(base, scene=scene, scene_depth=self.depths[key])

    def prepare(self, specs: list[SessionSpec]) -> None:
        for sp in specs:
            self(sp)


def pool_records(spec: SessionSpec) -> int:
    """Segment pool of a session, in records: room for every segment in four
    tiles, plus one record per tile (no record of these workloads drops;
    the server reports drops)."""
    tiles = -(-spec.width // 16) * -(-spec.height // 16)
    return 4 * spec.strands * (spec.points - 1) + tiles + 1


@dataclasses.dataclass
class Session:
    spec: SessionSpec
    inst: synthetic.Instance | None = None
    renderer: Renderer | None = None
    bytes: int = 0
    admitted_s: float = -1.0
    done: int = 0
    finished_s: float = -1.0


@dataclasses.dataclass
class ServeStats:
    frames: int
    wall_s: float
    busy_s: float
    ticks: int
    frame_ms: list[float]          # per frame: the tick that rendered it
    admit_wait_ms: list[float]     # per session: arrival -> admission
    peak_sessions: int
    peak_bytes: int
    budget_bytes: int
    dropped: int

    @property
    def frames_per_s(self) -> float:
        return self.frames / self.wall_s if self.wall_s > 0 else 0.0

    def pct(self, q: float, which: str = "frame_ms") -> float:
        v = sorted(getattr(self, which))
        return v[min(len(v) - 1, int(round(q * (len(v) - 1))))] if v else 0.0


class Server:
    """Sessions on one context (one pass config for all of them)."""

    def __init__(self, cfg: HairConfig, device: int = 0, budget_bytes: int = 150 << 30, stream=None,
                 groups: int = 1, make_instance=None, hair_depth: bool = True):
        """hair_depth: each session's frame draws the hair depth for its
        shading (the reference's frame); False shades with the scene depth."""
        self.cfg = cfg
        self.hair_depth = hair_depth
        self.device = device
        self.ctx = Context(cfg.to_c(), device)
        if stream is not None:
            self.ctx.set_stream(stream)
        self.ctx.set_batch_groups(groups)
        self.stream = stream
        self.budget = int(budget_bytes)
        self.used = 0
        self._make = make_instance or self._synthetic

    def _synthetic(self, spec: SessionSpec) -> synthetic.Instance:
        rng = np.random.Generator(np.random.PCG64(spec.seed))
        c = self.cfg
        return synthetic.make_instance(rng, strands=spec.strands, points=spec.points, width=spec.width,
                                       height=spec.height, tile_size=c.tile_size, depth_bins=c.tile_depth_bins,
                                       slices=c.slices_per_pixel, shading_points=c.shading_points,
                                       grid_dims=c.grid_dims, avg_segments_per_tile=c.avg_segments_per_tile)

    def session_bytes(self, spec: SessionSpec) -> int:
        """Device memory of an admitted session: hair buffers, grids, SDF,
        scene (and hair) depth and its raster buffers."""
        c = self.cfg
        n = spec.strands * spec.points
        hair = n * 16 * 4 + n * 4 + spec.strands * c.shading_points * 16  # 3 positions + tangents, lengths, shading
        grids = 2 * 16 * c.grid_dims ** 3
        sdf = 4 * 32 ** 3
        depth = 4 * spec.width * spec.height * (2 if self.hair_depth else 1)
        tx, ty = -(-spec.width // c.tile_size), -(-spec.height // c.tile_size)
        T = tx * ty
        md = pool_records(spec)
        raster = (T * c.tile_depth_bins * 16 + 4 + md * 8 + T * 4 + c.sort_buckets * 8 + (4 + T) * 4
                  + 16 + spec.width * spec.height * 16
                  + self.ctx.lib.hfb_raster_scratch_bytes_for(ctypes.byref(self.ctx.cfg), spec.width, spec.height, md))
        return hair + grids + sdf + depth + raster

    def admit(self, s: Session, now: float) -> None:
        s.inst = self._make(s.spec)
        s.renderer = Renderer(s.inst, self.device, ctx=self.ctx, max_drawn=pool_records(s.spec),
                              hair_depth=self.hair_depth)
        s.renderer.before_first_frame()
        s.admitted_s = now
        self.used += s.bytes

    def retire(self, s: Session) -> None:
        s.renderer.rb.close()
        s.renderer = None
        s.inst = None
        self.used -= s.bytes

    def run(self, specs: list[SessionSpec], frame_done=None) -> ServeStats:
        """Serves every session to its last frame.  `frame_done(session)` is
        called after each of a session's frames (tests read state there)."""
        pending = collections.deque(sorted(specs, key=lambda sp: sp.arrival_s))
        waiting: collections.deque[Session] = collections.deque()
        active: list[Session] = []
        frame_ms, waits = [], []
        ticks = frames = peak_sessions = peak_bytes = 0
        busy = 0.0
        d0 = self.ctx.counters()["tileRecordsDropped"]
        t0 = time.perf_counter()
        while pending or waiting or active:
            now = time.perf_counter() - t0
            while pending and pending[0].arrival_s <= now:
                sp = pending.popleft()
                s = Session(sp)
                s.bytes = self.session_bytes(sp)
                if s.bytes > self.budget:
                    raise RuntimeError(f"session {sp.sid} needs {s.bytes} B, more than the whole budget")
                waiting.append(s)
            while waiting and self.used + waiting[0].bytes <= self.budget:
                s = waiting.popleft()
                self.admit(s, now)
                waits.append(1000.0 * (now - s.spec.arrival_s))
                active.append(s)
            if not active:
                if pending:
                    time.sleep(max(0.0, min(pending[0].arrival_s - now, 0.01)))
                continue
            peak_sessions = max(peak_sessions, len(active))
            peak_bytes = max(peak_bytes, self.used)
            ta = time.perf_counter()
            for k in range(0, len(active), 1024):  # hfb_frame_batch takes up to 1024 instances
                BatchRenderer([s.renderer for s in active[k:k + 1024]]).frame()
            torch.cuda.synchronize()
            dt = time.perf_counter() - ta
            busy += dt
            ticks += 1
            frame_ms += [1000.0 * dt] * len(active)
            frames += len(active)
            still = []
            for s in active:
                s.done += 1
                if frame_done:
                    frame_done(s)
                if s.done >= s.spec.frames:
                    s.finished_s = time.perf_counter() - t0
                    self.retire(s)
                else:
                    still.append(s)
            active = still
        wall = time.perf_counter() - t0
        dropped = self.ctx.counters()["tileRecordsDropped"] - d0
        return ServeStats(frames, wall, busy, ticks, frame_ms, waits, peak_sessions, peak_bytes, self.budget,
                          dropped)

    def close(self) -> None:
        self.ctx.close()
