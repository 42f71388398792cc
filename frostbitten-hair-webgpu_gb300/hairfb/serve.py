"""Serving many hair sessions on one GPU: admission under a device-memory
budget, and frame requests batched as they arrive (continuous batching).

The reference renders one hair object per frame for one viewer: its frame
is ``Renderer.cmdRender`` (src/renderer.ts:171-210), submitted once per
frame (src/index.deno.ts:95-109).  A server runs many such viewers
("sessions") at once.  Each session is one hair instance with its own
camera, viewport and simulation state, resident on the device for its whole
life; its client asks for frames one at a time.  The server

- admits a waiting session (first come, first served) as soon as its device
  memory fits in what the budget leaves.  Admission (allocation, upload and
  the first-frame set-up, ``beforeFirstFrame``) runs on a host thread and a
  stream of its own, beside the frames already on the GPU, and allocates
  from torch's caching allocator, so neither the GPU nor the loop that
  launches frames waits for it;
- serves frame requests: each admitted session's client sends requests as a
  Poisson process from the moment its state is on the device.  Work runs
  in "ticks", one ``hfb_frame_batch`` call each, on a few "lanes" (contexts
  with their own streams).  When a lane is free it takes the oldest pending
  requests, one frame per session, until an estimate of the tick's GPU time
  reaches a budget, and launches them; requests that arrive while ticks
  run go into the next free lane's tick, and the lanes' ticks overlap on
  the device;
- watches completions through CUDA events (no device-wide synchronisation):
  a request's latency runs from its arrival to the moment the host sees its
  tick's event complete;
- retires a session after its last frame, once the GPU is done with it, and
  returns its memory to the budget.

A session is in at most one tick at a time, so its frames stay in order
whichever lane runs them, and a session's frames are exactly those it
renders alone (the batched kernels run each instance's own arithmetic);
``tests/test_serve.py`` checks that against hfb_frame.
"""
from __future__ import annotations

import collections
import ctypes
import dataclasses
import gc
import heapq
import math
import queue
import sys
import threading
import time

import numpy as np
import torch

from . import synthetic
from .config import HairConfig
from .lib import Context, HfbInstance
from .renderer import Renderer


@dataclasses.dataclass
class SessionSpec:
    """One viewer's hair instance and how many frames it asks for."""
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
        self.orders: dict = {}

    def grid_order(self, inst: synthetic.Instance):
        """The asset's strand order for the grid splat (computed once per asset)."""
        a = inst.hair.asset
        key = id(a)
        if key not in self.orders:
            from .lib import strand_grid_order
            self.orders[key] = (a, strand_grid_order(a.positions, a.strands, a.points_per_strand).view(np.int32))
        return self.orders[key][1]

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
        return dataclasses.replace(base, cfg=self.cfg, scene=scene, scene_depth=self.depths[key])

    def prepare(self, specs: list[SessionSpec]) -> None:
        for sp in specs:
            self(sp)


def pool_records(spec: SessionSpec) -> int:
    """Segment pool of a session, in records: room for every segment in four
    tiles, plus one record per tile (no record of these workloads drops;
    the server reports drops)."""
    tiles = -(-spec.width // 16) * -(-spec.height // 16)
    return 4 * spec.strands * (spec.points - 1) + tiles + 1


def request_times(spec: SessionSpec, rate_hz: float, seed: int) -> np.ndarray:
    """Offsets (s) of a session's frame requests from the moment it is ready:
    a Poisson process of rate `rate_hz` (its share of the total request rate)."""
    rng = np.random.Generator(np.random.PCG64((seed, 7919, spec.sid)))
    return np.cumsum(rng.exponential(1.0 / rate_hz, spec.frames))


@dataclasses.dataclass
class Session:
    spec: SessionSpec
    inst: synthetic.Instance | None = None
    renderer: Renderer | None = None
    bytes: int = 0
    admitted_s: float = -1.0   # admission call made
    ready_s: float = -1.0      # state on the device: requests start
    ready_ev: torch.cuda.Event | None = None
    offsets: np.ndarray | None = None
    issued: int = 0            # requests that have arrived
    done: int = 0              # frames completed
    pending: collections.deque = dataclasses.field(default_factory=collections.deque)
    busy: bool = False         # in a tick on the GPU
    finished_s: float = -1.0
    work: tuple = (0.0, 0.0)   # a frame's (points, pixels): the cost model's units


@dataclasses.dataclass
class Tick:
    lane: int
    sessions: list
    arrivals: list
    start: torch.cuda.Event
    end: torch.cuda.Event
    launched_s: float
    units: tuple


@dataclasses.dataclass
class ServeStats:
    frames: int
    wall_s: float
    ticks: int
    latency_ms: list[float]        # per frame request: arrival -> completion seen by the host
    admit_wait_ms: list[float]     # per session: arrival -> admission
    peak_sessions: int
    peak_bytes: int
    budget_bytes: int
    dropped: int
    lanes: int
    offered_hz: float
    frames_per_tick: float
    tick_gpu_ms: list[float]
    first_request_s: float = 0.0
    last_done_s: float = 0.0
    done_s: list = dataclasses.field(default_factory=list)  # per frame: when the host saw it complete
    arrival_s: list = dataclasses.field(default_factory=list)  # per frame: when its request arrived
    all_active_s: float = 0.0      # the last session started asking for frames
    first_finished_s: float = 0.0  # the first session had all its frames

    @property
    def frames_per_s(self) -> float:
        """Frames over the time from the first request to the last frame."""
        span = self.last_done_s - self.first_request_s
        return self.frames / span if span > 0 else 0.0

    @property
    def steady_frames_per_s(self) -> float:
        """Frames completed per second while every session was asking for
        frames (from the last session's first request to the first
        session's last frame): the rate at the full offered load."""
        t0, t1 = self.all_active_s, self.first_finished_s
        if not t1 > t0:
            return 0.0
        return sum(1 for t in self.done_s if t0 <= t <= t1) / (t1 - t0)

    def steady_pct(self, q: float) -> float:
        """Latency percentile (ms) of the requests that arrived and completed
        while every session was asking for frames (the steady window of
        steady_frames_per_s): the start, when sessions are still being
        admitted, and the end, when they retire, are left out."""
        t0, t1 = self.all_active_s, self.first_finished_s
        v = sorted(l for l, a, d in zip(self.latency_ms, self.arrival_s, self.done_s) if a >= t0 and d <= t1)
        return v[min(len(v) - 1, int(round(q * (len(v) - 1))))] if v else 0.0

    def pct(self, q: float, which: str = "latency_ms") -> float:
        v = sorted(getattr(self, which))
        return v[min(len(v) - 1, int(round(q * (len(v) - 1))))] if v else 0.0


class CostModel:
    """GPU milliseconds of a tick as a + b * points + c * pixels, refitted by
    least squares over the recent ticks (their event-timed durations); used
    to keep each tick inside the budget.  Starts from a prior that
    overestimates, so the first ticks are small."""

    def __init__(self, a=1.0, b=1.2e-6, c=3.0e-7, window: int = 400):
        self.coef = np.array([a, b, c])
        self.rows: collections.deque = collections.deque(maxlen=window)

    def ms(self, points: float, pixels: float, n: int = 1) -> float:
        return float(self.coef[0] * (1 if n else 0) + self.coef[1] * points + self.coef[2] * pixels)

    def add(self, points: float, pixels: float, ms: float) -> None:
        self.rows.append((1.0, points, pixels, ms))
        if len(self.rows) >= 16 and len(self.rows) % 8 == 0:
            A = np.array(self.rows)
            x, *_ = np.linalg.lstsq(A[:, :3], A[:, 3], rcond=None)
            if np.all(np.isfinite(x)) and x[1] > 0 and x[2] >= 0:
                self.coef = np.array([max(x[0], 0.0), x[1], x[2]])


class Server:
    """Sessions served on `lanes` contexts of one pass config."""

    def __init__(self, cfg: HairConfig, device: int = 0, budget_bytes: int = 150 << 30, lanes: int = 3,
                 tick_budget_ms: float = 8.0, make_instance=None, hair_depth: bool = True, groups: int = 1):
        """hair_depth: each session's frame draws the hair depth for its
        shading (the reference's frame); False shades with the scene depth.
        tick_budget_ms: the estimated GPU time a tick may hold (at least one
        frame).  groups: instance groups of each lane's batched frame."""
        self.cfg = cfg
        self.hair_depth = hair_depth
        self.device = device
        torch.cuda.set_device(device)
        self.streams = [torch.cuda.Stream(device) for _ in range(lanes)]
        self.ctxs = []
        for st in self.streams:
            c = Context(cfg.to_c(), device)
            c.set_stream(st)
            c.set_batch_groups(groups)
            self.ctxs.append(c)
        # admission: its own stream and context (uploads, first-frame set-up)
        self.admit_stream = torch.cuda.Stream(device)
        self.admit_ctx = Context(cfg.to_c(), device)
        self.admit_ctx.set_stream(self.admit_stream)
        self.ctx = self.admit_ctx
        self.budget = int(budget_bytes)
        self.tick_budget_ms = float(tick_budget_ms)
        self.used = 0
        self.cost = CostModel()
        self._make = make_instance or self._synthetic
        self._arrs: dict = {}

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
        hair = n * 16 * 4 + n * 4 + spec.strands * 4 + spec.strands * c.shading_points * 16
        grids = 2 * 16 * c.grid_dims ** 3
        sdf = 4 * 32 ** 3
        depth = 4 * spec.width * spec.height * (2 if self.hair_depth else 1)
        tx, ty = -(-spec.width // c.tile_size), -(-spec.height // c.tile_size)
        T = tx * ty
        md = pool_records(spec)
        scratch = self.ctx.lib.hfb_raster_scratch_bytes_for(ctypes.byref(self.ctx.cfg), spec.width, spec.height, md)
        parts = [T * c.tile_depth_bins * 16, 4 + md * 8, T * 4, c.sort_buckets * 8, (4 + T) * 4,
                 16 + spec.width * spec.height * 16, scratch]
        raster = sum((p + 255) // 256 * 256 for p in parts)
        return hair + grids + sdf + depth + raster

    # ---- sessions ----
    def admit(self, s: Session) -> None:
        """Allocates and uploads the session's state and runs its first-frame
        set-up, all on the admission stream (the admission thread calls it);
        s.ready_ev completes when the state is on the device."""
        s.inst = self._make(s.spec)
        order = self._make.grid_order(s.inst) if hasattr(self._make, "grid_order") else None
        with torch.cuda.stream(self.admit_stream):
            s.renderer = Renderer(s.inst, self.device, ctx=self.admit_ctx, max_drawn=pool_records(s.spec),
                                  hair_depth=self.hair_depth, pooled=True, grid_order=order)
            s.renderer.before_first_frame()
            s.ready_ev = torch.cuda.Event()
            s.ready_ev.record(self.admit_stream)

    def _admission_worker(self, todo: queue.Queue, loaded: queue.Queue) -> None:
        torch.cuda.set_device(self.device)
        while True:
            s = todo.get()
            if s is None:
                return
            try:
                self.admit(s)
                loaded.put(s)
            except BaseException as e:  # handed to the serving loop, which raises it
                loaded.put(e)
                return

    def retire(self, s: Session) -> None:
        """After the GPU finished the session's last frame: its memory goes
        back to torch's cache and to the budget."""
        s.renderer.rb.close()
        s.renderer = None
        s.inst = None
        self.used -= s.bytes

    # ---- ticks ----
    def _launch(self, lane: int, group: list, now: float) -> Tick:
        ctx, stream = self.ctxs[lane], self.streams[lane]
        n = len(group)
        arr = self._arrs.get((lane, n))
        if arr is None:
            arr = self._arrs[(lane, n)] = (HfbInstance * n)()
        for k, s in enumerate(group):
            arr[k] = s.renderer.instance()
        start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        start.record(stream)
        ctx.call("hfb_frame_batch", arr, n)
        end.record(stream)
        arrivals = []
        for s, inst in zip(group, arr):
            s.renderer.after_native_frame(inst)
            s.busy = True
            arrivals.append(s.pending.popleft())
        pts = sum(s.work[0] for s in group)
        pix = sum(s.work[1] for s in group)
        return Tick(lane, group, arrivals, start, end, now, (pts, pix))

    def _form(self, ready: list) -> list:
        """The oldest pending requests, one per session, within the budget."""
        cands = sorted((s for s in ready if s.pending and not s.busy), key=lambda s: s.pending[0])
        group, pts, pix = [], 0.0, 0.0
        for s in cands:
            p2, x2 = pts + s.work[0], pix + s.work[1]
            if group and (self.cost.ms(p2, x2) > self.tick_budget_ms or len(group) >= 1024):
                break
            group.append(s)
            pts, pix = p2, x2
        return group

    def run(self, specs: list[SessionSpec], rate_hz: float = 2000.0, seed: int = 0, frame_done=None,
            per_session_rate_hz: float | None = None) -> ServeStats:
        """Serves every session to its last frame.  Frame requests total
        `rate_hz` when every session is active (each session's share is
        rate_hz / len(specs), or per_session_rate_hz).  `frame_done(session)`
        is called once the host sees a session's frame complete (tests read
        state there)."""
        per = per_session_rate_hz or rate_hz / max(1, len(specs))
        todo: queue.Queue = queue.Queue()
        loaded: queue.Queue = queue.Queue()
        worker = threading.Thread(target=self._admission_worker, args=(todo, loaded), daemon=True)
        worker.start()
        switch = sys.getswitchinterval()
        sys.setswitchinterval(1e-4)  # the loop gets the interpreter back quickly from the admission thread
        # no garbage-collector pauses inside the request loop (its objects are freed by
        # reference counting; one collection runs after it)
        collecting = gc.isenabled()
        gc.disable()
        try:
            return self._serve(specs, per, seed, frame_done, todo, loaded)
        finally:
            todo.put(None)
            worker.join()
            sys.setswitchinterval(switch)
            if collecting:
                gc.enable()
                gc.collect()

    def _serve(self, specs, per, seed, frame_done, todo, loaded) -> ServeStats:
        pending = collections.deque(sorted(specs, key=lambda sp: sp.arrival_s))
        waiting: collections.deque[Session] = collections.deque()
        loading: list[Session] = []       # admitted, state still uploading
        active: list[Session] = []        # ready: issuing requests
        heap: list = []                   # (next request time, sid, session)
        ticks: list[Tick | None] = [None] * len(self.ctxs)
        lat, waits, tick_ms, done_t, arr_t = [], [], [], [], []
        all_active, first_finished = 0.0, math.inf
        n_ticks = frames = peak_sessions = peak_bytes = admitting = 0
        first_req, last_done = math.inf, 0.0
        d0 = sum(c.counters()["tileRecordsDropped"] for c in self.ctxs)
        remaining = len(specs)
        t0 = time.perf_counter()
        while remaining:
            now = time.perf_counter() - t0
            progressed = False
            # session arrivals
            while pending and pending[0].arrival_s <= now:
                sp = pending.popleft()
                s = Session(sp)
                s.bytes = self.session_bytes(sp)
                if s.bytes > self.budget:
                    raise RuntimeError(f"session {sp.sid} needs {s.bytes} B, more than the whole budget")
                waiting.append(s)
            # completions
            for li, tk in enumerate(ticks):
                if tk is not None and tk.end.query():
                    now = time.perf_counter() - t0
                    ticks[li] = None
                    progressed = True
                    n_ticks += 1
                    ms = tk.start.elapsed_time(tk.end)
                    tick_ms.append(ms)
                    self.cost.add(tk.units[0], tk.units[1], ms)
                    for s, a in zip(tk.sessions, tk.arrivals):
                        lat.append(1000.0 * (now - a))
                        done_t.append(now)
                        arr_t.append(a)
                        last_done = max(last_done, now)
                        s.busy = False
                        s.done += 1
                        frames += 1
                        if frame_done:
                            frame_done(s)
                        if s.done >= s.spec.frames:
                            s.finished_s = now
                            first_finished = min(first_finished, now)
                            self.retire(s)
                            active.remove(s)
                            remaining -= 1
            # sessions whose state reached the device start asking for frames
            while not loaded.empty():
                s = loaded.get()
                if isinstance(s, BaseException):
                    raise s
                loading.append(s)
            for s in list(loading):
                if s.ready_ev.query():
                    s.ready_s = time.perf_counter() - t0
                    s.offsets = s.ready_s + request_times(s.spec, per, seed)
                    all_active = max(all_active, float(s.offsets[0]))
                    heapq.heappush(heap, (float(s.offsets[0]), s.spec.sid, s))
                    loading.remove(s)
                    active.append(s)
                    admitting -= 1
                    progressed = True
            # frame requests
            now = time.perf_counter() - t0
            while heap and heap[0][0] <= now:
                t_req, _, s = heapq.heappop(heap)
                s.pending.append(t_req)
                first_req = min(first_req, t_req)
                s.issued += 1
                if s.issued < s.spec.frames:
                    heapq.heappush(heap, (float(s.offsets[s.issued]), s.spec.sid, s))
            # free lanes take the oldest requests
            for li in range(len(ticks)):
                if ticks[li] is None:
                    group = self._form(active)
                    if group:
                        ticks[li] = self._launch(li, group, now)
                        progressed = True
            # admission, first come first served while the budget allows: the
            # admission thread builds the sessions in order
            while waiting and self.used + waiting[0].bytes <= self.budget:
                s = waiting.popleft()
                s.admitted_s = now
                s.work = (s.spec.strands * s.spec.points, s.spec.width * s.spec.height)
                self.used += s.bytes
                waits.append(1000.0 * (now - s.spec.arrival_s))
                todo.put(s)
                admitting += 1
                progressed = True
                peak_bytes = max(peak_bytes, self.used)
                peak_sessions = max(peak_sessions, len(active) + admitting)
            if not progressed:
                time.sleep(5e-5)
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
        dropped = sum(c.counters()["tileRecordsDropped"] for c in self.ctxs) - d0
        st = ServeStats(frames, wall, n_ticks, lat, waits, peak_sessions, peak_bytes, self.budget, dropped,
                        len(self.ctxs), per * len(specs), frames / max(1, n_ticks), tick_ms)
        st.first_request_s = first_req if math.isfinite(first_req) else 0.0
        st.last_done_s = last_done
        st.done_s = done_t
        st.arrival_s = arr_t
        st.all_active_s = all_active
        st.first_finished_s = first_finished if math.isfinite(first_finished) else 0.0
        return st

    def close(self) -> None:
        for c in self.ctxs:
            c.close()
        self.admit_ctx.close()
