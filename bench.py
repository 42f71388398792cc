"""Benchmark of the hair hot path (one JSON line on rank 0).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--workload NAME] [--impl ours|reference]

A step is one frame of the hot path for the workload: GridPreSim ->
SimIntegration -> GridPostSim -> clear -> Tiles -> TileSort -> Fine ->
Shading (src/renderer.ts:171-295 order).  ``value`` is device-timed
frames/s with every input resident in HBM; the L2 is flushed (a 256 MiB
write) between timed frames, outside the timed events.  ``e2e`` is the same
metric through the public API with the per-frame inputs (both uniform blocks
and the scene depth buffer) copied from pinned host memory and the frame's
image (the rasterizer result) read back every step.

Under torchrun each rank renders its own instance (replicas, weak scaling):
value = frames of all ranks / max over ranks of the timed region.

``--impl reference`` times the reference's algorithm on the host cores: the
reference is TypeScript + WGSL that needs a WebGPU adapter (none exists on
these machines), so its path runs as the C restatement of its WGSL passes,
built with OpenMP, on all host threads -- on the same workload and metric.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "frostbitten-hair-webgpu_gb300")
for _p in (ROOT, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import numpy as np  # noqa: E402

WORKLOADS = {
    # 64 instances of uneven sizes in one batched frame (the headline)
    "batched64": "64 instances, strands U[1k, 20k], points in {16, 24, 32}, resolutions in {256^2, 512^2, "
                 "1024^2}, own camera and own 32^3 sphere SDF each, 64^3 grids, 4 slices, 8 shading points, "
                 "7 iterations; tile size and depth bins autotuned over {8, 16, 32} x {4, 8, 16, 32}",
    # serving: Poisson arrivals, continuous batching under a memory budget
    "served256": "256 sessions arriving as a Poisson process of 2,000/s, strands log-uniform [500, 50k] "
                 "(8 levels), 32 points, square viewports of log-uniform area [256^2, 2048^2] (8 levels), "
                 "600 frames each, 150 GB device-memory budget, 16 px tiles, 8 depth bins, 4 slices, "
                 "8 shading points, 64^3 grids, 32^3 SDF",
    # one full frame: 10k strands at 1080p
    "plain_full": "10,000 x 32 curly strands, 1920x1080, 16 px tiles, 16 depth bins, 4 slices, "
                  "16 shading points, 4 iterations, 64^3 SDF, 64^3 grids, sinusoidal wind",
    # the small case the reference also runs on a CPU adapter
    "plain_small": "2,000 x 16 strands, 640x480, 16 px tiles, 8 depth bins, 4 slices, 8 shading points",
    # the 4K stress frame: 200k strands
    "stress": "200,000 x 32 strands (60% ponytail), 3840x2160, 32 depth bins, 8 slices, 32 shading points",
    # a hair asset in the reference's formats (--tfx, --sdf) with the reference's default constants
    "asset": "a TFX hair asset (+ binary SDF) at 1920x1080 with the reference's default CONFIG: 8 px tiles, "
             "32 depth bins, 8 slices, 64 shading points, 64^3 grids, 7 iterations",
}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--workload", default="batched64", choices=sorted(WORKLOADS))
    ap.add_argument("--tune-budget", type=float, default=90.0, help="seconds for the autotuner sweep")
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-seconds", type=float, default=15.0, help="bounded CPU-baseline sample")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--serve-frames", type=int, default=60,
                    help="frames per session of the serving run in the batched64 line (0 = none)")
    ap.add_argument("--capture-frames", type=int, default=0,
                    help="profiler runs: set up the workload, render this many frames (batched64: batched "
                         "frames at --tile-size/--depth-bins, no tuning), print 'ok' and exit; no timing")
    ap.add_argument("--tfx", help="hair asset (TFX file) of the asset workload")
    ap.add_argument("--sdf", help="binary SDF of the asset workload's head (optional)")
    ap.add_argument("--tile-size", type=int, default=16)
    ap.add_argument("--depth-bins", type=int, default=8)
    return ap.parse_args()


def capture(args):
    """A fixed number of frames for an ncu capture: the workload's renderers
    (hair depth on), the first-frame setup, then `--capture-frames` frames."""
    import dataclasses
    import torch
    from hairfb import renderer as R
    from hairfb.lib import Context
    if args.workload == "batched64":
        insts = batched_instances(seed=0)
        cfg = dataclasses.replace(insts[0].cfg, tile_size=args.tile_size, tile_depth_bins=args.depth_bins)
        insts = [dataclasses.replace(i, cfg=cfg) for i in insts]
        ctx = Context(cfg.to_c(), 0)
        rs = [R.Renderer(i, 0, ctx=ctx, hair_depth=True) for i in insts]
        for r in rs:
            r.before_first_frame()
        b = R.BatchRenderer(rs)
        for _ in range(args.capture_frames):
            b.frame()
    else:
        inst = make_instance(args.workload, seed=0)
        r = R.Renderer(inst, 0, hair_depth=True)
        r.before_first_frame()
        for _ in range(args.capture_frames):
            r.frame_native()
        ctx = r.ctx
    ctx.sync()
    print(f"ok: {args.capture_frames} frames of {args.workload}, "
          f"{torch.cuda.max_memory_allocated() / 1e9:.2f} GB allocated by torch", flush=True)


ASSET_FILES = {}  # --tfx / --sdf of the "asset" workload


def data_label(wl):
    if wl == "asset":
        return f"hair asset {os.path.basename(ASSET_FILES.get('tfx', ''))} (+ SDF " \
               f"{os.path.basename(ASSET_FILES.get('sdf') or '') or 'none'}), the user's files"
    return "synthetic (seeded; no public dataset exists for this path)"


def make_instance(name, seed):
    from hairfb import synthetic
    if name == "asset":
        if "tfx" not in ASSET_FILES:
            raise SystemExit("the asset workload needs --tfx FILE (and optionally --sdf FILE)")
        with open(ASSET_FILES["tfx"], "rb") as f:
            tfx = f.read()
        sdf = None
        if ASSET_FILES.get("sdf"):
            with open(ASSET_FILES["sdf"], "rb") as f:
                sdf = f.read()
        return synthetic.asset_instance(tfx, sdf)
    return getattr(synthetic, name)(seed=seed)


# ----------------------------------------------------------------------------
# algorithmic bytes per pass (the compulsory traffic of each kernel)
# ----------------------------------------------------------------------------

def algorithmic_bytes(inst, K):
    """Compulsory DRAM bytes of one launch of each pass (inputs read once,
    outputs written once).  K = stored (segment, tile-bin) records."""
    cfg = inst.cfg
    S, P = inst.hair.asset.strands, inst.hair.asset.points_per_strand
    Npt = S * P
    SP = cfg.shading_points
    W, H = inst.width, inst.height
    tx, ty = cfg.tile_count(W, H)
    T, B = tx * ty, cfg.tile_depth_bins
    G3 = cfg.grid_dims ** 3
    D3 = inst.sdf.dims ** 3
    return {
        "grid_pre": 16 * G3 + 16 * G3 + 4 * D3,
        "integrate": Npt * (16 + 16 + 16 + 4 + 16) + 2 * 16 * G3 + 4 * D3,
        "grid_post": Npt * 32 + 16 * G3,
        "clear": T * B * 16 + T * 4 + W * H * 16,
        # positions + tangents, depth, records staged (8 w + 8 r), keys (4 w + 4 r),
        # lists written (8), heads (16), per-bin counts/offsets (3 x 4), per-tile counts
        "tiles": Npt * 32 + W * H * 4 + K * (8 + 8 + 4 + 4 + 8) + T * B * (16 + 12) + T * 4,
        "sort": T * 4 + (4 + T) * 4 + cfg.sort_buckets * 8,
        # lists read (8), heads (16), shading read, depth read, result write
        "fine": Npt * 32 + S * SP * 16 + W * H * (4 + 16) + K * 8 + T * B * 16,
        # positions + tangents, scene depth read and hair depth written
        "hair_depth": Npt * 32 + W * H * 8,
        "shading": Npt * 32 + S * SP * (16 + 8),
    }


# ----------------------------------------------------------------------------
# clocks sampling (nvidia-smi during the timed region)
# ----------------------------------------------------------------------------

REASON_BITS = {
    0x1: "gpu_idle", 0x2: "applications_clocks_setting", 0x4: "sw_power_cap", 0x8: "hw_slowdown",
    0x10: "sync_boost", 0x20: "sw_thermal_slowdown", 0x40: "hw_thermal_slowdown",
    0x80: "hw_power_brake_slowdown", 0x100: "display_clock_setting",
}


class ClockSampler:
    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.samples = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu),
                 "--query-gpu=clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 4:
                self.samples.append(parts)

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        for s in self.samples:
            try:
                sm.append(float(s[0]))
                mx.append(float(s[1]))
                bits = int(s[3], 16) if s[3].startswith("0x") else int(s[3])
                for b, n in REASON_BITS.items():
                    if bits & b:
                        reasons.add(n)
            except ValueError:
                continue
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["not sampled"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


# ----------------------------------------------------------------------------
# CPU leg (the reference algorithm on host cores)
# ----------------------------------------------------------------------------

def cpu_frame_runner(inst, from_rest=False):
    """One frame of the restated reference passes on the host (OpenMP build);
    from_rest: every frame starts from the asset at rest (the stress frame)."""
    from hairfb import uniforms as UN
    from oracle import oracle as O
    O.use_threads(True)
    cfg, hb = inst.cfg, inst.hair
    u = UN.pack_render_uniforms(inst.scene, cfg)
    md = cfg.max_drawn_segments(inst.width, inst.height)
    st = {"prev": hb.asset.positions.copy(), "now": hb.asset.positions.copy(), "f": 0}
    su0 = UN.pack_sim_uniforms(inst.sim, inst.scene.model_matrix, inst.scene.sdf_bounds,
                               inst.scene.grid_bounds, 0, wind_dir=inst.wind_dir)
    st["dv"] = O.grid_post_sim(cfg, su0, hb.hair_data, st["prev"], st["now"])
    hd = O.hair_depth(u, hb.hair_data, st["now"], hb.tangents, hb.asset.strands, inst.scene_depth)
    st["shade"] = O.shading(cfg, u, hb.hair_data, st["now"], hb.tangents, hd, hb.asset.strands)
    rest = dict(st)

    def frame():
        if from_rest:
            st.update(rest)
        f = st["f"]
        su = UN.pack_sim_uniforms(inst.sim, inst.scene.model_matrix, inst.scene.sdf_bounds,
                                  inst.scene.grid_bounds, f, wind_dir=inst.wind_dir,
                                  wind_strength=inst.wind_strength(f))
        gw = O.grid_pre_sim(cfg, su, st["dv"], inst.sdf.distances, inst.sdf.dims)
        new = O.sim_integrate(cfg, su, hb.hair_data, st["prev"], st["now"], hb.asset.positions,
                              hb.segment_lengths, st["dv"], gw, inst.sdf.distances, inst.sdf.dims)
        st["prev"], st["now"] = st["now"], new
        st["dv"] = O.grid_post_sim(cfg, su, hb.hair_data, st["prev"], st["now"])
        tiles, segs, cnt = O.tiles_pass(cfg, u, hb.hair_data, st["now"], hb.tangents, inst.scene_depth,
                                        hb.asset.strands, inst.width, inst.height, md)
        _, tl = O.tile_sort(cfg, inst.width, inst.height, cnt)
        O.fine_pass(cfg, u, hb.hair_data, st["now"], hb.tangents, st["shade"], inst.scene_depth, tiles,
                    segs, tl, inst.width, inst.height)
        hd = O.hair_depth(u, hb.hair_data, st["now"], hb.tangents, hb.asset.strands, inst.scene_depth)
        st["shade"] = O.shading(cfg, u, hb.hair_data, st["now"], hb.tangents, hd, hb.asset.strands)
        st["f"] = f + 1
    return frame


def time_cpu(inst, seconds, min_frames=1, max_frames=None, from_rest=False):
    frame = cpu_frame_runner(inst, from_rest)
    frame()  # warm-up (page-in, thread pool)
    n, t0 = 0, time.perf_counter()
    while True:
        frame()
        n += 1
        el = time.perf_counter() - t0
        if (el >= seconds and n >= min_frames) or (max_frames and n >= max_frames):
            break
    return n, el


def host_threads():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


# ----------------------------------------------------------------------------
# GPU leg
# ----------------------------------------------------------------------------

def run_ours(args, rank, world, dist):
    import torch
    from hairfb import renderer as R
    from hairfb.lib import Context

    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    inst = make_instance(args.workload, seed=rank)
    stream = torch.cuda.Stream()  # the library, the events and torch all run on it
    torch.cuda.set_stream(stream)
    ctx = Context(inst.cfg.to_c(), dev)
    ctx.set_stream(stream)
    r = R.Renderer(inst, ctx=ctx, hair_depth=True)
    r.before_first_frame()
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    names = ["grid_pre", "integrate", "grid_post", "clear", "tiles", "sort", "fine", "hair_depth", "shading"]

    def timed_frame(ev):
        su = r.sim_uniforms(r.frame_idx)
        ev[0].record(stream)
        r.grid_pre.cmd_update_grids_before_sim(su, r.grids, r.sdf)
        ev[1].record(stream)
        r.integrate.cmd_simulate_hair_positions(su, r.hair, r.grids, r.sdf)
        ev[2].record(stream)
        r.grid_post.cmd_update_grids_after_sim(su, r.hair, r.grids)
        ev[3].record(stream)
        R.clear_before_render(r.ctx, r.rb)
        ev[4].record(stream)
        r.tiles.cmd_draw_hair_to_tiles(r.uniforms, r.hair, r.scene_depth, r.rb)
        ev[5].record(stream)
        r.sort.cmd_sort_hair_tiles(r.rb)
        ev[6].record(stream)
        r.fine.cmd_rasterize_slices_hair(r.uniforms, r.hair, r.scene_depth, r.rb)
        ev[7].record(stream)
        r.hw_hair.cmd_draw_hair_depth(r.uniforms, r.hair, r.scene_depth, r.hair_depth, r.rb)
        ev[8].record(stream)
        r.shading.cmd_compute_shading_points(r.uniforms, r.hair, r.shading_depth)
        ev[9].record(stream)
        r.frame_idx += 1

    # the stress frame is timed from rest: its 120k-strand ponytail overflows the
    # reference's i32 fixed-point density within a few frames and the hair
    # blows apart (reference arithmetic, reproduced), so every frame there
    # starts from the asset at rest, reset outside the timed region
    from_rest = args.workload == "stress"

    def rest():
        if from_rest:
            r.hair.reset_simulation()
            r.hair._current = 0
            r.grids.clear()
            r.frame_idx = 0
            r.before_first_frame()

    for _ in range(args.warmup):
        rest()
        r.frame()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    launches0 = ctx.counters()["launches"]
    rec0 = ctx.counters()["tileRecords"]
    frame_ms, pass_ms = [], {n: [] for n in names}
    with ClockSampler(dev) as clk:
        torch.cuda.synchronize()
        for _ in range(args.steps):
            if from_rest:  # the reset's launches are not the frame's
                l_a = ctx.counters()["launches"]
                rest()
                launches0 += ctx.counters()["launches"] - l_a
            flush.fill_(1.0)  # L2 flush, outside the timed events
            ev = [torch.cuda.Event(enable_timing=True) for _ in range(len(names) + 1)]
            timed_frame(ev)
            torch.cuda.synchronize()
            frame_ms.append(ev[0].elapsed_time(ev[len(names)]))
            for i, n in enumerate(names):
                pass_ms[n].append(ev[i].elapsed_time(ev[i + 1]))
    launches = ctx.counters()["launches"] - launches0
    records = (ctx.counters()["tileRecords"] - rec0) / args.steps
    total_s = sum(frame_ms) / 1000.0

    # ---- e2e through the public API with host buffers ----
    from hairfb import uniforms as UN
    depth_h = torch.from_numpy(inst.scene_depth).pin_memory()
    img_h = torch.empty(4 + 4 * inst.width * inst.height, dtype=torch.float32).pin_memory()
    depth_d = torch.empty_like(depth_h, device="cuda")
    e2e_ms = []
    for k in range(args.warmup + args.steps):
        rest()
        t0 = torch.cuda.Event(enable_timing=True)
        t1 = torch.cuda.Event(enable_timing=True)
        t0.record(stream)
        u = UN.pack_render_uniforms(inst.scene, inst.cfg)      # host-built uniform blocks
        su = r.sim_uniforms(r.frame_idx)
        depth_d.copy_(depth_h, non_blocking=True)               # scene depth H2D
        r.uniforms = u
        r.scene_depth = depth_d
        r.grid_pre.cmd_update_grids_before_sim(su, r.grids, r.sdf)
        r.integrate.cmd_simulate_hair_positions(su, r.hair, r.grids, r.sdf)
        r.grid_post.cmd_update_grids_after_sim(su, r.hair, r.grids)
        R.clear_before_render(r.ctx, r.rb)
        r.tiles.cmd_draw_hair_to_tiles(u, r.hair, depth_d, r.rb)
        r.sort.cmd_sort_hair_tiles(r.rb)
        r.fine.cmd_rasterize_slices_hair(u, r.hair, depth_d, r.rb)
        r.hw_hair.cmd_draw_hair_depth(u, r.hair, depth_d, r.hair_depth, r.rb)
        r.shading.cmd_compute_shading_points(u, r.hair, r.shading_depth)
        r.frame_idx += 1
        ctx.call("hfb_buffer_download", img_h.data_ptr(), r.rb.rb.rasterizerResult, img_h.numel() * 4)
        t1.record(stream)
        torch.cuda.synchronize()
        if k >= args.warmup:
            e2e_ms.append(t0.elapsed_time(t1))
    h2d = depth_h.numel() * 4 + UN.RENDER_UNIFORMS_BYTES + UN.SIM_UNIFORMS_BYTES
    d2h = img_h.numel() * 4

    out = dict(frame_ms=frame_ms, pass_ms=pass_ms, total_s=total_s, launches=launches, records=records,
               e2e_ms=e2e_ms, h2d=h2d, d2h=d2h, clocks=clk.summary(), inst=inst)
    ctx.close()
    return out


# ----------------------------------------------------------------------------
# batched64: many instances per frame (hfb_frame_batch) vs one at a time (hfb_frame)
# ----------------------------------------------------------------------------

def batched_instances(seed):
    from hairfb import synthetic
    # 2048 records per 16x16 tile (the densest instance holds ~500): the pool
    # scales with the tile area for the autotuner's 8 and 32 px tiles, and no
    # candidate drops a record
    return synthetic.batched_instances(seed=seed, count=64, tile_size=16, depth_bins=8, grid_dims=64,
                                       slices=4, shading_points=8, avg_segments_per_tile=2048)


def read_records(r):
    import ctypes
    out = (ctypes.c_uint32 * 1)()
    r.ctx.call("hfb_buffer_download", ctypes.addressof(out), r.rb.rb.tileSegments, 4)
    return int(out[0])


def run_batched(args, rank, world, dist):
    import ctypes
    import torch
    from hairfb import autotune as AT
    from hairfb import renderer as R
    from hairfb.lib import Context, HfbInstance

    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    insts = batched_instances(seed=rank)
    n = len(insts)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    base = insts[0].cfg
    ctx0 = Context(base.to_c(), dev)
    ctx0.set_stream(stream)
    rs = [R.Renderer(i, dev, ctx=ctx0, hair_depth=True) for i in insts]
    for r in rs:
        r.before_first_frame()
    torch.cuda.synchronize()
    t_tune = time.perf_counter()
    cfg, ctx, trials = AT.tune(rs, base, dev, stream, budget_s=args.tune_budget)
    t_tune = time.perf_counter() - t_tune
    ctx0.close()
    batch = R.BatchRenderer(rs)
    ev = lambda: torch.cuda.Event(enable_timing=True)  # noqa: E731

    # ---- batched frames ----
    for _ in range(args.warmup):
        batch.frame()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    c0 = ctx.counters()
    # frames back to back (the host prepares the next frame while the GPU
    # renders); an event between frames gives each frame's GPU time
    evs = [ev() for _ in range(args.steps + 1)]
    with ClockSampler(dev) as clk:
        torch.cuda.synchronize()
        evs[0].record(stream)
        for k in range(args.steps):
            batch.frame()
            evs[k + 1].record(stream)
        torch.cuda.synchronize()
    step_ms = [evs[k].elapsed_time(evs[k + 1]) for k in range(args.steps)]
    c1 = ctx.counters()
    # latency: one frame submitted and waited for at a time (host work included)
    lat_ms = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        batch.frame()
        torch.cuda.synchronize()
        lat_ms.append(1000.0 * (time.perf_counter() - t0))
    launches = c1["launches"] - c0["launches"]
    dropped = c1["tileRecordsDropped"] - c0["tileRecordsDropped"]

    # ---- the plain per-frame path: hfb_frame on one instance after another ----
    for r in rs:
        r.frame_native()
    torch.cuda.synchronize()
    plain_round_ms, plain_frame_ms = [], []
    for _ in range(args.steps):
        evs = [ev() for _ in range(n + 1)]
        evs[0].record(stream)
        for j, r in enumerate(rs):
            r.frame_native()
            evs[j + 1].record(stream)
        torch.cuda.synchronize()
        plain_round_ms.append(evs[0].elapsed_time(evs[n]))
        plain_frame_ms += [evs[j].elapsed_time(evs[j + 1]) for j in range(n)]

    # ---- per-pass times of one batched frame (plain launches + events) ----
    arr = (HfbInstance * n)(*[r.instance() for r in rs])
    names = ["grid_pre", "integrate", "grid_post", "clear", "tiles", "sort", "fine", "hair_depth", "shading"]
    pm = (ctypes.c_float * len(names))()
    ctx.call("hfb_frame_batch_profile", arr, n, pm)
    for r, inst in zip(rs, arr):
        r.after_native_frame(inst)
    pass_ms = {k: float(pm[i]) for i, k in enumerate(names)}
    K = [read_records(r) for r in rs]

    # ---- e2e: the public call with host inputs, every image read back ----
    imgs = [torch.empty(4 + 4 * i.width * i.height, dtype=torch.float32).pin_memory() for i in insts]
    e2e_ms = []
    for k in range(args.warmup + args.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        batch.frame()  # uniform blocks go up from host memory inside the call
        for r, h in zip(rs, imgs):
            ctx.call("hfb_buffer_download", h.data_ptr(), r.rb.rb.rasterizerResult, h.numel() * 4)
        torch.cuda.synchronize()
        if k >= args.warmup:
            e2e_ms.append(1000.0 * (time.perf_counter() - t0))
    from hairfb import uniforms as UN
    h2d = n * (UN.RENDER_UNIFORMS_BYTES + UN.SIM_UNIFORMS_BYTES)
    d2h = sum(h.numel() * 4 for h in imgs)
    served = None
    if args.serve_frames > 0 and world == 1:
        served = run_served(args.serve_frames, dev, groups=getattr(ctx, "batch_groups", 1))
    out = dict(served=served, step_ms=step_ms, lat_ms=lat_ms, plain_round_ms=plain_round_ms, plain_frame_ms=plain_frame_ms,
               pass_ms=pass_ms, K=K, e2e_ms=e2e_ms, h2d=h2d, d2h=d2h, clocks=clk.summary(), insts=insts,
               cfg=cfg, trials=[t.as_dict() for t in trials], tune_s=t_tune, launches=launches,
               groups=getattr(ctx, "batch_groups", 1), pipelined=getattr(ctx, "batch_pipeline", False),
               dropped=dropped, n=n)
    ctx.close()
    return out


def run_served(frames_per_session, device, groups=1, seed=0):
    """The serving workload: sessions admitted under the memory budget, one
    hfb_frame_batch call per tick over every admitted session.  Host assets
    are generated before the clock starts (a server loads them)."""
    import torch
    from hairfb import serve
    from hairfb.config import HairConfig
    cfg = HairConfig(tile_size=16, tile_depth_bins=8, slices_per_pixel=4, shading_points=8, grid_dims=64)
    specs = serve.snap(serve.poisson_sessions(seed=seed, count=256, rate_hz=2000.0, frames=frames_per_session))
    factory = serve.SessionFactory(cfg, seed=seed)
    t0 = time.perf_counter()
    factory.prepare(specs)
    prep_s = time.perf_counter() - t0
    server = serve.Server(cfg, device, budget_bytes=150 << 30, groups=groups, make_instance=factory)
    torch.cuda.synchronize()
    st = server.run(specs)
    server.close()
    torch.cuda.empty_cache()
    return {"frames_per_s": st.frames_per_s, "frames": st.frames, "wall_s": st.wall_s, "ticks": st.ticks,
            "frame_p50_ms": st.pct(0.5), "frame_p99_ms": st.pct(0.99),
            "admit_wait_p50_ms": st.pct(0.5, "admit_wait_ms"), "admit_wait_p99_ms": st.pct(0.99, "admit_wait_ms"),
            "peak_sessions": st.peak_sessions, "peak_bytes": st.peak_bytes, "budget_bytes": st.budget_bytes,
            "records_dropped": st.dropped, "frames_per_session": frames_per_session, "sessions": len(specs),
            "host_asset_prep_s": round(prep_s, 1),
            "note": "frames/s over the wall clock from the first arrival to the last frame (admission, uploads "
                    "and first-frame setup included); frame latency = the tick that rendered the frame"}


def report_batched_peer(res, dist):
    """Non-zero ranks join the max-over-ranks reduction of report_batched."""
    from hairfb import replicas
    replicas.max_over_ranks([sum(res["step_ms"]) / 1000.0, sum(res["plain_round_ms"]) / 1000.0,
                             sum(res["e2e_ms"]) / 1000.0], dist, "cuda")


def cpu_batched(insts, seconds):
    """Instance frames/s of the restated reference on the host, on a bounded
    sample: the instances in order, one frame each, for ~`seconds`."""
    frames = [cpu_frame_runner(i) for i in insts[:8]]
    for f in frames:
        f()  # warm-up
    k, t0 = 0, time.perf_counter()
    while True:
        frames[k % len(frames)]()
        k += 1
        el = time.perf_counter() - t0
        if el >= seconds:
            return k, el


def report_batched(args, res, world, dist):
    import dataclasses
    from hairfb import autotune as AT  # noqa: F401
    step_s = sum(res["step_ms"]) / 1000.0
    plain_s = sum(res["plain_round_ms"]) / 1000.0
    e2e_s = sum(res["e2e_ms"]) / 1000.0
    from hairfb import replicas
    step_s, plain_s, e2e_s = replicas.max_over_ranks([step_s, plain_s, e2e_s], dist, "cuda")
    n = res["n"]
    fps = replicas.job_throughput(n * len(res["step_ms"]), world, step_s)
    plain_fps = replicas.job_throughput(n * len(res["plain_round_ms"]), world, plain_s)
    cfg = res["cfg"]
    insts = [dataclasses.replace(i, cfg=cfg) for i in res["insts"]]
    alg = {}
    for inst, k in zip(insts, res["K"]):
        for key, v in algorithmic_bytes(inst, k).items():
            alg[key] = alg.get(key, 0) + v
    pm = res["pass_ms"]
    dominant = max(pm, key=pm.get)
    peaks_path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(peaks_path):
        peak, peak_src = json.load(open(peaks_path))["hbm_gbs"], "measured"
    else:
        peak, peak_src = 6800.0, "fallback"
    achieved = alg[dominant] / (pm[dominant] / 1000.0) / 1e9
    traffic = None
    tp = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(tp):
        # measured at one pass config; the raster passes' figure is reported only
        # when the tuner chose that config, the simulation's does not depend on it
        tj = json.load(open(tp))
        traffic = tj.get(f"batched64:ts{cfg.tile_size}_b{cfg.tile_depth_bins}:{dominant}")
        if traffic is None and dominant in ("grid_pre", "integrate", "grid_post"):
            traffic = next((v for k, v in tj.items() if k.startswith("batched64:") and k.endswith(":" + dominant)),
                           None)
    srt = sorted(res["step_ms"])
    q = lambda v, x: v[min(len(v) - 1, int(round(x * (len(v) - 1))))]  # noqa: E731
    psrt = sorted(res["plain_frame_ms"])
    segments = sum(i.hair.asset.strands * (i.hair.asset.points_per_strand - 1) for i in insts)
    frame_bytes = sum(alg.values())
    cpu = None
    if not args.no_cpu_baseline:
        k, el = cpu_batched(res["insts"], args.cpu_seconds)
        cpu = {"value": k / el, "unit": "frames/s", "cores": host_threads(), "kind": "port",
               "sample": f"{k} instance frames (the first 8 instances in turn) on the host, C restatement of "
                         f"the reference WGSL with OpenMP, {el:.1f} s"}
    line = {
        "metric": "frames/s", "value": fps, "unit": "frames/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": step_s * 1000.0 / len(res["step_ms"]),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded; no public dataset exists for this path)",
        "config": {"workload": "batched64", "describe": WORKLOADS["batched64"],
                   "step": f"one batched frame of all {n} instances (hfb_frame_batch, captured CUDA graph)",
                   "l2": "inputs larger than L2 (all instances' positions, grids and buffers ~ several GB)",
                   "frames_per_step": n, "tuned": {"tile_size": cfg.tile_size, "depth_bins": cfg.tile_depth_bins,
                                                   "slices": cfg.slices_per_pixel,
                                                   "avg_segments_per_tile": cfg.avg_segments_per_tile,
                                                   "groups": res["groups"], "pipelined": res["pipelined"],
                                                   "tune_s": round(res["tune_s"], 1)},
                   "autotune_trials": [{k: (round(v, 3) if isinstance(v, float) else v) for k, v in t.items()}
                                       for t in res["trials"]],
                   "plain_frames_per_s": plain_fps, "batched_over_plain": fps / plain_fps,
                   "p50_ms": q(srt, 0.5), "p99_ms": q(srt, 0.99),
                   "latency_p50_ms": q(sorted(res["lat_ms"]), 0.5), "latency_p99_ms": q(sorted(res["lat_ms"]), 0.99),
                   "plain_frame_p50_ms": q(psrt, 0.5), "plain_frame_p99_ms": q(psrt, 0.99),
                   "segments_per_s": world * segments * len(srt) / step_s,
                   "tile_records_per_step": sum(res["K"]), "records_dropped": res["dropped"],
                   "pass_ms": {k: round(v, 4) for k, v in pm.items()},
                   "step_algorithmic_bytes": frame_bytes,
                   "served": res["served"],
                   "step_hbm_roofline_frac": frame_bytes * (fps / n) / world / (peak * 1e9)},
        "e2e": {"value": world * n * len(res["e2e_ms"]) / e2e_s, "unit": "frames/s",
                "h2d_bytes_per_step": res["h2d"], "d2h_bytes_per_step": res["d2h"]},
        "roofline": {"bound": "hbm", "kernel": dominant, "achieved": achieved, "peak": peak,
                     "peak_source": peak_src, "unit": "GB/s", "frac": achieved / peak, "traffic": traffic,
                     "algorithmic_bytes": alg[dominant]},
        "cpu_baseline": cpu,
        "clocks": res["clocks"],
        "gpu_launches": res["launches"],
    }
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    if args.tfx:
        ASSET_FILES.update(tfx=args.tfx, sdf=args.sdf)
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    dist = None
    if world > 1:
        import torch
        import torch.distributed as dist_
        dist = dist_
        if args.impl == "reference":
            # the host reference runs once, on rank 0
            if rank != 0:
                return
            world = 1
            dist = None
        else:
            torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
            dist.init_process_group("nccl")

    wl = args.workload
    if args.capture_frames > 0:
        capture(args)
        return
    if args.impl == "reference" and wl == "batched64":
        insts = batched_instances(seed=0)
        frames = [cpu_frame_runner(i) for i in insts]
        w = max(1, min(args.warmup, 3))
        for k in range(w):
            frames[k % len(frames)]()
        t0 = time.perf_counter()
        for k in range(args.steps):
            frames[k % len(frames)]()
        el = time.perf_counter() - t0
        fps = args.steps / el
        line = {
            "impl": "reference", "metric": "frames/s", "value": fps, "unit": "frames/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": w, "ms_per_step": 1000.0 * el / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic",
            "config": {"workload": wl, "describe": WORKLOADS[wl],
                       "step": "one instance frame, the instances in turn",
                       "implementation": "C restatement of the reference WGSL passes, OpenMP"},
            "cpu_baseline": {"value": fps, "unit": "frames/s", "cores": host_threads(), "kind": "port",
                             "sample": f"{args.steps} instance frames (instances 0..{args.steps - 1} mod 64)"},
            "e2e": {"value": fps, "unit": "frames/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        }
        print(json.dumps(line), flush=True)
        return
    if args.impl == "reference":
        inst = make_instance(wl, seed=0)
        frame = cpu_frame_runner(inst, from_rest=wl == "stress")
        for _ in range(max(1, min(args.warmup, 3))):
            frame()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            frame()
        el = time.perf_counter() - t0
        n = args.steps
        fps = n / el
        cores = host_threads()
        line = {
            "impl": "reference", "metric": "frames/s", "value": fps, "unit": "frames/s",
            "n_gpus": args.gpus, "steps": n, "warmup": max(1, min(args.warmup, 3)), "ms_per_step": 1000.0 * el / n,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": data_label(wl),
            "config": {"workload": wl, "describe": WORKLOADS[wl],
                       "implementation": "C restatement of the reference WGSL passes, OpenMP"},
            "cpu_baseline": {"value": fps, "unit": "frames/s", "cores": cores, "kind": "port",
                             "sample": f"{n} full frames of {wl} after warm-up frames"},
            "e2e": {"value": fps, "unit": "frames/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        }
        print(json.dumps(line), flush=True)
        return

    if wl == "served256":
        import torch
        dev = int(os.environ.get("LOCAL_RANK", "0"))
        torch.cuda.set_device(dev)
        sv = run_served(600, dev, groups=4, seed=rank)
        from hairfb import replicas
        sv["wall_s"] = replicas.max_over_ranks([sv["wall_s"]], dist, "cuda")[0]
        if rank == 0:
            fps = replicas.job_throughput(sv["frames"], world, sv["wall_s"])
            line = {"metric": "frames/s", "value": fps, "unit": "frames/s", "n_gpus": world, "steps": sv["ticks"],
                    "warmup": 0, "ms_per_step": 1000.0 * sv["wall_s"] / max(1, sv["ticks"]),
                    "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
                    "data": "synthetic (seeded Poisson sessions; no public dataset exists for this path)",
                    "config": {"workload": wl, "describe": WORKLOADS[wl], "served": sv,
                               "step": "one tick: every admitted session's next frame (hfb_frame_batch)"},
                    "e2e": {"value": fps, "unit": "frames/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
                    "roofline": None, "cpu_baseline": None, "gpu_launches": None}
            print(json.dumps(line), flush=True)
        if dist:
            dist.barrier()
            dist.destroy_process_group()
        return

    if wl == "batched64":
        res = run_batched(args, rank, world, dist)
        if rank == 0:
            report_batched(args, res, world, dist)
        elif dist:
            report_batched_peer(res, dist)
        if dist:
            dist.barrier()
            dist.destroy_process_group()
        return

    res = run_ours(args, rank, world, dist)
    total = res["total_s"]
    e2e_total = sum(res["e2e_ms"]) / 1000.0
    from hairfb import replicas
    total, e2e_total = replicas.max_over_ranks([total, e2e_total], dist, "cuda")
    if dist:
        dist.barrier()
    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return

    inst = res["inst"]
    K = res["records"]
    alg = algorithmic_bytes(inst, int(K))
    pass_avg = {n: sum(v) / len(v) for n, v in res["pass_ms"].items()}
    frame_avg = sum(res["frame_ms"]) / len(res["frame_ms"])
    dominant = max(pass_avg, key=pass_avg.get)
    peaks_path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(peaks_path):
        peak = json.load(open(peaks_path))["hbm_gbs"]
        peak_src = "measured"
    else:
        peak, peak_src = 6800.0, "fallback"
    achieved = alg[dominant] / (pass_avg[dominant] / 1000.0) / 1e9
    traffic = None
    tp = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(tp):
        traffic = json.load(open(tp)).get(f"{wl}:{dominant}")
    fps = world * len(res["frame_ms"]) / total
    frame_bytes = sum(alg.values())
    segments = inst.hair.asset.strands * (inst.hair.asset.points_per_strand - 1)
    srt = sorted(res["frame_ms"])
    p = lambda q: srt[min(len(srt) - 1, int(round(q * (len(srt) - 1))))]

    cpu = None
    if not args.no_cpu_baseline:
        n, el = time_cpu(inst, args.cpu_seconds, from_rest=wl == "stress")
        cpu = {"value": n / el, "unit": "frames/s", "cores": host_threads(), "kind": "port",
               "sample": f"{n} full frames of {wl} on the host (C restatement of the reference "
                         f"WGSL, OpenMP) after 1 warm-up frame, {el:.1f} s"
                         + (", each from the asset at rest" if wl == "stress" else "")}

    line = {
        "metric": "frames/s", "value": fps, "unit": "frames/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": frame_avg,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": data_label(wl),
        "config": {"workload": wl, "describe": WORKLOADS[wl], "l2": "flushed (256 MiB write) between frames",
                   "p50_ms": p(0.5), "p99_ms": p(0.99), "segments_per_s": world * segments * len(srt) / total,
                   "tile_records_per_frame": K, "pass_ms": {k: round(v, 4) for k, v in pass_avg.items()},
                   "frame_algorithmic_bytes": frame_bytes,
                   "frame_hbm_roofline_frac": frame_bytes * fps / world / (peak * 1e9),
                   **({"frames": "each timed frame starts from the asset at rest (positions, grids and the "
                                 "first-frame setup reset before it, outside the timed region): the hair blows "
                                 "apart after a few frames on the reference's i32 density arithmetic"}
                      if wl == "stress" else {})},
        "e2e": {"value": world * len(res["e2e_ms"]) / e2e_total, "unit": "frames/s",
                "h2d_bytes_per_step": res["h2d"], "d2h_bytes_per_step": res["d2h"]},
        "roofline": {"bound": "hbm", "kernel": dominant, "achieved": achieved, "peak": peak,
                     "peak_source": peak_src, "unit": "GB/s", "frac": achieved / peak, "traffic": traffic,
                     "algorithmic_bytes": alg[dominant]},
        "cpu_baseline": cpu,
        "clocks": res["clocks"],
        "gpu_launches": res["launches"],
    }
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
