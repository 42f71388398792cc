"""Accuracy of whole frames on four of the workloads (the 2,000 x 16
640x480 frame, the 10,000 x 32 1920x1080 frame with 64^3 grids and with the
32^3 grids the configuration names, and the largest instance of the
64-instance batch), against the oracle over 60 frames -- or, for the 32^3
grids, as many frames as the reference's arithmetic stays finite (its i32
fixed-point density wraps there and blows the hair apart):

- positions after 60 frames of simulation within 1e-5 relative (the bar;
  the per-step arithmetic is bit-exact, `test_gpu_parity.py`);
- the 60th frame's image within 1/255 per channel of the oracle's raster
  passes run on the same positions and shading;
- the hair depth bit-exact and the shading within 1e-5 of the oracle's on
  the same positions.

With HAIRFB_ACCURACY_JSON set, each case appends its measured maxima to that
file (one JSON object per line).
"""
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

from hairfb import synthetic  # noqa: E402
from hairfb.renderer import Renderer  # noqa: E402



@pytest.fixture(scope="module")
def oracle():
    from oracle import oracle as o
    o.use_threads(True)
    o.load()
    return o


def _workload(name):
    if name == "plain_small":
        return synthetic.plain_small()
    if name == "plain_full":
        return synthetic.plain_full()
    if name == "plain_full_grid32":
        return synthetic.plain_full(grid_dims=32)
    insts = synthetic.batched_instances(seed=0, count=64, tile_size=16, depth_bins=8, grid_dims=64, slices=4,
                                        shading_points=8, avg_segments_per_tile=2048)
    return max(insts, key=lambda i: i.hair.asset.strands * i.hair.asset.points_per_strand)


def _finite_frames(oracle, inst, r, limit):
    """Frames (up to limit) after which the oracle's positions are all finite."""
    cfg, hb = inst.cfg, inst.hair
    prev = hb.asset.positions.copy()
    now = hb.asset.positions.copy()
    dv = oracle.grid_post_sim(cfg, r.sim_uniforms(0), hb.hair_data, prev, now)
    for f in range(limit):
        su = r.sim_uniforms(f)
        gw = oracle.grid_pre_sim(cfg, su, dv, inst.sdf.distances, inst.sdf.dims)
        new = oracle.sim_integrate(cfg, su, hb.hair_data, prev, now, hb.asset.positions, hb.segment_lengths, dv, gw,
                                   inst.sdf.distances, inst.sdf.dims)
        if not np.isfinite(new).all():
            return f
        prev, now = now, new
        dv = oracle.grid_post_sim(cfg, su, hb.hair_data, prev, now)
    return limit


@pytest.mark.parametrize("name", ["plain_small", "plain_full", "plain_full_grid32", "batched64_largest"])
def test_frames_against_the_oracle(oracle, name):
    inst = _workload(name)
    cfg, hb = inst.cfg, inst.hair
    S, P = hb.asset.strands, hb.asset.points_per_strand
    r = Renderer(inst, 0, hair_depth=True)
    FRAMES = _finite_frames(oracle, inst, r, 60) if name == "plain_full_grid32" else 60
    assert FRAMES >= 2, f"{name}: the reference arithmetic leaves finite values for {FRAMES} frames only"
    r.before_first_frame()
    for _ in range(FRAMES - 1):
        r.frame()
    r.ctx.sync()  # the library's stream is not torch's: wait for it before reading its buffers
    shade_in = r.hair.shading.cpu().numpy()  # the shading the last frame's fine pass reads
    r.frame()
    r.ctx.sync()
    g_pos = r.hair.positions.cpu().numpy()
    g_img = r.rb.read_result()[4:].reshape(-1, 4)
    g_depth = r.hair_depth.cpu().numpy()
    g_shade = r.hair.shading.cpu().numpy()

    # the oracle's simulation over the same frames
    u = r.uniforms
    prev = hb.asset.positions.copy()
    now = hb.asset.positions.copy()
    dv = oracle.grid_post_sim(cfg, r.sim_uniforms(0), hb.hair_data, prev, now)
    for f in range(FRAMES):
        su = r.sim_uniforms(f)
        gw = oracle.grid_pre_sim(cfg, su, dv, inst.sdf.distances, inst.sdf.dims)
        new = oracle.sim_integrate(cfg, su, hb.hair_data, prev, now, hb.asset.positions, hb.segment_lengths, dv, gw,
                                   inst.sdf.distances, inst.sdf.dims)
        prev, now = now, new
        dv = oracle.grid_post_sim(cfg, su, hb.hair_data, prev, now)
    pos_rel = float(np.abs(g_pos[:, :3].astype(np.float64) - now[:, :3]).max() / np.abs(now[:, :3]).max())
    moved = float(np.abs(now[:, :3] - hb.asset.positions[:, :3]).max())

    # the raster passes of the last frame, on the GPU's positions and the shading they read
    md = r.rb.max_drawn_segments
    tiles, segs, cnt = oracle.tiles_pass(cfg, u, hb.hair_data, g_pos, hb.tangents, inst.scene_depth, S, inst.width,
                                         inst.height, md)
    _, tl = oracle.tile_sort(cfg, inst.width, inst.height, cnt)
    o_img = oracle.fine_pass(cfg, u, hb.hair_data, g_pos, hb.tangents, shade_in, inst.scene_depth, tiles, segs, tl,
                             inst.width, inst.height)[4:].reshape(-1, 4)
    px_err = float(np.abs(g_img - o_img).max())
    covered = int((o_img[:, 3] > 0).sum())
    o_depth = oracle.hair_depth(u, hb.hair_data, g_pos, hb.tangents, S, inst.scene_depth)
    depth_diff = int((g_depth.view(np.uint32) != o_depth.view(np.uint32)).sum())
    o_shade = oracle.shading(cfg, u, hb.hair_data, g_pos, hb.tangents, o_depth, S)
    shade_err = float((np.abs(g_shade - o_shade) / (1.0 + np.abs(o_shade))).max())

    out = os.environ.get("HAIRFB_ACCURACY_JSON")
    if out:
        with open(out, "a") as f:
            f.write(json.dumps({"workload": name, "strands": S, "points": P, "width": inst.width,
                                "height": inst.height, "frames": FRAMES, "max_rel_position_error": pos_rel,
                                "max_moved": moved, "max_pixel_error": px_err, "covered_pixels": covered,
                                "hair_depth_pixels_differing": depth_diff, "max_shading_error": shade_err}) + "\n")
    assert moved > 1e-4, "the simulation did not move the hair"
    assert pos_rel <= 1e-5, f"relative position error {pos_rel:.3g} after {FRAMES} frames"
    assert covered > 1000
    assert px_err <= 1.0 / 255.0, f"max pixel error {px_err:.4g}"
    assert depth_diff == 0
    assert shade_err <= 1e-5, f"shading error {shade_err:.3g}"
