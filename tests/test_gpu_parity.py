"""GPU parity: every pass of libhairfb.so against the CPU oracle, called
through the C-ABI on the same seeded inputs.

Bars (the reference's own: integer work bit-exact, pixels within 1/255,
positions within 1e-5 relative after 60 steps):
- tiles pass: drawnSegmentsCount, segmentCountPerTile, per-bin min/max depth
  bit-exact; per-bin lists equal as walked sequences (canonical order);
- tile sort: buckets and tile list bit-exact (stable order on both sides);
- grids: density/velocity grid bit-exact (integer splat); gradient/wind
  grid bit-exact;
- integration: bit-exact after one step (same fp32 op order, no FMA), and
  within 1e-5 relative after 60 steps of the whole simulation;
- shading: within 1e-5 (absolute + relative) -- exp/pow are not
  correctly rounded on either side;
- fine pass: every pixel channel within 1/255.
"""
import ctypes

import numpy as np
import pytest

from helpers import INVALID, frame_of, small_instance, walk_lists
from hairfb import uniforms as UN

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

from hairfb.lib import Context, byref, ptr  # noqa: E402
from hairfb.passes import (GridPostSimPass, GridPreSimPass, HairFinePass, HairObject,  # noqa: E402
                           HairShadingPass, HairSimIntegrationPass, HairTileSortPass, HairTilesPass,
                           PhysicsGrids, RasterBuffers, SdfCollider, clear_before_render)


@pytest.fixture(scope="module")
def oracle():
    from oracle import oracle as o
    o.load()
    return o


def _ctx(inst):
    return Context(inst.cfg.to_c(), 0)


def _raster_gpu(inst, fr, hair=None, depth=None):
    ctx = _ctx(inst)
    hair = hair or HairObject(inst.hair, inst.cfg.shading_points)
    rb = RasterBuffers(ctx, inst.width, inst.height)
    d = torch.as_tensor(inst.scene_depth if depth is None else depth).cuda()
    clear_before_render(ctx, rb)
    HairTilesPass(ctx).cmd_draw_hair_to_tiles(fr.uniforms, hair, d, rb)
    HairTileSortPass(ctx).cmd_sort_hair_tiles(rb)
    ctx.sync()
    return ctx, hair, rb, d


def _compare_tiles(o, inst, fr, rb):
    hb = inst.hair
    ot, osg, oc = o.tiles_pass(inst.cfg, fr.uniforms, hb.hair_data, hb.asset.positions, hb.tangents,
                               inst.scene_depth, hb.asset.strands, inst.width, inst.height, fr.max_drawn)
    gt, gsg, gc = rb.read_tiles(), rb.read_tile_segments(), rb.read_segment_counts()
    assert int(osg[0]) > 0, "workload draws nothing"
    assert int(osg[0]) < fr.max_drawn, "parity cases must not overflow the segment pool"
    assert gsg[0] == osg[0], f"drawnSegmentsCount {gsg[0]} != {osg[0]}"
    assert np.array_equal(gc, oc), "segmentCountPerTile differs"
    assert np.array_equal(gt[:, 0], ot[:, 0]), "per-bin minDepth differs"
    assert np.array_equal(gt[:, 1], ot[:, 1]), "per-bin maxDepth differs"
    assert np.array_equal(gt[:, 2] != 0, ot[:, 2] != 0), "non-empty bins differ"
    gl = walk_lists(gt, gsg, fr.max_drawn)
    ol = walk_lists(ot, osg, fr.max_drawn)
    assert gl.keys() == ol.keys()
    bad = [k for k in ol if gl[k] != ol[k]]
    assert not bad, f"{len(bad)} bins list segments in a different order"
    assert sum(len(v) for v in gl.values()) == int(gsg[0])
    return ot, osg, oc


@pytest.mark.parametrize("tile,bins", [(16, 8), (8, 32), (32, 4)])
def test_tiles_pass_bit_exact(oracle, tile, bins):
    inst = small_instance(tile_size=tile, depth_bins=bins)
    fr = frame_of(inst)
    ctx, hair, rb, _ = _raster_gpu(inst, fr)
    _compare_tiles(oracle, inst, fr, rb)


def test_tiles_pass_crowded_bins_bit_exact(oracle):
    """40,000 strands in a 192x160 viewport with 32 px tiles and 4 depth bins:
    bins of every size class the list builder sorts differently -- up to 32
    records (one warp's registers), up to 1,024 (a warp in shared memory),
    more (a block), and more than 16,384 (sorted in runs, then merged)."""
    inst = small_instance(strands=40000, width=192, height=160, tile_size=32, depth_bins=4,
                          avg_segments_per_tile=65536)
    fr = frame_of(inst)
    ctx, hair, rb, _ = _raster_gpu(inst, fr)
    ot, osg, _ = _compare_tiles(oracle, inst, fr, rb)
    n = np.array([len(v) for v in walk_lists(ot, osg, fr.max_drawn).values()])
    assert ((n > 8) & (n <= 32)).any() and ((n > 32) & (n <= 1024)).any(), "no small or medium bins"
    assert (n > 1024).sum() >= 4 and (n > 16384).any(), f"largest bin {n.max()}: the test does not test"


@pytest.mark.parametrize("entry,value", [(None, None), (2, 2e-5), (7, -2e-4), (10, 0.05), (10, 1e-12)])
def test_tiles_pass_bins_for_any_inverse_projection(oracle, entry, value):
    """The record's depth bin, the smallest over its passing pixels, is taken
    from the depths' two ends when the inverse projection's z and w rows do
    not read the pixel (a perspective projection, entry None), and pixel by
    pixel otherwise: a non-zero x / y entry of those rows, or a depth term
    in the z row large enough to round into it (entry 10 = 0.05; 1e-12
    rounds away).  Both give the oracle's bins and lists."""
    import dataclasses
    inst = small_instance(strands=1200, tile_size=8, depth_bins=32)
    fr = frame_of(inst)
    if entry is not None:
        u = bytearray(fr.uniforms)
        off = UN.OFF["projMatrixInv"] + 4 * entry
        u[off:off + 4] = np.float32(value).tobytes()
        fr = dataclasses.replace(fr, uniforms=bytes(u))
    ctx, hair, rb, _ = _raster_gpu(inst, fr)
    ot, _, _ = _compare_tiles(oracle, inst, fr, rb)
    assert len(np.unique(np.nonzero(ot[:, 2])[0] % inst.cfg.tile_depth_bins)) > 10, "too few bins in use"


def test_tiles_pass_partial_tiles_and_lod(oracle):
    # 1000x700 with 16px tiles leaves partial edge tiles; LOD renders 70%
    inst = small_instance(width=1000, height=700)
    fr = frame_of(inst)
    ctx = _ctx(inst)
    hair = HairObject(inst.hair, inst.cfg.shading_points)
    hair.lod_render_percent = 70.0
    rb = RasterBuffers(ctx, inst.width, inst.height)
    d = torch.as_tensor(inst.scene_depth).cuda()
    clear_before_render(ctx, rb)
    HairTilesPass(ctx).cmd_draw_hair_to_tiles(fr.uniforms, hair, d, rb)
    ctx.sync()
    hb = inst.hair
    n = hair.rendered_strand_count()
    assert n == 1400
    ot, osg, oc = oracle.tiles_pass(inst.cfg, fr.uniforms, hb.hair_data, hb.asset.positions, hb.tangents,
                                    inst.scene_depth, n, inst.width, inst.height, fr.max_drawn)
    assert rb.read_tile_segments()[0] == osg[0]
    assert np.array_equal(rb.read_segment_counts(), oc)
    gl = walk_lists(rb.read_tiles(), rb.read_tile_segments(), fr.max_drawn)
    assert gl == walk_lists(ot, osg, fr.max_drawn)


def test_tiles_pass_empty_and_offscreen(oracle):
    inst = small_instance(strands=50)
    # move the camera away: nothing on screen
    inst.scene.camera.eye = inst.scene.camera.eye + np.array([50.0, 0.0, 0.0])
    fr = frame_of(inst)
    ctx, hair, rb, _ = _raster_gpu(inst, fr)
    assert rb.read_tile_segments()[0] == 0
    assert not rb.read_segment_counts().any()
    assert rb.read_tile_list()[0] == 0


def test_tile_sort_bit_exact(oracle):
    inst = small_instance()
    fr = frame_of(inst)
    ctx, hair, rb, _ = _raster_gpu(inst, fr)
    ob, otl = oracle.tile_sort(inst.cfg, inst.width, inst.height, rb.read_segment_counts())
    assert np.array_equal(rb.read_sort_buckets(), ob)
    assert np.array_equal(rb.read_tile_list(), otl)


def test_tile_sort_reference_case():
    """hairTileSortPass.test.ts:25-128 through the CUDA kernel."""
    from hairfb.config import HairConfig
    cfg = HairConfig(tile_size=8, sort_buckets=8)
    ctx = Context(cfg.to_c(), 0)
    rb = RasterBuffers(ctx, 16 * 8, 1)
    seg = np.zeros(16, np.uint32)
    seg[1], seg[6], seg[2], seg[3], seg[8] = 1, 15, 16, 17, 4096
    ctx.call("hfb_buffer_upload", rb.rb.segmentCountPerTile, seg.ctypes.data, seg.nbytes)
    HairTileSortPass(ctx).cmd_sort_hair_tiles(rb)
    b = rb.read_sort_buckets()
    tl = rb.read_tile_list()
    exp = np.zeros(8, np.uint32)
    for c in seg:
        if c:
            exp[min(c // 16, 7)] += 1
    assert np.array_equal(b[0::2], exp)
    n = int(tl[0])
    buckets = [min(int(seg[t]) // 16, 7) for t in tl[1:1 + n]]
    assert n == 5 and all(buckets[i] <= buckets[i - 1] for i in range(1, n))


def _sim_inputs(inst, frame_idx=0):
    return UN.pack_sim_uniforms(inst.sim, inst.scene.model_matrix, inst.scene.sdf_bounds,
                                inst.scene.grid_bounds, frame_idx, wind_dir=inst.wind_dir,
                                wind_strength=inst.wind_strength(frame_idx))


@pytest.mark.parametrize("maker", ["small", "curly_wind", "many_strands", "odd"])
def test_grids_and_one_step_bit_exact(oracle, maker):
    """Both integration kernels: warp per strand (moderate strand counts)
    and thread per strand (many strands); "odd": 24-point strands that
    straddle warps and a point count that ends in a partial warp."""
    if maker == "small":
        inst = small_instance()
    elif maker == "odd":
        inst = small_instance(strands=1001, points=24)
    elif maker == "many_strands":
        inst = small_instance(strands=24000, points=16, iterations=3)
    else:
        inst = small_instance(strands=3000, points=32, curl=True, ellipsoid=True, wind_amplitude=1.0,
                              iterations=4, sdf_dims=64)
    hb = inst.hair
    su = _sim_inputs(inst, 7)
    ctx = _ctx(inst)
    hair = HairObject(hb, inst.cfg.shading_points)
    grids = PhysicsGrids(inst.cfg.grid_dims)
    sdf = SdfCollider(inst.sdf)
    # perturb "now" so velocities are non-zero: prev = initial, now = initial + noise
    rng = np.random.default_rng(1)
    now = hb.asset.positions.copy()
    now[:, :3] += rng.normal(0, 2e-3, now[:, :3].shape).astype(np.float32) * (now[:, 3:] > 0)
    hair.positions.copy_(torch.as_tensor(now))
    GridPostSimPass(ctx).cmd_update_grids_after_sim(su, hair, grids)
    ctx.sync()
    odv = oracle.grid_post_sim(inst.cfg, su, hb.hair_data, hb.asset.positions, now)
    assert np.array_equal(grids.density_velocity.cpu().numpy(), odv), "density/velocity grid differs"
    GridPreSimPass(ctx).cmd_update_grids_before_sim(su, grids, sdf)
    ctx.sync()
    ogw = oracle.grid_pre_sim(inst.cfg, su, odv, inst.sdf.distances, inst.sdf.dims)
    assert np.array_equal(grids.density_grad_wind.cpu().numpy().view(np.uint32), ogw.view(np.uint32))
    HairSimIntegrationPass(ctx).cmd_simulate_hair_positions(su, hair, grids, sdf)
    ctx.sync()
    onew = oracle.sim_integrate(inst.cfg, su, hb.hair_data, hb.asset.positions, now, hb.asset.positions,
                                hb.segment_lengths, odv, ogw, inst.sdf.distances, inst.sdf.dims)
    g = hair.positions.cpu().numpy()
    assert np.array_equal(g.view(np.uint32), onew.view(np.uint32)), \
        f"max abs diff {np.abs(g - onew).max()}"


def test_density_grid_wraps_like_the_reference(oracle):
    """10,000 x 32 strands on a 32^3 grid overflow the reference's i32
    fixed-point density (atomicAdd<i32> of i32(w * 1e6) wraps): the CUDA splat
    wraps identically (two's complement), node for node."""
    from hairfb import synthetic
    inst = synthetic.plain_full(grid_dims=32)
    hb = inst.hair
    su = _sim_inputs(inst, 0)
    ctx = _ctx(inst)
    hair = HairObject(hb, inst.cfg.shading_points)
    grids = PhysicsGrids(inst.cfg.grid_dims)
    GridPostSimPass(ctx).cmd_update_grids_after_sim(su, hair, grids)
    ctx.sync()
    o = oracle.grid_post_sim(inst.cfg, su, hb.hair_data, hb.asset.positions, hb.asset.positions)
    assert (o[:, 3] < 0).sum() > 0, "no node wrapped: the case does not test the overflow"
    assert np.array_equal(grids.density_velocity.cpu().numpy(), o)


@pytest.mark.parametrize("order", ["identity", "reversed", "random"])
def test_grid_splat_does_not_depend_on_strand_order(oracle, order):
    """The grid splat visits the strands in a given order (Morton order of
    the roots by default): the identity, a reversed and a random order give
    the oracle's grid bit for bit."""
    from hairfb.passes import _dev
    inst = small_instance(strands=5000, points=24)
    hb = inst.hair
    su = _sim_inputs(inst, 3)
    ctx = _ctx(inst)
    hair = HairObject(hb, inst.cfg.shading_points)
    grids = PhysicsGrids(inst.cfg.grid_dims)
    rng = np.random.default_rng(4)
    now = hb.asset.positions.copy()
    now[:, :3] += rng.normal(0, 2e-3, now[:, :3].shape).astype(np.float32) * (now[:, 3:] > 0)
    hair.positions.copy_(torch.as_tensor(now))
    S = hb.asset.strands
    perm = {"identity": np.arange(S), "reversed": np.arange(S)[::-1],
            "random": rng.permutation(S)}[order].astype(np.int32)
    from hairfb.lib import byref, ptr
    ctx.call("hfb_grid_post_sim_ordered", ctypes_ub(su), byref(hair.hair_data), ptr(hair.positions_prev),
             ptr(hair.positions), ptr(grids.density_velocity), ptr(_dev(perm)))
    ctx.sync()
    odv = oracle.grid_post_sim(inst.cfg, su, hb.hair_data, hb.asset.positions, now)
    assert np.array_equal(grids.density_velocity.cpu().numpy(), odv)
    # the default (Morton) order and the unordered entry point agree too
    morton = PhysicsGrids(inst.cfg.grid_dims)
    GridPostSimPass(ctx).cmd_update_grids_after_sim(su, hair, morton)
    plain = PhysicsGrids(inst.cfg.grid_dims)
    ctx.call("hfb_grid_post_sim", ctypes_ub(su), byref(hair.hair_data), ptr(hair.positions_prev),
             ptr(hair.positions), ptr(plain.density_velocity))
    ctx.sync()
    assert np.array_equal(morton.density_velocity.cpu().numpy(), odv)
    assert np.array_equal(plain.density_velocity.cpu().numpy(), odv)


def ctypes_ub(b: bytes):
    from hairfb.passes import _ub
    return _ub(b)


def test_simulation_60_steps(oracle):
    inst = small_instance(strands=1500, points=24, curl=True, wind_amplitude=1.0, iterations=4)
    hb = inst.hair
    ctx = _ctx(inst)
    hair = HairObject(hb, inst.cfg.shading_points)
    grids = PhysicsGrids(inst.cfg.grid_dims)
    sdf = SdfCollider(inst.sdf)
    pre, integ, post = GridPreSimPass(ctx), HairSimIntegrationPass(ctx), GridPostSimPass(ctx)
    # oracle state
    o_prev = hb.asset.positions.copy()
    o_now = hb.asset.positions.copy()
    o_dv = oracle.grid_post_sim(inst.cfg, _sim_inputs(inst, 0), hb.hair_data, o_prev, o_now)
    post.cmd_update_grids_after_sim(_sim_inputs(inst, 0), hair, grids)
    for f in range(60):
        su = _sim_inputs(inst, f)
        pre.cmd_update_grids_before_sim(su, grids, sdf)
        integ.cmd_simulate_hair_positions(su, hair, grids, sdf)
        post.cmd_update_grids_after_sim(su, hair, grids)
        o_gw = oracle.grid_pre_sim(inst.cfg, su, o_dv, inst.sdf.distances, inst.sdf.dims)
        o_new = oracle.sim_integrate(inst.cfg, su, hb.hair_data, o_prev, o_now, hb.asset.positions,
                                     hb.segment_lengths, o_dv, o_gw, inst.sdf.distances, inst.sdf.dims)
        o_prev, o_now = o_now, o_new
        o_dv = oracle.grid_post_sim(inst.cfg, su, hb.hair_data, o_prev, o_now)
    ctx.sync()
    g = hair.positions.cpu().numpy()[:, :3].astype(np.float64)
    o = o_now[:, :3].astype(np.float64)
    moved = np.abs(o - hb.asset.positions[:, :3]).max()
    assert moved > 1e-4, "the simulation did not move the hair"
    rel = np.abs(g - o).max() / np.abs(o).max()
    assert rel <= 1e-5, f"relative position error {rel:.3g} after 60 steps"


def test_shading_parity(oracle):
    inst = small_instance()
    fr = frame_of(inst)
    hb = inst.hair
    ctx = _ctx(inst)
    hair = HairObject(hb, inst.cfg.shading_points)
    # depth buffer slightly behind the hair so attenuation stays in range
    depth = np.full(inst.width * inst.height, 0.9995, np.float32)
    d = torch.as_tensor(depth).cuda()
    ao = np.linspace(0.2, 1.0, 160 * 120, dtype=np.float32)
    HairShadingPass(ctx).cmd_compute_shading_points(fr.uniforms, hair, d, torch.as_tensor(ao).cuda(), (160, 120))
    ctx.sync()
    o = oracle.shading(inst.cfg, fr.uniforms, hb.hair_data, hb.asset.positions, hb.tangents, depth,
                       hb.asset.strands, ao=ao, ao_size=(160, 120))
    g = hair.shading.cpu().numpy()
    assert np.isfinite(g).all()
    assert np.abs(o).max() > 1e-3, "shading is all black: bad test input"
    err = np.abs(g - o)
    assert (err <= 1e-5 + 1e-5 * np.abs(o)).all(), f"max shading error {err.max():.3g}"


def test_shading_parity_with_shadow_map(oracle):
    inst = small_instance(strands=300)
    inst.scene.use_pcss = True
    fr = frame_of(inst)
    hb = inst.hair
    ctx = _ctx(inst)
    hair = HairObject(hb, inst.cfg.shading_points)
    depth = np.full(inst.width * inst.height, 0.9995, np.float32)
    rng = np.random.default_rng(3)
    sm = rng.uniform(0.3, 1.0, 256 * 256).astype(np.float32)
    HairShadingPass(ctx).cmd_compute_shading_points(fr.uniforms, hair, torch.as_tensor(depth).cuda(),
                                                    shadow_map=torch.as_tensor(sm).cuda(), shadow_size=256)
    ctx.sync()
    o = oracle.shading(inst.cfg, fr.uniforms, hb.hair_data, hb.asset.positions, hb.tangents, depth,
                       hb.asset.strands, shadow_map=sm, shadow_size=256)
    g = hair.shading.cpu().numpy()
    err = np.abs(g - o)
    assert (err <= 1e-5 + 1e-5 * np.abs(o)).all(), f"max shading error {err.max():.3g}"


def _shading_input(inst):
    """Non-trivial strand colours for the fine pass (shared by both sides)."""
    rng = np.random.default_rng(5)
    S, SP = inst.hair.asset.strands, inst.cfg.shading_points
    c = rng.uniform(0.05, 1.0, (S * SP, 4)).astype(np.float32)
    c[:, 3] = 1.0
    c.reshape(S, SP, 4)[:, -1, 3] = 0.0
    return c


@pytest.mark.parametrize("tile,bins,slices", [(16, 8, 4), (8, 16, 8), (32, 4, 4)])
def test_fine_pass_within_1_255(oracle, tile, bins, slices):
    inst = small_instance(tile_size=tile, depth_bins=bins, slices=slices)
    fr = frame_of(inst)
    ctx, hair, rb, d = _raster_gpu(inst, fr)
    shade = _shading_input(inst)
    hair.shading.copy_(torch.as_tensor(shade))
    HairFinePass(ctx).cmd_rasterize_slices_hair(fr.uniforms, hair, d, rb)
    ctx.sync()
    hb = inst.hair
    ot, osg, oc = oracle.tiles_pass(inst.cfg, fr.uniforms, hb.hair_data, hb.asset.positions, hb.tangents,
                                    inst.scene_depth, hb.asset.strands, inst.width, inst.height, fr.max_drawn)
    ob, otl = oracle.tile_sort(inst.cfg, inst.width, inst.height, oc)
    ores = oracle.fine_pass(inst.cfg, fr.uniforms, hb.hair_data, hb.asset.positions, hb.tangents, shade,
                            inst.scene_depth, ot, osg, otl, inst.width, inst.height)
    g = rb.read_result()[4:].reshape(-1, 4)
    o = ores[4:].reshape(-1, 4)
    assert (o[:, 3] > 0).sum() > 1000, "too few covered pixels for a meaningful test"
    err = np.abs(g - o)
    assert err.max() <= 1.0 / 255.0, f"max pixel error {err.max():.4g} (> 1/255) at {np.argmax(err.max(1))}"
    assert np.array_equal(g[:, 3] > 0, o[:, 3] > 0), "coverage differs"


def test_fine_pass_pool_capacity(oracle):
    """A tiny fragment pool forces the list walk to stop early, exactly as the
    reference's PPLL-full break does."""
    inst = small_instance(strands=4000, tile_size=16, depth_bins=2, slices=2)
    inst.cfg.avg_fragments_per_slice = 1  # 1 * 2 * 256 = 512 fragments per bin
    fr = frame_of(inst)
    ctx, hair, rb, d = _raster_gpu(inst, fr)
    shade = _shading_input(inst)
    hair.shading.copy_(torch.as_tensor(shade))
    HairFinePass(ctx).cmd_rasterize_slices_hair(fr.uniforms, hair, d, rb)
    ctx.sync()
    assert ctx.counters()["finePoolFullBins"] > 0, "the pool never filled: the test does not test"
    hb = inst.hair
    ot, osg, oc = oracle.tiles_pass(inst.cfg, fr.uniforms, hb.hair_data, hb.asset.positions, hb.tangents,
                                    inst.scene_depth, hb.asset.strands, inst.width, inst.height, fr.max_drawn)
    ob, otl = oracle.tile_sort(inst.cfg, inst.width, inst.height, oc)
    ores = oracle.fine_pass(inst.cfg, fr.uniforms, hb.hair_data, hb.asset.positions, hb.tangents, shade,
                            inst.scene_depth, ot, osg, otl, inst.width, inst.height)
    err = np.abs(rb.read_result()[4:] - ores[4:])
    assert err.max() <= 1.0 / 255.0, f"max pixel error {err.max():.4g}"


def _fine_vs_oracle(oracle, inst):
    fr = frame_of(inst)
    ctx, hair, rb, d = _raster_gpu(inst, fr)
    shade = _shading_input(inst)
    hair.shading.copy_(torch.as_tensor(shade))
    HairFinePass(ctx).cmd_rasterize_slices_hair(fr.uniforms, hair, d, rb)
    ctx.sync()
    hb = inst.hair
    ot, osg, oc = oracle.tiles_pass(inst.cfg, fr.uniforms, hb.hair_data, hb.asset.positions, hb.tangents,
                                    inst.scene_depth, hb.asset.strands, inst.width, inst.height, fr.max_drawn)
    ob, otl = oracle.tile_sort(inst.cfg, inst.width, inst.height, oc)
    ores = oracle.fine_pass(inst.cfg, fr.uniforms, hb.hair_data, hb.asset.positions, hb.tangents, shade,
                            inst.scene_depth, ot, osg, otl, inst.width, inst.height)
    g = rb.read_result()[4:].reshape(-1, 4)
    o = ores[4:].reshape(-1, 4)
    return ctx.counters(), g, o


def test_fine_pass_split_tiles(oracle):
    """Dense tiles (far more records than a CTA's share) are split into
    groups of depth bins on several CTAs and merged front to back."""
    inst = small_instance(strands=6000, points=32, width=320, height=240, depth_bins=16, slices=4)
    cnt, g, o = _fine_vs_oracle(oracle, inst)
    assert cnt["fineSplitTiles"] > 0, "no tile was split: the test does not test"
    assert cnt["fineSplitRedone"] == 0
    err = np.abs(g - o)
    assert err.max() <= 1.0 / 255.0, f"max pixel error {err.max():.4g} (> 1/255)"
    assert np.array_equal(g[:, 3] > 0, o[:, 3] > 0), "coverage differs"


def test_fine_pass_split_tiles_with_full_pools(oracle):
    """A split tile whose later group could fill a fragment pool is redone in
    order by one CTA, so the pool's cut stays the reference's."""
    inst = small_instance(strands=6000, points=32, width=320, height=240, depth_bins=4, slices=2)
    inst.cfg.avg_fragments_per_slice = 1  # 1 * 2 * 256 = 512 fragments per bin
    cnt, g, o = _fine_vs_oracle(oracle, inst)
    assert cnt["fineSplitTiles"] > 0 and cnt["fineSplitRedone"] > 0, cnt
    assert cnt["finePoolFullBins"] > 0, cnt
    err = np.abs(g - o)
    assert err.max() <= 1.0 / 255.0, f"max pixel error {err.max():.4g} (> 1/255)"


@pytest.mark.parametrize("strands,width,height", [(300, 320, 240), (400, 512, 512)])
def test_fine_schedule_items_match_the_tile_list(oracle, strands, width, height):
    """Without split tiles the fine pass's work list holds exactly one item
    per drawn tile (the schedule once counted the idle threads of its last
    1024-entry chunk as items, and the fine pass read them from stale
    scratch memory)."""
    inst = small_instance(strands=strands, width=width, height=height)
    fr = frame_of(inst)
    ctx, hair, rb, d = _raster_gpu(inst, fr)
    hair.shading.copy_(torch.as_tensor(_shading_input(inst)))
    HairFinePass(ctx).cmd_rasterize_slices_hair(fr.uniforms, hair, d, rb)
    ctx.sync()
    cnt = ctx.counters()
    assert cnt["fineSplitTiles"] == 0, "the case splits tiles: the item count is not the tile count"
    drawn = int(rb.read_tile_list()[0])
    assert 0 < drawn < rb.tile_count() and drawn % 1024 != 0, drawn
    items = int(rb._download(rb.rb.scratch, 1, np.uint32)[0])  # the fine scratch header: [0] = work items
    assert items == drawn, (items, drawn)
    assert cnt["badWorkItems"] == 0


def test_fine_pass_reads_arbitrary_list_order(oracle):
    """The fine pass walks whatever list it is given: feed it the oracle's
    LIFO lists (not the tiles pass's contiguous layout)."""
    inst = small_instance(strands=1000)
    fr = frame_of(inst)
    hb = inst.hair
    ot, osg, oc = oracle.tiles_pass(inst.cfg, fr.uniforms, hb.hair_data, hb.asset.positions, hb.tangents,
                                    inst.scene_depth, hb.asset.strands, inst.width, inst.height, fr.max_drawn)
    ob, otl = oracle.tile_sort(inst.cfg, inst.width, inst.height, oc)
    shade = _shading_input(inst)
    ctx = _ctx(inst)
    hair = HairObject(hb, inst.cfg.shading_points)
    hair.shading.copy_(torch.as_tensor(shade))
    rb = RasterBuffers(ctx, inst.width, inst.height)
    clear_before_render(ctx, rb)
    for addr, arr in ((rb.rb.tiles, ot), (rb.rb.tileSegments, osg), (rb.rb.tileList, otl)):
        a = np.ascontiguousarray(arr)
        ctx.call("hfb_buffer_upload", addr, a.ctypes.data, a.nbytes)
    d = torch.as_tensor(inst.scene_depth).cuda()
    HairFinePass(ctx).cmd_rasterize_slices_hair(fr.uniforms, hair, d, rb)
    ctx.sync()
    ores = oracle.fine_pass(inst.cfg, fr.uniforms, hb.hair_data, hb.asset.positions, hb.tangents, shade,
                            inst.scene_depth, ot, osg, otl, inst.width, inst.height)
    err = np.abs(rb.read_result()[4:] - ores[4:])
    assert err.max() <= 1.0 / 255.0


def test_fine_pass_debug_slices_mode(oracle):
    """displayMode USED_SLICES: the result counts fragments per pixel."""
    inst = small_instance(strands=800)
    inst.scene.display_mode = UN.DISPLAY_MODE_USED_SLICES
    inst.scene.display_mode_extra = 50
    fr = frame_of(inst)
    ctx, hair, rb, d = _raster_gpu(inst, fr)
    shade = _shading_input(inst)
    hair.shading.copy_(torch.as_tensor(shade))
    HairFinePass(ctx).cmd_rasterize_slices_hair(fr.uniforms, hair, d, rb)
    ctx.sync()
    hb = inst.hair
    ot, osg, oc = oracle.tiles_pass(inst.cfg, fr.uniforms, hb.hair_data, hb.asset.positions, hb.tangents,
                                    inst.scene_depth, hb.asset.strands, inst.width, inst.height, fr.max_drawn)
    ob, otl = oracle.tile_sort(inst.cfg, inst.width, inst.height, oc)
    ores = oracle.fine_pass(inst.cfg, fr.uniforms, hb.hair_data, hb.asset.positions, hb.tangents, shade,
                            inst.scene_depth, ot, osg, otl, inst.width, inst.height)
    assert np.array_equal(rb.read_result()[4:], ores[4:])


def test_constant_division_forms_equal_ieee_division():
    """The simulation divides by 3 and 1e6 as correctly rounded multiplications
    by the reciprocal; over all 2^32 inputs they equal the device's IEEE
    division bit for bit (x / 3 for every non-NaN x, (float)v / 1e6 for every
    int32 v, x / 1e6 for every finite |x| >= 2^-92)."""
    ctx = _ctx(small_instance(strands=10))
    out = (ctypes.c_uint64 * 3)()
    ctx.call("hfb_check_constant_division", out)
    assert list(out) == [0, 0, 0]
    ctx.close()


def test_invalid_arguments_return_errors():
    from hairfb.lib import HfbError
    inst = small_instance(strands=10)
    fr = frame_of(inst)
    ctx = _ctx(inst)
    hair = HairObject(inst.hair, inst.cfg.shading_points)
    rb = RasterBuffers(ctx, 320, 240)  # viewport does not match the uniforms
    d = torch.zeros(320 * 240, device="cuda")
    with pytest.raises(HfbError) as e:
        HairTilesPass(ctx).cmd_draw_hair_to_tiles(fr.uniforms, hair, d, rb)
    assert "viewport" in str(e.value)
    misaligned = torch.zeros(4 * 100 + 1, device="cuda")[1:]
    with pytest.raises(HfbError):
        ctx.call("hfb_grid_post_sim", None, None, misaligned.data_ptr(), misaligned.data_ptr(),
                 misaligned.data_ptr())
    # the later passes: NULL buffers, a viewport that does not match, a bad AO scale
    from hairfb.passes import _ub
    with pytest.raises(HfbError) as e:
        ctx.call("hfb_present", _ub(fr.uniforms), byref(rb.rb), None, None)
    assert "NULL" in str(e.value)
    with pytest.raises(HfbError) as e:
        ctx.call("hfb_hair_depth", _ub(fr.uniforms), byref(hair.hair_data), ptr(hair.positions), ptr(hair.tangents),
                 hair.rendered_strand_count(), ptr(d), ptr(d), byref(rb.rb))
    assert "viewport" in str(e.value)
    with pytest.raises(HfbError) as e:
        ctx.call("hfb_gtao", _ub(fr.uniforms), ptr(d), ptr(d), ctypes.c_float(0.0), ptr(d))
    assert "scale" in str(e.value)
    ctx.sync()  # the context stays usable


@pytest.mark.parametrize("kw,lod", [(dict(), 100.0), (dict(width=1000, height=700), 70.0),
                                    (dict(strands=300, fiber_radius=0.02), 100.0)])
def test_hair_depth_bit_exact(oracle, kw, lod):
    """HwHairPass's depth (hfb_hair_depth) against the oracle, bit for bit:
    the 2,000-strand case, partial edge tiles with LOD, and quads wide enough
    (fiber radius 0.02) that their triangles take the block-per-triangle path."""
    from hairfb.passes import HwHairPass
    inst = small_instance(**kw)
    fr = frame_of(inst)
    ctx = _ctx(inst)
    hair = HairObject(inst.hair, inst.cfg.shading_points)
    hair.lod_render_percent = lod
    rb = RasterBuffers(ctx, inst.width, inst.height)
    scene = torch.as_tensor(inst.scene_depth).cuda()
    out = torch.empty_like(scene)
    HwHairPass(ctx).cmd_draw_hair_depth(fr.uniforms, hair, scene, out, rb)
    ctx.sync()
    o = oracle.hair_depth(fr.uniforms, inst.hair.hair_data, inst.hair.asset.positions, inst.hair.tangents,
                          hair.rendered_strand_count(), inst.scene_depth)
    g = out.cpu().numpy()
    assert (o < inst.scene_depth).sum() > 100, "the hair covers nothing: the case does not test"
    assert np.array_equal(g.view(np.uint32), o.view(np.uint32)), f"{int((g != o).sum())} pixels differ"


def test_hair_depth_exploded_strands_bit_exact(oracle):
    """Points thrown far apart (as a simulation that blows up leaves them):
    long segments whose triangles cover large parts of the viewport take the
    block-per-triangle path and its row spans; still bit-exact."""
    from hairfb.passes import HwHairPass
    inst = small_instance(strands=400, points=16)
    fr = frame_of(inst)
    ctx = _ctx(inst)
    hair = HairObject(inst.hair, inst.cfg.shading_points)
    rng = np.random.default_rng(9)
    pos = inst.hair.asset.positions.copy()
    far = rng.random(len(pos)) < 0.05
    pos[far, :3] += rng.normal(0, 0.3, (int(far.sum()), 3)).astype(np.float32)
    hair.positions.copy_(torch.as_tensor(pos))
    rb = RasterBuffers(ctx, inst.width, inst.height)
    scene = torch.as_tensor(inst.scene_depth).cuda()
    out = torch.empty_like(scene)
    HwHairPass(ctx).cmd_draw_hair_depth(fr.uniforms, hair, scene, out, rb)
    ctx.sync()
    o = oracle.hair_depth(fr.uniforms, inst.hair.hair_data, pos, inst.hair.tangents, inst.hair.asset.strands,
                          inst.scene_depth)
    g = out.cpu().numpy()
    assert (o < inst.scene_depth).sum() > 20000, "the long segments cover little: the case does not test"
    assert np.array_equal(g.view(np.uint32), o.view(np.uint32)), f"{int((g != o).sum())} pixels differ"


@pytest.mark.parametrize("tile", [8, 16])
def test_tiles_and_fine_pass_exploded_strands(oracle, tile):
    """Points thrown far apart, some of them next to and behind the camera:
    long segments across many tiles, quads with huge or non-finite projected
    corners, edges nearly parallel to the rows.  The tiles pass stays
    bit-exact and the fine pass (whose edge tests list each box row's
    passing interval) within 1/255."""
    inst = small_instance(strands=1000, points=16, tile_size=tile, depth_bins=8)
    fr = frame_of(inst)
    rng = np.random.default_rng(11)
    pos = inst.hair.asset.positions.copy()
    far = rng.random(len(pos)) < 0.05
    pos[far, :3] += rng.normal(0, 0.3, (int(far.sum()), 3)).astype(np.float32)
    eye = np.asarray(inst.scene.camera.eye, np.float32)
    near = np.nonzero(rng.random(len(pos)) < 0.004)[0]
    pos[near, :3] = eye + rng.normal(0, 0.02, (len(near), 3)).astype(np.float32)
    hair = HairObject(inst.hair, inst.cfg.shading_points)
    hair.positions.copy_(torch.as_tensor(pos))
    ctx, hair, rb, d = _raster_gpu(inst, fr, hair=hair)
    hb = inst.hair
    ot, osg, oc = oracle.tiles_pass(inst.cfg, fr.uniforms, hb.hair_data, pos, hb.tangents, inst.scene_depth,
                                    hb.asset.strands, inst.width, inst.height, fr.max_drawn)
    gt, gsg = rb.read_tiles(), rb.read_tile_segments()
    assert int(osg[0]) > 0 and gsg[0] == osg[0] and int(osg[0]) < fr.max_drawn
    assert np.array_equal(rb.read_segment_counts(), oc)
    assert np.array_equal(gt[:, :2], ot[:, :2])
    assert walk_lists(gt, gsg, fr.max_drawn) == walk_lists(ot, osg, fr.max_drawn)
    shade = _shading_input(inst)
    hair.shading.copy_(torch.as_tensor(shade))
    HairFinePass(ctx).cmd_rasterize_slices_hair(fr.uniforms, hair, d, rb)
    ctx.sync()
    _, otl = oracle.tile_sort(inst.cfg, inst.width, inst.height, oc)
    ores = oracle.fine_pass(inst.cfg, fr.uniforms, hb.hair_data, pos, hb.tangents, shade, inst.scene_depth, ot, osg,
                            otl, inst.width, inst.height)
    g = rb.read_result()[4:].reshape(-1, 4)
    o = ores[4:].reshape(-1, 4)
    assert (o[:, 3] > 0).sum() > 15000, "the frame covers little: the case does not test"
    assert np.abs(g - o).max() <= 1.0 / 255.0
    assert np.array_equal(g[:, 3] > 0, o[:, 3] > 0), "coverage differs"


@pytest.mark.parametrize("scene", [False, True])
def test_present_within_1_255(oracle, scene, tmp_path):
    """HairCombinePass + PresentPass on a rendered frame (over black, and over
    a scene colour image): every channel within 1 of the oracle's unorm8
    (pow is not correctly rounded on either side); the image is written as
    a PNG."""
    from hairfb import formats
    from hairfb.passes import PresentPass
    from hairfb.renderer import Renderer
    inst = small_instance(strands=1500)
    r = Renderer(inst, 0, hair_depth=True)
    r.before_first_frame()
    r.frame()
    r.frame()
    rng = np.random.default_rng(1)
    sc = rng.uniform(0.0, 2.0, (inst.height, inst.width, 4)).astype(np.float32) if scene else None
    img = PresentPass(r.ctx).cmd_draw(r.uniforms, r.rb, torch.as_tensor(sc).cuda() if scene else None)
    r.ctx.sync()
    g = img.cpu().numpy()
    o = oracle.present(r.uniforms, r.rb.read_result()[4:], sc)
    assert g.shape == o.shape == (inst.height, inst.width, 4)
    diff = np.abs(g.astype(np.int32) - o.astype(np.int32))
    assert diff.max() <= 1, f"max difference {diff.max()} at {np.unravel_index(diff.argmax(), diff.shape)}"
    assert (g[..., 3] == 255).all()
    assert len(np.unique(g[..., :3].reshape(-1, 3), axis=0)) > 50, "a flat image: the case does not test"
    png = formats.write_png(g)
    (tmp_path / "frame.png").write_bytes(png)
    assert png[:8] == b"\x89PNG\r\n\x1a\n"


def test_present_batch_equals_present():
    """hfb_present_batch: three rendered frames of different viewports, one
    over a scene colour image, in one launch; each image equals hfb_present's
    on the same arguments, byte for byte."""
    from hairfb.lib import HfbError
    from hairfb.passes import PresentPass
    from hairfb.renderer import Renderer
    rng = np.random.default_rng(2)
    items = []
    ctx = None
    for k, (w, h, scene) in enumerate([(320, 240, False), (200, 150, True), (97, 61, False)]):
        inst = small_instance(seed=k, strands=600, width=w, height=h)
        r = Renderer(inst, 0, ctx=ctx)
        ctx = r.ctx
        r.before_first_frame()
        r.frame()
        sc = torch.as_tensor(rng.uniform(0.0, 2.0, (h, w, 4)).astype(np.float32)).cuda() if scene else None
        alone = PresentPass(ctx).cmd_draw(r.uniforms, r.rb, sc)
        items.append((r, sc, alone, torch.zeros_like(alone)))
    PresentPass(ctx).cmd_draw_batch([(r.uniforms, r.rb, sc, out) for r, sc, _, out in items])
    ctx.sync()
    for k, (r, sc, alone, batched) in enumerate(items):
        a, b = alone.cpu().numpy(), batched.cpu().numpy()
        assert len(np.unique(a[..., :3].reshape(-1, 3), axis=0)) > 20, f"image {k} is flat: the case does not test"
        assert np.array_equal(a, b), f"image {k}: {(a != b).any(-1).sum()} pixels differ"
    with pytest.raises(HfbError, match="item 1"):
        PresentPass(ctx).cmd_draw_batch([(items[0][0].uniforms, items[0][0].rb, None, items[0][3]),
                                         (items[0][0].uniforms, items[1][0].rb, None, items[1][3])])


@pytest.mark.parametrize("kw", [dict(), dict(strands=300, fiber_radius=0.02)])
def test_hair_normals_and_gtao(oracle, kw):
    """HwHairPass's normals (bit-exact: the winner of each pixel, the
    perspective-correct tangent, the f16 octahedron encoding) and GTAO on
    the hair depth and those normals (the transcendentals differ by an ulp
    or so, which can move a sample by a pixel: nearly every texel within
    4e-3, the mean far below)."""
    from hairfb.passes import AoPass, HwHairPass
    inst = small_instance(**kw)
    fr = frame_of(inst)
    ctx = _ctx(inst)
    hair = HairObject(inst.hair, inst.cfg.shading_points)
    rb = RasterBuffers(ctx, inst.width, inst.height)
    scene = torch.as_tensor(inst.scene_depth).cuda()
    hd = torch.empty_like(scene)
    hw = HwHairPass(ctx)
    hw.cmd_draw_hair_depth(fr.uniforms, hair, scene, hd, rb)
    rng = np.random.default_rng(6)
    base = rng.uniform(0.0, 1.0, (inst.width * inst.height, 2)).astype(np.float32)  # the scene's normals
    normals = torch.as_tensor(base).cuda()
    hw.cmd_draw_hair_normals(fr.uniforms, hair, hd, normals, rb)
    ctx.sync()
    hdn = hd.cpu().numpy()
    on = oracle.hair_normals(fr.uniforms, inst.hair.hair_data, inst.hair.asset.positions, inst.hair.tangents,
                             inst.hair.asset.strands, hdn, base)
    gn = normals.cpu().numpy()
    changed = (on != base).any(1)
    assert changed.sum() > 1000, "few hair pixels: the case does not test"
    assert np.array_equal(gn.view(np.uint32), on.view(np.uint32)), f"{int((gn != on).any(1).sum())} normals differ"
    ao = AoPass(ctx).cmd_calc_ao(fr.uniforms, hd, normals, inst.width, inst.height)
    ctx.sync()
    oao = oracle.gtao(fr.uniforms, hdn, on)
    g = ao.cpu().numpy()
    assert g.shape == oao.shape and np.isfinite(oao).all() and np.isfinite(g).all()
    assert np.abs(oao).max() > 0.05, "no occlusion anywhere: the case does not test"
    err = np.abs(g - oao)
    assert (err <= 4e-3).mean() >= 0.995 and err.mean() < 1e-3, (float(err.max()), float(err.mean()))


def test_frame_with_ao_matches_the_oracle_chain(oracle):
    """A frame with the hair depth, the hair's normals and GTAO before the
    shading (Renderer(ao=True)): the oracle's chain on the frame's positions
    (hair depth, normals, GTAO, shading with that AO) gives the same shading
    within 1e-5 where the GPU and oracle AO agree."""
    from hairfb.renderer import Renderer
    inst = small_instance(strands=1500)
    r = Renderer(inst, 0, hair_depth=True, ao=True)
    r.before_first_frame()
    r.frame()
    r.ctx.sync()
    pos = r.hair.positions.cpu().numpy()
    tan = r.hair.tangents.cpu().numpy()
    hb = inst.hair
    od = oracle.hair_depth(r.uniforms, hb.hair_data, pos, tan, hb.asset.strands, inst.scene_depth)
    assert np.array_equal(r.hair_depth.cpu().numpy().view(np.uint32), od.view(np.uint32))
    on = oracle.hair_normals(r.uniforms, hb.hair_data, pos, tan, hb.asset.strands, od)
    assert np.array_equal(r.normals.cpu().numpy().view(np.uint32), on.view(np.uint32))
    gao = r.ao.cpu().numpy()
    oao = oracle.gtao(r.uniforms, od, on)
    assert (np.abs(gao - oao) <= 4e-3).mean() >= 0.995
    # the shading on the GPU's AO (the AO's own tolerance is checked above)
    osh = oracle.shading(inst.cfg, r.uniforms, hb.hair_data, pos, tan, od, hb.asset.strands, ao=gao.reshape(-1),
                         ao_size=(gao.shape[1], gao.shape[0]))
    g = r.hair.shading.cpu().numpy()
    assert np.allclose(g, osh, rtol=1e-5, atol=1e-5), float(np.abs(g - osh).max())


def test_shading_reads_the_hair_depth(oracle):
    """A frame with the hair depth prepass: the depth it leaves is the
    oracle's for the frame's positions, and the shading computed from it
    matches the oracle's shading on that depth."""
    from hairfb.renderer import Renderer
    inst = small_instance(strands=1500)
    r = Renderer(inst, 0, hair_depth=True)
    r.before_first_frame()
    r.frame()
    torch.cuda.synchronize()
    pos = r.hair.positions.cpu().numpy()
    tan = r.hair.tangents.cpu().numpy()
    o = oracle.hair_depth(r.uniforms, inst.hair.hair_data, pos, tan, inst.hair.asset.strands, inst.scene_depth)
    assert (o < inst.scene_depth).sum() > 100
    assert np.array_equal(r.hair_depth.cpu().numpy().view(np.uint32), o.view(np.uint32))
    osh = oracle.shading(inst.cfg, r.uniforms, inst.hair.hair_data, pos, tan, o, inst.hair.asset.strands)
    g = r.hair.shading.cpu().numpy()
    assert np.allclose(g, osh, rtol=1e-5, atol=1e-5), float(np.abs(g - osh).max())
