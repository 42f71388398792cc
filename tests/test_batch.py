"""Whole frames: hfb_frame (one instance, one call) and hfb_frame_batch (many
instances, one persistent launch per pass, replayed as a captured CUDA
graph) against the pass-by-pass path on the same instances.

Bars: positions, density grid, tile counts, per-bin depth bounds, lists and
the tile list bit-exact (the same kernels run the same arithmetic);
shading within 1e-6; pixels within 1/255.
"""

import numpy as np
import pytest

from helpers import walk_lists

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

from hairfb import synthetic  # noqa: E402
import ctypes  # noqa: E402

from hairfb.lib import Context, HfbInstance  # noqa: E402
from hairfb.renderer import BatchRenderer, Renderer  # noqa: E402


def _instances(seed=3):
    rng = np.random.Generator(np.random.PCG64(seed))
    common = dict(tile_size=16, depth_bins=8, slices=4, shading_points=8, grid_dims=32, iterations=4,
                  wind_amplitude=1.0)
    return [synthetic.make_instance(rng, strands=1500, points=16, width=320, height=240, **common),
            synthetic.make_instance(rng, strands=600, points=24, width=256, height=256, curl=True, **common),
            synthetic.make_instance(rng, strands=2500, points=32, width=512, height=384, **common)]


def _state(r: Renderer):
    rb = r.rb
    return dict(pos=r.hair.positions.cpu().numpy(), dv=r.grids.density_velocity.cpu().numpy(),
                shading=r.hair.shading.cpu().numpy(), tiles=rb.read_tiles(),
                counts=rb.read_segment_counts(), segs=rb.read_tile_segments(), tl=rb.read_tile_list(),
                px=rb.read_result()[4:].reshape(-1, 4))


def _compare(a, b, r: Renderer, frame):
    tag = f"frame {frame}"
    assert np.array_equal(a["pos"], b["pos"]), f"{tag}: positions differ"
    assert np.array_equal(a["dv"], b["dv"]), f"{tag}: density grid differs"
    assert np.array_equal(a["counts"], b["counts"]), f"{tag}: segment counts differ"
    ta, tb = a["tiles"].reshape(-1, 4), b["tiles"].reshape(-1, 4)
    assert np.array_equal(ta[:, :2], tb[:, :2]), f"{tag}: depth bounds differ"
    md = r.rb.max_drawn_segments
    assert a["segs"][0] == b["segs"][0], f"{tag}: drawnSegmentsCount differs"
    assert walk_lists(ta, a["segs"], md) == walk_lists(tb, b["segs"], md), f"{tag}: lists differ"
    n = int(a["tl"][0])
    assert n == int(b["tl"][0]) and np.array_equal(a["tl"][1:1 + n], b["tl"][1:1 + n]), f"{tag}: tile list"
    assert np.abs(a["shading"] - b["shading"]).max() <= 1e-6, f"{tag}: shading differs"
    err = np.abs(a["px"] - b["px"]).max()
    assert err <= 1.0 / 255.0, f"{tag}: pixel error {err:.4g}"


@pytest.mark.parametrize("hair_depth", [False, True])
def test_frame_matches_pass_by_pass(hair_depth):
    insts = _instances()
    for inst in insts:
        ref = Renderer(inst, 0, hair_depth=hair_depth)
        nat = Renderer(inst, 0, hair_depth=hair_depth)
        ref.before_first_frame()
        nat.before_first_frame()
        for f in range(3):
            ref.frame()
            nat.frame_native()
            torch.cuda.synchronize()
            _compare(_state(ref), _state(nat), ref, f)
            if hair_depth:
                assert np.array_equal(ref.hair_depth.cpu().numpy(), nat.hair_depth.cpu().numpy()), f"frame {f}"


def test_contexts_with_different_strand_lengths_interleave():
    """The integration's shared-memory limit is a per-kernel setting of the
    process: contexts whose strands differ in length (so in staging size)
    run in any order, each again after the other."""
    insts = _instances()
    rs = [Renderer(inst, 0) for inst in insts]
    for r in rs:
        r.before_first_frame()
    for order in (rs, rs[::-1], rs):
        for r in order:
            r.frame()
    torch.cuda.synchronize()


def _batch_vs_alone(insts, frames, profile_frame=None, groups=1, pipeline=False):
    alone = [Renderer(inst, 0) for inst in insts]
    ctx = Context(insts[0].cfg.to_c(), 0)
    ctx.set_batch_groups(groups)
    ctx.set_batch_pipeline(pipeline)
    batch = BatchRenderer([Renderer(inst, 0, ctx=ctx) for inst in insts])
    for r in alone:
        r.before_first_frame()
    batch.before_first_frame()
    l0 = ctx.counters()["launches"]
    for f in range(frames):
        for r in alone:
            r.frame()
        if f == profile_frame:  # pass by pass on the context's stream, timed
            n = len(batch.renderers)
            arr = (HfbInstance * n)(*[r.instance() for r in batch.renderers])
            pm = (ctypes.c_float * 9)()
            ctx.call("hfb_frame_batch_profile", arr, n, pm)
            for r, inst in zip(batch.renderers, arr):
                r.after_native_frame(inst)
            assert all(v >= 0.0 for v in pm) and sum(pm) > 0.0, list(pm)
        else:
            batch.frame()
        torch.cuda.synchronize()
        for ra, rb in zip(alone, batch.renderers):
            _compare(_state(ra), _state(rb), ra, f)
            assert ra.hair._current == rb.hair._current
    # one persistent launch per pass kind and group, every frame
    per_frame = (ctx.counters()["launches"] - l0) / frames
    assert per_frame <= 20 * groups, per_frame
    return ctx


def test_frame_batch_matches_each_instance_alone():
    _batch_vs_alone(_instances(), 4, profile_frame=1)


@pytest.mark.parametrize("groups", [1, 3])
def test_frame_batch_many_small_instances(groups):
    """12 instances of uneven sizes, several frames through the captured
    graph, in one group or in three groups side by side."""
    rng = np.random.Generator(np.random.PCG64(11))
    common = dict(tile_size=16, depth_bins=8, slices=4, shading_points=8, grid_dims=32, iterations=4)
    insts = [synthetic.make_instance(rng, strands=int(rng.integers(200, 1500)), points=int(rng.choice([16, 24, 32])),
                                     width=int(rng.choice([128, 256])), height=int(rng.choice([128, 192])), **common)
             for _ in range(12)]
    _batch_vs_alone(insts, 3, groups=groups)


def _lists(tiles, segs):
    """Every non-empty (tile, bin) list, vectorised: (bins, lengths, the
    records in list order).  The builder stores a list of n records in n
    consecutive slots ending at its head, each linked to the one before
    (checked here), so a list is its slots read backwards."""
    heads = tiles[:, 2].astype(np.int64)
    bins = np.nonzero(heads)[0]
    n = tiles[bins, 3].astype(np.int64)
    assert (n > 0).all(), "a list without its length"
    first = np.cumsum(n) - n
    k = np.arange(int(n.sum())) - np.repeat(first, n)         # position in its list, 0 = head
    slot = np.repeat(heads[bins] - 1, n) - k                  # head first, then backwards
    nxt = segs[2 + 2 * slot].astype(np.int64)
    last = k == np.repeat(n - 1, n)
    assert (nxt[last] == 0xFFFFFFFF).all() and (nxt[~last] == slot[~last] - 1).all(), "a list is not linked backwards"
    return bins, n, segs[1 + 2 * slot]


def test_frame_batch_of_the_64_instance_workload():
    """All 64 instances of the benchmark's batched workload (strands
    U[1k, 20k], points in {16, 24, 32}, viewports 256^2-1024^2) at the
    constants the autotuner picks for it (8 px tiles, 4 depth bins), hair
    depth on: two batched frames equal each instance's frames alone --
    positions, grids, counts, per-bin depth bounds, every list walked from
    its head, tile list bit-exact, shading within 1e-6, pixels within
    1/255; no record dropped."""
    insts = synthetic.batched_instances(seed=0, count=64, tile_size=8, depth_bins=4, grid_dims=64, slices=4,
                                        shading_points=8, iterations=7, avg_segments_per_tile=512)
    alone = [Renderer(inst, 0, hair_depth=True) for inst in insts]
    ctx = Context(insts[0].cfg.to_c(), 0)
    batch = BatchRenderer([Renderer(inst, 0, ctx=ctx, hair_depth=True) for inst in insts])
    for r in alone:
        r.before_first_frame()
    batch.before_first_frame()
    for f in range(2):
        for r in alone:
            r.frame()
        batch.frame()
        torch.cuda.synchronize()
        for k, (ra, rb) in enumerate(zip(alone, batch.renderers)):
            tag = f"frame {f}, instance {k}"
            assert torch.equal(ra.hair.positions, rb.hair.positions), f"{tag}: positions differ"
            assert torch.equal(ra.grids.density_velocity, rb.grids.density_velocity), f"{tag}: density grid differs"
            assert np.array_equal(ra.rb.read_segment_counts(), rb.rb.read_segment_counts()), f"{tag}: counts"
            tla, tlb = ra.rb.read_tiles().reshape(-1, 4), rb.rb.read_tiles().reshape(-1, 4)
            assert np.array_equal(tla[:, :2], tlb[:, :2]), f"{tag}: depth bounds differ"
            sa, sb = ra.rb.read_tile_segments(), rb.rb.read_tile_segments()
            assert sa[0] == sb[0], f"{tag}: drawnSegmentsCount differs"
            la, lb = _lists(tla, sa), _lists(tlb, sb)
            assert all(np.array_equal(x, y) for x, y in zip(la, lb)), f"{tag}: lists differ"
            ta, tb = ra.rb.read_tile_list(), rb.rb.read_tile_list()
            assert np.array_equal(ta[:1 + int(ta[0])], tb[:1 + int(tb[0])]), f"{tag}: tile list differs"
            assert (ra.hair.shading - rb.hair.shading).abs().max().item() <= 1e-6, f"{tag}: shading differs"
            err = np.abs(ra.rb.read_result()[4:] - rb.rb.read_result()[4:]).max()
            assert err <= 1.0 / 255.0, f"{tag}: pixel error {err:.4g}"
    assert ctx.counters()["tileRecordsDropped"] == 0, "a pool overflowed: which records drop depends on timing"
    for r in alone:
        r.rb.close()
    for r in batch.renderers:
        r.rb.close()


def test_frame_batch_crowded_bins():
    """An instance whose tiles hold bins of more than 1,024 and 16,384 records
    beside a sparse one: the batched list builder (blocks of 32 bins, the
    larger bins queued per block, the largest one block each) links every
    bin as the single-instance launches do."""
    rng = np.random.Generator(np.random.PCG64(5))
    common = dict(tile_size=32, depth_bins=4, slices=4, shading_points=8, grid_dims=32, iterations=4,
                  avg_segments_per_tile=65536)
    insts = [synthetic.make_instance(rng, strands=40000, points=16, width=192, height=160, **common),
             synthetic.make_instance(rng, strands=1500, points=16, width=320, height=240, **common)]
    _batch_vs_alone(insts, 2)


def test_frame_batch_with_hair_depth():
    """Instances that draw the hair depth after the fine pass and shade with
    it: the batched frames equal each instance's frames alone."""
    insts = _instances()
    alone = [Renderer(inst, 0, hair_depth=True) for inst in insts]
    ctx = Context(insts[0].cfg.to_c(), 0)
    batch = BatchRenderer([Renderer(inst, 0, ctx=ctx, hair_depth=True) for inst in insts])
    for r in alone:
        r.before_first_frame()
    batch.before_first_frame()
    for f in range(3):
        for r in alone:
            r.frame()
        batch.frame()
        torch.cuda.synchronize()
        for ra, rb in zip(alone, batch.renderers):
            _compare(_state(ra), _state(rb), ra, f)
            assert np.array_equal(ra.hair_depth.cpu().numpy(), rb.hair_depth.cpu().numpy()), f"frame {f}: depth"


def test_frame_batch_pipelined_each_frame():
    """Simulation and raster passes on two streams, two tables in turn; the
    first frames run plain launches, the later ones the captured graphs."""
    _batch_vs_alone(_instances(), 6, pipeline=True)


def test_frame_batch_pipelined_back_to_back():
    """Frames submitted without waiting in between, so that each frame's
    simulation overlaps the previous frame's raster passes: the state after
    the last frame equals each instance's alone."""
    insts = _instances()
    frames = 7
    alone = [Renderer(inst, 0) for inst in insts]
    ctx = Context(insts[0].cfg.to_c(), 0)
    ctx.set_batch_pipeline(True)
    batch = BatchRenderer([Renderer(inst, 0, ctx=ctx) for inst in insts])
    for r in alone:
        r.before_first_frame()
        for _ in range(frames):
            r.frame()
    batch.before_first_frame()
    for _ in range(frames):
        batch.frame()
    torch.cuda.synchronize()
    for ra, rb in zip(alone, batch.renderers):
        _compare(_state(ra), _state(rb), ra, frames - 1)


def test_frame_batch_rejects_bad_instances():
    insts = _instances()[:2]
    ctx = Context(insts[0].cfg.to_c(), 0)
    rs = [Renderer(inst, 0, ctx=ctx) for inst in insts]
    arr = (HfbInstance * 2)(*[r.instance() for r in rs])
    arr[1].current = 2
    with pytest.raises(Exception, match="instance 1: current"):
        ctx.call("hfb_frame_batch", arr, 2)
    arr[1].current = 0
    arr[0].positions[1] = arr[0].positions[0]
    with pytest.raises(Exception, match="instance 0"):
        ctx.call("hfb_frame_batch", arr, 2)
    with pytest.raises(Exception, match="1024"):
        ctx.call("hfb_frame_batch", arr, 5000)
    assert ctx.lib.hfb_frame_batch(ctx.handle, None, 0) == 0
    for bad in (0, 5):
        with pytest.raises(Exception, match="groups"):
            ctx.set_batch_groups(bad)
    with pytest.raises(Exception, match="pipeline"):
        ctx.call("hfb_ctx_set_batch_pipeline", 2)

