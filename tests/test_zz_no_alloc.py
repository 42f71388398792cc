"""hfb_tiles_pass_noalloc: the tiles pass for callers that cannot allocate
device memory (a render thread that must not take cudaMalloc's device-wide
synchronisation, a host whose allocator owns every device byte, code about
to record a stream capture).  Its working memory is a fixed array inside the
library instead of HfbRasterBuffers.scratch.

Checked through the C-ABI against hfb_tiles_pass on the same inputs, on
calls in a row on two different frames (another viewport, strand count and
segment pool, so the bins and records of one call land elsewhere in the
array than the other's: the array keeps the previous call's contents, and a
pass that read any of them would differ).  The device's free memory is the
same before and after the calls: the array and the pass's code were made
resident when the context was created.  The tiles pass is integer work:
the bar is bit-exact, as for hfb_tiles_pass itself.  This file is collected
last so a failing run that stops at the first failure has run every other
test first.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

from helpers import frame_of, small_instance  # noqa: E402
from hairfb.lib import Context, HfbError, HfbRasterBuffers, byref, ptr  # noqa: E402
from hairfb.passes import HairObject, RasterBuffers, clear_before_render  # noqa: E402

NOALLOC_LIMIT = 16 << 20  # HFB_NOALLOC_SCRATCH_BYTES


def _outputs(rb: RasterBuffers):
    return rb.read_tiles().copy(), rb.read_tile_segments().copy(), rb.read_segment_counts().copy()


def _run(ctx, fn, fr, hair, depth, rb):
    clear_before_render(ctx, rb)
    ctx.call(fn, ctypes.cast(ctypes.c_char_p(fr.uniforms), ctypes.c_void_p), byref(hair.hair_data),
             ptr(hair.positions), ptr(hair.tangents), ptr(depth), hair.rendered_strand_count(), byref(rb.rb))
    ctx.sync()
    return _outputs(rb)


def test_noalloc_tiles_pass_matches_allocating_entry_point():
    # frame A, then frame B (other viewport, strands and pool), then A again
    insts = [small_instance(), small_instance(seed=1, strands=1200, width=512, height=400)]
    assert insts[0].cfg == insts[1].cfg
    ctx = Context(insts[0].cfg.to_c(), 0)
    frames = []
    for inst in insts:
        fr = frame_of(inst)
        hair = HairObject(inst.hair, inst.cfg.shading_points)
        depth = torch.as_tensor(inst.scene_depth).cuda()
        rb = RasterBuffers(ctx, inst.width, inst.height)
        assert ctx.lib.hfb_raster_scratch_bytes(byref(ctx.cfg), inst.width, inst.height) <= NOALLOC_LIMIT
        ref = _run(ctx, "hfb_tiles_pass", fr, hair, depth, rb)
        assert ref[1][0] > 0, "nothing was binned: the comparison would be empty"
        frames.append((fr, hair, depth, rb, ref))
    assert frames[0][4][1][0] != frames[1][4][1][0], "the two frames must differ in their records"
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    for call, k in enumerate((0, 1, 0)):  # consecutive calls share the fixed array
        fr, hair, depth, rb, ref = frames[k]
        got = _run(ctx, "hfb_tiles_pass_noalloc", fr, hair, depth, rb)
        for name, a, b in zip(("tiles", "tileSegments", "segmentCountPerTile"), got, ref):
            assert np.array_equal(a, b), f"call {call + 1} (frame {k}): {name} differs from hfb_tiles_pass"
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0, "the device's free memory changed across the calls"
    for fr, hair, depth, rb, ref in frames:
        rb.close()
    ctx.close()


def test_noalloc_rejects_viewports_beyond_the_fixed_array():
    inst = small_instance(strands=20, width=4096, height=4096)
    fr = frame_of(inst)
    ctx = Context(inst.cfg.to_c(), 0)
    need = ctx.lib.hfb_raster_scratch_bytes(byref(ctx.cfg), 4096, 4096)
    assert need > NOALLOC_LIMIT
    hair = HairObject(inst.hair, inst.cfg.shading_points)
    depth = torch.ones(4096 * 4096, device="cuda")
    rb = HfbRasterBuffers()  # only the outputs; no scratch
    rb.width, rb.height, rb.maxDrawnSegments = 4096, 4096, fr.max_drawn
    rb.tiles = rb.tileSegments = rb.segmentCountPerTile = ptr(depth)
    with pytest.raises(HfbError) as e:
        ctx.call("hfb_tiles_pass_noalloc", ctypes.cast(ctypes.c_char_p(fr.uniforms), ctypes.c_void_p),
                 byref(hair.hair_data), ptr(hair.positions), ptr(hair.tangents), ptr(depth), 20, byref(rb))
    assert "working memory" in str(e.value)
    ctx.sync()
    ctx.close()
