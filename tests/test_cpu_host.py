"""CPU tests: host-side logic, byte layouts, the C-ABI library's exports."""
import ctypes
import os
import re
import struct
import time

import numpy as np
import pytest

from hairfb import formats, hair_object as HO, synthetic, uniforms as UN
from hairfb.config import HairConfig, HfbConfig

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "hairfb.h")


def test_uniform_block_sizes_and_offsets():
    inst = synthetic.plain_small(strands=50)
    u = UN.pack_render_uniforms(inst.scene, inst.cfg)
    assert len(u) == 1184  # renderUniformsBuffer.ts BUFFER_SIZE
    vp = np.frombuffer(u, np.float32, 4, UN.OFF["viewport"])
    assert tuple(vp) == (640.0, 480.0, 0.0, 0.0)
    assert struct.unpack_from("<f", u, UN.OFF["fiberRadius"])[0] == np.float32(5e-4)
    md = struct.unpack_from("<I", u, UN.OFF["maxDrawnHairSegments"])[0]
    assert md == 1 + 40 * 30 * 128
    cam = np.frombuffer(u, np.float32, 3, UN.OFF["cameraPosition"])
    assert np.allclose(cam, inst.scene.camera.eye)
    # projMatrixInv is the inverse of projMatrix
    P = np.frombuffer(u, np.float32, 16, UN.OFF["projMatrix"]).reshape(4, 4).T
    Pi = np.frombuffer(u, np.float32, 16, UN.OFF["projMatrixInv"]).reshape(4, 4).T
    assert np.allclose(P.astype(np.float64) @ Pi, np.eye(4), atol=1e-4)
    s = UN.pack_sim_uniforms(inst.sim, inst.scene.model_matrix, inst.scene.sdf_bounds,
                             inst.scene.grid_bounds, 12)
    assert len(s) == 304
    assert struct.unpack_from("<f", s, UN.SIM_OFF["deltaTime"])[0] == np.float32(1 / 60)
    assert struct.unpack_from("<I", s, UN.SIM_OFF["frameIdx"])[0] == 12
    assert struct.unpack_from("<I", s, UN.SIM_OFF["constraintIterations"])[0] == 7


def test_patched_sim_uniforms_equal_a_full_pack():
    """The per-frame patch of the cached SimulationUniforms block (frameIdx,
    wind strength) gives the bytes of a full pack of that frame."""
    rng = np.random.Generator(np.random.PCG64(2))
    inst = synthetic.make_instance(rng, strands=50, points=8, width=64, height=64, wind_amplitude=1.0)

    def pack(k):
        return UN.pack_sim_uniforms(inst.sim, inst.scene.model_matrix, inst.scene.sdf_bounds,
                                    inst.scene.grid_bounds, k, wind_dir=inst.wind_dir,
                                    wind_strength=inst.wind_strength(k))
    block = bytearray(pack(0))
    for k in (1, 2, 17, 1000, 123456):
        UN.patch_sim_uniforms(block, k, inst.wind_strength(k))
        assert bytes(block) == pack(k), k


def test_config_struct_matches_header():
    assert ctypes.sizeof(HfbConfig) == 64
    txt = open(HEADER).read()
    body = re.search(r"typedef struct HfbConfig \{(.*?)\} HfbConfig;", txt, re.S).group(1)
    names = re.findall(r"(?:uint32_t|float)\s+([\w, ]+);", body)
    flat = [n.strip() for group in names for n in group.split(",")]
    assert flat == [f for f, _ in HfbConfig._fields_]
    c = HairConfig().to_c()  # reference defaults, constants.ts
    assert (c.tileSize, c.tileDepthBins, c.slicesPerPixel, c.shadingPoints) == (8, 32, 8, 64)
    assert (c.sortBuckets, c.sortBucketSize, c.processorCount) == (64, 16, 512)


def test_ctypes_structs_match_the_header_sizes():
    """The host mirrors of the C-ABI structs have the sizes include/hairfb.h
    static-asserts (a mismatch would shift every field the library reads)."""
    from hairfb.lib import HfbHairData, HfbInstance, HfbPresentItem
    txt = open(HEADER).read()
    asserted = dict((k, int(v)) for k, v in re.findall(r"static_assert\(sizeof\((\w+)\) == (\d+)", txt))
    for cls in (HfbConfig, HfbHairData, HfbInstance, HfbPresentItem):
        assert ctypes.sizeof(cls) == asserted[cls.__name__], cls.__name__


def test_max_drawn_segments_formula():
    # getLengthOfHairTileSegmentsBuffer, hairTileSegmentsBuffer.ts:81-87
    cfg = HairConfig(tile_size=16, avg_segments_per_tile=128)
    assert cfg.max_drawn_segments(1920, 1080) == 1 + 120 * 68 * 128
    assert cfg.slice_data_per_processor() == 16 * 8 * 16 * 16


def test_tangents_lengths_bounds():
    rng = np.random.Generator(np.random.PCG64(3))
    a = synthetic.grow_hair(rng, 20, 8)
    t = HO.tangents(a)
    p = a.positions[:, :3].reshape(20, 8, 3).astype(np.float64)
    d = p[:, 1:] - p[:, :-1]
    exp = d / np.linalg.norm(d, axis=-1, keepdims=True)
    tt = t.reshape(20, 8, 4)
    assert np.allclose(tt[:, :-1, :3], exp, atol=1e-6)
    assert np.array_equal(tt[:, -1], tt[:, -2])          # tip copies the previous tangent
    assert np.all(tt[..., 3] == 0)
    L = HO.segment_lengths(a).reshape(20, 8)
    assert np.allclose(L[:, :-1], np.linalg.norm(d, axis=-1), rtol=1e-6)
    assert np.array_equal(L[:, -1], L[:, -2])
    bmin, bmax = HO.bounding_box(a.positions)
    c, r = HO.bounding_sphere(bmin, bmax)
    assert np.allclose(c, (bmin + bmax) / 2)
    assert np.isclose(r, np.linalg.norm(bmax - c), rtol=1e-6)
    gmin, gmax = HO.scale_bounding_box(bmin, bmax, 2.0)
    assert np.allclose(gmax - gmin, 2 * (bmax - bmin), rtol=1e-5)


def test_growth_model():
    rng = np.random.Generator(np.random.PCG64(0))
    a = synthetic.grow_hair(rng, 500, 16)
    p = a.positions.reshape(500, 16, 4)
    assert np.all(p[:, 0, 3] == 0) and np.all(p[:, 1:, 3] == 1)
    seg = np.linalg.norm(np.diff(p[..., :3], axis=1), axis=-1)
    assert np.allclose(seg, 0.01, rtol=1e-4)
    root_r = np.linalg.norm(p[:, 0, :3], axis=-1)
    assert np.allclose(root_r, 0.1, rtol=1e-5)
    assert np.all(p[:, 0, 1] >= 0)                         # upper hemisphere


def test_tfx_round_trip_and_errors():
    rng = np.random.Generator(np.random.PCG64(1))
    a = synthetic.grow_hair(rng, 30, 16)
    data = formats.write_tfx(a)
    assert len(data) == formats.TFX_HEADER_BYTES + 30 * 16 * 16
    b = formats.parse_tfx(data)
    assert (b.strands, b.points_per_strand) == (30, 16)
    assert np.array_equal(a.positions, b.positions)
    with pytest.raises(ValueError):
        formats.parse_tfx(data[:200])
    with pytest.raises(ValueError):
        formats.parse_tfx(b"\0" * 16)


def test_sphere_depth_input():
    inst = synthetic.plain_small(strands=10)
    d = inst.scene_depth.reshape(inst.height, inst.width)
    assert d.min() > 0.0 and d.max() == 1.0
    # the head sphere covers a disc of the image, the corners are empty
    assert (d < 1.0).sum() > 5000 and d[0, 0] == 1.0


def _declared_symbols():
    txt = open(HEADER).read()
    return sorted(set(re.findall(r"HFB_API\s+[\w\s\*]+?\b(hfb_\w+)\s*\(", txt)))


def test_library_exports_every_declared_symbol():
    """The C-ABI library loads without a GPU and exports every entry point
    include/hairfb.h declares (no compute call is made here)."""
    from hairfb import build as B
    from hairfb import lib as L
    try:
        path = B.build()
    except RuntimeError as e:  # no CUDA toolkit on this machine
        pytest.skip(str(e))
    so = ctypes.CDLL(path)
    syms = _declared_symbols()
    assert len(syms) >= 20
    missing = [s for s in syms if not hasattr(so, s)]
    assert not missing, missing
    assert set(syms) == set(L.SIGNATURES), set(syms) ^ set(L.SIGNATURES)
    assert so.hfb_version() == 1
    so.hfb_raster_scratch_bytes.restype = ctypes.c_size_t
    so.hfb_raster_scratch_bytes.argtypes = [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint32]
    cfg = HairConfig(tile_size=16, tile_depth_bins=8).to_c()
    n = so.hfb_raster_scratch_bytes(ctypes.byref(cfg), 640, 480)
    assert n >= 2 * 1200 * 8 * 4 + 4 * (1 + 1200 * 128)
    # invalid config is rejected before touching CUDA
    bad = HairConfig(tile_size=12).to_c()
    h = ctypes.c_void_p()
    so.hfb_ctx_create.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
    assert so.hfb_ctx_create(ctypes.byref(bad), -1, ctypes.byref(h)) == -1


def test_product_has_no_cpu_fallback(tmp_path):
    """The host package fails loudly when the CUDA library is missing."""
    from hairfb import lib as L
    with pytest.raises(FileNotFoundError):
        L.open_library(str(tmp_path / "libhairfb.so"))


def test_strand_grid_order_is_a_morton_permutation():
    """hfb_strand_grid_order (host code, no GPU): a permutation of the
    strands whose roots' Morton codes do not decrease."""
    from hairfb import synthetic
    from hairfb.lib import strand_grid_order
    rng = np.random.Generator(np.random.PCG64(3))
    inst = synthetic.make_instance(rng, strands=3000, points=16, width=64, height=64)
    a = inst.hair.asset
    order = strand_grid_order(a.positions, a.strands, a.points_per_strand)
    assert np.array_equal(np.sort(order), np.arange(a.strands))
    roots = a.positions.reshape(a.strands, a.points_per_strand, 4)[:, 0, :3].astype(np.float64)
    lo, hi = roots.min(0), roots.max(0)
    q = np.clip(((roots - lo) / (hi - lo) * 1023.0).astype(np.int64), 0, 1023)

    def spread(v):
        out = np.zeros_like(v)
        for b in range(10):
            out |= ((v >> b) & 1) << (3 * b)
        return out
    code = spread(q[:, 0]) | (spread(q[:, 1]) << 1) | (spread(q[:, 2]) << 2)
    assert (np.diff(code[order]) >= 0).all()
    # neighbours in the order are near each other: far closer than in strand order
    d_order = np.linalg.norm(np.diff(roots[order], axis=0), axis=1).mean()
    d_plain = np.linalg.norm(np.diff(roots, axis=0), axis=1).mean()
    assert d_order < 0.5 * d_plain


def test_asset_instance_from_reference_formats():
    """synthetic.asset_instance on files in the reference's formats (a TFX
    written from a grown asset and the binary SDF of a sphere): the
    reference's default pass constants, and a scene depth that hits the
    head where the SDF's zero surface is in view."""
    rng = np.random.Generator(np.random.PCG64(5))
    grown = synthetic.grow_hair(rng, 500, 16, center=(0.0, 1.5, 0.0), head_radius=0.1)
    tfx = formats.write_tfx(grown)
    vol = synthetic.sdf_from_function(synthetic.sphere_sdf(np.array([0.0, 1.5, 0.0]), 0.1), 32,
                                      np.array([-0.2, 1.3, -0.2]), np.array([0.2, 1.7, 0.2]))
    inst = synthetic.asset_instance(tfx, formats.write_sdf(vol), width=320, height=180)
    assert inst.hair.asset.strands == 500 and inst.hair.asset.points_per_strand == 16
    assert (inst.cfg.tile_size, inst.cfg.tile_depth_bins, inst.cfg.slices_per_pixel, inst.cfg.shading_points) \
        == (8, 32, 8, 64)
    assert inst.scene_depth.shape == (320 * 180,)
    hit = inst.scene_depth < 1.0
    assert 0.01 < hit.mean() < 0.9 and (inst.scene_depth[hit] > 0.0).all()


def test_png_writer():
    """formats.write_png: signature, IHDR fields and the pixels back through zlib."""
    import zlib
    img = np.random.default_rng(2).integers(0, 256, (7, 5, 4), dtype=np.uint8)
    png = formats.write_png(img)
    assert png[:8] == b"\x89PNG\r\n\x1a\n"
    w, h, depth, ctype = struct.unpack(">IIBB", png[16:26])
    assert (w, h, depth, ctype) == (5, 7, 8, 6)
    idat = png.index(b"IDAT")
    n = struct.unpack(">I", png[idat - 4:idat])[0]
    raw = zlib.decompress(png[idat + 4:idat + 4 + n])
    rows = np.frombuffer(raw, np.uint8).reshape(7, 1 + 5 * 4)
    assert (rows[:, 0] == 0).all() and np.array_equal(rows[:, 1:].reshape(7, 5, 4), img)


def test_autotuner_stages_keep_only_clear_gains(monkeypatch):
    """The tuner's stages 1-3 (host logic, timings faked, no GPU): the fastest
    tile size x depth bins that drops no record, the base constants kept
    unless a candidate is 3 % faster, then slices and the persistent CTA
    count each kept only when 3 % faster than the choice so far."""
    from hairfb import autotune as AT

    class FakeCtx:
        def __init__(self, cfg, device):
            self.cfg = cfg

        def set_stream(self, s):
            pass

        def close(self):
            pass

    class FakeRenderer:
        def use_config(self, cfg, ctx):
            self.cfg = cfg

    def fake_time(cfg):
        table = {(16, 8): (10.0, 0), (8, 4): (9.0, 0), (8, 8): (9.9, 0), (32, 4): (5.0, 7)}  # 32 px drops records
        ms, dropped = table.get((cfg.tileSize, cfg.tileDepthBins), (12.0, 0))  # the context's C config
        if cfg.slicesPerPixel == 2:
            ms *= 0.99  # 1 %: not kept
        if cfg.processorCount == 512:
            ms *= 0.9   # 10 %: kept
        return ms, dropped

    monkeypatch.setattr(AT, "Context", FakeCtx)
    monkeypatch.setattr(AT, "time_batch", lambda rs, ctx, stream, frames, warmup: fake_time(ctx.cfg))
    monkeypatch.setattr(AT.torch.cuda, "synchronize", lambda *a: None)
    base = HairConfig(tile_size=16, tile_depth_bins=8, slices_per_pixel=4)
    rs = [FakeRenderer(), FakeRenderer()]
    trials = []
    ms, cfg, ctx = AT._tune_config(rs, base, 0, None, (8, 16, 32), (4, 8), (2, 4, 8), (0, 512), 2, 1,
                                   time.perf_counter() + 60.0, "all", trials)
    assert (cfg.tile_size, cfg.tile_depth_bins, cfg.slices_per_pixel, cfg.processor_count) == (8, 4, 4, 512)
    assert abs(ms - 9.0 * 0.9) < 1e-9 and all(r.cfg == cfg for r in rs)
    assert len(trials) == 6 + 2 + 1  # the grid, two other slice counts, one other CTA count
    # a winner within 3 % of the base constants leaves the base in place
    monkeypatch.setattr(AT, "time_batch", lambda rs, ctx, stream, frames, warmup:
                        (9.8 if (ctx.cfg.tileSize, ctx.cfg.tileDepthBins) == (8, 4) else 10.0, 0))
    ms, cfg, ctx = AT._tune_config(rs, base, 0, None, (8, 16), (4, 8), (4,), (0,), 2, 1,
                                   time.perf_counter() + 60.0, "all", [])
    assert (cfg.tile_size, cfg.tile_depth_bins) == (16, 8) and ms == 10.0
