"""Pins the CPU oracle against the reference's own golden vectors.

- sw-raster utility snapshot: src/passes/swHair/swRasterizer.test.ts:57-144
- tile-sort invariants:        src/passes/swHair/hairTileSortPass.test.ts:25-128
- SDF binary format:           src/scene/sdfCollider/createSdfColliderFromBinary.test.ts:14-57
"""
import os
import struct

import numpy as np

from hairfb import HairConfig, formats, hair_object, uniforms as UN

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _sw_raster_inputs():
    # swRasterizer.test.ts:63-75: 1 strand x 4 points, w = 1, fiberRadius 0.1
    pos = np.array([[-0.7, -0.7, 0.0, 1.0], [-0.2, 0.2, 0.0, 1.0],
                    [0.2, 0.2, 0.0, 1.0], [0.7, -0.7, 0.0, 1.0]], np.float32)
    asset = hair_object.HairAsset(1, 4, pos)
    hb = hair_object.build_hair_buffers(asset)
    u = bytearray(UN.RENDER_UNIFORMS_BYTES)
    eye = np.eye(4, dtype=np.float32).reshape(16)
    # identity proj / view / vp (:105-107) and identity model matrix
    for k in ("vpMatrix", "vpMatrixInv", "viewMatrix", "projMatrix", "projMatrixInv",
              "modelMatrix", "modelViewMat", "mvpMatrix"):
        u[UN.OFF[k]:UN.OFF[k] + 64] = eye.tobytes()
    struct.pack_into("<4f", u, UN.OFF["viewport"], 128.0, 128.0, 0.0, 0.0)
    # camera position = CONFIG.camera.position.position (src/constants.ts:128)
    struct.pack_into("<4f", u, UN.OFF["cameraPosition"], 0.25, 1.6, 0.6, 0.0)
    struct.pack_into("<f", u, UN.OFF["fiberRadius"], 0.1)
    return bytes(u), hb


def test_sw_raster_snapshot_bit_exact(oracle):
    u, hb = _sw_raster_inputs()
    out = oracle.sw_raster_test(u, hb.hair_data, hb.asset.positions, hb.tangents, 128, 128)
    g = np.load(os.path.join(GOLD, "swRasterizer.snapshot.npz"))
    expected = np.zeros(int(g["size"][0]) * int(g["size"][1]), np.uint32)
    expected[g["index"]] = g["value"]
    assert np.count_nonzero(expected) == 1116
    lit_o = set(np.nonzero(out)[0].tolist())
    lit_e = set(np.nonzero(expected)[0].tolist())
    assert lit_o == lit_e, f"coverage differs: +{len(lit_o - lit_e)} -{len(lit_e - lit_o)}"
    # every channel is u32(saturate(w) * 255): bit-exact
    assert np.array_equal(out, expected), f"{np.count_nonzero(out != expected)} pixels differ"


def _calc_bucket(count, buckets, size):
    return min(max(count // size, 0), buckets - 1)


def test_tile_sort_reference_case(oracle):
    # hairTileSortPass.test.ts:26-53: 8 buckets, 16 tiles, 1-px-tall viewport
    cfg = HairConfig(tile_size=8, sort_buckets=8)
    seg = np.zeros(16, np.uint32)
    seg[1], seg[6], seg[2], seg[3], seg[8] = 1, 15, 16, 17, 4096
    buckets, tile_list = oracle.tile_sort(cfg, 16 * 8, 1, seg)
    exp = np.zeros(8, np.uint32)
    for c in seg:
        if c:
            exp[_calc_bucket(int(c), 8, 16)] += 1
    assert np.array_equal(buckets[0::2], exp)                 # assertBucketCount
    n = int(tile_list[0])
    assert n == 5
    tiles = tile_list[1:1 + n]
    b = [_calc_bucket(int(seg[t]), 8, 16) for t in tiles]
    assert all(b[i] <= b[i - 1] for i in range(1, n))         # non-increasing buckets
    assert sorted(tiles.tolist()) == [1, 2, 3, 6, 8]
    assert np.array_equal(buckets[1::2], exp)                 # writeOffset ends at tileCount


def test_sdf_binary_format():
    data = open(os.path.join(GOLD, "test-sdf.bin"), "rb").read()
    vol = formats.parse_sdf(data)
    assert vol.dims == 5
    f = np.float32
    assert vol.bounds_min[0] == f(-0.07146620005369186)
    assert vol.bounds_min[1] == f(1.3298900127410889)
    assert vol.bounds_min[2] == f(-0.11404839903116226)
    assert vol.bounds_max[0] == f(0.07146620005369186)
    assert vol.bounds_max[1] == f(1.6911249160766602)
    assert vol.bounds_max[2] == f(0.11287439614534378)
    assert abs(float(vol.distances[0]) - 0.05447781831026077) < 1e-7
    # the reference snapshot stores Uint8Array(Float32Array) = each value truncated to u8
    snap = np.frombuffer(open(os.path.join(GOLD, "sdf-binary.snapshot.bin"), "rb").read(), np.uint8)
    trunc = np.array([int(np.trunc(x)) & 0xFF for x in vol.distances.astype(np.float64)], np.uint8)
    assert np.array_equal(snap, trunc)
    # round trip through the writer
    assert formats.write_sdf(vol) == data


def test_sdf_binary_rejects_bad_size():
    data = open(os.path.join(GOLD, "test-sdf.bin"), "rb").read()
    import pytest
    with pytest.raises(ValueError):
        formats.parse_sdf(data[:-4])


def test_threaded_oracle_matches_serial(oracle):
    """The OpenMP build of the oracle (CPU baseline) computes exactly what the
    serial build does: the canonical list order survives the parallel raster."""
    import helpers
    inst = helpers.small_instance(strands=600)
    fr = helpers.frame_of(inst)
    hb = inst.hair
    out = {}
    for t in (False, True):
        oracle.use_threads(t)
        try:
            tl = oracle.tiles_pass(inst.cfg, fr.uniforms, hb.hair_data, hb.asset.positions, hb.tangents,
                                   inst.scene_depth, hb.asset.strands, inst.width, inst.height, fr.max_drawn)
            b, lst = oracle.tile_sort(inst.cfg, inst.width, inst.height, tl[2])
            sh = oracle.shading(inst.cfg, fr.uniforms, hb.hair_data, hb.asset.positions, hb.tangents,
                                inst.scene_depth, hb.asset.strands)
            fine = oracle.fine_pass(inst.cfg, fr.uniforms, hb.hair_data, hb.asset.positions, hb.tangents,
                                    sh + 0.25, inst.scene_depth, tl[0], tl[1], lst, inst.width, inst.height)
            dv = oracle.grid_post_sim(inst.cfg, fr.uniforms[:304], hb.hair_data, hb.asset.positions,
                                      hb.asset.positions * 1.001)
        finally:
            oracle.use_threads(False)
        out[t] = (tl, lst, sh, fine, dv)
    for a, b in zip(out[False], out[True]):
        if isinstance(a, tuple):
            for x, y in zip(a, b):
                assert np.array_equal(x, y)
        else:
            assert np.array_equal(a, b)
