"""A hair asset in the reference's own file formats, through a whole frame.

A seeded hair is written as a TFX file (parseTfxFile's layout,
src/scene/hair/tfxFileLoader.ts:19-69) and its head as the binary SDF
(createSdfColliderFromBinary.ts:5-43); both are parsed back by
hairfb.formats and set up as the reference's default scene
(synthetic.asset_instance).  One frame through hfb_frame (simulation, tiles,
sort, fine, hair depth, shading) is compared with the oracle's frame on the
parsed data: positions, the density grid, tile records and the hair depth
bit-exact, pixels within 1/255, the shading within 1e-5.
"""
import numpy as np
import pytest

from helpers import walk_lists
from hairfb import formats, synthetic
from hairfb import uniforms as UN
from hairfb.hair_object import HairAsset

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("needs a CUDA GPU", allow_module_level=True)


@pytest.fixture(scope="module")
def oracle():
    from oracle import oracle as o
    o.load()
    return o


def _asset_files(strands=1500, points=16, seed=3):
    """A grown hair (TFX bytes) and the SDF of its head sphere (binary SDF bytes)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    a = synthetic.grow_hair(rng, strands, points, center=(0.0, 0.0, 0.0), head_radius=0.1)
    vol = synthetic.sdf_from_function(synthetic.sphere_sdf((0.0, 0.0, 0.0), 0.1), 32,
                                      (-0.25, -0.25, -0.25), (0.25, 0.25, 0.25))
    return formats.write_tfx(a), formats.write_sdf(vol), a, vol


def test_tfx_and_sdf_asset_frame_matches_the_oracle(oracle):
    from hairfb.renderer import Renderer
    tfx, sdf, grown, vol = _asset_files()
    inst = synthetic.asset_instance(tfx, sdf, width=480, height=360, tile_size=16, tile_depth_bins=8,
                                    slices_per_pixel=4, shading_points=8, grid_dims=32)
    # the loaders' view of the files is the data that was written
    assert inst.hair.asset.strands == grown.strands and inst.hair.asset.points_per_strand == grown.points_per_strand
    assert np.array_equal(inst.hair.asset.positions.view(np.uint32), grown.positions.view(np.uint32))
    assert inst.sdf.dims == vol.dims and np.array_equal(inst.sdf.distances, vol.distances)
    cfg, hb = inst.cfg, inst.hair

    r = Renderer(inst, 0, hair_depth=True)
    r.before_first_frame()
    torch.cuda.synchronize()
    shade0 = r.hair.shading.cpu().numpy().copy()
    r.frame_native()  # hfb_frame
    torch.cuda.synchronize()

    # the oracle's frame: the first-frame set-up, then the passes in the reference's order
    u = r.uniforms
    md = r.rb.max_drawn_segments
    p0 = hb.asset.positions
    su0 = UN.pack_sim_uniforms(inst.sim, inst.scene.model_matrix, inst.scene.sdf_bounds, inst.scene.grid_bounds, 0,
                               wind_dir=inst.wind_dir)
    dv = oracle.grid_post_sim(cfg, su0, hb.hair_data, p0, p0)
    hd0 = oracle.hair_depth(u, hb.hair_data, p0, hb.tangents, hb.asset.strands, inst.scene_depth)
    osh0 = oracle.shading(cfg, u, hb.hair_data, p0, hb.tangents, hd0, hb.asset.strands)
    assert np.allclose(shade0, osh0, rtol=1e-5, atol=1e-5), float(np.abs(shade0 - osh0).max())
    gw = oracle.grid_pre_sim(cfg, su0, dv, inst.sdf.distances, inst.sdf.dims)
    new = oracle.sim_integrate(cfg, su0, hb.hair_data, p0, p0, p0, hb.segment_lengths, dv, gw, inst.sdf.distances,
                               inst.sdf.dims)
    dv1 = oracle.grid_post_sim(cfg, su0, hb.hair_data, p0, new)
    gpos = r.hair.positions.cpu().numpy()
    assert np.array_equal(gpos.view(np.uint32), new.view(np.uint32)), "positions after the step differ"
    assert np.array_equal(r.grids.density_velocity.cpu().numpy().reshape(-1), dv1.reshape(-1)), "density grid"
    assert not np.array_equal(new, p0), "the step moved nothing"

    ot, osg, oc = oracle.tiles_pass(cfg, u, hb.hair_data, new, hb.tangents, inst.scene_depth, hb.asset.strands,
                                    inst.width, inst.height, md)
    gt, gsg, gc = r.rb.read_tiles(), r.rb.read_tile_segments(), r.rb.read_segment_counts()
    assert int(osg[0]) > 0 and gsg[0] == osg[0]
    assert np.array_equal(gc, oc) and np.array_equal(gt[:, :2], ot[:, :2])
    assert walk_lists(gt, gsg, md) == walk_lists(ot, osg, md)
    _, otl = oracle.tile_sort(cfg, inst.width, inst.height, oc)
    ores = oracle.fine_pass(cfg, u, hb.hair_data, new, hb.tangents, shade0, inst.scene_depth, ot, osg, otl,
                            inst.width, inst.height)
    err = float(np.abs(r.rb.read_result()[4:] - ores[4:]).max())
    assert err <= 1.0 / 255.0, err
    assert (np.abs(ores[4:]) > 0).sum() > 1000, "the frame covers too few pixels to compare"

    hd1 = oracle.hair_depth(u, hb.hair_data, new, hb.tangents, hb.asset.strands, inst.scene_depth)
    assert np.array_equal(r.hair_depth.cpu().numpy().view(np.uint32), hd1.view(np.uint32)), "hair depth"
    osh1 = oracle.shading(cfg, u, hb.hair_data, new, hb.tangents, hd1, hb.asset.strands)
    g = r.hair.shading.cpu().numpy()
    assert np.allclose(g, osh1, rtol=1e-5, atol=1e-5), float(np.abs(g - osh1).max())
    r.rb.close()
    r.ctx.close()


def test_tfx_round_trip_keeps_every_bit():
    """write_tfx / parse_tfx and write_sdf / parse_sdf are lossless (CPU side of the asset path)."""
    tfx, sdf, grown, vol = _asset_files(strands=200, points=24)
    a = formats.parse_tfx(tfx)
    assert isinstance(a, HairAsset) and a.positions.shape == (200 * 24, 4)
    assert np.array_equal(a.positions.view(np.uint32), grown.positions.view(np.uint32))
    v = formats.parse_sdf(sdf)
    assert v.dims == 32 and np.array_equal(v.bounds_min, vol.bounds_min) and np.array_equal(v.distances, vol.distances)
