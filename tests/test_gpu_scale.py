"""The largest configuration (200,000 x 32 strands, 60 % in a ponytail,
3840x2160, 32 depth bins, 8 slices, 32 shading points, 128^3 SDF, 64^3
grids, 8 iterations) through size-independent properties:

- one simulation step (grid post-sim, grid pre-sim, integration) bit-exact
  against the oracle at full size;
- a whole frame is deterministic: two contexts on the same inputs give the
  same positions, grids, tile heads, lists, tile list and image;
- the tiles pass's lists are canonical (walked from the head, keys strictly
  decrease), their lengths sum to the record count, no record dropped, and
  every tile's count equals the lengths of its bins' lists.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

from hairfb import synthetic, uniforms as UN  # noqa: E402
from hairfb.lib import Context  # noqa: E402
from hairfb.passes import (GridPostSimPass, GridPreSimPass, HairObject, HairSimIntegrationPass,  # noqa: E402
                           PhysicsGrids, SdfCollider)
from hairfb.renderer import Renderer  # noqa: E402

INVALID = 0xFFFFFFFF


@pytest.fixture(scope="module")
def stress():
    return synthetic.stress()


@pytest.fixture(scope="module")
def oracle():
    from oracle import oracle as o
    o.use_threads(True)  # the OpenMP build: 6.4 M points
    o.load()
    return o


def test_stress_one_step_bit_exact(stress, oracle):
    inst = stress
    hb = inst.hair
    su = UN.pack_sim_uniforms(inst.sim, inst.scene.model_matrix, inst.scene.sdf_bounds, inst.scene.grid_bounds, 3,
                              wind_dir=inst.wind_dir, wind_strength=inst.wind_strength(3))
    ctx = Context(inst.cfg.to_c(), 0)
    hair = HairObject(hb, inst.cfg.shading_points)
    grids = PhysicsGrids(inst.cfg.grid_dims)
    sdf = SdfCollider(inst.sdf)
    rng = np.random.default_rng(2)
    now = hb.asset.positions.copy()
    now[:, :3] += rng.normal(0, 2e-3, now[:, :3].shape).astype(np.float32) * (now[:, 3:] > 0)
    hair.positions.copy_(torch.as_tensor(now))
    GridPostSimPass(ctx).cmd_update_grids_after_sim(su, hair, grids)
    GridPreSimPass(ctx).cmd_update_grids_before_sim(su, grids, sdf)
    HairSimIntegrationPass(ctx).cmd_simulate_hair_positions(su, hair, grids, sdf)
    ctx.sync()
    odv = oracle.grid_post_sim(inst.cfg, su, hb.hair_data, hb.asset.positions, now)
    assert np.array_equal(grids.density_velocity.cpu().numpy(), odv), "density/velocity grid differs"
    ogw = oracle.grid_pre_sim(inst.cfg, su, odv, inst.sdf.distances, inst.sdf.dims)
    assert np.array_equal(grids.density_grad_wind.cpu().numpy().view(np.uint32), ogw.view(np.uint32))
    onew = oracle.sim_integrate(inst.cfg, su, hb.hair_data, hb.asset.positions, now, hb.asset.positions,
                                hb.segment_lengths, odv, ogw, inst.sdf.distances, inst.sdf.dims)
    g = hair.positions.cpu().numpy()
    assert np.array_equal(g.view(np.uint32), onew.view(np.uint32)), f"max abs diff {np.abs(g - onew).max()}"
    ctx.close()


def _frame_state(inst):
    r = Renderer(inst, 0)
    r.before_first_frame()
    r.frame()
    torch.cuda.synchronize()
    rb = r.rb
    st = dict(pos=r.hair.positions.cpu().numpy(), dv=r.grids.density_velocity.cpu().numpy(),
              tiles=rb.read_tiles(), segs=rb.read_tile_segments(), counts=rb.read_segment_counts(),
              tl=rb.read_tile_list(), px=rb.read_result(), cnt=r.ctx.counters(), md=rb.max_drawn_segments)
    rb.close()
    r.ctx.close()
    return st


def test_stress_frame_deterministic_and_lists_canonical(stress):
    a = _frame_state(stress)
    b = _frame_state(stress)
    for k in ("pos", "dv", "tiles", "counts", "tl", "px"):
        assert np.array_equal(a[k], b[k]), f"{k} differs between two runs"
    n = int(a["segs"][0])
    assert n == int(b["segs"][0]) and np.array_equal(a["segs"][:1 + 2 * n], b["segs"][:1 + 2 * n])
    assert a["cnt"]["tileRecordsDropped"] == 0 and n < a["md"], "the stress frame overflowed its segment pool"

    tiles = a["tiles"].reshape(-1, 4).astype(np.int64)
    recs = a["segs"][1:1 + 2 * n].reshape(-1, 2).astype(np.int64)
    heads, lens = tiles[:, 2], tiles[:, 3]
    used = heads != 0
    assert int(lens[used].sum()) == n, "list lengths do not add up to the record count"
    # the tiles pass writes each list as a contiguous run ending at its head:
    # entries head-1-j, next pointer head-2-j, the last one INVALID
    starts = heads[used] - lens[used]              # first (smallest) slot of each list
    assert (starts >= 0).all()
    order = np.argsort(starts)
    s_sorted, l_sorted = starts[order], lens[used][order]
    assert s_sorted[0] == 0 and np.array_equal(s_sorted[1:], (s_sorted + l_sorted)[:-1]), "lists overlap or leave gaps"
    nxt = recs[:, 1]
    is_first = np.zeros(n, bool)
    is_first[starts] = True
    idx = np.arange(n)
    assert (nxt[is_first] == INVALID).all(), "a list's last entry does not end the list"
    assert (nxt[~is_first] == idx[~is_first] - 1).all(), "a link does not point at the previous slot"
    # canonical order: inside each list the keys (strand << 8 | segment) increase with the slot,
    # so walking from the head they strictly decrease
    enc = recs[:, 0]
    key = ((enc & 0x00FFFFFF) << 8) | (enc >> 24)
    inc = key[1:] > key[:-1]
    boundary = is_first[1:]
    assert (inc | boundary).all(), "keys are not in canonical order inside a list"
    # per-tile counts equal the lengths of the tile's bins
    B = stress.cfg.tile_depth_bins
    assert np.array_equal(lens.reshape(-1, B).sum(axis=1), a["counts"].astype(np.int64))
    # the image: alpha in [0, 1 + 1e-6], zero where no tile was drawn
    px = a["px"][4:].reshape(-1, 4)
    assert np.isfinite(px).all() and (px[:, 3] >= 0).all() and (px[:, 3] <= 1.0 + 1e-6).all()
