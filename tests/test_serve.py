"""Serving: admission under a memory budget and continuous batching
(hairfb/serve.py).  A session's frames in the served mix equal the same
session's frames rendered alone through hfb_frame: positions and density
grid bit-exact, pixels within 1/255."""

import numpy as np
import pytest

from hairfb import serve
from hairfb.config import HairConfig

CFG = HairConfig(tile_size=16, tile_depth_bins=8, slices_per_pixel=4, shading_points=8, grid_dims=32)


def _specs():
    sp = serve.poisson_sessions(seed=5, count=6, rate_hz=400.0, frames=3, strands=(200, 1500), points=16,
                                side=(128, 320))
    for k, s in enumerate(sp):
        s.frames = 2 + k % 3  # sessions of 2..4 frames: they leave at different ticks
    return sp


def test_poisson_sessions_and_snap():
    sp = serve.poisson_sessions(seed=0, count=256)
    assert len(sp) == 256 and all(b.arrival_s > a.arrival_s for a, b in zip(sp, sp[1:]))
    assert all(500 <= s.strands <= 50000 and 256 <= s.width <= 2048 and s.width % 16 == 0 for s in sp)
    snapped = serve.snap(sp)
    assert len({s.strands for s in snapped}) <= 8 and len({s.width for s in snapped}) <= 8
    assert all(abs(np.log(a.strands / b.strands)) < 0.4 for a, b in zip(sp, snapped))


@pytest.mark.gpu
def test_served_sessions_equal_sessions_alone():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA GPU")
    from hairfb.renderer import Renderer

    specs = _specs()
    factory = serve.SessionFactory(CFG, seed=1)
    factory.prepare(specs)
    probe = serve.Server(CFG, 0, budget_bytes=1 << 40, make_instance=factory)
    sizes = sorted(probe.session_bytes(s) for s in specs)
    probe.close()
    # room for about three sessions at a time: later arrivals queue for admission
    server = serve.Server(CFG, 0, budget_bytes=sum(sizes[-3:]), make_instance=factory)
    final = {}

    def frame_done(s):
        if s.done == s.spec.frames:
            r = s.renderer
            final[s.spec.sid] = (r.hair.positions.cpu().numpy().copy(),
                                 r.grids.density_velocity.cpu().numpy().copy(),
                                 r.rb.read_result()[4:].copy(), r.hair.shading.cpu().numpy().copy())

    st = server.run(specs, frame_done)
    assert st.frames == sum(s.frames for s in specs)
    assert st.dropped == 0
    assert st.peak_bytes <= server.budget and st.peak_sessions < len(specs), (st.peak_sessions, st.peak_bytes)
    assert max(st.admit_wait_ms) > 0.0  # someone waited for memory
    server.close()

    for sp in specs:
        r = Renderer(factory(sp), 0, max_drawn=serve.pool_records(sp), hair_depth=True)
        r.before_first_frame()
        for _ in range(sp.frames):
            r.frame_native()
        torch.cuda.synchronize()
        pos, dv, px, shade = final[sp.sid]
        assert np.array_equal(r.hair.positions.cpu().numpy(), pos), f"session {sp.sid}: positions"
        assert np.array_equal(r.grids.density_velocity.cpu().numpy(), dv), f"session {sp.sid}: density grid"
        assert np.abs(r.hair.shading.cpu().numpy() - shade).max() <= 1e-6, f"session {sp.sid}: shading"
        err = np.abs(r.rb.read_result()[4:] - px).max()
        assert err <= 1.0 / 255.0, f"session {sp.sid}: pixel error {err}"
        r.rb.close()
        r.ctx.close()
