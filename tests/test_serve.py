"""Serving: admission under a memory budget and continuous batching of
frame requests (hairfb/serve.py).  A session's frames in the served mix
equal the same session's frames rendered alone through hfb_frame: positions
and density grid bit-exact, pixels within 1/255."""

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


def test_request_times_are_a_poisson_process():
    sp = serve.SessionSpec(3, 0.0, 1000, 32, 256, 256, 4000, 0)
    t = serve.request_times(sp, 8.0, seed=0)
    assert len(t) == 4000 and np.all(np.diff(t) > 0)
    gaps = np.diff(np.concatenate([[0.0], t]))
    assert abs(gaps.mean() - 1 / 8.0) < 0.01 and abs(gaps.std() / gaps.mean() - 1.0) < 0.05  # exponential
    assert np.array_equal(t, serve.request_times(sp, 8.0, seed=0))  # seeded


def test_cost_model_fits_tick_times():
    cm = serve.CostModel()
    rng = np.random.Generator(np.random.PCG64(1))
    for _ in range(64):
        pts, pix = rng.uniform(1e4, 2e6), rng.uniform(6e4, 4e6)
        cm.add(pts, pix, 0.3 + 2e-7 * pts + 1e-7 * pix)
    assert abs(cm.ms(1e6, 1e6) - (0.3 + 0.2 + 0.1)) < 1e-6


def test_tick_takes_the_oldest_requests_one_per_session_within_the_budget():
    """Server._form (host logic, no GPU): the sessions with a pending request
    and no frame on the GPU, oldest request first, one frame each, until the
    cost model's estimate would pass the tick budget -- and at least one."""
    import types
    cm = serve.CostModel(a=0.0, b=1e-3, c=0.0)  # 1 ms per 1,000 points
    fake = types.SimpleNamespace(cost=cm, tick_budget_ms=3.0)

    def session(sid, points, requests, busy=False):
        s = serve.Session(serve.SessionSpec(sid, 0.0, points, 1, 16, 16, 10, 0))
        s.work = (float(points), 0.0)
        s.pending.extend(requests)
        s.busy = busy
        return s

    ready = [session(0, 1000, [0.5, 0.6]), session(1, 1000, [0.2]), session(2, 1000, [0.1], busy=True),
             session(3, 1000, []), session(4, 1000, [0.3]), session(5, 1000, [0.4])]
    group = serve.Server._form(fake, ready)
    assert [s.spec.sid for s in group] == [1, 4, 5]  # oldest first; busy and idle sessions skipped; 3 ms
    fake.tick_budget_ms = 0.5
    assert [s.spec.sid for s in serve.Server._form(fake, ready)] == [1]  # over budget alone: still one
    assert serve.Server._form(fake, [ready[2], ready[3]]) == []


def test_steady_rate_counts_the_window_where_every_session_asks():
    """steady_frames_per_s: frames completed between the last session's first
    request and the first session's last frame, per second of that window."""
    st = serve.ServeStats(frames=7, wall_s=10.0, ticks=7, latency_ms=[1.0] * 7, admit_wait_ms=[0.0],
                          peak_sessions=2, peak_bytes=0, budget_bytes=1, dropped=0, lanes=1, offered_hz=2.0,
                          frames_per_tick=1.0, tick_gpu_ms=[1.0] * 7)
    st.done_s = [0.5, 1.5, 2.0, 2.5, 3.0, 3.5, 9.0]
    st.all_active_s, st.first_finished_s = 1.0, 3.0
    assert st.steady_frames_per_s == pytest.approx(4 / 2.0)
    st.latency_ms = [9.0, 1.0, 2.0, 3.0, 4.0, 5.0, 9.0]
    st.arrival_s = [0.4, 1.4, 1.9, 2.4, 2.9, 2.9, 8.0]
    # the window holds the requests that arrived at or after 1.0 and completed by 3.0
    assert st.steady_pct(0.0) == 1.0 and st.steady_pct(1.0) == 4.0
    st.first_finished_s = 0.5  # no window: a session finished before the last one started
    assert st.steady_frames_per_s == 0.0 and st.steady_pct(0.99) == 0.0


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

    st = server.run(specs, frame_done=frame_done, per_session_rate_hz=300.0)
    assert st.frames == sum(s.frames for s in specs) == len(st.latency_ms)
    assert all(v > 0.0 for v in st.latency_ms)
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
