"""Serving loop (nes_server_*): continuous batching of mono and stereo
requests of mixed resolutions.  A request's frame must be the same rendered
alone and rendered in a batch with others (the march is per ray; batching
only changes which rays share a tile), and the same as the synchronous
pose->YUV call.  Admission against the memory budget drops requests instead of
stalling, and recovers once slots are released."""
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def views_for(nes_lib, pose, w, h, fov, stereo):
    f = nes_lib.focal_from_fov(w, fov)
    poses = nes_lib.stereo_pair(pose, 0.063) if stereo else [pose]
    return [nes_lib.make_view(m, w, h, f) for m in poses]


@pytest.fixture(scope="module")
def server(nes_lib, rtc):
    srv = nes_lib.Server(rtc, max_inflight_batches=1, max_batch_pixels=2 * 1920 * 1832,
                         hbm_budget_bytes=4 << 30)
    yield srv
    srv.close()


def test_same_alone_and_in_the_mix(nes_lib, server):
    poses = nes_lib.shell_poses(12, 5, 1.2, 2.0)
    big = views_for(nes_lib, poses[0], 1920, 1832, 100.0, True)  # keeps the single slot busy
    a = views_for(nes_lib, poses[1], 640, 360, 90.0, False)
    b = views_for(nes_lib, poses[2], 1280, 720, 90.0, False)
    c = views_for(nes_lib, poses[3], 320, 180, 100.0, True)
    tb = server.submit(big)
    ta, tb2, tc = server.submit(a), server.submit(b), server.submit(c)
    assert None not in (tb, ta, tb2, tc)
    mixed = {t: server.wait(t) for t in (tb, ta, tb2, tc)}
    ra = mixed[ta]
    assert ra.status == 0 and ra.batch_requests >= 2, "A should have shared a batch"
    assert mixed[tb2].batch_id == ra.batch_id
    got_mixed = server.fetch(ra)
    got_c = [server.fetch(mixed[tc], v) for v in (0, 1)]
    # A again, alone.
    ta2 = server.submit(a)
    ra2 = server.wait(ta2)
    assert ra2.batch_requests == 1
    alone = server.fetch(ra2)
    for x, y in zip(got_mixed, alone):
        assert np.array_equal(x, y)
    tc2 = server.submit(c)
    rc2 = server.wait(tc2)
    for v in (0, 1):
        for x, y in zip(got_c[v], server.fetch(rc2, v)):
            assert np.array_equal(x, y)
    for t in (tb, ta, tb2, tc, ta2, tc2):
        server.release(t)


def test_matches_synchronous_pose_to_yuv(nes_lib, server, rtc, cuda):
    torch = cuda
    pose = nes_lib.shell_poses(3, 1, 1.5, 1.5)[0]
    W, H = 1280, 720
    (view,) = views_for(nes_lib, pose, W, H, 90.0, False)
    t = server.submit([view])
    res = server.wait(t)
    y, u, v, d = server.fetch(res)
    ls = list(res.linesize)
    ch = (H + 1) // 2
    hy = torch.empty(ls[0] * H, dtype=torch.uint8).pin_memory()
    hu = torch.empty(ls[1] * ch, dtype=torch.uint8).pin_memory()
    hv = torch.empty(ls[2] * ch, dtype=torch.uint8).pin_memory()
    hd = torch.empty(W * H, dtype=torch.int16).pin_memory()
    rtc.render_yuv(view, hy.data_ptr(), hu.data_ptr(), hv.data_ptr(), ls, hd.data_ptr())
    rows = lambda a, l, w, h: a.reshape(-1, l)[:h, :w]
    assert np.array_equal(rows(y, ls[0], W, H), rows(hy.numpy(), ls[0], W, H))
    assert np.array_equal(rows(u, ls[1], W // 2, ch), rows(hu.numpy(), ls[1], W // 2, ch))
    assert np.array_equal(d, hd.numpy().view(np.uint16))
    server.release(t)


def test_one_graph_serves_every_batch_shape(nes_lib, server, cuda):
    """Each slot's graph is instantiated once at creation and replayed for
    batches of any shape (the kernels read the batch from a device-side
    descriptor): batches of four different shapes add no instantiation and
    no update, and serving them allocates no device memory (outputs come
    from the arena reserved at creation)."""
    torch = cuda
    pose = nes_lib.shell_poses(4, 4, 1.2, 2.0)
    before = server.stats()
    assert before["graph_instantiations"] == 1  # one slot
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    ts = []
    for i, (w, h, stereo) in enumerate([(96, 64, False), (640, 360, False), (200, 100, True), (1280, 720, False)]):
        t = server.submit(views_for(nes_lib, pose[i], w, h, 90.0, stereo))
        assert server.wait(t).status == 0
        ts.append(t)
    free1, _ = torch.cuda.mem_get_info()
    after = server.stats()
    assert after["graph_instantiations"] == before["graph_instantiations"]
    assert after["graph_updates"] == before["graph_updates"] == 0
    assert free1 == free0
    for t in ts:
        server.release(t)


def test_admission_budget_drops_and_recovers(nes_lib, rtc):
    # The fixed per-slot cost of this configuration (a server's budget use
    # right after creation), then a budget of that plus exactly two 640x360
    # outputs: Y 640x360 + U, V 320x180 + uint16 depth = 806,400 bytes each.
    cfg = dict(max_inflight_batches=1, max_batch_pixels=640 * 360 * 2)
    with nes_lib.Server(rtc, hbm_budget_bytes=1 << 30, **cfg) as probe:
        fixed = probe.stats()["budget_used_bytes"]
    srv = nes_lib.Server(rtc, hbm_budget_bytes=fixed + 2 * 806_400 + 1000, **cfg)
    try:
        pose = nes_lib.shell_poses(5, 1, 1.5, 1.5)[0]
        v = views_for(nes_lib, pose, 640, 360, 90.0, False)
        t1, t2 = srv.submit(v), srv.submit(v)
        assert t1 is not None and t2 is not None
        assert srv.submit(v) is None  # over budget: dropped, not queued
        st = srv.stats()
        assert st["rejected"] == 1 and st["submitted"] == 2
        srv.wait(t1)
        srv.release(t1)
        t3 = srv.submit(v)
        assert t3 is not None
        for t in (t2, t3):
            assert srv.wait(t).status == 0
            srv.release(t)
    finally:
        srv.close()


def test_wait_timeout_and_bad_ticket(nes_lib, server):
    pose = nes_lib.shell_poses(6, 1, 1.2, 2.0)[0]
    t = server.submit(views_for(nes_lib, pose, 1920, 1832, 100.0, True))
    r = server.wait(t, timeout_ns=1000)  # 1 us: the stereo frame cannot be done yet
    assert r is None
    assert server.wait(t).status == 0
    server.release(t)
    with pytest.raises(nes_lib.NesError):
        server.release(t)  # already released
    with pytest.raises(nes_lib.NesError):
        server.wait(10 ** 12)


def test_invalid_requests(nes_lib, server):
    pose = nes_lib.shell_poses(7, 1, 1.5, 1.5)[0]
    f = nes_lib.focal_from_fov(64, 90.0)
    left = nes_lib.make_view(pose, 64, 64, f)
    right = nes_lib.make_view(pose, 32, 64, f)
    with pytest.raises(nes_lib.NesError):
        server.submit([left, right])  # stereo eyes must match in size
    with pytest.raises(nes_lib.NesError):
        server.submit([nes_lib.make_view(pose, 0, 64, f)])
    # Non-finite poses and focal lengths are refused at submission, so they
    # never reach (and fail) a batch shared with other requests.
    bad = list(pose)
    bad[3] = float("nan")
    for views in ([nes_lib.make_view(bad, 64, 64, f)], [left, nes_lib.make_view(bad, 64, 64, f)],
                  [nes_lib.make_view(pose, 64, 64, float("inf"))]):
        with pytest.raises(nes_lib.NesError) as e:
            server.submit(views)
        assert e.value.code == nes_lib.NES_EINVAL
    t = server.submit([left])
    assert server.wait(t).status == 0
    server.release(t)


def test_smallest_batch_size(nes_lib, rtc):
    """max_batch_pixels at its minimum (64): the slot buffers still hold the
    creation-time warm-up batch, and an 8x8 request is served."""
    pose = nes_lib.shell_poses(8, 1, 1.5, 1.5)[0]
    with nes_lib.Server(rtc, max_inflight_batches=1, max_batch_pixels=64, hbm_budget_bytes=1 << 26) as srv:
        t = srv.submit([nes_lib.make_view(pose, 8, 8, nes_lib.focal_from_fov(8, 90.0))])
        assert t is not None
        r = srv.wait(t)
        assert r.status == 0 and r.width == 8 and r.height == 8
        srv.release(t)
        with pytest.raises(nes_lib.NesError):
            srv.submit([nes_lib.make_view(pose, 16, 8, nes_lib.focal_from_fov(16, 90.0))])  # > 64 pixels


def test_queue_delay_bound_rejects_late_requests(nes_lib, rtc):
    """max_queue_ms: once a batch has completed (the throughput estimate), a
    burst of stereo 2x1920x1832 requests (~30 ms each) is admitted only while
    the expected pose -> YUV time stays within 100 ms; without the bound the
    same burst is admitted in full."""
    pose = nes_lib.shell_poses(21, 1, 1.5, 1.5)[0]
    big = views_for(nes_lib, pose, 1920, 1832, 100.0, True)
    admitted = {}
    for bound in (0.0, 100.0):
        srv = nes_lib.Server(rtc, max_inflight_batches=1, max_batch_pixels=2 * 1920 * 1832,
                             hbm_budget_bytes=8 << 30, max_pending=64, max_queue_ms=bound)
        try:
            t0 = srv.submit(big)
            assert t0 is not None
            srv.wait(t0)
            srv.release(t0)
            tickets = [srv.submit(big) for _ in range(8)]
            ok = [t for t in tickets if t is not None]
            for t in ok:
                assert srv.wait(t).status == 0
                srv.release(t)
            admitted[bound] = len(ok)
            assert srv.stats()["rejected"] == 8 - len(ok)
        finally:
            srv.close()
    assert admitted[0.0] == 8
    assert 1 <= admitted[100.0] < 8, admitted


def test_plane_padding_is_zero(nes_lib, server):
    """Served planes carry zeros in their row padding: the output arena is
    reused from request to request, and no request sees bytes of an earlier
    frame there."""
    poses = nes_lib.shell_poses(4, 2, 1.5, 1.5)
    t = server.submit(views_for(nes_lib, poses[0], 1280, 720, 90.0, False))
    assert server.wait(t).status == 0
    server.release(t)
    for W, H in ((33, 17), (650, 31)):
        t = server.submit(views_for(nes_lib, poses[1], W, H, 90.0, False))
        res = server.wait(t)
        assert res.status == 0
        y, u, v, _ = server.fetch(res)
        ls, ch, cw = list(res.linesize), (H + 1) // 2, (W + 1) // 2
        assert ls[0] > W and ls[1] > cw
        assert not y.reshape(H, ls[0])[:, W:].any()
        assert not u.reshape(ch, ls[1])[:, cw:].any() and not v.reshape(ch, ls[2])[:, cw:].any()
        server.release(t)
