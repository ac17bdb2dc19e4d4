"""A bounded device wait that runs out: the kernel reports NES_ETIMEDOUT
through the scratch error word instead of hanging, frees its tensor memory on
the way out, and the same context renders correctly afterwards.  neserver's
analogue is the 1 s LockTimeout of its frame queue
(src/base/video/frame_queue.cc:14-22).  Nothing faults or hangs: the wait is
on an mbarrier nothing arrives at, with a short poll limit."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _render_small(nes_lib, r, torch, M, W, H, f):
    rgb = torch.empty(W * H * 3, device="cuda")
    dep = torch.empty(W * H, device="cuda")
    r.render_views([nes_lib.make_view(M, W, H, f)], [rgb.data_ptr()], [dep.data_ptr()])
    torch.cuda.synchronize()
    return rgb.cpu().numpy().reshape(-1, 3), dep.cpu().numpy(), r.last_sample_count()


@pytest.mark.parametrize("which", ["rtc", "r32"])
def test_wait_runs_out_then_context_renders(nes_lib, oracle_mod, scene0, cuda, request, which):
    r = request.getfixturevalue(which)
    lib = nes_lib.load()
    # Positive control: the barrier was completed, the wait succeeds.
    assert lib.nes_selftest_bounded_wait(r.h, 1000, 1) == nes_lib.NES_OK
    # Nothing arrives: the wait gives up after 1,000 polls.
    for _ in range(3):
        assert lib.nes_selftest_bounded_wait(r.h, 1000, 0) == nes_lib.NES_ETIMEDOUT
    assert lib.nes_selftest_bounded_wait(r.h, 0, 0) == nes_lib.NES_EINVAL
    # The context still renders, matching the oracle (and the error word of
    # the probe does not leak into the render's status).
    M = nes_lib.shell_poses(0, 1, 1.5, 1.5)[0]
    W, H = 32, 24
    f = nes_lib.focal_from_fov(W, 90.0)
    g_rgb, g_dep, samples = _render_small(nes_lib, r, cuda, M, W, H, f)
    o_rgb, o_dep, o_samples = scene0.render(M, W, H, f)
    assert samples == o_samples
    assert oracle_mod.psnr(g_rgb, o_rgb) >= 45.0
    assert float(np.abs(g_dep - o_dep).max()) <= 1e-3
