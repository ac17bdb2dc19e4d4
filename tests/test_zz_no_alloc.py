"""nes_render_view_noalloc: the render for callers that may not allocate
device memory themselves (their host application owns the device memory and
hands out fixed buffers, or their frame loop cannot take an allocation's
implicit synchronisation).  It must give the same frame as the regular entry
point, nes_render_views, within the render tolerance of the other tests,
on consecutive calls (the shared static scratch keeps the previous call's
contents, so each call has to clear what must start at zero).

This file sorts last so a run that stops at the first failure has already run
every other test."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

PSNR_MIN = 45.0
DEPTH_TOL = 1e-3


@pytest.fixture(scope="module")
def scene_on_device(nes_lib, cuda):
    torch = cuda
    log2T = 19
    table, weights = nes_lib.scene_generate(0, log2T)
    with nes_lib.Renderer(precision=nes_lib.PREC_FP32, max_pixels=512 * 512) as r:
        occ = r.occupancy()
    dev = dict(table=torch.from_numpy(table).cuda(), weights=torch.from_numpy(weights).cuda(),
               occ=torch.from_numpy(occ.view(np.int32)).cuda(), log2T=log2T)
    torch.cuda.synchronize()
    return dev


def noalloc_render(nes_lib, torch, sc, M, W, H, f):
    view = nes_lib.make_view(M, W, H, f)
    rgb = torch.full((H * W * 3,), -1.0, device="cuda")
    dep = torch.full((H * W,), -1.0, device="cuda")
    rc = nes_lib.load().nes_render_view_noalloc(sc["table"].data_ptr(), sc["log2T"], sc["weights"].data_ptr(),
                                                sc["occ"].data_ptr(), ctypes.byref(view), rgb.data_ptr(),
                                                dep.data_ptr(), None)
    assert rc == nes_lib.NES_OK
    torch.cuda.synchronize()
    return rgb.cpu().numpy().reshape(-1, 3), dep.cpu().numpy()


def regular_render(nes_lib, torch, M, W, H, f):
    with nes_lib.Renderer(precision=nes_lib.PREC_FP32, max_pixels=W * H) as r:
        rgb = torch.empty(H * W * 3, device="cuda")
        dep = torch.empty(H * W, device="cuda")
        r.render_views([nes_lib.make_view(M, W, H, f)], [rgb.data_ptr()], [dep.data_ptr()])
        torch.cuda.synchronize()
        return rgb.cpu().numpy().reshape(-1, 3), dep.cpu().numpy()


def test_noalloc_matches_regular_entry_on_consecutive_calls(nes_lib, oracle_mod, cuda, scene_on_device):
    torch = cuda
    poses = nes_lib.shell_poses(3, 2, 1.2, 2.0)
    # Two calls in a row; the second uses the largest accepted view.
    for M, (W, H) in zip(poses, [(256, 192), (512, 512)]):
        f = nes_lib.focal_from_fov(W, 90.0)
        got_rgb, got_dep = noalloc_render(nes_lib, torch, scene_on_device, M, W, H, f)
        ref_rgb, ref_dep = regular_render(nes_lib, torch, M, W, H, f)
        assert np.all(got_dep >= 0)  # every pixel written
        assert oracle_mod.psnr(got_rgb, ref_rgb) >= PSNR_MIN
        assert np.abs(got_dep - ref_dep).max() <= DEPTH_TOL


def test_noalloc_rejects_views_beyond_the_scratch(nes_lib, cuda, scene_on_device):
    sc = scene_on_device
    lib = nes_lib.load()
    M = nes_lib.shell_poses(0, 1, 1.5, 1.5)[0]
    view = nes_lib.make_view(M, 513, 512, 256.0)  # 262,656 > NES_NOALLOC_MAX_PIXELS
    out = cuda.empty(513 * 512 * 3, device="cuda")
    rc = lib.nes_render_view_noalloc(sc["table"].data_ptr(), sc["log2T"], sc["weights"].data_ptr(),
                                     sc["occ"].data_ptr(), ctypes.byref(view), out.data_ptr(), None, None)
    assert rc == nes_lib.NES_EINVAL
