"""nes_render_view_noalloc: the render for callers that may not allocate
device memory themselves (their host application owns the device memory and
hands out fixed buffers, or their frame loop cannot take an allocation's
implicit synchronisation).  It runs the same kernels as the regular entry
point, nes_render_views, on the same inputs, so its frames must equal that
entry point's bit for bit and meet the render tolerance against the FP64
oracle, on consecutive calls (the shared static scratch keeps the previous
call's contents, so each call has to clear what must start at zero), also
when two calls follow each other on one stream with no host synchronisation
in between, and repeated calls must not change the device's free memory.

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


def noalloc_call(nes_lib, sc, view, rgb, dep, stream=None):
    return nes_lib.load().nes_render_view_noalloc(sc["table"].data_ptr(), sc["log2T"], sc["weights"].data_ptr(),
                                                  sc["occ"].data_ptr(), ctypes.byref(view), rgb.data_ptr(),
                                                  dep.data_ptr(), ctypes.c_void_p(stream) if stream else None)


def noalloc_render(nes_lib, torch, sc, M, W, H, f):
    view = nes_lib.make_view(M, W, H, f)
    rgb = torch.full((H * W * 3,), -1.0, device="cuda")
    dep = torch.full((H * W,), -1.0, device="cuda")
    assert noalloc_call(nes_lib, sc, view, rgb, dep) == nes_lib.NES_OK
    torch.cuda.synchronize()
    return rgb.cpu().numpy().reshape(-1, 3), dep.cpu().numpy()


def regular_render(nes_lib, torch, M, W, H, f):
    with nes_lib.Renderer(precision=nes_lib.PREC_FP32, max_pixels=W * H) as r:
        rgb = torch.empty(H * W * 3, device="cuda")
        dep = torch.empty(H * W, device="cuda")
        r.render_views([nes_lib.make_view(M, W, H, f)], [rgb.data_ptr()], [dep.data_ptr()])
        torch.cuda.synchronize()
        return rgb.cpu().numpy().reshape(-1, 3), dep.cpu().numpy()


def test_noalloc_matches_regular_entry_on_consecutive_calls(nes_lib, oracle_mod, scene0, cuda, scene_on_device):
    torch = cuda
    poses = nes_lib.shell_poses(3, 2, 1.2, 2.0)
    # Two calls in a row; the second uses the largest accepted view.
    for M, (W, H) in zip(poses, [(256, 192), (512, 512)]):
        f = nes_lib.focal_from_fov(W, 90.0)
        got_rgb, got_dep = noalloc_render(nes_lib, torch, scene_on_device, M, W, H, f)
        ref_rgb, ref_dep = regular_render(nes_lib, torch, M, W, H, f)
        assert np.all(got_dep >= 0)  # every pixel written
        # Same kernels, same inputs: the same bits as the regular entry point.
        assert np.array_equal(got_rgb, ref_rgb) and np.array_equal(got_dep, ref_dep)
        # And the render tolerance against the FP64 oracle on a pixel sample.
        pix = np.random.default_rng(W).choice(W * H, 4096, replace=False).astype(np.int32)
        o_rgb, o_dep, _ = scene0.render(M, W, H, f, pixels=pix)
        assert oracle_mod.psnr(got_rgb[pix], o_rgb) >= PSNR_MIN
        assert np.abs(got_dep[pix] - o_dep).max() <= DEPTH_TOL


def test_noalloc_back_to_back_on_one_stream(nes_lib, cuda, scene_on_device):
    """Two calls queued on one non-default stream with no host sync between
    them: the second call's counter reset is ordered after the first call's
    march on that stream, so both frames equal the regular entry's."""
    torch = cuda
    poses = nes_lib.shell_poses(5, 2, 1.2, 2.0)
    W, H = 320, 240
    f = nes_lib.focal_from_fov(W, 90.0)
    st = torch.cuda.Stream()
    outs = [(torch.full((H * W * 3,), -1.0, device="cuda"), torch.full((H * W,), -1.0, device="cuda"))
            for _ in poses]
    torch.cuda.synchronize()
    views = [nes_lib.make_view(M, W, H, f) for M in poses]
    for v, (rgb, dep) in zip(views, outs):
        assert noalloc_call(nes_lib, scene_on_device, v, rgb, dep, st.cuda_stream) == nes_lib.NES_OK
    st.synchronize()
    for M, (rgb, dep) in zip(poses, outs):
        ref_rgb, ref_dep = regular_render(nes_lib, torch, M, W, H, f)
        assert np.array_equal(rgb.cpu().numpy().reshape(-1, 3), ref_rgb)
        assert np.array_equal(dep.cpu().numpy(), ref_dep)


def test_noalloc_calls_leave_free_memory_unchanged(nes_lib, cuda, scene_on_device):
    torch = cuda
    M = nes_lib.shell_poses(7, 1, 1.5, 1.5)[0]
    W, H = 512, 512
    view = nes_lib.make_view(M, W, H, nes_lib.focal_from_fov(W, 90.0))
    rgb = torch.empty(H * W * 3, device="cuda")
    dep = torch.empty(H * W, device="cuda")
    # One call first: the library's device code (and its static scratch) may
    # be loaded lazily on its first launch.
    assert noalloc_call(nes_lib, scene_on_device, view, rgb, dep) == nes_lib.NES_OK
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(5):
        assert noalloc_call(nes_lib, scene_on_device, view, rgb, dep) == nes_lib.NES_OK
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0


def test_noalloc_rejects_views_beyond_the_scratch(nes_lib, cuda, scene_on_device):
    sc = scene_on_device
    lib = nes_lib.load()
    M = nes_lib.shell_poses(0, 1, 1.5, 1.5)[0]
    view = nes_lib.make_view(M, 513, 512, 256.0)  # 262,656 > NES_NOALLOC_MAX_PIXELS
    out = cuda.empty(513 * 512 * 3, device="cuda")
    rc = lib.nes_render_view_noalloc(sc["table"].data_ptr(), sc["log2T"], sc["weights"].data_ptr(),
                                     sc["occ"].data_ptr(), ctypes.byref(view), out.data_ptr(), None, None)
    assert rc == nes_lib.NES_EINVAL
