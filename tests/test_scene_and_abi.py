"""Host-side checks that need no GPU: the product's scene generator against
the oracle's independent one, the C ABI's exported symbols and argument
validation, pose helpers."""
import ctypes
import math

import numpy as np
import pytest


@pytest.mark.parametrize("seed,log2T", [(0, 19), (0, 14), (1, 14), (2, 16)])
def test_scene_generator_matches_oracle(nes_lib, oracle_mod, seed, log2T):
    table, weights = nes_lib.scene_generate(seed, log2T)
    s = oracle_mod.Scene(seed, log2T)
    assert np.array_equal(table, s.param(0))
    offs = [0, 2048, 3072, 5120, 9216, 9408]
    for i in range(5):
        assert np.array_equal(weights[offs[i]:offs[i + 1]], s.param(i + 1))


def test_scene_value_ranges(nes_lib):
    table, w = nes_lib.scene_generate(0, 14)
    assert table.min() >= -0.5 and table.max() < 0.5
    assert abs(float(table.mean())) < 0.01
    a = math.sqrt(6 / (32 + 64))
    assert np.abs(w[:2048]).max() <= a
    cw1 = w[3072:5120].reshape(64, 32)
    assert np.all(cw1[:, 31] == 0)


def test_header_symbols_exported(nes_lib):
    lib = nes_lib.load()
    syms = nes_lib.header_symbols()
    assert len(syms) >= 20
    for s in syms:
        assert hasattr(lib, s), "missing export " + s


def test_glue_rejects_bad_arguments_without_gpu(nes_lib):
    lib = nes_lib.load()
    ls = (ctypes.c_int * 3)(64, 32, 32)
    assert lib.nes_rgb24_to_yuv420p(None, 64, 64, 192, None, None, None, ls, None) == nes_lib.NES_EINVAL
    dummy = ctypes.c_void_p(16)
    assert lib.nes_rgb24_to_yuv420p(dummy, 0, 64, 192, dummy, dummy, dummy, ls, None) == nes_lib.NES_EINVAL
    bad = (ctypes.c_int * 3)(63, 32, 32)  # luma linesize below width
    assert lib.nes_rgb24_to_yuv420p(dummy, 64, 64, 192, dummy, dummy, dummy, bad, None) == nes_lib.NES_EINVAL
    assert lib.nes_depth_pack_u16mm(None, 10, None, None) == nes_lib.NES_EINVAL
    assert lib.nes_depth_to_gray8(dummy, 10, 0.0, dummy, None) == nes_lib.NES_EINVAL
    assert lib.nes_depth_pack_u16mm(None, 0, None, None) == nes_lib.NES_OK


def test_batched_glue_and_set_param_reject_bad_arguments_without_gpu(nes_lib):
    """The batched frame glue and nes_scene_set_param validate before any
    CUDA call: frame counts outside 1..NES_MAX_BATCH_FRAMES, null pointer
    arrays or frames, bad geometry, a null context."""
    lib = nes_lib.load()
    ls = (ctypes.c_int * 3)(64, 32, 32)
    dummy = ctypes.c_void_p(0x1000)
    one = (ctypes.c_void_p * 1)(dummy)
    many = (ctypes.c_void_p * 65)(*([dummy] * 65))
    for fn in (lib.nes_rgb24_to_yuv420p_batch, lib.nes_gray8_to_yuv420p_batch):
        assert fn(0, one, 64, 64, 192, one, one, one, ls, None) == nes_lib.NES_EINVAL
        assert fn(nes_lib.NES_MAX_BATCH_FRAMES + 1, many, 64, 64, 192, many, many, many, ls, None) == nes_lib.NES_EINVAL
        assert fn(1, None, 64, 64, 192, one, one, one, ls, None) == nes_lib.NES_EINVAL
        assert fn(1, one, 0, 64, 192, one, one, one, ls, None) == nes_lib.NES_EINVAL
        null_frame = (ctypes.c_void_p * 1)(None)
        assert fn(1, null_frame, 64, 64, 192, one, one, one, ls, None) == nes_lib.NES_EINVAL
    assert lib.nes_rgb24_to_yuv420p_batch(1, one, 64, 64, 100, one, one, one, ls, None) == nes_lib.NES_EINVAL  # < 3w
    assert lib.nes_depth_pack_u16mm_batch(0, one, 10, one, None) == nes_lib.NES_EINVAL
    assert lib.nes_depth_pack_u16mm_batch(65, many, 10, many, None) == nes_lib.NES_EINVAL
    assert lib.nes_depth_pack_u16mm_batch(1, None, 10, one, None) == nes_lib.NES_EINVAL
    assert lib.nes_depth_pack_u16mm_batch(1, one, 0, one, None) == nes_lib.NES_OK  # nothing to do
    buf = np.zeros(4, np.float32)
    assert lib.nes_scene_set_param(None, 1, buf.ctypes.data, 4) == nes_lib.NES_EINVAL


def test_create_validates_config(nes_lib):
    lib = nes_lib.load()
    h = ctypes.c_void_p()
    cfg = nes_lib.default_config(log2_table_size=30)
    assert lib.nes_create(ctypes.byref(cfg), ctypes.byref(h)) == nes_lib.NES_EINVAL
    cfg = nes_lib.default_config(precision=7)
    assert lib.nes_create(ctypes.byref(cfg), ctypes.byref(h)) == nes_lib.NES_EINVAL
    cfg = nes_lib.default_config(fov_deg=180.0)
    assert lib.nes_create(ctypes.byref(cfg), ctypes.byref(h)) == nes_lib.NES_EINVAL
    for levels in (1, 9, 11, 12, 14, 16):  # records cover levels 0..9 or 0..12 (or the default, 0)
        cfg = nes_lib.default_config(precision=nes_lib.PREC_FP16_TC, record_levels=levels)
        assert lib.nes_create(ctypes.byref(cfg), ctypes.byref(h)) == nes_lib.NES_EINVAL
    assert nes_lib.default_config().record_levels == 13


def test_server_create_validates_config(nes_lib):
    """nes_server_create checks its configuration before it touches the
    context or the GPU (the context here is a zeroed stand-in)."""
    lib = nes_lib.load()
    ctx = ctypes.create_string_buffer(4096)
    h = ctypes.c_void_p()
    for field, value in (("max_batch_pixels", 0), ("max_batch_pixels", 63), ("max_batch_pixels", (1 << 27) + 1),
                         ("max_inflight_batches", 0), ("max_inflight_batches", 5), ("max_pending", 0),
                         ("max_queue_ms", -1.0), ("max_queue_ms", float("nan"))):
        cfg = nes_lib.NesServerConfig()
        lib.nes_server_config_default(ctypes.byref(cfg))
        setattr(cfg, field, value)
        assert lib.nes_server_create(ctx, ctypes.byref(cfg), ctypes.byref(h)) == nes_lib.NES_EINVAL, (field, value)
        assert not h.value
    cfg = nes_lib.NesServerConfig()
    lib.nes_server_config_default(ctypes.byref(cfg))
    assert lib.nes_server_create(None, ctypes.byref(cfg), ctypes.byref(h)) == nes_lib.NES_EINVAL


def test_noalloc_render_rejects_bad_arguments_without_gpu(nes_lib):
    """nes_render_view_noalloc validates its arguments and the view before
    any CUDA call: missing arrays, a table size outside 2^10..2^24, a view
    the renderer rejects (zero or over-16384 sides, non-finite pose or
    focal length) and views above NES_NOALLOC_MAX_PIXELS."""
    lib = nes_lib.load()
    fn = lib.nes_render_view_noalloc
    d = 0x1000  # device addresses are never dereferenced on these paths
    M = [1, 0, 0, 0.5, 0, -1, 0, 0.5, 0, 0, -1, 0.5]
    good = nes_lib.make_view(M, 64, 64, 32.0)
    E = nes_lib.NES_EINVAL
    assert fn(None, 19, d, d, ctypes.byref(good), d, d, None) == E
    assert fn(d, 19, None, d, ctypes.byref(good), d, d, None) == E
    assert fn(d, 19, d, None, ctypes.byref(good), d, d, None) == E
    assert fn(d, 19, d, d, None, d, d, None) == E
    assert fn(d, 19, d, d, ctypes.byref(good), None, None, None) == E  # no output at all
    assert fn(d, 9, d, d, ctypes.byref(good), d, d, None) == E
    assert fn(d, 25, d, d, ctypes.byref(good), d, d, None) == E
    bad_pose = list(M)
    bad_pose[7] = float("inf")
    for v in (nes_lib.make_view(M, 0, 64, 32.0), nes_lib.make_view(M, 16385, 1, 32.0),
              nes_lib.make_view(M, 64, 64, float("inf")), nes_lib.make_view(M, 64, 64, float("nan")),
              nes_lib.make_view(M, 64, 64, 0.0), nes_lib.make_view(bad_pose, 64, 64, 32.0),
              nes_lib.make_view(M, 513, 512, 256.0)):  # 262,656 > NES_NOALLOC_MAX_PIXELS
        assert fn(d, 19, d, d, ctypes.byref(v), d, d, None) == E


def test_create_without_gpu_fails_cleanly(nes_lib):
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(nes_lib.NesError) as e:
        nes_lib.Renderer()
    assert e.value.code == nes_lib.NES_ENODEV


def test_render_server_binary_fails_cleanly_without_gpu(nes_lib):
    import os
    import subprocess
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    import nes_build
    r = subprocess.run([nes_build.SERVER_BIN, "--port", "0"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 1 and "no usable CUDA device" in r.stderr
    r = subprocess.run([nes_build.SERVER_BIN, "--bogus", "1"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 2
    # Values are checked before the GPU is touched: out-of-range ports and
    # table sizes, unknown precisions, FOVs outside (0, 180), trailing options.
    for bad in (["--port", "70000"], ["--port", "12x"], ["--port"], ["--precision", "bf16"],
                ["--fov", "180"], ["--fov", "abc"], ["--log2-table", "30"], ["--device", "-1"]):
        r = subprocess.run([nes_build.SERVER_BIN] + bad, capture_output=True, text=True, timeout=60)
        assert r.returncode == 2 and ("bad value" in r.stderr or "needs a value" in r.stderr), bad


def test_focal_and_capacity(nes_lib):
    assert nes_lib.focal_from_fov(1920, 90.0) == pytest.approx(960.0, rel=1e-6)
    assert nes_lib.focal_from_fov(256, 90.0) == np.float32(128.0)
    lib = nes_lib.load()
    assert lib.nes_rendered_frame_capacity(1280, 720) >= 1280 * 720 * 4 + 32


def test_poses_on_shell(nes_lib):
    poses = nes_lib.shell_poses(0, 100, 1.5, 1.5)
    for M in poses:
        M = np.asarray(M).reshape(3, 4)
        eye = M[:, 3]
        assert abs(np.linalg.norm(eye - 0.5) - 1.5) < 1e-12
        R = M[:, :3]
        assert np.allclose(R.T @ R, np.eye(3), atol=1e-12)
        # forward column looks at the centre
        assert np.allclose(R[:, 2], (0.5 - eye) / 1.5, atol=1e-12)
    shell = nes_lib.shell_poses(5, 200, 1.2, 2.0)
    r = [np.linalg.norm(np.asarray(M).reshape(3, 4)[:, 3] - 0.5) for M in shell]
    assert 1.2 <= min(r) and max(r) <= 2.0
    left, right = nes_lib.stereo_pair(shell[0], 0.063)
    assert abs(np.linalg.norm(np.asarray(left)[[3, 7, 11]] - np.asarray(right)[[3, 7, 11]]) - 0.063) < 1e-12


def test_linesizes(nes_lib):
    assert nes_lib.linesizes(1280) == [1280, 640, 640]
    assert nes_lib.linesizes(1920) == [1920, 960, 960]
    assert nes_lib.linesizes(33) == [64, 32, 32]


def test_probe_and_selftest_entries_reject_bad_arguments_without_gpu(nes_lib):
    """The gather probes, the bounded-wait self-test and the multi-view
    pose->YUV call check their arguments before any CUDA call."""
    lib = nes_lib.load()
    sink = ctypes.c_void_p(0x1000)
    table = ctypes.c_void_p(0x2000)
    EINVAL = nes_lib.NES_EINVAL
    assert lib.nes_probe_gather(None, 1 << 25, 4, 16, 256, sink, None) == EINVAL
    assert lib.nes_probe_gather(table, 1 << 25, 4, 16, 256, None, None) == EINVAL
    assert lib.nes_probe_gather(table, 1 << 25, 4, 0, 256, sink, None) == EINVAL
    assert lib.nes_probe_gather(table, 1 << 25, 8, 16, 256, sink, None) == EINVAL      # 4, 16 or 32 bytes
    assert lib.nes_probe_gather(table, 3 << 20, 4, 16, 256, sink, None) == EINVAL      # not a power of two
    assert lib.nes_probe_gather(table, 1 << 25, 16, 16, 100, sink, None) == EINVAL     # threads % 256
    ms = ctypes.c_float(0)
    assert lib.nes_probe_gather_replay(None, None, 1, 512, sink, 1 << 20, ctypes.byref(ms)) == EINVAL
    assert lib.nes_selftest_bounded_wait(None, 100, 0) == EINVAL
    ls = (ctypes.c_int * 3)(64, 32, 32)
    views = (nes_lib.NesView * 2)()
    ptrs = (ctypes.c_void_p * 2)(0x1000, 0x2000)
    assert lib.nes_render_yuv_views(None, views, 2, ptrs, ptrs, ptrs, ls, None) == EINVAL
