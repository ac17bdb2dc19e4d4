"""Frame glue on the GPU, bit-exact against the oracle's integer restatement
(swscale itself is not installed anywhere this runs: swscale parity is
unpinned).  Covers odd sizes, padded linesizes, the 1x1 frame, the configured
frame sizes and depth-packing edge values."""
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu


def synth_frame(rng, w, h):
    """50/50 blend of uniform bytes and a horizontal gradient."""
    noise = rng.integers(0, 256, (h, w, 3)).astype(np.uint16)
    grad = np.broadcast_to((np.arange(w) * 255 // max(1, w - 1)).astype(np.uint16)[None, :, None], (h, w, 3))
    return ((noise + grad) // 2).astype(np.uint8)


def gpu_yuv(torch, nes_lib, img, w, h, rgb_ls, ls, gray=False):
    ch = (h + 1) // 2
    src = torch.from_numpy(np.ascontiguousarray(img).reshape(-1)).cuda()
    y = torch.full((ls[0] * h,), 7, dtype=torch.uint8, device="cuda")
    u = torch.full((ls[1] * ch,), 7, dtype=torch.uint8, device="cuda")
    v = torch.full((ls[2] * ch,), 7, dtype=torch.uint8, device="cuda")
    fn = nes_lib.gray8_to_yuv420p if gray else nes_lib.rgb24_to_yuv420p
    fn(src.data_ptr(), w, h, rgb_ls, y.data_ptr(), u.data_ptr(), v.data_ptr(), ls)
    torch.cuda.synchronize()
    return y.cpu().numpy(), u.cpu().numpy(), v.cpu().numpy()


def visible(plane, ls, w, h):
    return plane.reshape(-1, ls)[:h, :w]


# Row strides that are multiples of 8 take the vector kernel (8x2 pixel
# blocks); (33, 17, 5), (30, 20, 6) and (1922, 1081, 2) do so with blocks
# cut by the right and bottom edges.  The others take the per-sample kernel.
@pytest.mark.parametrize("w,h,pad", [(1280, 720, 0), (1920, 1080, 0), (1920, 1832, 0), (640, 360, 0),
                                      (33, 17, 0), (31, 1, 5), (1, 1, 0), (2, 2, 3), (257, 255, 32),
                                      (33, 17, 5), (30, 20, 6), (1922, 1081, 2)])
def test_rgb24_to_yuv420p_bit_exact(cuda, nes_lib, oracle_mod, w, h, pad):
    rng = np.random.default_rng(w * 7919 + h)
    img = synth_frame(rng, w, h)
    rgb_ls = 3 * w + pad
    buf = np.zeros((h, rgb_ls), np.uint8)
    buf[:, :3 * w] = img.reshape(h, 3 * w)
    ls = nes_lib.linesizes(w)
    gy, gu, gv = gpu_yuv(cuda, nes_lib, buf, w, h, rgb_ls, ls)
    oy, ou, ov = oracle_mod.rgb24_to_yuv420p(buf, w, h, rgb_ls, ls)
    cw, ch = (w + 1) // 2, (h + 1) // 2
    assert np.array_equal(visible(gy, ls[0], w, h), visible(oy, ls[0], w, h))
    assert np.array_equal(visible(gu, ls[1], cw, ch), visible(ou, ls[1], cw, ch))
    assert np.array_equal(visible(gv, ls[2], cw, ch), visible(ov, ls[2], cw, ch))
    # Padding bytes past each row's width are left untouched.
    if ls[0] > w:
        assert np.all(gy.reshape(-1, ls[0])[:, w:] == 7)


def test_golden_yuv_on_gpu(cuda, nes_lib):
    g = np.load(os.path.join(GOLDEN, "yuv_small.npz"))
    w, h, ls = int(g["w"]), int(g["h"]), [int(v) for v in g["ls"]]
    y, u, v = gpu_yuv(cuda, nes_lib, g["rgb"], w, h, w * 3, ls)
    cw, ch = (w + 1) // 2, (h + 1) // 2
    assert np.array_equal(visible(y, ls[0], w, h), visible(g["y"], ls[0], w, h))
    assert np.array_equal(visible(u, ls[1], cw, ch), visible(g["u"], ls[1], cw, ch))
    assert np.array_equal(visible(v, ls[2], cw, ch), visible(g["v"], ls[2], cw, ch))


@pytest.mark.parametrize("w,h,pad", [(1280, 720, 0), (33, 17, 0), (1, 1, 0), (33, 17, 7), (1922, 1081, 6)])
def test_gray8_to_yuv420p_bit_exact(cuda, nes_lib, oracle_mod, w, h, pad):
    rng = np.random.default_rng(w + h)
    g = np.zeros((h, w + pad), np.uint8)
    g[:, :w] = rng.integers(0, 256, (h, w), dtype=np.uint8)
    ls = nes_lib.linesizes(w)
    gy, gu, gv = gpu_yuv(cuda, nes_lib, g, w, h, w + pad, ls, gray=True)
    oy, ou, ov = oracle_mod.gray8_to_yuv420p(g, w, h, w + pad, ls)
    cw, ch = (w + 1) // 2, (h + 1) // 2
    assert np.array_equal(visible(gy, ls[0], w, h), visible(oy, ls[0], w, h))
    assert np.array_equal(visible(gu, ls[1], cw, ch), visible(ou, ls[1], cw, ch))


def test_depth_pack_bit_exact(cuda, nes_lib, oracle_mod):
    torch = cuda
    rng = np.random.default_rng(0)
    d = np.concatenate([rng.uniform(0.1, 10.0, 1280 * 720 * 30 // 16).astype(np.float32),
                        np.array([0.0, 0.0004, 0.0005, 1.2345, 65.5349, 65.535, 1e9, -1.0, np.nan, np.inf,
                                  -np.inf, -0.0], np.float32)])
    src = torch.from_numpy(d).cuda()
    out = torch.empty(d.size, dtype=torch.int16, device="cuda")
    nes_lib.depth_pack_u16mm(src.data_ptr(), d.size, out.data_ptr())
    torch.cuda.synchronize()
    got = out.cpu().numpy().view(np.uint16)
    assert np.array_equal(got, oracle_mod.depth_pack_u16mm(d))


def test_rgb24_and_gray8_quantisation(cuda, nes_lib, oracle_mod):
    torch = cuda
    lib = nes_lib.load()
    rng = np.random.default_rng(1)
    x = np.concatenate([rng.uniform(-0.2, 1.2, 100000), np.arange(256) / 255.0, [0.5 / 255, 1.5 / 255]])
    x = x.astype(np.float32)
    src = torch.from_numpy(x).cuda()
    out = torch.empty(x.size, dtype=torch.uint8, device="cuda")
    assert lib.nes_rgb_to_rgb24(src.data_ptr(), x.size, out.data_ptr(), None) == 0
    torch.cuda.synchronize()
    assert np.array_equal(out.cpu().numpy(), oracle_mod.rgb_to_rgb24(x))
    d = rng.uniform(-1, 6, 50000).astype(np.float32)
    src = torch.from_numpy(d).cuda()
    out = torch.empty(d.size, dtype=torch.uint8, device="cuda")
    assert lib.nes_depth_to_gray8(src.data_ptr(), d.size, 4.0, out.data_ptr(), None) == 0
    torch.cuda.synchronize()
    assert np.array_equal(out.cpu().numpy(), oracle_mod.depth_to_gray8(d, 4.0))


@pytest.mark.parametrize("offset,extra", [(0, 1), (1, 0), (2, 3), (3, 2)])
def test_elementwise_glue_any_alignment(cuda, nes_lib, oracle_mod, offset, extra):
    """Depth packing and both quantisers at every input alignment and with
    element counts that leave a tail after the 4-element vector steps."""
    torch = cuda
    lib = nes_lib.load()
    rng = np.random.default_rng(offset * 7 + extra)
    n = 4 * 12345 + extra
    x = np.concatenate([rng.uniform(-0.5, 70.0, n - 6), [np.nan, np.inf, -np.inf, 0.0005, 65.535, -0.0]])
    x = x.astype(np.float32)
    src = torch.zeros(n + 8, dtype=torch.float32, device="cuda")
    src[offset:offset + n] = torch.from_numpy(x).cuda()
    p = src.data_ptr() + 4 * offset
    o16 = torch.zeros(n + 8, dtype=torch.int16, device="cuda")
    nes_lib.depth_pack_u16mm(p, n, o16.data_ptr() + 2 * offset)
    o8 = torch.zeros(n + 8, dtype=torch.uint8, device="cuda")
    assert lib.nes_depth_to_gray8(p, n, 4.0, o8.data_ptr() + offset, None) == 0
    q8 = torch.zeros(n + 8, dtype=torch.uint8, device="cuda")
    assert lib.nes_rgb_to_rgb24(p, n, q8.data_ptr() + offset, None) == 0
    torch.cuda.synchronize()
    assert np.array_equal(o16.cpu().numpy()[offset:offset + n].view(np.uint16), oracle_mod.depth_pack_u16mm(x))
    assert np.array_equal(o8.cpu().numpy()[offset:offset + n], oracle_mod.depth_to_gray8(x, 4.0))
    assert np.array_equal(q8.cpu().numpy()[offset:offset + n], oracle_mod.rgb_to_rgb24(x))
    # Nothing written outside [offset, offset + n).
    assert not o16.cpu().numpy()[:offset].any() and not o16.cpu().numpy()[offset + n:].any()
    assert not o8.cpu().numpy()[offset + n:].any() and not q8.cpu().numpy()[offset + n:].any()


# Batched conversion: every frame of one launch equals the oracle's
# single-frame result.  (1280, 720, 0) and (33, 17, 5) take the vector path,
# (31, 9, 5) the per-sample path; frames are separate allocations.
@pytest.mark.parametrize("w,h,pad,gray", [(1280, 720, 0, False), (33, 17, 5, False), (31, 9, 5, False),
                                          (1280, 720, 0, True), (31, 9, 5, True)])
def test_yuv420p_batch_matches_oracle(cuda, nes_lib, oracle_mod, w, h, pad, gray):
    torch = cuda
    rng = np.random.default_rng(w + 31 * h + pad)
    nframes = 5
    ls = nes_lib.linesizes(w)
    ch, cw = (h + 1) // 2, (w + 1) // 2
    src_ls = (w if gray else 3 * w) + pad
    bufs, srcs, ys, us, vs = [], [], [], [], []
    for f in range(nframes):
        img = synth_frame(rng, w, h)
        buf = np.zeros((h, src_ls), np.uint8)
        buf[:, :(w if gray else 3 * w)] = img[:, :, 0] if gray else img.reshape(h, 3 * w)
        bufs.append(buf)
        srcs.append(torch.from_numpy(buf.reshape(-1)).cuda())
        ys.append(torch.full((ls[0] * h,), 7, dtype=torch.uint8, device="cuda"))
        us.append(torch.full((ls[1] * ch,), 7, dtype=torch.uint8, device="cuda"))
        vs.append(torch.full((ls[2] * ch,), 7, dtype=torch.uint8, device="cuda"))
    nes_lib.yuv420p_batch([t.data_ptr() for t in srcs], w, h, src_ls, [t.data_ptr() for t in ys],
                          [t.data_ptr() for t in us], [t.data_ptr() for t in vs], ls, gray=gray)
    torch.cuda.synchronize()
    ref = oracle_mod.gray8_to_yuv420p if gray else oracle_mod.rgb24_to_yuv420p
    for f in range(nframes):
        oy, ou, ov = ref(bufs[f], w, h, src_ls, ls)
        assert np.array_equal(visible(ys[f].cpu().numpy(), ls[0], w, h), visible(oy, ls[0], w, h))
        assert np.array_equal(visible(us[f].cpu().numpy(), ls[1], cw, ch), visible(ou, ls[1], cw, ch))
        assert np.array_equal(visible(vs[f].cpu().numpy(), ls[2], cw, ch), visible(ov, ls[2], cw, ch))


def test_depth_pack_batch_matches_oracle(cuda, nes_lib, oracle_mod):
    torch = cuda
    rng = np.random.default_rng(11)
    n = 1280 * 720 + 3  # a scalar tail after the float4 groups
    deps = [torch.from_numpy((rng.random(n) * 70.0 - 1.0).astype(np.float32)).cuda() for _ in range(4)]
    outs = [torch.zeros(n, dtype=torch.int16, device="cuda") for _ in range(4)]
    nes_lib.depth_pack_u16mm_batch([d.data_ptr() for d in deps], n, [o.data_ptr() for o in outs])
    torch.cuda.synchronize()
    for d, o in zip(deps, outs):
        assert np.array_equal(o.cpu().numpy().view(np.uint16), oracle_mod.depth_pack_u16mm(d.cpu().numpy()))


def test_batch_glue_rejects_bad_arguments(cuda, nes_lib):
    torch = cuda
    a = torch.zeros(64 * 64 * 3, dtype=torch.uint8, device="cuda")
    ls = nes_lib.linesizes(64)
    for n in (0, nes_lib.NES_MAX_BATCH_FRAMES + 1):
        p = [a.data_ptr()] * max(n, 1)
        with pytest.raises(nes_lib.NesError):
            nes_lib.yuv420p_batch(p[:n] if n else [], 64, 64, 192, p[:n], p[:n], p[:n], ls)
    with pytest.raises(nes_lib.NesError):  # a null frame pointer
        nes_lib.yuv420p_batch([a.data_ptr(), 0], 64, 64, 192, [a.data_ptr()] * 2, [a.data_ptr()] * 2,
                              [a.data_ptr()] * 2, ls)
