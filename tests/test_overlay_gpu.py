"""Debug text overlay on the GPU (the per-frame text of
src/encode.cpp:57-97 drawn by RenderTextContext::render_string_to_frame,
src/base/video/render_text.cc:35-111), bit-exact against the CPU
restatement: all five anchors, the multi-line camera-matrix block, clipping
at the frame edges, characters without a glyph, padded linesizes."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def camera_text(m):
    """The centre block of process_frame_thread: 12 matrix values, 4 per
    row, then the fixed last row (std::showpos, setprecision 5)."""
    vals = list(m) + [0.0, 0.0, 0.0, 1.0]
    rows = [" ".join("%+08.5f" % v for v in vals[r * 4:(r + 1) * 4]) + " " for r in range(4)]
    return "\n".join(rows)


CASES = [
    (4, "camera"), (1, "index=12345"), (0, "23:59:58.123"), (2, "direction=left"), (3, "direction=right"),
    (0, "Upper Case & symbols #!"),  # glyph-less characters only advance
]


@pytest.mark.parametrize("anchor,text", CASES)
@pytest.mark.parametrize("w,h,pad", [(1280, 720, 0), (640, 360, 9), (200, 90, 0)])
def test_overlay_bit_exact(cuda, nes_lib, oracle_mod, anchor, text, w, h, pad):
    torch = cuda
    if text == "camera":
        text = camera_text(nes_lib.shell_poses(0, 1, 1.5, 1.5)[0])
    ls = 3 * w + pad
    rng = np.random.default_rng(w + anchor)
    frame = rng.integers(0, 200, h * ls, dtype=np.uint8)
    dev = torch.from_numpy(frame.copy()).cuda()
    rc = nes_lib.load().nes_overlay_text(dev.data_ptr(), w, h, ls, text.encode(), anchor, None)
    assert rc == 0
    torch.cuda.synchronize()
    got = dev.cpu().numpy()
    want = oracle_mod.overlay_text(frame, w, h, ls, text, anchor)
    assert np.array_equal(got, want)
    if w >= 640:
        assert np.count_nonzero(got != frame) > 0  # something was drawn


def test_overlay_rejects_bad_arguments(nes_lib, cuda):
    lib = nes_lib.load()
    t = cuda.zeros(300, dtype=cuda.uint8, device="cuda")
    assert lib.nes_overlay_text(t.data_ptr(), 10, 10, 29, b"x", 0, None) == nes_lib.NES_EINVAL  # linesize < 3w
    assert lib.nes_overlay_text(t.data_ptr(), 10, 10, 30, b"x", 5, None) == nes_lib.NES_EINVAL  # anchor
    assert lib.nes_overlay_text(t.data_ptr(), 10, 10, 30, b"", 0, None) == 0
