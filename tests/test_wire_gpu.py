"""The wire-compatible renderer call (nes_render: FrameRequest bytes in,
RenderedFrame bytes out, replacing the TCP round trip of
src/server.cpp:161-194) and the pose->YUV end-to-end call."""
import ctypes
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu


def decode_rendered_frame(data):
    """Minimal proto3 decoder for RenderedFrame (field -> value)."""
    out, i = {}, 0

    def varint():
        nonlocal i
        r, s = 0, 0
        while True:
            b = data[i]
            i += 1
            r |= (b & 0x7F) << s
            s += 7
            if not b & 0x80:
                return r
    while i < len(data):
        key = varint()
        f, wt = key >> 3, key & 7
        if wt == 0:
            out[f] = varint()
        elif wt == 2:
            n = varint()
            out[f] = bytes(data[i:i + n])
            i += n
        else:
            raise ValueError("unexpected wire type")
    return out


def frame_request(index, is_left, w, h, matrix):
    import struct
    cam = b""
    if is_left:
        cam += bytes([2 << 3, 1])
    for f, v in ((3, w), (4, h)):
        cam += bytes([f << 3])
        while v >= 0x80:
            cam += bytes([v & 0x7F | 0x80])
            v >>= 7
        cam += bytes([v])
    cam += bytes([12 << 3 | 2, 48]) + struct.pack("<12f", *matrix)
    msg = b""
    if index:
        msg += bytes([1 << 3])
        v = index
        while v >= 0x80:
            msg += bytes([v & 0x7F | 0x80])
            v >>= 7
        msg += bytes([v])
    msg += bytes([2 << 3 | 2, len(cam)]) + cam
    if is_left:
        msg += bytes([3 << 3, 1])
    return msg


def test_render_pb_matches_device_render(r32, cuda, nes_lib, oracle_mod):
    torch = cuda
    M = nes_lib.shell_poses(0, 1, 1.5, 1.5)[0]
    W, H = 64, 36
    req = frame_request(12345, True, W, H, M)
    out = decode_rendered_frame(r32.render(req))
    assert out[1] == 12345 and out[3] == 1
    assert len(out[6]) == W * H * 3 and len(out[7]) == W * H
    # The echoed camera parses back to the request's camera.
    cam = nes_lib.NesFrameRequest()
    assert nes_lib.load().nes_parse_frame_request(req, len(req), ctypes.byref(cam)) == 0
    f = r32.cfg.fov_deg
    focal = nes_lib.focal_from_fov(W, f)
    rgb = torch.empty(W * H * 3, device="cuda")
    dep = torch.empty(W * H, device="cuda")
    r32.render_views([nes_lib.make_view(M, W, H, focal)], [rgb.data_ptr()], [dep.data_ptr()])
    torch.cuda.synchronize()
    assert np.frombuffer(out[6], np.uint8).tolist() == oracle_mod.rgb_to_rgb24(rgb.cpu().numpy()).tolist()
    assert np.array_equal(np.frombuffer(out[7], np.uint8), oracle_mod.depth_to_gray8(dep.cpu().numpy(), 4.0))


def test_render_pb_errors(r32, nes_lib):
    lib = nes_lib.load()
    n = ctypes.c_size_t(0)
    bad = b"\x12\x10\x18\x01"
    assert lib.nes_render(r32.h, bad, len(bad), None, 0, ctypes.byref(n)) == nes_lib.NES_EPROTO
    no_matrix = bytes([2 << 3 | 2, 4, 3 << 3, 8, 4 << 3, 8])
    assert lib.nes_render(r32.h, no_matrix, len(no_matrix), None, 0, ctypes.byref(n)) == nes_lib.NES_EPROTO
    M = nes_lib.shell_poses(0, 1, 1.5, 1.5)[0]
    req = frame_request(1, False, 16, 16, M)
    assert lib.nes_render(r32.h, req, len(req), None, 0, ctypes.byref(n)) == nes_lib.NES_ENOBUFS
    need = n.value
    small = ctypes.create_string_buffer(need - 1)
    assert lib.nes_render(r32.h, req, len(req), small, need - 1, ctypes.byref(n)) == nes_lib.NES_ENOBUFS
    huge = frame_request(1, False, 8192, 8192, M)
    assert lib.nes_render(r32.h, huge, len(huge), None, 0, ctypes.byref(n)) == nes_lib.NES_EINVAL


def _lpf_send(sock, payload):
    import struct
    sock.sendall(struct.pack("=Q", len(payload)) + payload)  # host-endian size_t, src/server.cpp:46-60


def _lpf_recv(sock):
    import struct

    def exact(n):
        buf = b""
        while len(buf) < n:
            chunk = sock.recv(n - len(buf))
            if not chunk:
                raise EOFError
            buf += chunk
        return buf
    (n,) = struct.unpack("=Q", exact(8))
    return exact(n)


def test_tcp_endpoint_speaks_the_renderer_protocol(r32, nes_lib):
    """Acts as neserver's socket_client_thread (src/server.cpp:132-209):
    alternating left/right requests on one connection, a second concurrent
    connection, and a malformed request that closes its connection."""
    import socket
    ep = nes_lib.TcpEndpoint(r32)
    try:
        poses = nes_lib.shell_poses(8, 4, 1.5, 1.5)
        a = socket.create_connection(("127.0.0.1", ep.port.value), timeout=30)
        b = socket.create_connection(("127.0.0.1", ep.port.value), timeout=30)
        for i, M in enumerate(poses[:3]):
            req = frame_request(i, i % 2 == 0, 48, 32, M)
            _lpf_send(a, req)
            got = _lpf_recv(a)
            assert got == r32.render(req)
        req = frame_request(99, False, 24, 16, poses[3])
        _lpf_send(b, req)
        assert _lpf_recv(b) == r32.render(req)
        _lpf_send(b, b"\x12\x10\x18\x01")  # truncated camera: the endpoint closes the connection
        with pytest.raises((EOFError, ConnectionError)):
            _lpf_recv(b)
        a.close()
        b.close()
    finally:
        served = ep.close()
    assert ep.rc == 0 and served == 4


def test_render_yuv_end_to_end(r32, cuda, nes_lib, oracle_mod):
    torch = cuda
    M = nes_lib.shell_poses(0, 100, 1.5, 1.5)[3]
    W, H = 1920, 1080
    focal = nes_lib.focal_from_fov(W, 90.0)
    view = nes_lib.make_view(M, W, H, focal)
    ls = nes_lib.linesizes(W)
    ch = (H + 1) // 2
    y = torch.empty(ls[0] * H, dtype=torch.uint8).pin_memory()
    u = torch.empty(ls[1] * ch, dtype=torch.uint8).pin_memory()
    v = torch.empty(ls[2] * ch, dtype=torch.uint8).pin_memory()
    dmm = torch.empty(W * H, dtype=torch.int16).pin_memory()
    r32.render_yuv(view, y.data_ptr(), u.data_ptr(), v.data_ptr(), ls, dmm.data_ptr())
    rgb = torch.empty(W * H * 3, device="cuda")
    dep = torch.empty(W * H, device="cuda")
    r32.render_views([view], [rgb.data_ptr()], [dep.data_ptr()])
    torch.cuda.synchronize()
    rgb24 = oracle_mod.rgb_to_rgb24(rgb.cpu().numpy())
    oy, ou, ov = oracle_mod.rgb24_to_yuv420p(rgb24, W, H, W * 3, ls)
    assert np.array_equal(y.numpy(), oy) and np.array_equal(u.numpy(), ou) and np.array_equal(v.numpy(), ov)
    assert np.array_equal(dmm.numpy().view(np.uint16), oracle_mod.depth_pack_u16mm(dep.cpu().numpy()))


def test_render_yuv_views_stereo_matches_single_views(rtc, cuda, nes_lib):
    """A stereo pair through nes_render_yuv_views (one batch, one march, one
    frame-output launch) gives each eye the bytes nes_render_yuv gives it
    alone."""
    torch = cuda
    W, H = 640, 366  # odd chroma height
    M = nes_lib.shell_poses(9, 1, 1.2, 2.0)[0]
    f = nes_lib.focal_from_fov(W, 100.0)
    views = [nes_lib.make_view(m, W, H, f) for m in nes_lib.stereo_pair(M, 0.063)]
    ls = nes_lib.linesizes(W)
    ch = (H + 1) // 2

    def bufs():
        return [torch.zeros(n, dtype=torch.uint8).pin_memory() for n in (ls[0] * H, ls[1] * ch, ls[2] * ch)] + \
               [torch.zeros(W * H, dtype=torch.int16).pin_memory()]

    pair = [bufs(), bufs()]
    rtc.render_yuv_views(views, [b[0].data_ptr() for b in pair], [b[1].data_ptr() for b in pair],
                         [b[2].data_ptr() for b in pair], ls, [b[3].data_ptr() for b in pair])
    for v, got in zip(views, pair):
        one = bufs()
        rtc.render_yuv(v, one[0].data_ptr(), one[1].data_ptr(), one[2].data_ptr(), ls, one[3].data_ptr())
        for a, b in zip(got, one):
            assert np.array_equal(a.numpy(), b.numpy())


@pytest.mark.parametrize("W,H", [(33, 17), (1, 1), (3, 5)])
@pytest.mark.parametrize("prec", ["fp32", "tc"])
def test_render_yuv_odd_sizes(cuda, nes_lib, oracle_mod, prec, W, H):
    """nes_render_yuv at odd widths and heights (chroma planes of ceil(W/2) x
    ceil(H/2)): the fused frame output gives the bytes of the separate
    conversions of the same render in the visible part of every row, and the
    row padding of the caller's planes is left as it was."""
    torch = cuda
    p = nes_lib.PREC_FP32 if prec == "fp32" else nes_lib.PREC_FP16_TC
    M = nes_lib.shell_poses(0, 100, 1.5, 1.5)[5]
    focal = nes_lib.focal_from_fov(W, 90.0)
    view = nes_lib.make_view(M, W, H, focal)
    ls = nes_lib.linesizes(W)
    ch = (H + 1) // 2
    y = torch.zeros(ls[0] * H, dtype=torch.uint8).pin_memory()
    u = torch.zeros(ls[1] * ch, dtype=torch.uint8).pin_memory()
    v = torch.zeros(ls[2] * ch, dtype=torch.uint8).pin_memory()
    dmm = torch.zeros(W * H, dtype=torch.int16).pin_memory()
    with nes_lib.Renderer(precision=p, max_pixels=64 * 64) as r:
        r.render_yuv(view, y.data_ptr(), u.data_ptr(), v.data_ptr(), ls, dmm.data_ptr())
        rgb = torch.empty(W * H * 3, device="cuda")
        dep = torch.empty(W * H, device="cuda")
        r.render_views([view], [rgb.data_ptr()], [dep.data_ptr()])
        torch.cuda.synchronize()
    rgb24 = oracle_mod.rgb_to_rgb24(rgb.cpu().numpy())
    oy, ou, ov = oracle_mod.rgb24_to_yuv420p(rgb24, W, H, W * 3, ls)
    cw = (W + 1) // 2
    for got, want, l, w, h in ((y, oy, ls[0], W, H), (u, ou, ls[1], cw, ch), (v, ov, ls[2], cw, ch)):
        g = got.numpy().reshape(h, l)
        assert np.array_equal(g[:, :w], want.reshape(h, l)[:, :w])
        assert not g[:, w:].any()  # the padding keeps the caller's zeros
    assert np.array_equal(dmm.numpy().view(np.uint16), oracle_mod.depth_pack_u16mm(dep.cpu().numpy()))
