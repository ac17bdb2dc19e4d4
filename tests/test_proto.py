"""The library's proto3 codec for nes.proto (proto/nes.proto:5-25) against
bytes serialised by the official protobuf runtime (committed fixtures, so the
GPU host without the protobuf package checks them too), plus malformed-input
handling (the reference drops a frame whose bytes fail to parse,
src/server.cpp:174-180)."""
import ctypes
import os
import struct

import numpy as np
import pytest

from conftest import GOLDEN


def _parse(nes_lib, data):
    lib = nes_lib.load()
    out = nes_lib.NesFrameRequest()
    buf = ctypes.create_string_buffer(bytes(data), max(1, len(data)))
    rc = lib.nes_parse_frame_request(buf, len(data), ctypes.byref(out))
    return rc, out


def _write(nes_lib, req, frame, depth, cap=None):
    lib = nes_lib.load()
    n = ctypes.c_size_t(0)
    rc = lib.nes_write_rendered_frame(ctypes.byref(req), frame, len(frame), depth, len(depth), None, 0,
                                      ctypes.byref(n))
    assert rc == nes_lib.NES_ENOBUFS
    size = n.value if cap is None else cap
    out = ctypes.create_string_buffer(max(1, size))
    rc = lib.nes_write_rendered_frame(ctypes.byref(req), frame, len(frame), depth, len(depth), out, size,
                                      ctypes.byref(n))
    return rc, out.raw[:n.value]


def _cases():
    g = np.load(os.path.join(GOLDEN, "nes_proto.npz"))
    for i in range(int(g["count"])):
        yield (g["req%d" % i].tobytes(), g["rf%d" % i].tobytes(), g["frame%d" % i].tobytes(),
               g["depth%d" % i].tobytes(), g["matrix%d" % i], [int(v) for v in g["meta%d" % i]])


def test_parse_golden_requests(nes_lib):
    for req, _, _, _, m, (idx, left, w, h) in _cases():
        rc, out = _parse(nes_lib, req)
        assert rc == 0
        assert out.index == idx and out.is_left == left and out.camera_is_left == left
        assert out.width == w and out.height == h and out.matrix_len == len(m)
        assert np.array_equal(np.array(out.matrix[:len(m)], np.float32), m)


def test_write_matches_protobuf_bytes(nes_lib):
    for req, rf, frame, depth, _, _ in _cases():
        rc, parsed = _parse(nes_lib, req)
        assert rc == 0
        rc, out = _write(nes_lib, parsed, frame, depth)
        assert rc == 0
        assert out == rf


def test_unknown_fields_and_unpacked_matrix(nes_lib):
    req, _, _, _, m, (idx, left, w, h) = list(_cases())[1]
    rc, ref = _parse(nes_lib, req)
    extra = bytes([15 << 3 | 0, 0x96, 0x01]) + bytes([0x85, 0x01]) + b"\0\0\0\0"  # field 16, fixed32
    rc, out = _parse(nes_lib, req + extra)
    assert rc == 0 and out.index == ref.index and list(out.matrix) == list(ref.matrix)
    # Camera with the repeated floats written unpacked (wire type 5).
    cam = bytes([3 << 3, w & 0x7F | 0x80, w >> 7]) + b"".join(
        bytes([12 << 3 | 5]) + struct.pack("<f", float(v)) for v in m)
    msg = bytes([2 << 3 | 2, len(cam)]) + cam
    rc, out = _parse(nes_lib, msg)
    assert rc == 0 and out.width == w and out.matrix_len == 12
    assert np.array_equal(np.array(out.matrix, np.float32), m)


@pytest.mark.parametrize("bad", [
    b"\x08",                      # truncated varint
    b"\x08" + b"\xff" * 11,       # varint longer than 10 bytes
    b"\x12\x10\x18\x01",          # camera length beyond the end
    b"\x0b\x00",                  # wire type 3 (group)
    b"\x00\x01",                  # field number 0
    b"\x12\x03\x62\x01\x00",      # packed matrix length not a multiple of 4
    b"\x80\x80\x80\x80\x10\x00",  # key 2^32: wider than 32 bits
    b"\x88\x80\x80\x80\x80\x10\x05",  # key 2^35 + 8: field 1 if truncated to 32 bits
    b"\x88\x80\x80\x80\x80\x00\x05",  # key of field 1 padded to 6 bytes
    b"\x08" + b"\x80" * 10 + b"\x00",   # 11-byte varint
])
def test_malformed_requests(nes_lib, bad):
    rc, _ = _parse(nes_lib, bad)
    assert rc == nes_lib.NES_EPROTO


@pytest.mark.parametrize("data,index", [
    (b"\x88\x80\x80\x80\x00\x05", 5),           # key padded to 5 bytes
    (b"\xf8\xff\xff\xff\x0f\x00\x08\x07", 7),  # field 2^29 - 1 (unknown, skipped)
    (b"\x08" + b"\xff" * 9 + b"\x02", 2 ** 63 - 1),  # 10th varint byte: bits past 64 dropped
    (b"\x08" + b"\x80" * 9 + b"\x00", 0),          # 10-byte zero
])
def test_edge_encodings_accepted_like_protobuf(nes_lib, data, index):
    """Outcomes of the official protobuf runtime (7.x, upb) on the same bytes."""
    rc, out = _parse(nes_lib, data)
    assert rc == 0 and out.index == index


def test_empty_request_parses_to_defaults(nes_lib):
    rc, out = _parse(nes_lib, b"")
    assert rc == 0 and out.index == 0 and out.has_camera == 0


def test_random_requests_against_protobuf(nes_lib):
    pytest.importorskip("google.protobuf")
    import sys
    sys.path.insert(0, GOLDEN)
    from make_golden import nes_proto_classes
    Camera, FrameRequest, RenderedFrame = nes_proto_classes()
    rng = np.random.default_rng(3)
    for _ in range(200):
        req = FrameRequest(index=int(rng.integers(0, 2 ** 63)), is_left=bool(rng.integers(0, 2)))
        if rng.integers(0, 4):
            req.camera.is_left = bool(rng.integers(0, 2))
            req.camera.width = int(rng.integers(0, 5000))
            req.camera.height = int(rng.integers(0, 5000))
            req.camera.matrix.extend(rng.uniform(-3, 3, int(rng.integers(0, 13))).astype(np.float32).tolist())
        data = req.SerializeToString()
        rc, out = _parse(nes_lib, data)
        assert rc == 0 and out.index == req.index and bool(out.is_left) == req.is_left
        assert bool(out.has_camera) == req.HasField("camera")
        frame = rng.integers(0, 256, int(rng.integers(0, 300)), dtype=np.uint8).tobytes()
        depth = rng.integers(0, 256, int(rng.integers(0, 100)), dtype=np.uint8).tobytes()
        rf = RenderedFrame(index=req.index, is_left=req.is_left, frame=frame, depth=depth)
        if req.HasField("camera"):
            rf.camera.CopyFrom(req.camera)
        rc, ours = _write(nes_lib, out, frame, depth)
        assert rc == 0 and ours == rf.SerializeToString()
        back = RenderedFrame()
        back.ParseFromString(ours)
        assert back == rf


def test_mutated_requests_against_protobuf(nes_lib):
    """Random FrameRequests with bytes overwritten, cut short or inserted:
    the library accepts exactly what the protobuf runtime accepts and decodes
    the same values."""
    pytest.importorskip("google.protobuf")
    import sys
    sys.path.insert(0, GOLDEN)
    from google.protobuf.message import DecodeError
    from make_golden import nes_proto_classes
    _, FrameRequest, _ = nes_proto_classes()
    rng = np.random.default_rng(5)
    checked = 0
    for _ in range(4000):
        req = FrameRequest(index=int(rng.integers(0, 2 ** 63)), is_left=bool(rng.integers(0, 2)))
        if rng.integers(0, 4):
            req.camera.is_left = bool(rng.integers(0, 2))
            req.camera.width = int(rng.integers(0, 5000))
            req.camera.height = int(rng.integers(0, 5000))
            req.camera.matrix.extend(rng.uniform(-3, 3, int(rng.integers(0, 13))).astype(np.float32).tolist())
        data = bytearray(req.SerializeToString())
        kind = int(rng.integers(0, 3))
        if kind == 0 and data:
            for _ in range(int(rng.integers(1, 4))):
                data[int(rng.integers(0, len(data)))] = int(rng.integers(0, 256))
        elif kind == 1 and data:
            data = data[:int(rng.integers(0, len(data)))]
        else:
            pos = int(rng.integers(0, len(data) + 1))
            data = data[:pos] + bytes(rng.integers(0, 256, int(rng.integers(1, 6)), dtype=np.uint8)) + data[pos:]
        ref = FrameRequest()
        try:
            ref.ParseFromString(bytes(data))
            ok_ref = True
        except DecodeError:
            ok_ref = False
        rc, out = _parse(nes_lib, data)
        assert (rc == 0) == ok_ref, bytes(data).hex()
        if not ok_ref:
            continue
        checked += 1
        assert out.index == ref.index and bool(out.is_left) == ref.is_left, bytes(data).hex()
        assert bool(out.has_camera) == ref.HasField("camera"), bytes(data).hex()
        if ref.HasField("camera"):
            m = np.array(list(ref.camera.matrix), np.float32)
            assert (out.width, out.height, out.matrix_len) == (ref.camera.width, ref.camera.height, len(m))
            assert bool(out.camera_is_left) == ref.camera.is_left
            k = min(12, len(m))
            assert np.array_equal(np.array(out.matrix[:k], np.float32).view(np.uint32), m[:k].view(np.uint32))
    assert checked > 500
