"""Generates the committed golden fixtures under tests/golden/.

Run in the build container (it needs the Python `protobuf` package, which the
GPU host lacks):

    python tests/golden/make_golden.py

Fixtures:
  nes_proto.npz        FrameRequest / RenderedFrame bytes serialised by the
                       official protobuf runtime from the nes.proto schema
                       (proto/nes.proto:5-25), pinning the library's own
                       proto3 codec.
  render_seed0.npz     FP64 oracle render of a 32x32 view (seed 0, 2^19),
                       pinning the oracle across hosts (x86 here, Arm on the
                       GPU host).
  yuv_small.npz        oracle YUV420P / depth packing of small seeded inputs.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "oracle"))
sys.path.insert(0, os.path.join(REPO, "ngp-encode-server_gb300"))


def nes_proto_classes():
    """Message classes for nes.proto built from a descriptor (no protoc)."""
    from google.protobuf import descriptor_pb2, descriptor_pool, message_factory
    F = descriptor_pb2.FieldDescriptorProto
    fdp = descriptor_pb2.FileDescriptorProto(name="nes.proto", package="nesproto", syntax="proto3")

    def msg(name, fields):
        m = fdp.message_type.add(name=name)
        for fname, num, ftype, label, tname in fields:
            f = m.field.add(name=fname, number=num, type=ftype, label=label)
            if tname:
                f.type_name = tname

    O, R = F.LABEL_OPTIONAL, F.LABEL_REPEATED
    msg("Camera", [("is_left", 2, F.TYPE_BOOL, O, None), ("width", 3, F.TYPE_UINT32, O, None),
                   ("height", 4, F.TYPE_UINT32, O, None), ("matrix", 12, F.TYPE_FLOAT, R, None)])
    msg("FrameRequest", [("index", 1, F.TYPE_UINT64, O, None),
                         ("camera", 2, F.TYPE_MESSAGE, O, ".nesproto.Camera"),
                         ("is_left", 3, F.TYPE_BOOL, O, None)])
    msg("RenderedFrame", [("index", 1, F.TYPE_UINT64, O, None),
                          ("camera", 2, F.TYPE_MESSAGE, O, ".nesproto.Camera"),
                          ("is_left", 3, F.TYPE_BOOL, O, None), ("frame", 6, F.TYPE_BYTES, O, None),
                          ("depth", 7, F.TYPE_BYTES, O, None)])
    pool = descriptor_pool.DescriptorPool()
    pool.Add(fdp)
    get = message_factory.GetMessageClass
    return (get(pool.FindMessageTypeByName("nesproto.Camera")),
            get(pool.FindMessageTypeByName("nesproto.FrameRequest")),
            get(pool.FindMessageTypeByName("nesproto.RenderedFrame")))


def make_proto():
    _, FrameRequest, RenderedFrame = nes_proto_classes()
    import nes
    rng = np.random.default_rng(7)
    cases = []
    init = [1.0, 0.0, 0.0, 0.5, 0.0, -1.0, 0.0, 0.5, 0.0, 0.0, -1.0, 0.5]  # camera_manager.h:18-19
    specs = [(0, True, 1280, 720, init), (1, False, 1920, 1080, nes.shell_poses(0, 1, 1.5, 1.5)[0]),
             (2 ** 40 + 3, True, 7, 5, list(rng.uniform(-2, 2, 12))), (0, False, 0, 0, [])]
    for idx, left, w, h, m in specs:
        req = FrameRequest(index=idx, is_left=left)
        req.camera.is_left = left
        req.camera.width = w
        req.camera.height = h
        req.camera.matrix.extend([float(np.float32(v)) for v in m])
        frame = bytes(rng.integers(0, 256, 3 * 4 * 3, dtype=np.uint8))
        depth = bytes(rng.integers(0, 256, 4 * 3, dtype=np.uint8))
        rf = RenderedFrame(index=idx, is_left=left, frame=frame, depth=depth)
        rf.camera.CopyFrom(req.camera)
        cases.append((req.SerializeToString(), rf.SerializeToString(), frame, depth,
                      np.asarray(m, np.float32), idx, left, w, h))
    out = {}
    for i, (rq, rf, fr, dp, m, idx, left, w, h) in enumerate(cases):
        out["req%d" % i] = np.frombuffer(rq, np.uint8)
        out["rf%d" % i] = np.frombuffer(rf, np.uint8)
        out["frame%d" % i] = np.frombuffer(fr, np.uint8)
        out["depth%d" % i] = np.frombuffer(dp, np.uint8)
        out["matrix%d" % i] = m
        out["meta%d" % i] = np.array([idx, int(left), w, h], dtype=np.uint64)
    np.savez(os.path.join(HERE, "nes_proto.npz"), count=np.array(len(cases)), **out)


def make_render():
    import nes
    import oracle
    scene = oracle.Scene(0, 19)
    pose = np.asarray(nes.shell_poses(0, 1, 1.5, 1.5)[0], np.float32)
    W = H = 32
    focal = np.float32(nes.focal_from_fov(W, 90.0))
    rgb, depth, samples = scene.render(pose, W, H, float(focal))
    np.savez(os.path.join(HERE, "render_seed0.npz"), pose=pose, W=W, H=H, focal=focal, rgb=rgb, depth=depth,
             samples=np.array(samples))


def make_yuv():
    import oracle
    rng = np.random.default_rng(11)
    w, h = 17, 9
    ls = [32, 32, 32]
    rgb = rng.integers(0, 256, (h, w * 3), dtype=np.uint8)
    y, u, v = oracle.rgb24_to_yuv420p(rgb, w, h, w * 3, ls)
    g = rng.integers(0, 256, (h, w), dtype=np.uint8)
    gy, gu, gv = oracle.gray8_to_yuv420p(g, w, h, w, ls)
    d = rng.uniform(0.1, 10.0, 64).astype(np.float32)
    np.savez(os.path.join(HERE, "yuv_small.npz"), w=w, h=h, ls=np.array(ls), rgb=rgb, y=y, u=u, v=v, gray=g,
             gy=gy, gu=gu, gv=gv, depth=d, depth_mm=oracle.depth_pack_u16mm(d))


if __name__ == "__main__":
    make_proto()
    make_render()
    make_yuv()
    print("fixtures written to", HERE)
