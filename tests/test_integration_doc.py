"""The integration guide's binding examples (the C++ and ctypes blocks a
neserver maintainer would add) against the real C ABI: every C++ block
compiles (g++ -fsyntax-only) against include/nes_gb300.h with stand-ins
for neserver's own types (protobuf messages, AVFrame, the RenderedFrame
constructor), and the raw ctypes stub resolves its symbol in the built
library.  No GPU is used."""
import ctypes
import os
import re
import shutil
import subprocess

import pytest

from conftest import REPO

DOC = os.path.join(REPO, "INTEGRATION.md")

# neserver-side names the examples use; only their shapes matter here.
PRELUDE = r"""
#include <cstdint>
#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>
#include "nes_gb300.h"
typedef void* cudaStream_t;
enum AVPixelFormat { AV_PIX_FMT_RGB24, AV_PIX_FMT_GRAY8 };
struct AVFrame { uint8_t* data[8]; int linesize[8]; };
struct SwsContextManager {};
namespace nesproto {
struct FrameRequest { std::string SerializeAsString() const; };
struct RenderedFrame { bool ParseFromString(const std::string&); };
struct FloatRep { const float* data() const; };
struct Camera { FloatRep matrix() const; uint32_t width() const; uint32_t height() const; };
}  // namespace nesproto
struct RenderedFrame {
  RenderedFrame(const nesproto::RenderedFrame&, AVPixelFormat, AVPixelFormat,
                std::shared_ptr<SwsContextManager>, std::shared_ptr<SwsContextManager>);
};
extern nesproto::FrameRequest req;
extern nesproto::Camera cam;
extern uint32_t w, h;
extern float fov_deg;
extern AVFrame* avframe;
extern AVFrame *left, *right;
extern uint16_t *left_depth_mm, *right_depth_mm;
extern uint16_t* depth_mm;
extern nes_ctx* nes;
extern nes_view left_view, right_view;
extern std::shared_ptr<SwsContextManager> ctxmgr_scene, ctxmgr_depth;
extern const uint8_t *left_rgb_dev, *right_rgb_dev;
extern uint8_t *ly, *lu, *lv, *ry, *ru, *rv;
extern int linesize[3];
extern cudaStream_t s;
"""


def _blocks(lang):
    text = open(DOC).read()
    return re.findall(r"```" + lang + r"\n(.*?)```", text, re.S)


def test_integration_cpp_examples_compile_against_header(tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ absent")
    blocks = _blocks("cpp")
    assert len(blocks) >= 4
    src = [PRELUDE]
    for i, b in enumerate(blocks):
        body = "\n".join(l for l in b.splitlines() if not l.lstrip().startswith("#include"))
        if re.match(r"\s*(inline\s+)?\w[\w:<>\s\*&]*\s+\w+\s*\(", body) and body.rstrip().endswith("}"):
            src.append(body)  # a function definition: top level
        else:
            src.append("void example_%d() {\n  for (;;) {\n%s\n    break;\n  }\n}" % (i, body))
    path = tmp_path / "integration_examples.cpp"
    path.write_text("\n".join(src))
    r = subprocess.run([gxx, "-std=c++20", "-fsyntax-only", "-Wall", "-Wno-unused-variable",
                        "-I", os.path.join(REPO, "include"), str(path)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_integration_ctypes_stub_binds(nes_lib):
    blocks = [b for b in _blocks("python") if "ctypes.CDLL" in b]
    assert len(blocks) == 1
    code = blocks[0].replace('"ngp-encode-server_gb300/libnes_gb300.so"', "LIBPATH")
    ns = {"ctypes": ctypes, "LIBPATH": nes_lib.load()._name}
    exec(code, ns)
    fn = ns["lib"].nes_rgb24_to_yuv420p
    ls = (ctypes.c_int * 3)(64, 32, 32)
    # argument validation runs before any CUDA call
    assert fn(None, 64, 64, 192, None, None, None, ls, None) == nes_lib.NES_EINVAL
