// overlay.cu -- the debug text overlay drawn into the RGB24 frame before the
// YUV conversion, on the GPU.
//
// Reference: process_frame_thread draws four strings into every scene frame
// (camera matrix at the centre, "index=N" bottom-left, a timestamp top-left,
// "direction=left|right" top-right; src/encode.cpp:57-97) with
// RenderTextContext::render_string_to_frame (src/base/video/render_text.cc:35-111):
// pen at one of five anchors (margin 50, box 300x100), a newline moves the
// pen back to the anchor column and 20 px down, and every pixel a glyph
// covers is set to white, clipped to the frame.  FreeType and the NotoMono
// font are not available here, so glyphs come from this file's own 5x7
// dot-matrix font drawn at 2x (10x14 px cells, 12 px advance, baseline at the
// pen); anchors, newline step, clipping and the white write follow the
// reference.  Characters without a glyph advance the pen and draw nothing.
#include <cstring>

#include "kernels.h"
#include "nes_gb300.h"

namespace nes {

namespace {

constexpr int kGlyphW = 5, kGlyphH = 7, kScale = 2, kAdvance = 12, kLineStep = 20;
constexpr int kMaxChars = 512;

// Rows top to bottom, bit 4 = leftmost column.  Index = ASCII code - 32.
struct Font {
  unsigned char rows[95][kGlyphH];
};

constexpr Font make_font() {
  Font f{};
  struct G {
    char c;
    unsigned char r[kGlyphH];
  };
  const G g[] = {
      {'0', {14, 17, 19, 21, 25, 17, 14}}, {'1', {4, 12, 4, 4, 4, 4, 14}},   {'2', {14, 17, 1, 2, 4, 8, 31}},
      {'3', {30, 1, 1, 14, 1, 1, 30}},     {'4', {2, 6, 10, 18, 31, 2, 2}},  {'5', {31, 16, 30, 1, 1, 17, 14}},
      {'6', {6, 8, 16, 30, 17, 17, 14}},   {'7', {31, 1, 2, 4, 8, 8, 8}},    {'8', {14, 17, 17, 14, 17, 17, 14}},
      {'9', {14, 17, 17, 15, 1, 2, 12}},   {'+', {0, 4, 4, 31, 4, 4, 0}},    {'-', {0, 0, 0, 31, 0, 0, 0}},
      {'.', {0, 0, 0, 0, 0, 12, 12}},      {':', {0, 12, 12, 0, 12, 12, 0}}, {'=', {0, 0, 31, 0, 31, 0, 0}},
      {'a', {0, 0, 14, 1, 15, 17, 15}},    {'b', {16, 16, 22, 25, 17, 17, 30}}, {'c', {0, 0, 14, 16, 16, 17, 14}},
      {'d', {1, 1, 13, 19, 17, 17, 15}},   {'e', {0, 0, 14, 17, 31, 16, 14}}, {'f', {6, 9, 8, 28, 8, 8, 8}},
      {'g', {0, 15, 17, 17, 15, 1, 14}},   {'h', {16, 16, 22, 25, 17, 17, 17}}, {'i', {4, 0, 12, 4, 4, 4, 14}},
      {'j', {2, 0, 6, 2, 2, 18, 12}},      {'k', {16, 16, 18, 20, 24, 20, 18}}, {'l', {12, 4, 4, 4, 4, 4, 14}},
      {'m', {0, 0, 26, 21, 21, 17, 17}},   {'n', {0, 0, 22, 25, 17, 17, 17}}, {'o', {0, 0, 14, 17, 17, 17, 14}},
      {'p', {0, 0, 30, 17, 30, 16, 16}},   {'q', {0, 0, 13, 19, 15, 1, 1}},  {'r', {0, 0, 22, 25, 16, 16, 16}},
      {'s', {0, 0, 14, 16, 14, 1, 30}},    {'t', {8, 8, 28, 8, 8, 9, 6}},    {'u', {0, 0, 17, 17, 17, 19, 13}},
      {'v', {0, 0, 17, 17, 17, 10, 4}},    {'w', {0, 0, 17, 17, 21, 21, 10}}, {'x', {0, 0, 17, 10, 4, 10, 17}},
      {'y', {0, 0, 17, 17, 15, 1, 14}},    {'z', {0, 0, 31, 2, 4, 8, 31}},
  };
  for (const G& x : g)
    for (int r = 0; r < kGlyphH; ++r) f.rows[x.c - 32][r] = x.r[r];
  return f;
}

__constant__ Font c_font = make_font();

struct GlyphList {
  int n;
  short x[kMaxChars], y[kMaxChars];  // pen (baseline-left) per character, frame pixels
  unsigned char code[kMaxChars];     // ASCII - 32
};

// One thread per (character, cell pixel).
__global__ void overlay_kernel(uint8_t* __restrict__ rgb, int w, int h, int ls, const GlyphList gl) {
  constexpr int cw = kGlyphW * kScale, chh = kGlyphH * kScale;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int ci = t / (cw * chh), p = t % (cw * chh);
  if (ci >= gl.n) return;
  const int px = p % cw, py = p / cw;
  const unsigned bits = c_font.rows[gl.code[ci]][py / kScale];
  if (!((bits >> (kGlyphW - 1 - px / kScale)) & 1u)) return;
  const int X = gl.x[ci] + px, Y = gl.y[ci] - chh + py;  // glyph sits on the baseline
  if (X < 0 || Y < 0 || X >= w || Y >= h) return;
  uint8_t* q = rgb + (size_t)Y * ls + (size_t)X * 3;
  q[0] = 255;
  q[1] = 255;
  q[2] = 255;
}

}  // namespace

}  // namespace nes

extern "C" int nes_overlay_text(uint8_t* rgb_dev, int width, int height, int linesize, const char* text, int anchor,
                                void* stream) {
  using namespace nes;
  if (!rgb_dev || !text || width <= 0 || height <= 0 || linesize < 3 * width) return NES_EINVAL;
  if (anchor < NES_TEXT_LEFT_TOP || anchor > NES_TEXT_CENTER) return NES_EINVAL;
  const int x_box = 300, y_box = 100, margin = 50;
  int pen_x = margin, pen_y = margin;
  switch (anchor) {
    case NES_TEXT_LEFT_TOP: pen_x = margin; pen_y = margin; break;
    case NES_TEXT_LEFT_BOTTOM: pen_x = margin; pen_y = height - y_box + margin; break;
    case NES_TEXT_RIGHT_TOP: pen_x = width - x_box + margin; pen_y = margin; break;
    case NES_TEXT_RIGHT_BOTTOM: pen_x = width - x_box + margin; pen_y = height - y_box + margin; break;
    case NES_TEXT_CENTER: pen_x = width / 2 - x_box; pen_y = height / 2 - y_box; break;
  }
  GlyphList gl;
  gl.n = 0;
  const int x0 = pen_x;
  for (const char* c = text; *c; ++c) {
    if (*c == '\n') {
      pen_x = x0;
      pen_y += kLineStep;
      continue;
    }
    const unsigned char u = (unsigned char)*c;
    if (u >= 33 && u <= 126) {
      if (gl.n >= kMaxChars) return NES_EINVAL;
      gl.x[gl.n] = (short)pen_x;
      gl.y[gl.n] = (short)pen_y;
      gl.code[gl.n] = (unsigned char)(u - 32);
      ++gl.n;
    }
    pen_x += kAdvance;
    if (pen_x > 32000 || pen_y > 32000) break;  // beyond any frame: nothing more can be visible
  }
  if (gl.n == 0) return NES_OK;
  const int threads = gl.n * kGlyphW * kScale * kGlyphH * kScale;
  overlay_kernel<<<(threads + 255) / 256, 256, 0, reinterpret_cast<cudaStream_t>(stream)>>>(rgb_dev, width, height,
                                                                                           linesize, gl);
  return cudaGetLastError() == cudaSuccess ? NES_OK : NES_EIO;
}
