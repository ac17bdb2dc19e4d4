// proto.cpp -- proto3 wire codec for nes.proto (see proto.h).
#include "proto.h"

#include <cstring>

namespace nes {

namespace {

struct Reader {
  const uint8_t* p;
  const uint8_t* end;
  bool varint(uint64_t* v) {
    uint64_t r = 0;
    for (int shift = 0; shift < 64; shift += 7) {
      if (p >= end) return false;
      uint8_t b = *p++;
      r |= (uint64_t)(b & 0x7f) << shift;
      if (!(b & 0x80)) {
        *v = r;
        return true;
      }
    }
    return false;  // more than 10 bytes
  }
  // A field key (field number << 3 | wire type).  Like the protobuf
  // runtime, rejects keys encoded in more than 5 bytes or wider than 32
  // bits, and field number 0.
  bool key(uint32_t* field, uint32_t* wire) {
    const uint8_t* const start = p;
    uint64_t k;
    if (!varint(&k) || p - start > 5 || k > 0xFFFFFFFFull || (k >> 3) == 0) return false;
    *field = (uint32_t)(k >> 3);
    *wire = (uint32_t)(k & 7);
    return true;
  }
  bool bytes(const uint8_t** data, size_t* len) {
    uint64_t l;
    if (!varint(&l)) return false;
    if (l > (uint64_t)(end - p)) return false;
    *data = p;
    *len = (size_t)l;
    p += l;
    return true;
  }
  bool skip(uint32_t wire) {
    uint64_t v;
    const uint8_t* d;
    size_t l;
    switch (wire) {
      case 0: return varint(&v);
      case 1: if (end - p < 8) return false; p += 8; return true;
      case 2: return bytes(&d, &l);
      case 5: if (end - p < 4) return false; p += 4; return true;
      default: return false;  // groups (3, 4) and reserved types
    }
  }
};

inline float read_f32(const uint8_t* p) {
  float f;
  std::memcpy(&f, p, 4);  // little-endian on both supported hosts
  return f;
}

size_t varint_size(uint64_t v) {
  size_t n = 1;
  while (v >= 0x80) {
    v >>= 7;
    ++n;
  }
  return n;
}

uint8_t* put_varint(uint8_t* o, uint64_t v) {
  while (v >= 0x80) {
    *o++ = (uint8_t)(v | 0x80);
    v >>= 7;
  }
  *o++ = (uint8_t)v;
  return o;
}

}  // namespace

bool parse_camera(const uint8_t* p, size_t n, PbCamera* out) {
  Reader r{p, p + n};
  while (r.p < r.end) {
    uint32_t field, wire;
    if (!r.key(&field, &wire)) return false;
    uint64_t v;
    if (field == 2 && wire == 0) {
      if (!r.varint(&v)) return false;
      out->is_left = v != 0;
    } else if (field == 3 && wire == 0) {
      if (!r.varint(&v)) return false;
      out->width = (uint32_t)v;
    } else if (field == 4 && wire == 0) {
      if (!r.varint(&v)) return false;
      out->height = (uint32_t)v;
    } else if (field == 12 && wire == 2) {  // packed
      const uint8_t* d;
      size_t l;
      if (!r.bytes(&d, &l) || (l % 4) != 0) return false;
      for (size_t i = 0; i < l; i += 4) out->matrix.push_back(read_f32(d + i));
    } else if (field == 12 && wire == 5) {  // unpacked element
      if (r.end - r.p < 4) return false;
      out->matrix.push_back(read_f32(r.p));
      r.p += 4;
    } else if (!r.skip(wire)) {
      return false;
    }
  }
  return true;
}

bool parse_frame_request(const uint8_t* p, size_t n, PbFrameRequest* out) {
  Reader r{p, p + n};
  while (r.p < r.end) {
    uint32_t field, wire;
    if (!r.key(&field, &wire)) return false;
    uint64_t v;
    if (field == 1 && wire == 0) {
      if (!r.varint(&v)) return false;
      out->index = v;
    } else if (field == 2 && wire == 2) {
      const uint8_t* d;
      size_t l;
      if (!r.bytes(&d, &l)) return false;
      out->has_camera = true;
      if (!parse_camera(d, l, &out->camera)) return false;
    } else if (field == 3 && wire == 0) {
      if (!r.varint(&v)) return false;
      out->is_left = v != 0;
    } else if (!r.skip(wire)) {
      return false;
    }
  }
  return true;
}

size_t camera_size(const PbCamera& c) {
  size_t n = 0;
  if (c.is_left) n += 2;
  if (c.width) n += 1 + varint_size(c.width);
  if (c.height) n += 1 + varint_size(c.height);
  if (!c.matrix.empty()) n += 1 + varint_size(4 * c.matrix.size()) + 4 * c.matrix.size();
  return n;
}

size_t write_camera(const PbCamera& c, uint8_t* out) {
  uint8_t* o = out;
  if (c.is_left) {
    *o++ = (2 << 3) | 0;
    *o++ = 1;
  }
  if (c.width) {
    *o++ = (3 << 3) | 0;
    o = put_varint(o, c.width);
  }
  if (c.height) {
    *o++ = (4 << 3) | 0;
    o = put_varint(o, c.height);
  }
  if (!c.matrix.empty()) {
    *o++ = (12 << 3) | 2;
    o = put_varint(o, 4 * c.matrix.size());
    std::memcpy(o, c.matrix.data(), 4 * c.matrix.size());
    o += 4 * c.matrix.size();
  }
  return (size_t)(o - out);
}

RenderedFrameLayout rendered_frame_layout(uint64_t index, const PbCamera* camera, bool is_left,
                                          size_t frame_len, size_t depth_len) {
  RenderedFrameLayout L;
  size_t n = 0;
  if (index) n += 1 + varint_size(index);
  if (camera) {
    const size_t cs = camera_size(*camera);
    n += 1 + varint_size(cs) + cs;
  }
  if (is_left) n += 2;
  if (frame_len) {
    n += 1 + varint_size(frame_len);
    L.frame_offset = n;
    n += frame_len;
  }
  if (depth_len) {
    n += 1 + varint_size(depth_len);
    L.depth_offset = n;
    n += depth_len;
  }
  L.total = n;
  return L;
}

RenderedFrameLayout write_rendered_frame_header(uint64_t index, const PbCamera* camera,
                                                bool is_left, size_t frame_len, size_t depth_len,
                                                uint8_t* out) {
  RenderedFrameLayout L = rendered_frame_layout(index, camera, is_left, frame_len, depth_len);
  uint8_t* o = out;
  if (index) {
    *o++ = (1 << 3) | 0;
    o = put_varint(o, index);
  }
  if (camera) {
    *o++ = (2 << 3) | 2;
    o = put_varint(o, camera_size(*camera));
    o += write_camera(*camera, o);
  }
  if (is_left) {
    *o++ = (3 << 3) | 0;
    *o++ = 1;
  }
  if (frame_len) {
    *o++ = (6 << 3) | 2;
    o = put_varint(o, frame_len);
    o += frame_len;  // payload filled by the caller
  }
  if (depth_len) {
    *o++ = (7 << 3) | 2;
    o = put_varint(o, depth_len);
    o += depth_len;
  }
  return L;
}

}  // namespace nes
