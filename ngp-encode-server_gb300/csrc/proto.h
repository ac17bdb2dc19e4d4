// proto.h -- a minimal proto3 codec for the three nes.proto messages
// (proto/nes.proto:5-25).  The reference links libprotobuf for them
// (CMakeLists.txt:32-50); only varint, 32-bit and length-delimited fields
// occur, so a hand-written codec keeps the library free of that dependency.
#pragma once
#include <cstddef>
#include <cstdint>
#include <vector>

namespace nes {

struct PbCamera {
  bool is_left = false;     // field 2
  uint32_t width = 0;       // field 3
  uint32_t height = 0;      // field 4
  std::vector<float> matrix;  // field 12 (packed or unpacked floats)
};

struct PbFrameRequest {
  uint64_t index = 0;       // field 1
  bool has_camera = false;  // field 2 present
  PbCamera camera;
  bool is_left = false;     // field 3
};

// Parses a serialised FrameRequest.  Unknown fields are skipped, repeated
// occurrences merge as proto3 does.  Returns false on malformed bytes.
bool parse_frame_request(const uint8_t* p, size_t n, PbFrameRequest* out);
bool parse_camera(const uint8_t* p, size_t n, PbCamera* out);

// Serialised size of a Camera message.
size_t camera_size(const PbCamera& c);
// Writes a Camera message body; returns bytes written.
size_t write_camera(const PbCamera& c, uint8_t* out);

// Layout of a serialised RenderedFrame{index, camera, is_left, frame, depth}
// whose frame/depth payloads are filled in place afterwards.
struct RenderedFrameLayout {
  size_t total = 0;
  size_t frame_offset = 0;  // where the frame payload bytes go
  size_t depth_offset = 0;  // where the depth payload bytes go
};
RenderedFrameLayout rendered_frame_layout(uint64_t index, const PbCamera* camera, bool is_left,
                                          size_t frame_len, size_t depth_len);
// Writes everything except the two payloads (caller fills them at the
// offsets of the returned layout).  out must hold layout.total bytes.
RenderedFrameLayout write_rendered_frame_header(uint64_t index, const PbCamera* camera,
                                                bool is_left, size_t frame_len, size_t depth_len,
                                                uint8_t* out);

}  // namespace nes
