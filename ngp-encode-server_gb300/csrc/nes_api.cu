// nes_api.cu -- the C ABI (include/nes_gb300.h): context life cycle, the
// wire-compatible render call, the device-native render calls and the frame
// glue entry points.
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <mutex>
#include <vector>

#include "ctx_internal.h"
#include "nes_gb300.h"
#include "kernels.h"
#include "proto.h"
#include "scene.h"

using namespace nes;

namespace {

#define NES_CUDA(call)                        \
  do {                                        \
    cudaError_t e_ = (call);                  \
    if (e_ != cudaSuccess) return NES_EIO;    \
  } while (0)

template <typename T>
int dalloc(T** p, size_t count) {
  if (count == 0) count = 1;
  return cudaMalloc(reinterpret_cast<void**>(p), count * sizeof(T)) == cudaSuccess ? NES_OK : NES_ENOMEM;
}

// Renders views on ctx->stream into the given device outputs.
int render_batch_locked(nes_ctx* c, const nes_view* views, int n, float* const* rgb, float* const* depth) {
  ViewBatch vb;
  uint64_t pixels = 0;
  const int rc = fill_view_batch(views, n, rgb, depth, c->cfg.max_pixels, &vb, &pixels);
  if (rc != NES_OK) return rc;
  if (c->profiling) NES_CUDA(cudaEventRecord(c->ev_t[0], c->stream));
  NES_CUDA(cudaMemsetAsync(c->scratch.counters, 0, kCtrWords * sizeof(uint32_t), c->stream));
  NES_CUDA(launch_raygen(vb, c->scratch, c->stream));
  if (c->profiling) NES_CUDA(cudaEventRecord(c->ev_t[1], c->stream));
  if (c->cfg.precision == NES_PREC_FP16_TC)
    NES_CUDA(launch_march_tc(vb, c->scene, c->scratch, c->num_sms, c->stream));
  else
    NES_CUDA(launch_march_fp32(vb, c->scene, c->scratch, c->num_sms, c->stream));
  if (c->profiling) {
    NES_CUDA(cudaEventRecord(c->ev_t[2], c->stream));
    c->timings_pending = true;
  }
  c->samples_pending = true;
  return NES_OK;
}

// After the stream is idle: reads the last render's sample count and the
// device error word (set when a bounded wait inside a kernel ran out).
int collect_status(nes_ctx* c) {
  if (!c->samples_pending) return NES_OK;
  uint32_t w[3] = {0, 0, 0};  // samples lo, samples hi, error
  NES_CUDA(cudaMemcpy(w, c->scratch.counters + kCtrSamples, sizeof(w), cudaMemcpyDeviceToHost));
  c->last_samples = (uint64_t)w[0] | ((uint64_t)w[1] << 32);
  c->samples_pending = false;
  return w[2] ? NES_ETIMEDOUT : NES_OK;
}

// Runs fn on ctx->stream ordered after everything already queued on `user`
// and makes `user` wait for its completion.
template <typename Fn>
int on_ctx_stream(nes_ctx* c, void* user, Fn fn) {
  cudaStream_t us = reinterpret_cast<cudaStream_t>(user);
  if (us && us != c->stream) {
    NES_CUDA(cudaEventRecord(c->ev_in, us));
    NES_CUDA(cudaStreamWaitEvent(c->stream, c->ev_in, 0));
  }
  const int rc = fn();
  if (rc != NES_OK) return rc;
  if (us && us != c->stream) {
    NES_CUDA(cudaEventRecord(c->ev_out, c->stream));
    NES_CUDA(cudaStreamWaitEvent(us, c->ev_out, 0));
  }
  return NES_OK;
}

void free_ctx(nes_ctx* c) {
  cudaFree(c->d_table32);
  cudaFree(c->d_table16);
  cudaFree(c->d_rec16);
  cudaFree(c->d_weights);
  cudaFree(c->d_tc_weights);
  cudaFree(c->d_occ);
  cudaFree(c->scratch.ray_dt);
  cudaFree(c->scratch.ray_meta);
  cudaFree(c->scratch.counters);
  cudaFree(c->d_rgb);
  cudaFree(c->d_depth);
  cudaFree(c->d_rgb8);
  cudaFree(c->d_gray);
  cudaFree(c->d_yuv);
  cudaFree(c->d_depth16);
  for (cudaEvent_t e : c->ev_t)
    if (e) cudaEventDestroy(e);
  if (c->ev_in) cudaEventDestroy(c->ev_in);
  if (c->ev_out) cudaEventDestroy(c->ev_out);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
}

bool planes_ok(int w, int h, const int ls[3]) {
  if (w <= 0 || h <= 0 || !ls) return false;
  const int cw = (w + 1) / 2;
  return ls[0] >= w && ls[1] >= cw && ls[2] >= cw;
}

}  // namespace

extern "C" {

void nes_config_default(nes_config* cfg) {
  std::memset(cfg, 0, sizeof(*cfg));
  cfg->seed = 0;
  cfg->log2_table_size = 19;
  cfg->precision = NES_PREC_FP32;
  cfg->fov_deg = 90.0f;
  cfg->depth_gray_max = 4.0f;
  cfg->device = 0;
  cfg->max_pixels = 2u * 1920u * 1832u;
  cfg->record_levels = kRecLevelsDefault;
}

const char* nes_strerror(int code) {
  switch (code) {
    case NES_OK: return "ok";
    case NES_EIO: return "CUDA call failed";
    case NES_EAGAIN: return "not ready";
    case NES_ENOMEM: return "allocation failed";
    case NES_ENODEV: return "no usable CUDA device";
    case NES_EINVAL: return "invalid argument";
    case NES_EPROTO: return "malformed nes.proto message";
    case NES_ENOBUFS: return "output buffer too small";
    case NES_ETIMEDOUT: return "timed out";
  }
  return "unknown error";
}

float nes_focal_from_fov(uint32_t width, float fov_deg) {
  const double half = 0.5 * (double)fov_deg * 3.14159265358979323846 / 180.0;
  return (float)(0.5 * (double)width / std::tan(half));
}

int nes_create(const nes_config* cfg, nes_ctx** out) {
  if (!cfg || !out) return NES_EINVAL;
  *out = nullptr;
  if (cfg->log2_table_size < 10 || cfg->log2_table_size > 24) return NES_EINVAL;
  if (cfg->precision != NES_PREC_FP32 && cfg->precision != NES_PREC_FP16_TC) return NES_EINVAL;
  if (cfg->max_pixels == 0 || cfg->max_pixels > (1u << 27)) return NES_EINVAL;
  if (!(cfg->fov_deg > 0.0f && cfg->fov_deg < 180.0f)) return NES_EINVAL;
  if (cfg->record_levels != 0 && cfg->record_levels != (uint32_t)kRecLevelsDefault &&
      cfg->record_levels != (uint32_t)kRecLevelsSmall)
    return NES_EINVAL;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= cfg->device || cfg->device < 0) return NES_ENODEV;
  if (cudaSetDevice(cfg->device) != cudaSuccess) return NES_ENODEV;

  nes_ctx* c = new (std::nothrow) nes_ctx;
  if (!c) return NES_ENOMEM;
  c->cfg = *cfg;
  if (!(c->cfg.depth_gray_max > 0.0f)) c->cfg.depth_gray_max = 4.0f;
  if (c->cfg.record_levels == 0) c->cfg.record_levels = kRecLevelsDefault;
  int rc = NES_OK;
  auto fail = [&](int code) {
    free_ctx(c);
    return code;
  };
  if (cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, cfg->device) != cudaSuccess)
    return fail(NES_EIO);
  if (cudaStreamCreateWithFlags(&c->stream, cudaStreamDefault) != cudaSuccess) return fail(NES_EIO);
  if (cudaEventCreateWithFlags(&c->ev_in, cudaEventDisableTiming) != cudaSuccess) return fail(NES_EIO);
  if (cudaEventCreateWithFlags(&c->ev_out, cudaEventDisableTiming) != cudaSuccess) return fail(NES_EIO);

  SceneHost host;
  if (!generate_scene(cfg->seed, cfg->log2_table_size, &host)) return fail(NES_EINVAL);
  const size_t entries = (size_t)kLevels * host.T;
  if ((rc = dalloc(&c->d_table32, entries)) != NES_OK) return fail(rc);
  if ((rc = dalloc(&c->d_weights, (size_t)kWeightFloats)) != NES_OK) return fail(rc);
  if ((rc = dalloc(&c->d_occ, (size_t)kOccWords)) != NES_OK) return fail(rc);
  if (cudaMemcpy(c->d_table32, host.table.data(), entries * sizeof(float2), cudaMemcpyHostToDevice) != cudaSuccess)
    return fail(NES_EIO);
  if (cudaMemcpy(c->d_weights, host.weights.data(), kWeightFloats * sizeof(float), cudaMemcpyHostToDevice) !=
      cudaSuccess)
    return fail(NES_EIO);
  c->scene.table32 = c->d_table32;
  c->scene.weights = c->d_weights;
  c->scene.occ = c->d_occ;
  c->scene.T = host.T;
  c->scene.dense_mask = dense_level_mask(host.T);
  if (cfg->precision == NES_PREC_FP16_TC) {
    if ((rc = dalloc(&c->d_table16, entries)) != NES_OK) return fail(rc);
    if (launch_table_to_fp16(c->d_table32, c->d_table16, entries, c->stream) != cudaSuccess) return fail(NES_EIO);
    c->scene.rec_levels = c->cfg.record_levels;
    if ((rc = dalloc(&c->d_rec16, tc_record_bytes((int)c->cfg.record_levels) / sizeof(uint4))) != NES_OK)
      return fail(rc);
    if (launch_build_records(c->d_table16, host.T, c->scene.dense_mask, (int)c->cfg.record_levels, c->d_rec16,
                             c->stream) != cudaSuccess)
      return fail(NES_EIO);
    if ((rc = dalloc(&c->d_tc_weights, tc_weight_bytes())) != NES_OK) return fail(rc);
    if (launch_pack_tc_weights(c->d_weights, c->d_tc_weights, c->stream) != cudaSuccess) return fail(NES_EIO);
    c->scene.table16 = c->d_table16;
    c->scene.rec16 = c->d_rec16;
    c->scene.tc_weights = c->d_tc_weights;
  }
  if (launch_occupancy(c->scene, kOccThreshold, c->d_occ, c->stream) != cudaSuccess) return fail(NES_EIO);

  const size_t P = cfg->max_pixels;
  if ((rc = dalloc(&c->scratch.ray_dt, P)) != NES_OK) return fail(rc);
  if ((rc = dalloc(&c->scratch.ray_meta, P)) != NES_OK) return fail(rc);
  if ((rc = dalloc(&c->scratch.counters, (size_t)kCtrWords)) != NES_OK) return fail(rc);
  c->scratch.max_rays = (uint32_t)P;
  if ((rc = dalloc(&c->d_rgb, P * 3)) != NES_OK) return fail(rc);
  if ((rc = dalloc(&c->d_depth, P)) != NES_OK) return fail(rc);
  if ((rc = dalloc(&c->d_rgb8, P * 3)) != NES_OK) return fail(rc);
  if ((rc = dalloc(&c->d_gray, P)) != NES_OK) return fail(rc);
  c->yuv_capacity = 2 * P + 65536;
  if ((rc = dalloc(&c->d_yuv, c->yuv_capacity)) != NES_OK) return fail(rc);
  if ((rc = dalloc(&c->d_depth16, P)) != NES_OK) return fail(rc);
  if (cudaStreamSynchronize(c->stream) != cudaSuccess) return fail(NES_EIO);
  *out = c;
  return NES_OK;
}

void nes_destroy(nes_ctx* ctx) {
  if (!ctx) return;
  cudaSetDevice(ctx->cfg.device);
  cudaStreamSynchronize(ctx->stream);
  free_ctx(ctx);
}

size_t nes_rendered_frame_capacity(uint32_t width, uint32_t height) {
  const size_t px = (size_t)width * height;
  return px * 4 + 256;
}

int nes_render(nes_ctx* c, const uint8_t* request, size_t request_len, uint8_t* frame_out, size_t frame_cap,
               size_t* frame_len) {
  if (!c || (!request && request_len) || !frame_len) return NES_EINVAL;
  PbFrameRequest req;
  if (!parse_frame_request(request, request_len, &req)) return NES_EPROTO;
  if (!req.has_camera || req.camera.matrix.size() != 12) return NES_EPROTO;
  nes_view v;
  std::memset(&v, 0, sizeof(v));
  std::memcpy(v.matrix, req.camera.matrix.data(), sizeof(v.matrix));
  v.width = req.camera.width;
  v.height = req.camera.height;
  if (v.width == 0 || v.height == 0) return NES_EINVAL;
  v.focal_px = nes_focal_from_fov(v.width, c->cfg.fov_deg);
  const size_t px = (size_t)v.width * v.height;
  if (px > c->cfg.max_pixels) return NES_EINVAL;
  const RenderedFrameLayout L = rendered_frame_layout(req.index, &req.camera, req.is_left, px * 3, px);
  *frame_len = L.total;
  if (!frame_out || frame_cap < L.total) return NES_ENOBUFS;

  std::lock_guard<std::mutex> lock(c->mu);
  NES_CUDA(cudaSetDevice(c->cfg.device));
  float* rgb[1] = {c->d_rgb};
  float* dep[1] = {c->d_depth};
  int rc = render_batch_locked(c, &v, 1, rgb, dep);
  if (rc != NES_OK) return rc;
  NES_CUDA(launch_rgb_to_rgb24(c->d_rgb, px * 3, c->d_rgb8, c->stream));
  NES_CUDA(launch_depth_to_gray8(c->d_depth, px, c->cfg.depth_gray_max, c->d_gray, c->stream));
  write_rendered_frame_header(req.index, &req.camera, req.is_left, px * 3, px, frame_out);
  NES_CUDA(cudaMemcpyAsync(frame_out + L.frame_offset, c->d_rgb8, px * 3, cudaMemcpyDeviceToHost, c->stream));
  NES_CUDA(cudaMemcpyAsync(frame_out + L.depth_offset, c->d_gray, px, cudaMemcpyDeviceToHost, c->stream));
  NES_CUDA(cudaStreamSynchronize(c->stream));
  return collect_status(c);
}

int nes_render_views(nes_ctx* c, const nes_view* views, int nviews, float* const* rgb_dev,
                     float* const* depth_dev, void* stream) {
  if (!c || !views) return NES_EINVAL;
  std::lock_guard<std::mutex> lock(c->mu);
  NES_CUDA(cudaSetDevice(c->cfg.device));
  return on_ctx_stream(c, stream, [&] { return render_batch_locked(c, views, nviews, rgb_dev, depth_dev); });
}

int nes_render_yuv_views(nes_ctx* c, const nes_view* views, int nviews, uint8_t* const* y_host,
                         uint8_t* const* u_host, uint8_t* const* v_host, const int linesize[3],
                         uint16_t* const* depth_mm_host) {
  if (!c || !views || !y_host || !u_host || !v_host || !linesize || nviews < 1 || nviews > kMaxViews)
    return NES_EINVAL;
  const int w = (int)views[0].width, h = (int)views[0].height;
  for (int i = 0; i < nviews; ++i) {
    if ((int)views[i].width != w || (int)views[i].height != h) return NES_EINVAL;
    if (!y_host[i] || !u_host[i] || !v_host[i]) return NES_EINVAL;
  }
  if (!planes_ok(w, h, linesize)) return NES_EINVAL;
  const int ch = (h + 1) / 2;
  const size_t ysz = (size_t)linesize[0] * h, usz = (size_t)linesize[1] * ch, vsz = (size_t)linesize[2] * ch;
  const size_t px = (size_t)w * h;
  if ((ysz + usz + vsz) * (size_t)nviews > c->yuv_capacity) return NES_EINVAL;
  if (px * (size_t)nviews > c->cfg.max_pixels) return NES_EINVAL;
  std::lock_guard<std::mutex> lock(c->mu);
  NES_CUDA(cudaSetDevice(c->cfg.device));
  float* rgb[kMaxViews];
  float* dep[kMaxViews];
  for (int i = 0; i < nviews; ++i) {
    rgb[i] = c->d_rgb + 3 * px * (size_t)i;
    dep[i] = c->d_depth + px * (size_t)i;
  }
  int rc = render_batch_locked(c, views, nviews, rgb, dep);
  if (rc != NES_OK) return rc;
  // RGB24 quantisation, YUV420P and depth packing of every view in one launch.
  FrameBatch fb;
  std::memset(&fb, 0, sizeof(fb));
  fb.n = nviews;
  for (int i = 0; i < nviews; ++i) {
    FrameOut& F = fb.f[i];
    F.rgb = rgb[i];
    F.depth = dep[i];
    F.y = c->d_yuv + (ysz + usz + vsz) * (size_t)i;
    F.u = F.y + ysz;
    F.v = F.u + usz;
    F.depth_mm = depth_mm_host && depth_mm_host[i] ? c->d_depth16 + px * (size_t)i : nullptr;
    F.w = w;
    F.h = h;
    F.ls0 = linesize[0];
    F.ls1 = linesize[1];
    F.ls2 = linesize[2];
  }
  frame_batch_index(&fb);
  NES_CUDA(launch_frame_out(fb, c->stream));
  // Only the visible bytes of each row go back: the caller's row padding is
  // left as it was (the device planes' padding holds nothing defined).
  const int cw = (w + 1) / 2;
  for (int i = 0; i < nviews; ++i) {
    const FrameOut& F = fb.f[i];
    NES_CUDA(cudaMemcpy2DAsync(y_host[i], linesize[0], F.y, linesize[0], w, h, cudaMemcpyDeviceToHost, c->stream));
    NES_CUDA(cudaMemcpy2DAsync(u_host[i], linesize[1], F.u, linesize[1], cw, ch, cudaMemcpyDeviceToHost, c->stream));
    NES_CUDA(cudaMemcpy2DAsync(v_host[i], linesize[2], F.v, linesize[2], cw, ch, cudaMemcpyDeviceToHost, c->stream));
    if (F.depth_mm)
      NES_CUDA(cudaMemcpyAsync(depth_mm_host[i], F.depth_mm, px * sizeof(uint16_t), cudaMemcpyDeviceToHost,
                               c->stream));
  }
  NES_CUDA(cudaStreamSynchronize(c->stream));
  return collect_status(c);
}

int nes_render_yuv(nes_ctx* c, const nes_view* view, uint8_t* y_host, uint8_t* u_host, uint8_t* v_host,
                   const int linesize[3], uint16_t* depth_mm_host) {
  if (!c || !view) return NES_EINVAL;
  uint8_t* y[1] = {y_host};
  uint8_t* u[1] = {u_host};
  uint8_t* v[1] = {v_host};
  uint16_t* d[1] = {depth_mm_host};
  return nes_render_yuv_views(c, view, 1, y, u, v, linesize, d);
}

int nes_rgb24_to_yuv420p(const uint8_t* rgb_dev, int width, int height, int rgb_linesize, uint8_t* y_dev,
                         uint8_t* u_dev, uint8_t* v_dev, const int linesize[3], void* stream) {
  if (!rgb_dev || !y_dev || !u_dev || !v_dev || !planes_ok(width, height, linesize)) return NES_EINVAL;
  if (rgb_linesize < 3 * width) return NES_EINVAL;
  NES_CUDA(launch_rgb24_to_yuv420p(rgb_dev, width, height, rgb_linesize, y_dev, u_dev, v_dev, linesize,
                                   reinterpret_cast<cudaStream_t>(stream)));
  return NES_OK;
}

int nes_gray8_to_yuv420p(const uint8_t* gray_dev, int width, int height, int gray_linesize, uint8_t* y_dev,
                         uint8_t* u_dev, uint8_t* v_dev, const int linesize[3], void* stream) {
  if (!gray_dev || !y_dev || !u_dev || !v_dev || !planes_ok(width, height, linesize)) return NES_EINVAL;
  if (gray_linesize < width) return NES_EINVAL;
  NES_CUDA(launch_gray8_to_yuv420p(gray_dev, width, height, gray_linesize, y_dev, u_dev, v_dev, linesize,
                                   reinterpret_cast<cudaStream_t>(stream)));
  return NES_OK;
}

int nes_depth_pack_u16mm(const float* depth_dev, size_t n, uint16_t* out_dev, void* stream) {
  if ((!depth_dev || !out_dev) && n) return NES_EINVAL;
  if (n == 0) return NES_OK;
  NES_CUDA(launch_depth_pack_u16mm(depth_dev, n, out_dev, reinterpret_cast<cudaStream_t>(stream)));
  return NES_OK;
}

namespace {

int yuv_batch(bool gray, int nframes, const uint8_t* const* src, int width, int height, int src_ls,
              uint8_t* const* y, uint8_t* const* u, uint8_t* const* v, const int linesize[3], void* stream) {
  if (nframes < 1 || nframes > NES_MAX_BATCH_FRAMES || !src || !y || !u || !v || !planes_ok(width, height, linesize))
    return NES_EINVAL;
  if (src_ls < (gray ? width : 3 * width)) return NES_EINVAL;
  FrameSet fs;
  std::memset(&fs, 0, sizeof(fs));
  for (int f = 0; f < nframes; ++f) {
    if (!src[f] || !y[f] || !u[f] || !v[f]) return NES_EINVAL;
    fs.src[f] = src[f];
    fs.y[f] = y[f];
    fs.u[f] = u[f];
    fs.v[f] = v[f];
  }
  NES_CUDA(launch_yuv420p_batch(gray, fs, nframes, width, height, src_ls, linesize,
                                reinterpret_cast<cudaStream_t>(stream)));
  return NES_OK;
}

}  // namespace

int nes_rgb24_to_yuv420p_batch(int nframes, const uint8_t* const* rgb_dev, int width, int height, int rgb_linesize,
                               uint8_t* const* y_dev, uint8_t* const* u_dev, uint8_t* const* v_dev,
                               const int linesize[3], void* stream) {
  return yuv_batch(false, nframes, rgb_dev, width, height, rgb_linesize, y_dev, u_dev, v_dev, linesize, stream);
}

int nes_gray8_to_yuv420p_batch(int nframes, const uint8_t* const* gray_dev, int width, int height,
                               int gray_linesize, uint8_t* const* y_dev, uint8_t* const* u_dev, uint8_t* const* v_dev,
                               const int linesize[3], void* stream) {
  return yuv_batch(true, nframes, gray_dev, width, height, gray_linesize, y_dev, u_dev, v_dev, linesize, stream);
}

int nes_depth_pack_u16mm_batch(int nframes, const float* const* depth_dev, size_t n, uint16_t* const* out_dev,
                               void* stream) {
  if (nframes < 1 || nframes > NES_MAX_BATCH_FRAMES || !depth_dev || !out_dev) return NES_EINVAL;
  DepthSet ds;
  std::memset(&ds, 0, sizeof(ds));
  for (int f = 0; f < nframes; ++f) {
    if ((!depth_dev[f] || !out_dev[f]) && n) return NES_EINVAL;
    ds.src[f] = depth_dev[f];
    ds.dst[f] = out_dev[f];
  }
  if (n == 0) return NES_OK;
  NES_CUDA(launch_depth_pack_u16mm_batch(ds, nframes, n, reinterpret_cast<cudaStream_t>(stream)));
  return NES_OK;
}

int nes_depth_to_gray8(const float* depth_dev, size_t n, float dmax, uint8_t* out_dev, void* stream) {
  if ((!depth_dev || !out_dev) && n) return NES_EINVAL;
  if (!(dmax > 0.0f)) return NES_EINVAL;
  if (n == 0) return NES_OK;
  NES_CUDA(launch_depth_to_gray8(depth_dev, n, dmax, out_dev, reinterpret_cast<cudaStream_t>(stream)));
  return NES_OK;
}

int nes_rgb_to_rgb24(const float* rgb_dev, size_t n, uint8_t* out_dev, void* stream) {
  if ((!rgb_dev || !out_dev) && n) return NES_EINVAL;
  if (n == 0) return NES_OK;
  NES_CUDA(launch_rgb_to_rgb24(rgb_dev, n, out_dev, reinterpret_cast<cudaStream_t>(stream)));
  return NES_OK;
}

int nes_parse_frame_request(const uint8_t* bytes, size_t len, nes_frame_request* out) {
  if ((!bytes && len) || !out) return NES_EINVAL;
  PbFrameRequest req;
  if (!parse_frame_request(bytes, len, &req)) return NES_EPROTO;
  std::memset(out, 0, sizeof(*out));
  out->index = req.index;
  out->is_left = req.is_left ? 1 : 0;
  out->has_camera = req.has_camera ? 1 : 0;
  out->camera_is_left = req.camera.is_left ? 1 : 0;
  out->width = req.camera.width;
  out->height = req.camera.height;
  out->matrix_len = (uint32_t)req.camera.matrix.size();
  const size_t k = req.camera.matrix.size() < 12 ? req.camera.matrix.size() : 12;
  if (k) std::memcpy(out->matrix, req.camera.matrix.data(), k * sizeof(float));
  return NES_OK;
}

int nes_write_rendered_frame(const nes_frame_request* req, const uint8_t* frame, size_t frame_len,
                             const uint8_t* depth, size_t depth_len, uint8_t* out, size_t cap, size_t* out_len) {
  if (!req || !out_len || (!frame && frame_len) || (!depth && depth_len)) return NES_EINVAL;
  PbCamera cam;
  cam.is_left = req->camera_is_left != 0;
  cam.width = req->width;
  cam.height = req->height;
  const uint32_t k = req->matrix_len < 12 ? req->matrix_len : 12;
  cam.matrix.assign(req->matrix, req->matrix + k);
  const PbCamera* cp = req->has_camera ? &cam : nullptr;
  const RenderedFrameLayout L = rendered_frame_layout(req->index, cp, req->is_left != 0, frame_len, depth_len);
  *out_len = L.total;
  if (!out || cap < L.total) return NES_ENOBUFS;
  write_rendered_frame_header(req->index, cp, req->is_left != 0, frame_len, depth_len, out);
  if (frame_len) std::memcpy(out + L.frame_offset, frame, frame_len);
  if (depth_len) std::memcpy(out + L.depth_offset, depth, depth_len);
  return NES_OK;
}

int nes_scene_generate(uint64_t seed, uint32_t log2_table_size, float* table_out, float* weights_out) {
  if (!table_out || !weights_out) return NES_EINVAL;
  SceneHost host;
  if (!generate_scene(seed, log2_table_size, &host)) return NES_EINVAL;
  std::memcpy(table_out, host.table.data(), host.table.size() * sizeof(float));
  std::memcpy(weights_out, host.weights.data(), host.weights.size() * sizeof(float));
  return NES_OK;
}

int nes_scene_param(nes_ctx* c, int which, float* host_out, size_t count) {
  if (!c || !host_out) return NES_EINVAL;
  std::lock_guard<std::mutex> lock(c->mu);
  NES_CUDA(cudaSetDevice(c->cfg.device));
  const float* src = nullptr;
  size_t n = 0;
  switch (which) {
    case 0: src = reinterpret_cast<const float*>(c->d_table32); n = (size_t)kLevels * c->scene.T * 2; break;
    case 1: src = c->d_weights + kOffDW1; n = kHid * kEnc; break;
    case 2: src = c->d_weights + kOffDW2; n = kDOut * kHid; break;
    case 3: src = c->d_weights + kOffCW1; n = kHid * kCIn; break;
    case 4: src = c->d_weights + kOffCW2; n = kHid * kHid; break;
    case 5: src = c->d_weights + kOffCW3; n = 3 * kHid; break;
    default: return NES_EINVAL;
  }
  if (count != n) return NES_EINVAL;
  NES_CUDA(cudaStreamSynchronize(c->stream));
  NES_CUDA(cudaMemcpy(host_out, src, n * sizeof(float), cudaMemcpyDeviceToHost));
  return NES_OK;
}

int nes_scene_set_param(nes_ctx* c, int which, const float* host_in, size_t count) {
  if (!c || !host_in) return NES_EINVAL;
  std::lock_guard<std::mutex> lock(c->mu);
  NES_CUDA(cudaSetDevice(c->cfg.device));
  float* dst = nullptr;
  size_t n = 0;
  switch (which) {
    case 0: dst = reinterpret_cast<float*>(c->d_table32); n = (size_t)kLevels * c->scene.T * 2; break;
    case 1: dst = c->d_weights + kOffDW1; n = kHid * kEnc; break;
    case 2: dst = c->d_weights + kOffDW2; n = kDOut * kHid; break;
    case 3: dst = c->d_weights + kOffCW1; n = kHid * kCIn; break;
    case 4: dst = c->d_weights + kOffCW2; n = kHid * kHid; break;
    case 5: dst = c->d_weights + kOffCW3; n = 3 * kHid; break;
    default: return NES_EINVAL;
  }
  if (count != n) return NES_EINVAL;
  NES_CUDA(cudaStreamSynchronize(c->stream));
  NES_CUDA(cudaMemcpy(dst, host_in, n * sizeof(float), cudaMemcpyHostToDevice));
  if (c->cfg.precision == NES_PREC_FP16_TC) {  // the tensor-core path's derived copies
    if (which == 0) {
      NES_CUDA(launch_table_to_fp16(c->d_table32, c->d_table16, (size_t)kLevels * c->scene.T, c->stream));
      NES_CUDA(launch_build_records(c->d_table16, c->scene.T, c->scene.dense_mask, (int)c->scene.rec_levels,
                                    c->d_rec16, c->stream));
    } else {
      NES_CUDA(launch_pack_tc_weights(c->d_weights, c->d_tc_weights, c->stream));
    }
    NES_CUDA(cudaStreamSynchronize(c->stream));
  }
  return NES_OK;
}

int nes_occupancy(nes_ctx* c, uint32_t* host_bits) {
  if (!c || !host_bits) return NES_EINVAL;
  std::lock_guard<std::mutex> lock(c->mu);
  NES_CUDA(cudaSetDevice(c->cfg.device));
  NES_CUDA(cudaStreamSynchronize(c->stream));
  NES_CUDA(cudaMemcpy(host_bits, c->d_occ, kOccWords * sizeof(uint32_t), cudaMemcpyDeviceToHost));
  return NES_OK;
}

int nes_rebuild_occupancy(nes_ctx* c, float threshold) {
  if (!c || !(threshold > 0.0f)) return NES_EINVAL;
  std::lock_guard<std::mutex> lock(c->mu);
  NES_CUDA(cudaSetDevice(c->cfg.device));
  NES_CUDA(launch_occupancy(c->scene, threshold, c->d_occ, c->stream));
  NES_CUDA(cudaStreamSynchronize(c->stream));
  return collect_status(c);
}

int nes_last_sample_count(nes_ctx* c, uint64_t* samples) {
  if (!c || !samples) return NES_EINVAL;
  std::lock_guard<std::mutex> lock(c->mu);
  NES_CUDA(cudaSetDevice(c->cfg.device));
  NES_CUDA(cudaStreamSynchronize(c->stream));
  const int rc = collect_status(c);
  *samples = c->last_samples;
  return rc;
}

int nes_selftest_bounded_wait(nes_ctx* c, uint32_t poll_limit, int arrive) {
  if (!c || poll_limit == 0 || poll_limit > (1u << 24)) return NES_EINVAL;
  std::lock_guard<std::mutex> lock(c->mu);
  NES_CUDA(cudaSetDevice(c->cfg.device));
  // Settle the previous render's sample count before the counters are reused.
  NES_CUDA(cudaStreamSynchronize(c->stream));
  const int prev = collect_status(c);
  if (prev != NES_OK) return prev;
  NES_CUDA(cudaMemsetAsync(c->scratch.counters, 0, kCtrWords * sizeof(uint32_t), c->stream));
  NES_CUDA(launch_bounded_wait_probe(poll_limit, arrive ? 1 : 0, c->scratch.counters, c->stream));
  uint32_t err = 0;
  NES_CUDA(cudaMemcpyAsync(&err, c->scratch.counters + kCtrError, sizeof(err), cudaMemcpyDeviceToHost, c->stream));
  NES_CUDA(cudaStreamSynchronize(c->stream));
  return err ? NES_ETIMEDOUT : NES_OK;
}

int nes_probe_gather(const void* table_dev, uint64_t table_bytes, int load_bytes, uint32_t loads_per_thread,
                     uint32_t threads, uint32_t* sink_dev, void* stream) {
  if (!table_dev || !sink_dev || loads_per_thread == 0) return NES_EINVAL;
  const cudaError_t e = launch_gather_probe(table_dev, table_bytes, load_bytes, loads_per_thread, sink_dev, threads,
                                            reinterpret_cast<cudaStream_t>(stream));
  return e == cudaSuccess ? NES_OK : (e == cudaErrorInvalidValue ? NES_EINVAL : NES_EIO);
}

int nes_probe_gather_replay(nes_ctx* c, const nes_view* views, int nviews, int threads, uint32_t* sink_dev,
                            size_t sink_words, float* replay_ms) {
  if (!c || !views || !sink_dev || !replay_ms) return NES_EINVAL;
  if (c->cfg.precision != NES_PREC_FP16_TC || (threads != 256 && threads != 512)) return NES_EINVAL;
  if (sink_words < (size_t)c->num_sms * (size_t)threads) return NES_EINVAL;
  std::lock_guard<std::mutex> lock(c->mu);
  NES_CUDA(cudaSetDevice(c->cfg.device));
  ViewBatch vb;
  uint64_t pixels = 0;
  float* none[kMaxViews] = {};
  const int rc = fill_view_batch(views, nviews, none, none, c->cfg.max_pixels, &vb, &pixels);
  if (rc != NES_OK) return rc;
  NES_CUDA(cudaStreamSynchronize(c->stream));
  const int prev = collect_status(c);
  if (prev != NES_OK) return prev;
  cudaEvent_t ev[2] = {nullptr, nullptr};
  NES_CUDA(cudaEventCreate(&ev[0]));
  if (cudaEventCreate(&ev[1]) != cudaSuccess) {
    cudaEventDestroy(ev[0]);
    return NES_EIO;
  }
  cudaError_t e = cudaMemsetAsync(c->scratch.counters, 0, kCtrWords * sizeof(uint32_t), c->stream);
  if (e == cudaSuccess) e = launch_raygen(vb, c->scratch, c->stream);
  if (e == cudaSuccess) e = cudaEventRecord(ev[0], c->stream);
  if (e == cudaSuccess) e = launch_gather_replay(vb, c->scene, c->scratch, c->num_sms, threads, sink_dev, c->stream);
  if (e == cudaSuccess) e = cudaEventRecord(ev[1], c->stream);
  if (e == cudaSuccess) e = cudaEventSynchronize(ev[1]);
  if (e == cudaSuccess) e = cudaEventElapsedTime(replay_ms, ev[0], ev[1]);
  cudaEventDestroy(ev[0]);
  cudaEventDestroy(ev[1]);
  return e == cudaSuccess ? NES_OK : NES_EIO;
}

int nes_set_profiling(nes_ctx* c, int enable) {
  if (!c) return NES_EINVAL;
  std::lock_guard<std::mutex> lock(c->mu);
  NES_CUDA(cudaSetDevice(c->cfg.device));
  for (cudaEvent_t& e : c->ev_t)
    if (!e) NES_CUDA(cudaEventCreate(&e));
  c->profiling = enable != 0;
  c->timings_pending = false;
  return NES_OK;
}

int nes_last_timings(nes_ctx* c, float* raygen_ms, float* march_ms) {
  if (!c || !raygen_ms || !march_ms) return NES_EINVAL;
  std::lock_guard<std::mutex> lock(c->mu);
  if (!c->timings_pending) return NES_EAGAIN;
  NES_CUDA(cudaSetDevice(c->cfg.device));
  NES_CUDA(cudaEventSynchronize(c->ev_t[2]));
  NES_CUDA(cudaEventElapsedTime(raygen_ms, c->ev_t[0], c->ev_t[1]));
  NES_CUDA(cudaEventElapsedTime(march_ms, c->ev_t[1], c->ev_t[2]));
  return NES_OK;
}

}  // extern "C"

namespace nes {

bool view_ok(const nes_view& v) {
  if (v.width == 0 || v.height == 0 || v.width > 16384 || v.height > 16384) return false;
  if (!(v.focal_px > 0.0f) || !std::isfinite(v.focal_px)) return false;
  for (float m : v.matrix)
    if (!std::isfinite(m)) return false;
  return true;
}

int fill_view_batch(const nes_view* views, int n, float* const* rgb, float* const* depth, uint64_t max_pixels,
                    ViewBatch* vb, uint64_t* pixels) {
  if (!views || n < 1 || n > kMaxViews) return NES_EINVAL;
  std::memset(vb, 0, sizeof(*vb));
  vb->n = n;
  uint64_t total = 0, threads = 0;
  for (int i = 0; i < n; ++i) {
    if (!view_ok(views[i])) return NES_EINVAL;
    DevView& d = vb->v[i];
    std::memcpy(d.M, views[i].matrix, sizeof(d.M));
    d.W = (int)views[i].width;
    d.H = (int)views[i].height;
    d.focal = views[i].focal_px;
    d.pix_offset = (uint32_t)threads;
    d.rgb = rgb ? rgb[i] : nullptr;
    d.depth = depth ? depth[i] : nullptr;
    total += (uint64_t)views[i].width * views[i].height;
    threads += view_threads(d.W, d.H);
  }
  if (total > max_pixels || threads > 0xFFFFFFFFull) return NES_EINVAL;
  vb->total_pixels = (uint32_t)threads;
  *pixels = total;
  return NES_OK;
}

cudaError_t enqueue_march(const ViewBatch& vb, const DevScene& scene, const DevScratch& s, int precision, int num_sms,
                          cudaStream_t stream) {
  cudaError_t e = cudaMemsetAsync(s.counters, 0, kCtrWords * sizeof(uint32_t), stream);
  if (e != cudaSuccess) return e;
  if ((e = launch_raygen(vb, s, stream)) != cudaSuccess) return e;
  return precision == NES_PREC_FP16_TC ? launch_march_tc(vb, scene, s, num_sms, stream)
                                       : launch_march_fp32(vb, scene, s, num_sms, stream);
}

}  // namespace nes
