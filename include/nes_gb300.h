/*
 * nes_gb300.h -- C ABI of the GB300 render-and-encode library.
 *
 * Two drop-in boundaries of neserver (moonsikpark/ngp-encode-server):
 *
 *  (i)  The renderer round trip.  neserver serialises a nesproto::FrameRequest,
 *       sends it length-prefixed to an external instant-ngp-renderer process
 *       and parses the nesproto::RenderedFrame it gets back
 *       (src/server.cpp:161-194, framing in src/server.cpp:46-60 and 91-112).
 *       nes_render() takes and returns the same nes.proto bytes
 *       (proto/nes.proto:5-25) in-process; nes_render_views() and
 *       nes_render_yuv() are the device-native forms.
 *
 *  (ii) The frame glue.  RenderedFrame::convert_frame converts the RGB24 scene
 *       and GRAY8 depth planes to YUV420P with libswscale
 *       (include/base/video/rendered_frame.h:24-33,
 *       src/base/video/type_managers.cc:143-153).  nes_rgb24_to_yuv420p() and
 *       nes_gray8_to_yuv420p() write the same YUV420P plane layout that
 *       AVCodecContextManager::send_frame consumes (src/encode.cpp:136-137,
 *       164-165); nes_depth_pack_u16mm() packs FP32 depth to uint16 mm.
 *
 * Conventions (mirroring src/server.cpp:23-43, which returns -errno):
 *  - every entry point returns an int status: NES_OK (0) or a negative
 *    errno-style NES_E* code; no C++ exception crosses this boundary;
 *  - pointers named *_dev are CUDA device pointers, everything else is host;
 *  - `stream` is a cudaStream_t passed as void*; NULL means the context's own
 *    stream (stream-free glue functions use the legacy default stream);
 *  - one nes_ctx may be used from several host threads; calls on one context
 *    are serialised internally.
 */
#ifndef NES_GB300_H_
#define NES_GB300_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define NES_OK 0
#define NES_EIO (-5)        /* a CUDA call failed */
#define NES_EAGAIN (-11)    /* nothing ready yet / queue full */
#define NES_ENOMEM (-12)    /* device or host allocation failed */
#define NES_ENODEV (-19)    /* no usable CUDA device */
#define NES_EINVAL (-22)    /* bad argument */
#define NES_EPROTO (-71)    /* malformed nes.proto message */
#define NES_ENOBUFS (-105)  /* caller's output buffer too small */
#define NES_ETIMEDOUT (-110)/* a bounded wait ran out */

enum nes_precision {
  NES_PREC_FP32 = 0,    /* plain path: FP32 table, FP32 MLP on CUDA cores */
  NES_PREC_FP16_TC = 1  /* FP16 table, FP16 MLP on tcgen05 tensor cores, FP32 accumulate */
};

typedef struct nes_ctx nes_ctx;

/* Scene and renderer configuration.  The scene is generated from `seed`
 * (SplitMix64 streams) and is identical for every precision. */
typedef struct nes_config {
  uint64_t seed;             /* scene seed (0 for the reference scene) */
  uint32_t log2_table_size;  /* hash-table entries per level = 2^this (10..24) */
  int32_t precision;         /* enum nes_precision */
  float fov_deg;             /* horizontal FOV for nes_render (nes.proto has no FOV field) */
  float depth_gray_max;      /* scene units mapped to 255 in GRAY8 depth */
  int32_t device;            /* CUDA device ordinal */
  uint32_t max_pixels;       /* largest single-call pixel count (sum over views) */
  uint32_t record_levels;    /* tensor-core path: hash-grid levels also kept as per-cell records
                              * of their 8 corner entries (one 32-byte read instead of eight
                              * scattered gathers): 13 = levels 0..12, 24.0 GB (the default),
                              * 10 = levels 0..9, 1.30 GB; 0 = the default */
} nes_config;

/* One view to render: the nes.proto Camera plus a focal length.
 * matrix: 3x4 row-major pose (include/base/camera_manager.h:18-19):
 * columns 0,1,2 = image right, image down, view direction; column 3 = eye.
 * Every entry point that takes views accepts one when width and height are
 * 1..16384, focal_px is finite and positive and all 12 matrix entries are
 * finite, and returns NES_EINVAL otherwise. */
typedef struct nes_view {
  float matrix[12];
  uint32_t width;
  uint32_t height;
  float focal_px;  /* focal length in pixels; see nes_focal_from_fov */
  uint32_t flags;  /* reserved, 0 */
} nes_view;

/* Fills cfg with the reference scene: seed 0, 2^19 entries, FP32, 90 deg,
 * 13 record levels. */
void nes_config_default(nes_config *cfg);

/* Creates a context on cfg->device: generates the scene, uploads it,
 * builds the 128^3 occupancy grid.  Replaces connecting to a renderer
 * (src/server.cpp:216-283). */
int nes_create(const nes_config *cfg, nes_ctx **out);
void nes_destroy(nes_ctx *ctx);
const char *nes_strerror(int code);

/* focal = (width/2) / tan(fov/2), computed in double, rounded to float. */
float nes_focal_from_fov(uint32_t width, float fov_deg);

/* ---------------- (i) renderer round trip ---------------- */

/* Upper bound of the RenderedFrame bytes nes_render writes for a w x h
 * camera (RGB24 frame + GRAY8 depth + header). */
size_t nes_rendered_frame_capacity(uint32_t width, uint32_t height);

/* Wire-compatible render: request = serialised nesproto::FrameRequest,
 * frame_out receives a serialised nesproto::RenderedFrame with the same
 * index/camera/is_left, frame = RGB24 (W*H*3) and depth = GRAY8 (W*H),
 * exactly the payload src/server.cpp:193-194 wraps.  Replaces
 * socket_send_blocking_lpf + socket_receive_blocking_lpf + ParseFromString
 * (src/server.cpp:161-177).  NES_EPROTO for a malformed request,
 * NES_ENOBUFS (with *frame_len = bytes needed) when cap is too small. */
int nes_render(nes_ctx *ctx, const uint8_t *request, size_t request_len, uint8_t *frame_out,
               size_t frame_cap, size_t *frame_len);

/* Renderer endpoint for an unmodified neserver (`--renderer ip:port`):
 * listens on bind_addr:port (port 0 picks a free one, reported in
 * *bound_port) and answers each connection's length-prefixed FrameRequests
 * with RenderedFrames through nes_render, exactly the framing of
 * socket_send_blocking_lpf / socket_receive_blocking_lpf (src/server.cpp:46-112).
 * Blocks until *stop becomes nonzero (checked every 100 ms), then closes the
 * listener, finishes the open connections and returns; *frames_served counts
 * answered requests.  Negative errno on socket errors. */
int nes_tcp_serve(nes_ctx *ctx, const char *bind_addr, uint16_t port, const volatile int *stop,
                  uint16_t *bound_port, uint64_t *frames_served);

/* Device-native render of n views in one batch (rays of all views share
 * one march): the renderer's work behind the round trip of
 * src/server.cpp:161-194 with the frame left on the device, and both eyes
 * of a stereo request at once where neserver asks for them one at a time
 * (src/server.cpp:144-153).  rgb_dev[i]: W*H*3 floats (HWC), depth_dev[i]:
 * W*H floats (expected depth, 0 for rays that miss); either may be NULL. */
int nes_render_views(nes_ctx *ctx, const nes_view *views, int nviews, float *const *rgb_dev,
                     float *const *depth_dev, void *stream);

/* Pose -> YUV end to end for one view: render, RGB24 quantise, convert to
 * YUV420P and pack depth to uint16 mm on the device, then copy the planes to
 * the caller's HOST buffers (pinned for best speed): the renderer round trip
 * (src/server.cpp:161-194) and RenderedFrame::convert_frame
 * (include/base/video/rendered_frame.h:24-33) in one call.  y/u/v follow
 * linesize[3] (chroma planes are ceil(W/2) x ceil(H/2)); only the visible
 * bytes of each row are written, the row padding up to the linesize is left
 * as it was.  depth_mm_host is W*H uint16 (may be NULL).  Blocks until the
 * host buffers are filled. */
int nes_render_yuv(nes_ctx *ctx, const nes_view *view, uint8_t *y_host, uint8_t *u_host,
                   uint8_t *v_host, const int linesize[3], uint16_t *depth_mm_host);

/* Pose -> YUV end to end for nviews views of one size rendered as one batch
 * (e.g. the left and right eye of a stereo request, which neserver asks the
 * renderer for one eye at a time, src/server.cpp:144-161): one march over all
 * views' rays, one frame-output launch for all views, then the planes of
 * view i are copied to y_host[i], u_host[i], v_host[i] (all with
 * linesize[3]) and, where depth_mm_host is not NULL and depth_mm_host[i] is
 * not NULL, its W*H uint16 depth to depth_mm_host[i].  Each view's bytes are
 * those nes_render_yuv gives for it alone.  Blocks until the host buffers are
 * filled.  NES_EINVAL for views of different sizes or beyond the context's
 * max_pixels. */
int nes_render_yuv_views(nes_ctx *ctx, const nes_view *views, int nviews, uint8_t *const *y_host,
                         uint8_t *const *u_host, uint8_t *const *v_host, const int linesize[3],
                         uint16_t *const *depth_mm_host);

/* Largest view (width * height) nes_render_view_noalloc accepts. */
#define NES_NOALLOC_MAX_PIXELS (1u << 18) /* 262,144 pixels, e.g. 512 x 512 */

/* Plain FP32 render of one view that allocates no device memory.  No
 * counterpart in the reference: it exists for callers that may not call
 * cudaMalloc/cudaFree (a host application that owns all device memory and
 * hands out fixed buffers, or a frame loop that cannot take the implicit
 * synchronisation of an allocation).  The caller passes the scene
 * (table_dev = 16 * 2^log2_table_size * 2 floats, weights_dev = the 9,408-float
 * blob of nes_scene_generate, occupancy_dev = 65,536 words as nes_occupancy
 * returns) and the outputs (rgb_dev W*H*3 floats, depth_dev W*H floats;
 * either may be NULL).  Work is queued on `stream` (NULL = legacy default
 * stream) on the calling thread's current device.  The ray list lives in a
 * static device array of the library (8 MiB + 256 B, held by every GPU that
 * loads the library's device code until exit): views above
 * NES_NOALLOC_MAX_PIXELS pixels return NES_EINVAL.  All calls on a device
 * share that array: calls whose GPU work overlaps race.  The first call on
 * a device looks up the array's address (make it before any stream capture
 * on that device) and keeps it for the life of the process, so a
 * cudaDeviceReset of that device after the first call is not supported. */
int nes_render_view_noalloc(const float *table_dev, uint32_t log2_table_size, const float *weights_dev,
                            const uint32_t *occupancy_dev, const nes_view *view, float *rgb_dev,
                            float *depth_dev, void *stream);

/* ---------------- serving: continuously batched request loop ----------------
 * Replaces neserver's request loop (src/server.cpp:116-214: one synchronous
 * FrameRequest in flight per renderer connection, frames handed on through a
 * bounded FrameQueue/FrameMap with 1 s lock timeouts, src/base/video/
 * frame_queue.cc:11-39, frame_map.cc:12-53).  Requests are admitted against a
 * device-memory budget; a scheduler thread flattens the views of all waiting
 * requests (mono or stereo, any resolution) into one ray queue per batch and
 * keeps up to max_inflight_batches batches on the GPU.  Each batch slot owns
 * one CUDA graph, captured and instantiated once at creation, whose kernels
 * read the batch (views, poses, output planes) from a device-side descriptor:
 * every batch of any shape replays it.  Outputs (YUV420P planes + uint16
 * depth) are carved at admission out of a device output arena allocated once
 * at creation (the budget minus the fixed per-slot buffers) and stay there
 * until the caller releases them: nothing is allocated on the request path. */

typedef struct nes_server nes_server;

typedef struct nes_server_config {
  uint64_t hbm_budget_bytes;     /* batch scratch + outputs of admitted requests */
  uint32_t max_batch_pixels;     /* pixels per batch (sum over its views), 64..2^27 */
  uint32_t max_inflight_batches; /* batches on the GPU at once (1..4) */
  uint32_t max_pending;          /* admitted requests waiting for a batch */
  int32_t use_graphs;            /* 1: CUDA graph per batch shape, 0: plain launches */
  float max_queue_ms;            /* > 0: reject a request whose estimated pose -> YUV time
                                  * (its expected samples plus those of every request queued
                                  * or in flight -- mean march length of a 16 x 16 grid of each
                                  * view's rays through the unit cube, times its pixels -- at
                                  * the measured sample throughput) exceeds this; 0: no bound */
} nes_server_config;

typedef struct nes_request {
  uint32_t nviews; /* 1 = mono, 2 = stereo (left, right) */
  nes_view views[2];
} nes_request;

typedef struct nes_result {
  uint64_t ticket;
  int32_t status;  /* NES_OK, or the error of the batch */
  uint32_t nviews;
  uint32_t width, height;
  int32_t linesize[3];        /* YUV420P plane linesizes (32-byte aligned; row padding zeroed) */
  uint8_t *y_dev[2], *u_dev[2], *v_dev[2];
  uint16_t *depth_mm_dev[2];  /* W*H uint16 millimetres per view */
  double latency_ms;          /* submit -> YUV ready on the device */
  uint64_t batch_id;
  uint32_t batch_requests;    /* requests that shared this request's batch */
  uint32_t batch_views;
} nes_result;

typedef struct nes_server_stats {
  uint64_t submitted, rejected, completed, batches;
  uint64_t pixels, samples;
  uint64_t graph_instantiations; /* one per slot, at creation (0 with use_graphs = 0) */
  uint64_t graph_updates;        /* graph updates after creation: always 0 */
  uint64_t budget_used_bytes;
} nes_server_stats;

/* Fills cfg with defaults: 8 GiB budget, 2x1920x1832 pixels per batch, two
 * batches in flight, 256 pending requests, graphs on. */
void nes_server_config_default(nes_server_config *cfg);

int nes_server_create(nes_ctx *ctx, const nes_server_config *cfg, nes_server **out);
/* Stops the scheduler, waits for the batches on the GPU and frees the
 * server.  Requests still pending (never batched) finish with NES_EIO.
 * nes_submit, nes_wait and nes_release must not run concurrently with it or
 * after it. */
void nes_server_destroy(nes_server *srv);

/* Admits a request.  NES_EAGAIN when the budget or the pending queue is
 * full, or when max_queue_ms is set and the request would wait longer (the
 * request is dropped and counted), NES_EINVAL for a bad request (a view
 * that nes_render_views would reject, stereo eyes of different sizes, more
 * than max_batch_pixels pixels): it is refused here and never reaches a
 * batch, so it cannot fail the requests batched with it.  Until the
 * first batch has completed (no throughput estimate yet) the bound admits at
 * most max_batch_pixels of queued and running pixels. */
int nes_submit(nes_server *srv, const nes_request *req, uint64_t *ticket);

/* Waits up to timeout_ns (< 0 or above 10^15: forever) for the request;
 * NES_ETIMEDOUT when it is not finished yet.  The output pointers stay valid
 * until release. */
int nes_wait(nes_server *srv, uint64_t ticket, int64_t timeout_ns, nes_result *out);

/* Frees a finished request's output slots and its budget share. */
int nes_release(nes_server *srv, uint64_t ticket);

int nes_server_stats_get(nes_server *srv, nes_server_stats *out);

/* Synchronous device -> host copy of n bytes, e.g. a served YUV plane for the
 * host H.264 encoder (AVCodecContextManager::send_frame, src/encode.cpp:136). */
int nes_copy_to_host(void *host_dst, const void *dev_src, size_t n);

/* ---------------- differentiation: refit a scene to target renders ----------------
 * No counterpart in neserver (which only renders); this is the training
 * form of the renderer: a hand-written backward through the volume
 * rendering (per-sample compositing adjoint from recorded sample states),
 * the MLPs (per-sample backpropagation; weight gradients as GEMMs over the
 * samples on the tensor cores, or exact FP32 reductions) and the hash grid (atomic float2 scatter-add
 * into an FP32 gradient table), then Adam on the student context's FP32
 * table and weights.  The occupancy grid is left as it is (rebuild it with
 * nes_rebuild_occupancy between steps where wanted).
 * Loss per ray: |C - C*|^2 + depth_weight (D - D*)^2, averaged over the batch.
 * Trainer calls hold the student context's lock; a nes_server must not be
 * serving the same context meanwhile. */

typedef struct nes_trainer nes_trainer;

typedef struct nes_train_config {
  uint32_t batch_rays;  /* rays per step (2^18 in the refit configuration) */
  float lr, beta1, beta2, eps;
  float depth_weight;
  /* 0 (default): the per-sample MLP on the tensor cores (tcgen05) -- the
   * forward's field evaluation as 3xTF32 products (FP32-level loss), the
   * backward's recompute, backpropagation and weight-gradient GEMMs in TF32;
   * 1: everything in FP32 on the CUDA cores (the strict parity mode). */
  int32_t exact_weight_grads;
} nes_train_config;

/* lr 1e-2, betas (0.9, 0.99), eps 1e-15, depth weight 0.1, 2^18 rays,
 * the tensor-core mode (exact_weight_grads = 0). */
void nes_train_config_default(nes_train_config *cfg);

/* The student must be an NES_PREC_FP32 context; its table and weights are
 * updated in place by the step calls.  batch_rays <= 2^20.  Device memory:
 * 64 B per ray per march step (1024 steps) of scratch (per-sample state and
 * the sample list / adjoint records), ~3.9 GB of per-sample staging for the
 * weight gradients, 4x the table for gradient and Adam moments, and ~160 KB
 * of weight operand images. */
int nes_trainer_create(nes_ctx *student, const nes_train_config *cfg, nes_trainer **out);
void nes_trainer_destroy(nes_trainer *tr);

/* Target images: nviews views (1..1024) with HWC FP32 RGB and FP32 depth on
 * the device, concatenated view after view (pointers are kept, not copied).
 * NES_EINVAL for a view that nes_render_views would reject. */
int nes_trainer_set_targets(nes_trainer *tr, const nes_view *views, int nviews, const float *rgb_dev,
                            const float *depth_dev);

/* One step: samples batch_rays (view, pixel) pairs from the seed, computes
 * the loss and gradients, applies Adam.  *loss = mean loss before the update. */
int nes_trainer_step(nes_trainer *tr, uint64_t seed, double *loss);

/* One step on the listed rays (n pairs of int32 view, pixel on the host). */
int nes_trainer_step_rays(nes_trainer *tr, const int32_t *rays, int n, double *loss);

/* Loss and gradient of the mean loss over the listed rays (rays: n pairs of
 * int32 view, pixel on the host), without updating anything.  Gradient
 * outputs (host, may be NULL): table 16*T*2 floats, weights 9,408 floats
 * (layout of nes_scene_generate). */
int nes_trainer_grad(nes_trainer *tr, const int32_t *rays, int n, double *loss, float *grad_table,
                     float *grad_weights);

/* The same loss evaluated in FP64 on the GPU with one parameter perturbed by
 * delta (which: 0 table, 1 weights blob; index into that array), for
 * central finite-difference checks. */
int nes_trainer_loss_fp64(nes_trainer *tr, const int32_t *rays, int n, int which, uint64_t index, double delta,
                          double *loss);

/* The same FP64 loss for m perturbations in one launch (1..65535):
 * perturbation j adds delta[j] to entry index[j] of array which[j] (0 table,
 * 1 weights blob); losses[j] receives its loss.  For checking many
 * parameters by central differences at once. */
int nes_trainer_loss_fp64_batch(nes_trainer *tr, const int32_t *rays, int n, int m, const int32_t *which,
                                const uint64_t *index, const double *delta, double *losses);

/* Samples evaluated (and backpropagated) by the last loss/gradient pass. */
uint64_t nes_trainer_last_samples(const nes_trainer *tr);

/* Device time of the last step's phases from CUDA events on the trainer's
 * stream: forward march + compositing adjoint, backward (recompute,
 * backpropagation, table scatter, weight-gradient reductions), Adam.
 * NES_EAGAIN before the first step. */
int nes_trainer_last_timings(const nes_trainer *tr, float *forward_ms, float *backward_ms, float *adam_ms);

/* ---------------- (ii) frame glue ---------------- */

/* RGB24 -> YUV420P, BT.601 studio range, 2x2 chroma average (edge pixels
 * replicated for odd sizes).  Replaces the scene SwsContextManager in
 * RenderedFrame::convert_frame (include/base/video/rendered_frame.h:28-29). */
int nes_rgb24_to_yuv420p(const uint8_t *rgb_dev, int width, int height, int rgb_linesize,
                         uint8_t *y_dev, uint8_t *u_dev, uint8_t *v_dev, const int linesize[3],
                         void *stream);

/* GRAY8 -> YUV420P (luma scaled to studio range, chroma 128).  Replaces the
 * depth SwsContextManager (include/base/video/rendered_frame.h:30-31). */
int nes_gray8_to_yuv420p(const uint8_t *gray_dev, int width, int height, int gray_linesize,
                         uint8_t *y_dev, uint8_t *u_dev, uint8_t *v_dev, const int linesize[3],
                         void *stream);

/* Batched frame glue.  neserver converts one frame per call (process_frame_thread
 * -> RenderedFrame::convert_frame, src/encode.cpp:42-119); these convert
 * nframes frames of one geometry in a single launch, each frame identical to
 * the single-frame call.  rgb_dev / gray_dev / y_dev / u_dev / v_dev (and
 * depth_dev / out_dev) are host arrays of nframes device pointers; at most
 * NES_MAX_BATCH_FRAMES frames per call. */
#define NES_MAX_BATCH_FRAMES 64
int nes_rgb24_to_yuv420p_batch(int nframes, const uint8_t *const *rgb_dev, int width, int height,
                               int rgb_linesize, uint8_t *const *y_dev, uint8_t *const *u_dev,
                               uint8_t *const *v_dev, const int linesize[3], void *stream);
int nes_gray8_to_yuv420p_batch(int nframes, const uint8_t *const *gray_dev, int width, int height,
                               int gray_linesize, uint8_t *const *y_dev, uint8_t *const *u_dev,
                               uint8_t *const *v_dev, const int linesize[3], void *stream);
int nes_depth_pack_u16mm_batch(int nframes, const float *const *depth_dev, size_t n, uint16_t *const *out_dev,
                               void *stream);

/* Debug text overlay into an RGB24 frame on the device, before conversion:
 * RenderTextContext::render_string_to_frame (src/base/video/render_text.cc:35-111)
 * with the same five anchors (margin 50, box 300x100), '\n' = back to the
 * anchor column and 20 px down, covered pixels set to white, clipped to the
 * frame.  Glyphs are this library's 5x7 font at 2x (10x14 px, 12 px advance,
 * baseline at the pen) for ' ', + - . : = 0-9 a-z; other characters advance
 * without drawing.  At most 512 drawn characters per call. */
enum nes_text_anchor {
  NES_TEXT_LEFT_TOP = 0,
  NES_TEXT_LEFT_BOTTOM = 1,
  NES_TEXT_RIGHT_TOP = 2,
  NES_TEXT_RIGHT_BOTTOM = 3,
  NES_TEXT_CENTER = 4
};
int nes_overlay_text(uint8_t *rgb_dev, int width, int height, int linesize, const char *text, int anchor,
                     void *stream);

/* FP32 depth (scene units = metres) -> uint16 millimetres, round half up,
 * NaN/negative -> 0, saturating at 65535. */
int nes_depth_pack_u16mm(const float *depth_dev, size_t n, uint16_t *out_dev, void *stream);

/* FP32 depth -> GRAY8 (round(clamp(d/dmax,0,1)*255)), the depth plane of
 * nesproto::RenderedFrame (src/server.cpp:193-194). */
int nes_depth_to_gray8(const float *depth_dev, size_t n, float dmax, uint8_t *out_dev,
                       void *stream);

/* FP32 RGB in [0,1] -> RGB24 bytes (round(clamp(x,0,1)*255)). */
int nes_rgb_to_rgb24(const float *rgb_dev, size_t n, uint8_t *out_dev, void *stream);

/* ---------------- nes.proto wire helpers (no GPU) ---------------- */

/* A parsed nesproto::FrameRequest (proto/nes.proto:12-16) with its Camera
 * (proto/nes.proto:5-10) flattened. */
typedef struct nes_frame_request {
  uint64_t index;
  int32_t is_left;
  int32_t has_camera;
  int32_t camera_is_left;
  uint32_t width;
  uint32_t height;
  uint32_t matrix_len;  /* floats present in Camera.matrix; 12 expected */
  float matrix[12];     /* the first min(12, matrix_len) floats */
} nes_frame_request;

/* Parses FrameRequest bytes, as the renderer side of src/server.cpp:161-168
 * receives them.  NES_EPROTO on malformed input. */
int nes_parse_frame_request(const uint8_t *bytes, size_t len, nes_frame_request *out);

/* Serialises RenderedFrame{index, camera, is_left, frame, depth}
 * (proto/nes.proto:18-25) echoing req's index/camera/is_left, as the renderer
 * answers src/server.cpp:170-177.  *out_len = bytes needed; NES_ENOBUFS when
 * cap is too small (out may then be NULL). */
int nes_write_rendered_frame(const nes_frame_request *req, const uint8_t *frame, size_t frame_len,
                             const uint8_t *depth, size_t depth_len, uint8_t *out, size_t cap,
                             size_t *out_len);

/* Generates the seeded scene on the host (no GPU): table = 16*2^log2T*2
 * floats (level-major), weights = 9408 floats: density W1 [64][32], density
 * W2 [16][64], colour W1 [64][32], colour W2 [64][64], colour W3 [3][64]. */
int nes_scene_generate(uint64_t seed, uint32_t log2_table_size, float *table_out, float *weights_out);

/* ---------------- scene access (tests, tools) ---------------- */

/* Copies one scene parameter array to host: which 0 = hash table
 * (16*T*2 floats, level-major), 1..5 = density W1 [64][32], density W2
 * [16][64], colour W1 [64][32] (column 31 zero), colour W2 [64][64],
 * colour W3 [3][64] (row-major [out][in]). */
int nes_scene_param(nes_ctx *ctx, int which, float *host_out, size_t count);

/* Replaces one scene parameter array from host memory (same `which`, count
 * and layout as nes_scene_param), e.g. to render a refitted student's table
 * and weights.  A tensor-core context re-derives its FP16 table, per-cell
 * corner records and MLP weight image.  The occupancy grid is kept: call
 * nes_rebuild_occupancy for the new field.  No counterpart in neserver, whose
 * scene lives in the external renderer. */
int nes_scene_set_param(nes_ctx *ctx, int which, const float *host_in, size_t count);

/* Copies the 128^3 occupancy bitfield (65536 uint32 words, x-fastest). */
int nes_occupancy(nes_ctx *ctx, uint32_t *host_bits);

/* Rebuilds the occupancy grid with a different density threshold
 * (the scene's own threshold is 0.01). */
int nes_rebuild_occupancy(nes_ctx *ctx, float threshold);

/* Number of field evaluations (samples) of the last render call. */
int nes_last_sample_count(nes_ctx *ctx, uint64_t *samples);

/* Self-test of the device-side bounded waits (every spin in the tensor-core
 * kernels gives up after a poll limit and reports NES_ETIMEDOUT instead of
 * hanging; neserver's analogue is the 1 s LockTimeout of its frame queue,
 * src/base/video/frame_queue.cc:14-22).  One CTA allocates tensor memory,
 * waits with the kernels' bounded mbarrier wait for at most poll_limit polls
 * (1..2^24) on a barrier nothing arrives at (arrive = 0) or one it completed
 * itself (arrive = 1), and leaves through the kernels' uniform exit.
 * Returns NES_ETIMEDOUT when the wait ran out, NES_OK when it completed; the
 * context stays usable either way.  Blocks until done. */
int nes_selftest_bounded_wait(nes_ctx *ctx, uint32_t poll_limit, int arrive);

/* Measured ceilings of the tensor-core march's gather stream (the roofline
 * term next to the MLP's tensor-core term; no counterpart in the reference,
 * whose renderer is external).  nes_probe_gather queues `threads` threads (a
 * multiple of 256) that each make loads_per_thread uniformly random loads of
 * load_bytes (4, 16, or 32 read as two 16-byte loads) over table_bytes of
 * device memory (table_bytes / load_bytes a power of two), XOR-folded into
 * sink_dev[thread]; the caller times it on `stream`.
 * nes_probe_gather_replay replays the march's own load stream for the views
 * on a tensor-core context -- the same rays, warp refills, sample positions,
 * record and table addresses, with no interpolation, MLP or compositing --
 * with `threads` (256 or 512) ray slots per SM, and returns its device time
 * (CUDA events) in *replay_ms; sink_dev holds at least (SM count) x threads
 * words.  Both write nothing but the sink. */
int nes_probe_gather(const void *table_dev, uint64_t table_bytes, int load_bytes, uint32_t loads_per_thread,
                     uint32_t threads, uint32_t *sink_dev, void *stream);
int nes_probe_gather_replay(nes_ctx *ctx, const nes_view *views, int nviews, int threads, uint32_t *sink_dev,
                            size_t sink_words, float *replay_ms);

/* Per-kernel timing with CUDA events recorded on the stream the kernels
 * run on (the reference's ScopedTimer averages, src/server.cpp:172-190,
 * in device time).  When enabled, every render records events around ray
 * generation and the march; nes_last_timings waits for the last render and
 * returns both durations in milliseconds. */
int nes_set_profiling(nes_ctx *ctx, int enable);
int nes_last_timings(nes_ctx *ctx, float *raygen_ms, float *march_ms);

#ifdef __cplusplus
}
#endif

#endif /* NES_GB300_H_ */
