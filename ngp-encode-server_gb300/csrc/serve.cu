// serve.cu -- the continuously batched serving loop (nes_server_* in
// include/nes_gb300.h).
//
// neserver serves poses with one synchronous FrameRequest in flight per
// renderer connection (src/server.cpp:116-214) and hands frames on through a
// bounded queue and a reorder map with 1 s lock timeouts
// (src/base/video/frame_queue.cc:11-39, frame_map.cc:12-53).  Here:
//  - nes_submit admits a request (mono or stereo, any resolution) if its
//    device output slots fit the memory budget and the pending queue has
//    room; otherwise it is dropped and counted (no silent stall);
//  - a scheduler thread forms a batch from the pending requests (FIFO, up to
//    max_batch_pixels) whenever one of max_inflight_batches stream slots is
//    free, so requests arriving while others run join the next batch and
//    overlap them on the device;
//  - a batch is one ray queue over all its views: ray generation with
//    compaction, one persistent march, then per view RGB24 quantisation,
//    YUV420P conversion and depth packing into the request's device slots;
//    the whole batch is captured as a CUDA graph and replayed per batch
//    shape (cudaGraphExecUpdate swaps in the new poses and pointers);
//  - a completion thread waits for each batch's event in launch order and
//    publishes its requests with their pose->YUV latency.
#include <cuda_runtime.h>

#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "ctx_internal.h"
#include "kernels.h"
#include "nes_gb300.h"

using namespace nes;
using Clock = std::chrono::steady_clock;

namespace {

constexpr int kMaxSlots = 4;
// The warm-up batch of nes_server_create: one 8x8 view, its RGB24 at byte 0
// of the slot's RGB24 buffer, Y/U/V planes (linesize 32) at 256/512/768 and
// uint16 depth at 1024; the buffer holds at least kWarmupBytes.
constexpr uint32_t kWarmupSide = 8;
constexpr size_t kWarmupBytes = 1024 + kWarmupSide * kWarmupSide * 2;

size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

struct ViewPlanes {
  uint32_t w, h;
  int ls[3];
  size_t off_y, off_u, off_v, off_d, bytes;
};

// Device output layout of one view: Y, U, V (av_image_alloc-style 32-byte
// aligned linesizes, include/base/video/type_managers.h:164) and uint16 depth.
ViewPlanes plan_view(uint32_t w, uint32_t h, size_t base) {
  ViewPlanes p;
  p.w = w;
  p.h = h;
  const uint32_t cw = (w + 1) / 2, ch = (h + 1) / 2;
  p.ls[0] = (int)align_up(w, 32);
  p.ls[1] = p.ls[2] = (int)align_up(cw, 32);
  p.off_y = base;
  p.off_u = align_up(p.off_y + (size_t)p.ls[0] * h, 256);
  p.off_v = align_up(p.off_u + (size_t)p.ls[1] * ch, 256);
  p.off_d = align_up(p.off_v + (size_t)p.ls[2] * ch, 256);
  p.bytes = align_up(p.off_d + (size_t)w * h * 2, 256) - base;
  return p;
}

enum class ReqState { Pending, Running, Done };

struct Req {
  nes_request r{};
  ViewPlanes planes[2];
  size_t bytes = 0;
  uint8_t* dev = nullptr;  // output slots (allocated when the batch forms)
  ReqState state = ReqState::Pending;
  int status = NES_OK;
  Clock::time_point t_submit, t_done;
  double pred_ms = 0.0;  // expected pose -> YUV time at admission (0: no estimate yet)
  uint64_t batch_id = 0;
  uint32_t batch_requests = 0, batch_views = 0;
};

struct Slot {
  cudaStream_t st = nullptr;
  cudaEvent_t done = nullptr;
  DevScratch scratch;
  float* rgb = nullptr;
  float* depth = nullptr;
  uint8_t* rgb8 = nullptr;
  uint32_t* h_counters = nullptr;  // pinned copy of the batch's counters
  bool busy = false;
  uint64_t batch_id = 0;
  std::vector<uint64_t> tickets;
  uint64_t pixels = 0;
  Clock::time_point t_launch;
  std::map<std::string, cudaGraphExec_t> graphs;
};

}  // namespace

struct nes_server {
  nes_ctx* ctx = nullptr;
  nes_server_config cfg{};
  std::vector<Slot> slots;
  cudaStream_t release_stream = nullptr;
  uint64_t fixed_bytes = 0;

  std::mutex mu;
  std::condition_variable cv_sched, cv_done;
  std::unordered_map<uint64_t, Req> reqs;
  std::deque<uint64_t> pending;
  std::deque<int> launch_order;  // slots in launch order (completion order)
  uint64_t next_ticket = 1, next_batch = 1;
  // Admission by expected delay: pixels admitted but not yet batched, pixels
  // of the batches on the GPU, and the measured service rate (pixels per ms,
  // an exponential average over completed batches; 0 until the first).  The
  // model leaves out host work between batches (graph updates, allocation)
  // and batching granularity, so its predictions are scaled by the running
  // ratio of measured to predicted latency of completed requests.
  uint64_t pending_pixels = 0, inflight_pixels = 0;
  double rate_px_per_ms = 0.0, delay_scale = 1.0;
  Clock::time_point last_done;
  // Batch shapes seen so far (scheduler thread only): a shape is launched
  // directly the first time and captured as a graph once it recurs, so
  // one-off mixes of resolutions cost no graph instantiation.
  std::unordered_map<std::string, uint32_t> shape_seen;
  bool stop = false;
  nes_server_stats stats{};
  std::thread sched, comp;
};

namespace {

#define SRV_CUDA(call)                     \
  do {                                     \
    cudaError_t e_ = (call);               \
    if (e_ != cudaSuccess) return NES_EIO; \
  } while (0)

// Queues one batch on the slot's stream (inside or outside stream capture).
int enqueue_batch(nes_server* s, Slot& sl, const ViewBatch& vb, const std::vector<Req*>& reqs) {
  nes_ctx* c = s->ctx;
  SRV_CUDA(enqueue_march(vb, c->scene, sl.scratch, c->cfg.precision, c->num_sms, sl.st));
  int vi = 0;
  for (Req* r : reqs) {
    for (uint32_t k = 0; k < r->r.nviews; ++k, ++vi) {
      const DevView& V = vb.v[vi];
      const ViewPlanes& p = r->planes[k];
      const size_t px = (size_t)p.w * p.h;
      uint8_t* rgb8 = sl.rgb8 + (size_t)(V.rgb - sl.rgb);  // same pixel offset, 1 byte per channel
      SRV_CUDA(launch_rgb_to_rgb24(V.rgb, px * 3, rgb8, sl.st));
      SRV_CUDA(launch_rgb24_to_yuv420p(rgb8, (int)p.w, (int)p.h, (int)p.w * 3, r->dev + p.off_y, r->dev + p.off_u,
                                       r->dev + p.off_v, p.ls, sl.st));
      SRV_CUDA(launch_depth_pack_u16mm(V.depth, px, reinterpret_cast<uint16_t*>(r->dev + p.off_d), sl.st));
    }
  }
  SRV_CUDA(cudaMemcpyAsync(sl.h_counters, sl.scratch.counters, kCtrWords * sizeof(uint32_t), cudaMemcpyDeviceToHost,
                           sl.st));
  return NES_OK;
}

std::string shape_key(const std::vector<Req*>& reqs) {
  std::string k;
  for (Req* r : reqs)
    for (uint32_t v = 0; v < r->r.nviews; ++v)
      k += std::to_string(r->planes[v].w) + "x" + std::to_string(r->planes[v].h) + ";";
  return k;
}

// Launches a batch: plain launches (graphs off, or a shape's first
// occurrence), or capture + instantiate/update + replay.  Runs outside the
// server lock (the scheduler thread is its only caller); graph counters go to
// *inst / *upd.
int launch_batch(nes_server* s, Slot& sl, const ViewBatch& vb, const std::vector<Req*>& reqs, uint64_t* inst,
                 uint64_t* upd) {
  for (Req* r : reqs) SRV_CUDA(cudaMallocAsync(reinterpret_cast<void**>(&r->dev), r->bytes, sl.st));
  const std::string key = shape_key(reqs);
  if (s->shape_seen.size() > 4096) s->shape_seen.clear();  // bounded memory for endless mixes
  const uint32_t seen = ++s->shape_seen[key];
  if (sl.graphs.size() > 256) {  // likewise for the executable graphs of this slot
    for (auto& kv : sl.graphs) cudaGraphExecDestroy(kv.second);
    sl.graphs.clear();
  }
  if (!s->cfg.use_graphs || (seen < 2 && sl.graphs.find(key) == sl.graphs.end())) {
    const int rc = enqueue_batch(s, sl, vb, reqs);
    if (rc != NES_OK) return rc;
  } else {
    SRV_CUDA(cudaStreamBeginCapture(sl.st, cudaStreamCaptureModeThreadLocal));
    const int rc = enqueue_batch(s, sl, vb, reqs);
    cudaGraph_t g = nullptr;
    const cudaError_t ec = cudaStreamEndCapture(sl.st, &g);
    if (rc != NES_OK || ec != cudaSuccess) {
      if (g) cudaGraphDestroy(g);
      return rc != NES_OK ? rc : NES_EIO;
    }
    auto it = sl.graphs.find(key);
    bool ok = false;
    if (it != sl.graphs.end()) {
      cudaGraphExecUpdateResultInfo info;
      if (cudaGraphExecUpdate(it->second, g, &info) == cudaSuccess) {
        ok = true;
        ++*upd;
      } else {
        cudaGetLastError();
        cudaGraphExecDestroy(it->second);
        sl.graphs.erase(it);
      }
    }
    if (!ok) {
      cudaGraphExec_t ex = nullptr;
      if (cudaGraphInstantiate(&ex, g, 0) != cudaSuccess) {
        cudaGraphDestroy(g);
        return NES_EIO;
      }
      sl.graphs[key] = ex;
      ++*inst;
    }
    const cudaError_t el = cudaGraphLaunch(sl.graphs[key], sl.st);
    cudaGraphDestroy(g);
    if (el != cudaSuccess) return NES_EIO;
  }
  SRV_CUDA(cudaEventRecord(sl.done, sl.st));
  return NES_OK;
}

void scheduler_main(nes_server* s) {
  cudaSetDevice(s->ctx->cfg.device);
  std::unique_lock<std::mutex> lk(s->mu);
  for (;;) {
    int free_slot = -1;
    s->cv_sched.wait(lk, [&] {
      if (s->stop) return true;
      if (s->pending.empty()) return false;
      for (size_t i = 0; i < s->slots.size(); ++i)
        if (!s->slots[i].busy) {
          free_slot = (int)i;
          return true;
        }
      return false;
    });
    if (s->stop) return;
    Slot& sl = s->slots[free_slot];
    // FIFO batch formation up to the pixel and view limits.
    std::vector<Req*> batch;
    std::vector<uint64_t> tickets;
    std::vector<nes_view> views;
    std::vector<float*> rgbp, depp;
    uint64_t pixels = 0;
    while (!s->pending.empty()) {
      Req& r = s->reqs[s->pending.front()];
      uint64_t px = 0;
      for (uint32_t v = 0; v < r.r.nviews; ++v) px += (uint64_t)r.planes[v].w * r.planes[v].h;
      if (!batch.empty() && (pixels + px > s->cfg.max_batch_pixels || views.size() + r.r.nviews > (size_t)kMaxViews))
        break;
      for (uint32_t v = 0; v < r.r.nviews; ++v) {
        views.push_back(r.r.views[v]);
        rgbp.push_back(sl.rgb + 3 * (pixels));
        depp.push_back(sl.depth + pixels);
        pixels += (uint64_t)r.planes[v].w * r.planes[v].h;
      }
      tickets.push_back(s->pending.front());
      batch.push_back(&r);
      s->pending.pop_front();
      s->pending_pixels -= px;
    }
    s->inflight_pixels += pixels;
    const uint64_t bid = s->next_batch++;
    for (Req* r : batch) {
      r->state = ReqState::Running;
      r->batch_id = bid;
      r->batch_requests = (uint32_t)batch.size();
      r->batch_views = (uint32_t)views.size();
    }
    sl.busy = true;
    sl.batch_id = bid;
    sl.tickets = tickets;
    sl.pixels = pixels;
    sl.t_launch = Clock::now();
    lk.unlock();

    ViewBatch vb;
    uint64_t npx = 0;
    int rc = fill_view_batch(views.data(), (int)views.size(), rgbp.data(), depp.data(), s->cfg.max_batch_pixels, &vb,
                             &npx);
    uint64_t inst = 0, upd = 0;
    if (rc == NES_OK) rc = launch_batch(s, sl, vb, batch, &inst, &upd);

    lk.lock();
    s->stats.batches++;
    s->stats.graph_instantiations += inst;
    s->stats.graph_updates += upd;
    if (rc != NES_OK) {  // publish the failure; nothing is in flight on this slot
      s->inflight_pixels -= sl.pixels;
      for (uint64_t t : tickets) {
        Req& r = s->reqs[t];
        r.state = ReqState::Done;
        r.status = rc;
        r.t_done = Clock::now();
      }
      sl.busy = false;
      sl.tickets.clear();
      s->cv_done.notify_all();
      continue;
    }
    s->launch_order.push_back(free_slot);
    s->cv_done.notify_all();  // wakes the completion thread
  }
}

void completion_main(nes_server* s) {
  cudaSetDevice(s->ctx->cfg.device);
  std::unique_lock<std::mutex> lk(s->mu);
  for (;;) {
    s->cv_done.wait(lk, [&] { return s->stop || !s->launch_order.empty(); });
    if (s->launch_order.empty() && s->stop) return;
    const int si = s->launch_order.front();
    Slot& sl = s->slots[si];
    lk.unlock();
    const cudaError_t e = cudaEventSynchronize(sl.done);
    const Clock::time_point now = Clock::now();
    lk.lock();
    s->launch_order.pop_front();
    int status = e == cudaSuccess ? NES_OK : NES_EIO;
    if (status == NES_OK && sl.h_counters[kCtrError]) status = NES_ETIMEDOUT;
    s->stats.samples += (uint64_t)sl.h_counters[kCtrSamples] | ((uint64_t)sl.h_counters[kCtrSamples + 1] << 32);
    s->stats.pixels += sl.pixels;
    s->inflight_pixels -= sl.pixels;
    {  // this batch's service time: from its launch, or from the previous
       // completion if the GPU was still busy with that one
      const Clock::time_point from = sl.t_launch > s->last_done ? sl.t_launch : s->last_done;
      const double ms = std::chrono::duration<double, std::milli>(now - from).count();
      if (status == NES_OK && ms > 0.0 && sl.pixels) {
        const double r = (double)sl.pixels / ms;
        s->rate_px_per_ms = s->rate_px_per_ms > 0.0 ? 0.8 * s->rate_px_per_ms + 0.2 * r : r;
      }
      s->last_done = now;
    }
    for (uint64_t t : sl.tickets) {
      Req& r = s->reqs[t];
      r.state = ReqState::Done;
      r.status = status;
      r.t_done = now;
      s->stats.completed++;
      if (status == NES_OK && r.pred_ms > 0.0) {
        const double ratio = std::chrono::duration<double, std::milli>(now - r.t_submit).count() / r.pred_ms;
        const double sc = 0.9 * s->delay_scale + 0.1 * ratio;
        s->delay_scale = sc < 0.5 ? 0.5 : (sc > 50.0 ? 50.0 : sc);
      }
    }
    sl.tickets.clear();
    sl.busy = false;
    s->cv_done.notify_all();
    s->cv_sched.notify_all();
  }
}

void destroy_slots(nes_server* s) {
  for (Slot& sl : s->slots) {
    if (sl.st) cudaStreamSynchronize(sl.st);
    for (auto& kv : sl.graphs) cudaGraphExecDestroy(kv.second);
    cudaFree(sl.scratch.ray_dt);
    cudaFree(sl.scratch.ray_meta);
    cudaFree(sl.scratch.counters);
    cudaFree(sl.rgb);
    cudaFree(sl.depth);
    cudaFree(sl.rgb8);
    if (sl.h_counters) cudaFreeHost(sl.h_counters);
    if (sl.done) cudaEventDestroy(sl.done);
    if (sl.st) cudaStreamDestroy(sl.st);
  }
  s->slots.clear();
}

}  // namespace

extern "C" {

void nes_server_config_default(nes_server_config* cfg) {
  std::memset(cfg, 0, sizeof(*cfg));
  cfg->hbm_budget_bytes = 8ull << 30;
  cfg->max_batch_pixels = 2u * 1920u * 1832u;
  cfg->max_inflight_batches = 2;
  cfg->max_pending = 256;
  cfg->use_graphs = 1;
  cfg->max_queue_ms = 0.0f;
}

int nes_server_create(nes_ctx* ctx, const nes_server_config* cfg, nes_server** out) {
  if (!ctx || !cfg || !out) return NES_EINVAL;
  *out = nullptr;
  if (cfg->max_inflight_batches < 1 || cfg->max_inflight_batches > kMaxSlots) return NES_EINVAL;
  if (cfg->max_batch_pixels < kWarmupSide * kWarmupSide || cfg->max_batch_pixels > (1u << 27) ||
      cfg->max_pending == 0)
    return NES_EINVAL;
  if (!(cfg->max_queue_ms >= 0.0f && cfg->max_queue_ms < 1e9f)) return NES_EINVAL;
  if (cudaSetDevice(ctx->cfg.device) != cudaSuccess) return NES_ENODEV;
  nes_server* s = new (std::nothrow) nes_server;
  if (!s) return NES_ENOMEM;
  s->ctx = ctx;
  s->cfg = *cfg;
  const size_t P = cfg->max_batch_pixels;
  // Per slot: 32 B ray record + 16 B FP32 colour/depth + 3 B RGB24 per pixel.
  s->fixed_bytes = (uint64_t)cfg->max_inflight_batches * (P * (32 + 16 + 3) + 4096);
  if (s->fixed_bytes > cfg->hbm_budget_bytes) {
    delete s;
    return NES_ENOMEM;
  }
  s->stats.budget_used_bytes = s->fixed_bytes;
  s->slots.resize(cfg->max_inflight_batches);
  auto fail = [&](int code) {
    destroy_slots(s);
    if (s->release_stream) cudaStreamDestroy(s->release_stream);
    delete s;
    return code;
  };
  for (Slot& sl : s->slots) {
    if (cudaStreamCreateWithFlags(&sl.st, cudaStreamNonBlocking) != cudaSuccess) return fail(NES_EIO);
    if (cudaEventCreateWithFlags(&sl.done, cudaEventDisableTiming | cudaEventBlockingSync) != cudaSuccess)
      return fail(NES_EIO);
    if (cudaMalloc(&sl.scratch.ray_dt, P * sizeof(float4)) != cudaSuccess) return fail(NES_ENOMEM);
    if (cudaMalloc(&sl.scratch.ray_meta, P * sizeof(RayMeta)) != cudaSuccess) return fail(NES_ENOMEM);
    if (cudaMalloc(&sl.scratch.counters, kCtrWords * sizeof(uint32_t)) != cudaSuccess) return fail(NES_ENOMEM);
    sl.scratch.max_rays = (uint32_t)P;
    if (cudaMalloc(&sl.rgb, P * 3 * sizeof(float)) != cudaSuccess) return fail(NES_ENOMEM);
    if (cudaMalloc(&sl.depth, P * sizeof(float)) != cudaSuccess) return fail(NES_ENOMEM);
    if (cudaMalloc(&sl.rgb8, P * 3 > kWarmupBytes ? P * 3 : kWarmupBytes) != cudaSuccess) return fail(NES_ENOMEM);
    if (cudaMallocHost(&sl.h_counters, kCtrWords * sizeof(uint32_t)) != cudaSuccess) return fail(NES_ENOMEM);
  }
  if (cudaStreamCreateWithFlags(&s->release_stream, cudaStreamNonBlocking) != cudaSuccess) return fail(NES_EIO);
  // Keep freed output slots in the pool for reuse instead of returning them.
  cudaMemPool_t pool;
  if (cudaDeviceGetDefaultMemPool(&pool, ctx->cfg.device) == cudaSuccess) {
    uint64_t thr = cfg->hbm_budget_bytes;
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
  }
  // Warm-up batch outside capture so every kernel's module is loaded and its
  // attributes set before the first capture.
  {
    nes_view v;
    std::memset(&v, 0, sizeof(v));
    const float M[12] = {1, 0, 0, 0.5f, 0, -1, 0, 0.5f, 0, 0, -1, 0.5f};
    std::memcpy(v.matrix, M, sizeof(M));
    v.width = v.height = kWarmupSide;
    v.focal_px = 0.5f * kWarmupSide;
    for (Slot& sl : s->slots) {
      ViewBatch vb;
      uint64_t px = 0;
      float* rgb[1] = {sl.rgb};
      float* dep[1] = {sl.depth};
      if (fill_view_batch(&v, 1, rgb, dep, P, &vb, &px) != NES_OK) return fail(NES_EIO);
      if (enqueue_march(vb, ctx->scene, sl.scratch, ctx->cfg.precision, ctx->num_sms, sl.st) != cudaSuccess)
        return fail(NES_EIO);
      const int ls[3] = {32, 32, 32};
      const size_t wpx = kWarmupSide * kWarmupSide;
      if (launch_rgb_to_rgb24(sl.rgb, wpx * 3, sl.rgb8, sl.st) != cudaSuccess ||
          launch_rgb24_to_yuv420p(sl.rgb8, kWarmupSide, kWarmupSide, 3 * kWarmupSide, sl.rgb8 + 256, sl.rgb8 + 512,
                                  sl.rgb8 + 768, ls, sl.st) != cudaSuccess ||
          launch_depth_pack_u16mm(sl.depth, wpx, reinterpret_cast<uint16_t*>(sl.rgb8 + 1024), sl.st) != cudaSuccess)
        return fail(NES_EIO);
      if (cudaStreamSynchronize(sl.st) != cudaSuccess) return fail(NES_EIO);
    }
  }
  s->sched = std::thread(scheduler_main, s);
  s->comp = std::thread(completion_main, s);
  *out = s;
  return NES_OK;
}

void nes_server_destroy(nes_server* s) {
  if (!s) return;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
  }
  s->cv_sched.notify_all();
  s->cv_done.notify_all();
  if (s->sched.joinable()) s->sched.join();
  if (s->comp.joinable()) s->comp.join();
  cudaSetDevice(s->ctx->cfg.device);
  // A batch launched while the stop was being set may still run (the
  // completion thread can have left first): its outputs are freed after it.
  for (Slot& sl : s->slots)
    if (sl.st) cudaStreamSynchronize(sl.st);
  for (auto& kv : s->reqs)
    if (kv.second.dev) cudaFreeAsync(kv.second.dev, s->release_stream);
  cudaStreamSynchronize(s->release_stream);
  destroy_slots(s);
  cudaStreamDestroy(s->release_stream);
  delete s;
}

int nes_submit(nes_server* s, const nes_request* req, uint64_t* ticket) {
  if (!s || !req || !ticket || req->nviews < 1 || req->nviews > 2) return NES_EINVAL;
  Req r;
  r.r = *req;
  uint64_t px = 0;
  for (uint32_t v = 0; v < req->nviews; ++v) {
    const nes_view& w = req->views[v];
    // Checked here, not at batch formation, so that a bad view cannot fail
    // the other requests of its batch.
    if (!view_ok(w)) return NES_EINVAL;
    if (req->nviews == 2 && (w.width != req->views[0].width || w.height != req->views[0].height)) return NES_EINVAL;
    r.planes[v] = plan_view(w.width, w.height, r.bytes);
    r.bytes += r.planes[v].bytes;
    px += (uint64_t)w.width * w.height;
  }
  if (px > s->cfg.max_batch_pixels) return NES_EINVAL;
  std::lock_guard<std::mutex> lk(s->mu);
  if (s->stop) return NES_EINVAL;
  const double pred = s->rate_px_per_ms > 0.0
                          ? (double)(s->pending_pixels + s->inflight_pixels + px) / s->rate_px_per_ms
                          : 0.0;
  // Before the first batch has completed there is no rate: keep at most one
  // batch's worth of pixels in the system.
  const bool late = s->cfg.max_queue_ms > 0.0f &&
                    (s->rate_px_per_ms > 0.0 ? pred * s->delay_scale > s->cfg.max_queue_ms
                                             : s->pending_pixels + s->inflight_pixels + px > s->cfg.max_batch_pixels);
  if (s->pending.size() >= s->cfg.max_pending || late ||
      s->stats.budget_used_bytes + r.bytes > s->cfg.hbm_budget_bytes) {
    s->stats.rejected++;
    return NES_EAGAIN;
  }
  s->pending_pixels += px;
  s->stats.submitted++;
  s->stats.budget_used_bytes += r.bytes;
  r.t_submit = Clock::now();
  r.pred_ms = pred;
  const uint64_t t = s->next_ticket++;
  s->reqs.emplace(t, r);
  s->pending.push_back(t);
  *ticket = t;
  s->cv_sched.notify_one();
  return NES_OK;
}

int nes_wait(nes_server* s, uint64_t ticket, int64_t timeout_ns, nes_result* out) {
  if (!s || !out) return NES_EINVAL;
  std::unique_lock<std::mutex> lk(s->mu);
  auto it = s->reqs.find(ticket);
  if (it == s->reqs.end()) return NES_EINVAL;
  // Looked up afresh on each wake-up: another thread may release the ticket
  // between its completion and this thread's return to the lock.
  auto done = [&] {
    it = s->reqs.find(ticket);
    return it == s->reqs.end() || it->second.state == ReqState::Done;
  };
  // Beyond ~11.6 days a timeout counts as none (now + timeout would
  // overflow the steady clock).
  if (timeout_ns < 0 || timeout_ns > 1000000000000000ll)
    s->cv_done.wait(lk, done);
  else if (!s->cv_done.wait_for(lk, std::chrono::nanoseconds(timeout_ns), done))
    return NES_ETIMEDOUT;
  if (it == s->reqs.end()) return NES_EINVAL;
  const Req& r = it->second;
  std::memset(out, 0, sizeof(*out));
  out->ticket = ticket;
  out->status = r.status;
  out->nviews = r.r.nviews;
  out->width = r.planes[0].w;
  out->height = r.planes[0].h;
  for (int k = 0; k < 3; ++k) out->linesize[k] = r.planes[0].ls[k];
  for (uint32_t v = 0; v < r.r.nviews && r.dev; ++v) {
    out->y_dev[v] = r.dev + r.planes[v].off_y;
    out->u_dev[v] = r.dev + r.planes[v].off_u;
    out->v_dev[v] = r.dev + r.planes[v].off_v;
    out->depth_mm_dev[v] = reinterpret_cast<uint16_t*>(r.dev + r.planes[v].off_d);
  }
  out->latency_ms = std::chrono::duration<double, std::milli>(r.t_done - r.t_submit).count();
  out->batch_id = r.batch_id;
  out->batch_requests = r.batch_requests;
  out->batch_views = r.batch_views;
  return NES_OK;
}

int nes_release(nes_server* s, uint64_t ticket) {
  if (!s) return NES_EINVAL;
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->reqs.find(ticket);
  if (it == s->reqs.end() || it->second.state != ReqState::Done) return NES_EINVAL;
  if (it->second.dev) {
    cudaSetDevice(s->ctx->cfg.device);
    if (cudaFreeAsync(it->second.dev, s->release_stream) != cudaSuccess) return NES_EIO;
  }
  s->stats.budget_used_bytes -= it->second.bytes;
  s->reqs.erase(it);
  s->cv_sched.notify_one();
  return NES_OK;
}

int nes_server_stats_get(nes_server* s, nes_server_stats* out) {
  if (!s || !out) return NES_EINVAL;
  std::lock_guard<std::mutex> lk(s->mu);
  *out = s->stats;
  return NES_OK;
}

int nes_copy_to_host(void* host_dst, const void* dev_src, size_t n) {
  if ((!host_dst || !dev_src) && n) return NES_EINVAL;
  if (n == 0) return NES_OK;
  return cudaMemcpy(host_dst, dev_src, n, cudaMemcpyDeviceToHost) == cudaSuccess ? NES_OK : NES_EIO;
}

}  // extern "C"
