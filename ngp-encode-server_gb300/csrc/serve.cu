// serve.cu -- the continuously batched serving loop (nes_server_* in
// include/nes_gb300.h).
//
// neserver serves poses with one synchronous FrameRequest in flight per
// renderer connection (src/server.cpp:116-214) and hands frames on through a
// bounded queue and a reorder map with 1 s lock timeouts
// (src/base/video/frame_queue.cc:11-39, frame_map.cc:12-53).  Here:
//  - nes_submit admits a request (mono or stereo, any resolution) if its
//    device output slots fit the memory budget and the pending queue has
//    room, carving them out of an output arena allocated once at creation;
//    otherwise it is dropped and counted (no silent stall, and no device
//    allocation on the request path);
//  - a scheduler thread forms a batch from the pending requests (FIFO, up to
//    max_batch_pixels) whenever one of max_inflight_batches stream slots is
//    free, so requests arriving while others run join the next batch and
//    overlap them on the device;
//  - a batch is one ray queue over all its views: ray generation with
//    compaction, one persistent march, then one fused launch for every
//    view's RGB24 quantisation, YUV420P conversion and depth packing into the
//    request's output slots;
//  - every kernel reads the batch from a device-side descriptor (views,
//    poses, output pointers) that the first node copies from the slot's
//    pinned host copy, and every grid is fixed by max_batch_pixels, so each
//    slot's CUDA graph is captured and instantiated once at creation and
//    replayed for every batch of any shape;
//  - a completion thread waits for each batch's event in launch order and
//    publishes its requests with their pose->YUV latency.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
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
  uint8_t* dev = nullptr;  // output slots, carved from the arena at admission
  size_t arena_off = 0;
  ReqState state = ReqState::Pending;
  int status = NES_OK;
  Clock::time_point t_submit, t_done;
  double pred_ms = 0.0;  // expected pose -> YUV time at admission (0: no estimate yet)
  double work = 0.0;     // expected cost (samples + pixels), see estimate_work
  uint64_t batch_id = 0;
  uint32_t batch_requests = 0, batch_views = 0;
};

// The batch descriptor every kernel of a slot reads at run time.
struct BatchDesc {
  ViewBatch vb;
  FrameBatch fb;
};

struct Slot {
  cudaStream_t st = nullptr;
  cudaEvent_t done = nullptr;
  DevScratch scratch;
  float* rgb = nullptr;
  float* depth = nullptr;
  uint8_t* warm = nullptr;         // outputs of the creation-time warm-up batch
  uint32_t* h_counters = nullptr;  // pinned copy of the batch's counters
  BatchDesc* h_desc = nullptr;     // pinned: written by the host per batch
  BatchDesc* d_desc = nullptr;     // device: copied from h_desc by the batch's first node
  cudaGraphExec_t graph = nullptr; // the slot's batch, instantiated once
  bool busy = false;
  uint64_t batch_id = 0;
  std::vector<uint64_t> tickets;
  uint64_t pixels = 0;
  double work = 0.0;
  Clock::time_point t_launch;
};

// Expected cost of a view in samples: the mean march length (chord through
// the unit cube / dt, at most the step limit) of a 16 x 16 grid of its rays,
// times its pixels, plus one per pixel for its ray generation and frame
// output.  Costs differ by more than 2x between poses of the serving mix
// (near poses fill the frame with long chords), so the delay bound
// predicts with this rather than with pixel counts.
double estimate_work(const nes_view& v) {
  constexpr int kGrid = 16;
  const float* M = v.matrix;
  double steps = 0.0;
  for (int gy = 0; gy < kGrid; ++gy) {
    for (int gx = 0; gx < kGrid; ++gx) {
      const double px = ((double)gx + 0.5) * v.width / kGrid, py = ((double)gy + 0.5) * v.height / kGrid;
      const double u = (px - 0.5 * v.width) / v.focal_px, w = (py - 0.5 * v.height) / v.focal_px;
      double d[3], nrm = 0.0;
      for (int a = 0; a < 3; ++a) {
        d[a] = M[a * 4 + 0] * u + M[a * 4 + 1] * w + M[a * 4 + 2];
        nrm += d[a] * d[a];
      }
      nrm = std::sqrt(nrm);
      double tn = -1e30, tf = 1e30;
      for (int a = 0; a < 3; ++a) {
        const double da = d[a] / nrm, oa = M[a * 4 + 3];
        if (std::fabs(da) < 1e-12) {  // parallel to this slab: inside it or a miss
          if (oa < 0.0 || oa > 1.0) tf = -1e30;
          continue;
        }
        const double t0 = (0.0 - oa) / da, t1 = (1.0 - oa) / da;
        tn = std::max(tn, std::min(t0, t1));
        tf = std::min(tf, std::max(t0, t1));
      }
      const double ts = std::max(tn, 0.0);
      if (nrm > 0.0 && tf > ts) steps += std::min((double)kMaxSteps, std::floor((tf - ts) / (double)kDt));
    }
  }
  return ((double)v.width * v.height) * (steps / (kGrid * kGrid) + 1.0);
}

// First-fit free list over one device allocation: request outputs are
// carved out at admission and handed back at release, so serving never
// calls the CUDA allocator after creation.  Offsets and sizes are multiples
// of 256 bytes; neighbouring free ranges are merged.
class Arena {
 public:
  static constexpr size_t kNone = ~size_t(0);
  void reset(size_t bytes) {
    free_.clear();
    if (bytes) free_[0] = bytes;
  }
  size_t alloc(size_t bytes) {
    for (auto it = free_.begin(); it != free_.end(); ++it) {
      if (it->second < bytes) continue;
      const size_t off = it->first, rest = it->second - bytes;
      free_.erase(it);
      if (rest) free_[off + bytes] = rest;
      return off;
    }
    return kNone;
  }
  void release(size_t off, size_t bytes) {
    auto next = free_.lower_bound(off);
    if (next != free_.end() && off + bytes == next->first) {
      bytes += next->second;
      next = free_.erase(next);
    }
    if (next != free_.begin()) {
      auto prev = std::prev(next);
      if (prev->first + prev->second == off) {
        prev->second += bytes;
        return;
      }
    }
    free_[off] = bytes;
  }

 private:
  std::map<size_t, size_t> free_;  // offset -> size
};

}  // namespace

struct nes_server {
  nes_ctx* ctx = nullptr;
  nes_server_config cfg{};
  std::vector<Slot> slots;
  uint64_t fixed_bytes = 0;
  uint8_t* arena_base = nullptr;  // device memory of the output arena
  Arena arena;                    // guarded by mu

  std::mutex mu;
  std::condition_variable cv_sched, cv_done;
  std::unordered_map<uint64_t, Req> reqs;
  std::deque<uint64_t> pending;
  std::deque<int> launch_order;  // slots in launch order (completion order)
  uint64_t next_ticket = 1, next_batch = 1;
  // Admission by expected delay: the expected cost (estimate_work) of the
  // requests admitted but not yet batched and of the batches on the GPU, and
  // the measured service rate (cost per ms, an exponential average over
  // completed batches; 0 until the first).  The model leaves out batching
  // granularity and host work between batches, so its predictions are
  // scaled by the running ratio of measured to predicted latency of
  // completed requests.  Pixel counts still bound the first batch.
  uint64_t pending_pixels = 0, inflight_pixels = 0;
  double pending_work = 0.0, inflight_work = 0.0;
  double rate_work_per_ms = 0.0, delay_scale = 1.0;
  Clock::time_point last_done;
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

// Queues one batch on the slot's stream, inside or outside stream capture.
// Nothing here depends on the batch: the kernels read it from d_desc.
int enqueue_batch(nes_server* s, Slot& sl) {
  nes_ctx* c = s->ctx;
  const uint32_t P = s->cfg.max_batch_pixels;
  SRV_CUDA(cudaMemcpyAsync(sl.d_desc, sl.h_desc, sizeof(BatchDesc), cudaMemcpyHostToDevice, sl.st));
  SRV_CUDA(cudaMemsetAsync(sl.scratch.counters, 0, kCtrWords * sizeof(uint32_t), sl.st));
  SRV_CUDA(launch_raygen(&sl.d_desc->vb, P, c->num_sms, sl.scratch, sl.st));
  if (c->cfg.precision == NES_PREC_FP16_TC)
    SRV_CUDA(launch_march_tc(&sl.d_desc->vb, c->scene, sl.scratch, c->num_sms, sl.st));
  else
    SRV_CUDA(launch_march_fp32(&sl.d_desc->vb, c->scene, sl.scratch, c->num_sms, sl.st));
  SRV_CUDA(launch_frame_out(&sl.d_desc->fb, c->num_sms, sl.st));
  SRV_CUDA(cudaMemcpyAsync(sl.h_counters, sl.scratch.counters, kCtrWords * sizeof(uint32_t), cudaMemcpyDeviceToHost,
                           sl.st));
  return NES_OK;
}

// Fills the slot's pinned descriptor for a batch of views whose FP32 render
// goes to the slot's buffers and whose frames go to the given planes.
int fill_desc(nes_server* s, Slot& sl, const nes_view* views, const ViewPlanes* planes, uint8_t* const* out_base,
              int n) {
  float* rgbp[kMaxViews];
  float* depp[kMaxViews];
  uint64_t px = 0;
  for (int i = 0; i < n; ++i) {
    rgbp[i] = sl.rgb + 3 * px;
    depp[i] = sl.depth + px;
    px += (uint64_t)planes[i].w * planes[i].h;
  }
  uint64_t npx = 0;
  const int rc = fill_view_batch(views, n, rgbp, depp, s->cfg.max_batch_pixels, &sl.h_desc->vb, &npx);
  if (rc != NES_OK) return rc;
  FrameBatch& fb = sl.h_desc->fb;
  std::memset(&fb, 0, sizeof(fb));
  fb.n = n;
  for (int i = 0; i < n; ++i) {
    const ViewPlanes& p = planes[i];
    FrameOut& F = fb.f[i];
    F.rgb = rgbp[i];
    F.depth = depp[i];
    F.y = out_base[i] + p.off_y;
    F.u = out_base[i] + p.off_u;
    F.v = out_base[i] + p.off_v;
    F.depth_mm = reinterpret_cast<uint16_t*>(out_base[i] + p.off_d);
    F.w = (int)p.w;
    F.h = (int)p.h;
    F.ls0 = p.ls[0];
    F.ls1 = p.ls[1];
    F.ls2 = p.ls[2];
  }
  frame_batch_index(&fb);
  return NES_OK;
}

// Launches the batch whose descriptor is in sl.h_desc: the slot's graph, or
// the same launches one by one when graphs are off.
int launch_batch(nes_server* s, Slot& sl) {
  if (sl.graph) {
    SRV_CUDA(cudaGraphLaunch(sl.graph, sl.st));
  } else {
    const int rc = enqueue_batch(s, sl);
    if (rc != NES_OK) return rc;
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
    nes_view views[kMaxViews];
    ViewPlanes planes[kMaxViews];
    uint8_t* outs[kMaxViews];
    int nv = 0;
    uint64_t pixels = 0;
    double work = 0.0;
    while (!s->pending.empty()) {
      Req& r = s->reqs[s->pending.front()];
      uint64_t px = 0;
      for (uint32_t v = 0; v < r.r.nviews; ++v) px += (uint64_t)r.planes[v].w * r.planes[v].h;
      if (!batch.empty() && (pixels + px > s->cfg.max_batch_pixels || nv + (int)r.r.nviews > kMaxViews)) break;
      for (uint32_t v = 0; v < r.r.nviews; ++v, ++nv) {
        views[nv] = r.r.views[v];
        planes[nv] = r.planes[v];
        outs[nv] = r.dev;
      }
      pixels += px;
      work += r.work;
      tickets.push_back(s->pending.front());
      batch.push_back(&r);
      s->pending.pop_front();
      s->pending_pixels -= px;
      s->pending_work -= r.work;
    }
    s->inflight_pixels += pixels;
    s->inflight_work += work;
    const uint64_t bid = s->next_batch++;
    for (Req* r : batch) {
      r->state = ReqState::Running;
      r->batch_id = bid;
      r->batch_requests = (uint32_t)batch.size();
      r->batch_views = (uint32_t)nv;
    }
    sl.busy = true;
    sl.batch_id = bid;
    sl.tickets = tickets;
    sl.pixels = pixels;
    sl.work = work;
    sl.t_launch = Clock::now();
    lk.unlock();

    // The slot is idle (its last batch completed), so its pinned descriptor
    // can be rewritten.
    int rc = fill_desc(s, sl, views, planes, outs, nv);
    if (rc == NES_OK) rc = launch_batch(s, sl);
    // A failed launch may have queued part of the batch: let that finish
    // before the requests (and their output slots) are handed back.
    if (rc != NES_OK) cudaStreamSynchronize(sl.st);

    lk.lock();
    s->stats.batches++;
    if (rc != NES_OK) {  // publish the failure; the slot's stream is idle
      s->inflight_pixels -= sl.pixels;
      s->inflight_work -= sl.work;
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
    s->inflight_work -= sl.work;
    {  // this batch's service time: from its launch, or from the previous
       // completion if the GPU was still busy with that one
      const Clock::time_point from = sl.t_launch > s->last_done ? sl.t_launch : s->last_done;
      const double ms = std::chrono::duration<double, std::milli>(now - from).count();
      if (status == NES_OK && ms > 0.0 && sl.work > 0.0) {
        const double r = sl.work / ms;
        s->rate_work_per_ms = s->rate_work_per_ms > 0.0 ? 0.8 * s->rate_work_per_ms + 0.2 * r : r;
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
    if (sl.graph) cudaGraphExecDestroy(sl.graph);
    cudaFree(sl.scratch.ray_dt);
    cudaFree(sl.scratch.ray_meta);
    cudaFree(sl.scratch.counters);
    cudaFree(sl.rgb);
    cudaFree(sl.depth);
    cudaFree(sl.warm);
    cudaFree(sl.d_desc);
    if (sl.h_desc) cudaFreeHost(sl.h_desc);
    if (sl.h_counters) cudaFreeHost(sl.h_counters);
    if (sl.done) cudaEventDestroy(sl.done);
    if (sl.st) cudaStreamDestroy(sl.st);
  }
  s->slots.clear();
  cudaFree(s->arena_base);
  s->arena_base = nullptr;
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
  // Per slot: 32 B ray record + 16 B FP32 colour/depth per pixel, the
  // descriptor and the warm-up outputs.
  s->fixed_bytes = (uint64_t)cfg->max_inflight_batches * (P * (32 + 16) + sizeof(BatchDesc) + kWarmupBytes + 4096);
  if (s->fixed_bytes > cfg->hbm_budget_bytes) {
    delete s;
    return NES_ENOMEM;
  }
  s->stats.budget_used_bytes = s->fixed_bytes;
  s->slots.resize(cfg->max_inflight_batches);
  auto fail = [&](int code) {
    destroy_slots(s);
    delete s;
    return code;
  };
  // The output arena: the rest of the budget, reserved up front.
  const size_t arena_bytes = (size_t)(cfg->hbm_budget_bytes - s->fixed_bytes) / 256 * 256;
  if (arena_bytes && cudaMalloc(&s->arena_base, arena_bytes) != cudaSuccess) return fail(NES_ENOMEM);
  s->arena.reset(arena_bytes);
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
    if (cudaMalloc(&sl.warm, kWarmupBytes) != cudaSuccess) return fail(NES_ENOMEM);
    if (cudaMalloc(&sl.d_desc, sizeof(BatchDesc)) != cudaSuccess) return fail(NES_ENOMEM);
    if (cudaMallocHost(&sl.h_desc, sizeof(BatchDesc)) != cudaSuccess) return fail(NES_ENOMEM);
    if (cudaMallocHost(&sl.h_counters, kCtrWords * sizeof(uint32_t)) != cudaSuccess) return fail(NES_ENOMEM);
  }
  // Per slot: one warm-up batch of plain launches (loads every kernel's
  // module and sets its attributes outside capture), then the capture and
  // the one instantiation of the slot's graph.
  {
    nes_view v;
    std::memset(&v, 0, sizeof(v));
    const float M[12] = {1, 0, 0, 0.5f, 0, -1, 0, 0.5f, 0, 0, -1, 0.5f};
    std::memcpy(v.matrix, M, sizeof(M));
    v.width = v.height = kWarmupSide;
    v.focal_px = 0.5f * kWarmupSide;
    for (Slot& sl : s->slots) {
      ViewPlanes p = plan_view(kWarmupSide, kWarmupSide, 0);
      uint8_t* base[1] = {sl.warm};
      if (p.bytes > kWarmupBytes) return fail(NES_EIO);
      if (fill_desc(s, sl, &v, &p, base, 1) != NES_OK) return fail(NES_EIO);
      if (enqueue_batch(s, sl) != NES_OK) return fail(NES_EIO);
      if (cudaStreamSynchronize(sl.st) != cudaSuccess) return fail(NES_EIO);
      if (cfg->use_graphs) {
        if (cudaStreamBeginCapture(sl.st, cudaStreamCaptureModeThreadLocal) != cudaSuccess) return fail(NES_EIO);
        const int rc = enqueue_batch(s, sl);
        cudaGraph_t g = nullptr;
        const cudaError_t ec = cudaStreamEndCapture(sl.st, &g);
        if (rc != NES_OK || ec != cudaSuccess) {
          if (g) cudaGraphDestroy(g);
          return fail(NES_EIO);
        }
        const cudaError_t ei = cudaGraphInstantiate(&sl.graph, g, 0);
        cudaGraphDestroy(g);
        if (ei != cudaSuccess) {
          sl.graph = nullptr;
          return fail(NES_EIO);
        }
        s->stats.graph_instantiations++;
      }
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
    // Requests never batched finish now with an error, so no waiter sleeps
    // on a request that will not run.
    for (uint64_t t : s->pending) {
      Req& r = s->reqs[t];
      r.state = ReqState::Done;
      r.status = NES_EIO;
      r.t_done = Clock::now();
    }
    s->pending.clear();
  }
  s->cv_sched.notify_all();
  s->cv_done.notify_all();
  if (s->sched.joinable()) s->sched.join();
  if (s->comp.joinable()) s->comp.join();
  cudaSetDevice(s->ctx->cfg.device);
  // A batch launched while the stop was being set may still run (the
  // completion thread can have left first): its outputs live in the arena,
  // which destroy_slots frees after synchronising every slot stream.
  destroy_slots(s);
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
  for (uint32_t v = 0; v < req->nviews; ++v) r.work += estimate_work(req->views[v]);
  std::lock_guard<std::mutex> lk(s->mu);
  if (s->stop) return NES_EINVAL;
  const double pred = s->rate_work_per_ms > 0.0
                          ? (s->pending_work + s->inflight_work + r.work) / s->rate_work_per_ms
                          : 0.0;
  // Before the first batch has completed there is no rate: keep at most one
  // batch's worth of pixels in the system.
  const bool late = s->cfg.max_queue_ms > 0.0f &&
                    (s->rate_work_per_ms > 0.0 ? pred * s->delay_scale > s->cfg.max_queue_ms
                                             : s->pending_pixels + s->inflight_pixels + px > s->cfg.max_batch_pixels);
  size_t off = Arena::kNone;
  if (s->pending.size() < s->cfg.max_pending && !late &&
      s->stats.budget_used_bytes + r.bytes <= s->cfg.hbm_budget_bytes)
    off = s->arena.alloc(r.bytes);
  if (off == Arena::kNone) {
    s->stats.rejected++;
    return NES_EAGAIN;
  }
  r.arena_off = off;
  r.dev = s->arena_base + off;
  s->pending_pixels += px;
  s->pending_work += r.work;
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
  // Done means the request's batch has finished on the GPU (or its slot's
  // stream was synchronised after a failed launch): the slots are free.
  if (it->second.dev) s->arena.release(it->second.arena_off, it->second.bytes);
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
