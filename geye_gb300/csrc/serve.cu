// serve.cu -- asynchronous frame submission and the multi-stream detection
// server (no counterpart in the reference, whose car_detection handles one
// frame at a time from main.cpp's loop).
//
// A context is a slot: geye_detect_submit stages a frame through pinned
// memory, replays the frame graph on the context's stream and queues the
// result copies; a completion event tells when it is done.  The server keeps a
// pool of slots and a FIFO of submitted frames.  A frame goes to a free slot
// that already holds a plan for its size, else to a new slot while the device
// memory held by slots stays within the budget, else to any free slot, which
// builds a plan for the size beside the ones it holds (or in their place once
// the memory held reaches the budget).  Frames in different slots overlap on
// the GPU; a stream's frames are
// dispatched in submission order and its tracker updates are chained with
// events so they run in that order too.
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <deque>
#include <map>
#include <string>
#include <vector>

#include "runtime.h"
#include "tracker.h"

namespace geye {
geye_status run_frame(geye_ctx *ctx, Plan &P, const uint8_t *d_bgr, int width_step, float thresh, float overlap,
                      const float *const *h_ascore_init);
geye_status frame_plan(geye_ctx *ctx, geye_model *const *models, int n, int w, int h, Plan **out);
void drop_frame_plans(geye_ctx *ctx, int w, int h);   // the context's whole-path plans for frames of w x h
size_t plan_device_bytes(const Plan &P);

constexpr int kHostRes = 4096;   // records per model returned through pinned memory

// pinned result block: ints [0, 32) boxes before NMS per model, [32, 64) kept
// per model, then per model point[4R], or_point[4R], type[R], scale[R], score[R]
static size_t res_block_ints(int n_models) { return 64 + (size_t)n_models * 11 * kHostRes; }

static long long now_ns() {
  return std::chrono::duration_cast<std::chrono::nanoseconds>(std::chrono::steady_clock::now().time_since_epoch())
      .count();
}

// queue everything of one frame on the context's stream (the frame already in P.h_bgr)
// (from h_src, pinned and kept until the frame completes, when given)
// (copy_in false: the frame is on the device already)
static geye_status enqueue_frame(geye_ctx *ctx, Plan &P, float thresh, float overlap, TrackerSet *trk, int stream,
                                 cudaEvent_t after, cudaEvent_t tracked, bool record_done = true,
                                 const void *h_src = nullptr, bool copy_in = true) {
  const int n_models = (int)P.models.size();
  if (copy_in)
    CUDA_TRY(cudaMemcpyAsync(P.d_bgr.p, h_src ? h_src : P.h_bgr, (size_t)3 * P.width * P.height,
                             cudaMemcpyHostToDevice, ctx->stream));
  GEYE_TRY(run_frame(ctx, P, P.d_bgr.as<uint8_t>(), 3 * P.width, thresh, overlap, nullptr));
  if (trk) {
    if (after) CUDA_TRY(cudaStreamWaitEvent(ctx->stream, after, 0));
    GEYE_TRY(tracker_update(*trk, stream, P.d_result.as<int>(), P.max_cap, P.d_small.as<int>() + 32, n_models,
                            P.d_ascore.as<float>(), P.width, P.height, ctx->stream));
    CUDA_TRY(cudaEventRecord(tracked, ctx->stream));
  }
  int *h = static_cast<int *>(P.h_res);
  CUDA_TRY(cudaMemcpyAsync(h, P.d_small.p, sizeof(int) * 64, cudaMemcpyDeviceToHost, ctx->stream));
  const size_t R = (size_t)std::min(P.max_cap, kHostRes);
  for (int mi = 0; mi < n_models; mi++) {
    const int *res = P.d_result.as<int>() + (size_t)mi * P.max_cap * 11;
    int *dst = h + 64 + (size_t)mi * 11 * kHostRes;
    CUDA_TRY(cudaMemcpyAsync(dst, res, sizeof(int) * 4 * R, cudaMemcpyDeviceToHost, ctx->stream));
    CUDA_TRY(cudaMemcpyAsync(dst + 4 * kHostRes, res + 4 * (size_t)P.max_cap, sizeof(int) * 4 * R,
                             cudaMemcpyDeviceToHost, ctx->stream));
    for (int f = 8; f < 11; f++)   // type, scale, score (max_cap apart on the device, kHostRes apart here)
      CUDA_TRY(cudaMemcpyAsync(dst + f * kHostRes, res + f * (size_t)P.max_cap, sizeof(int) * R,
                               cudaMemcpyDeviceToHost, ctx->stream));
  }
  if (record_done) CUDA_TRY(cudaEventRecord(P.ev_done, ctx->stream));
  ctx->pending = &P;
  return GEYE_OK;
}

static geye_status ensure_staging(Plan &P) {
  const int n_models = (int)P.models.size();
  if (!P.h_bgr) CUDA_TRY(cudaMallocHost(&P.h_bgr, (size_t)3 * P.width * P.height));
  if (!P.h_res) CUDA_TRY(cudaMallocHost(&P.h_res, sizeof(int) * res_block_ints(n_models)));
  if (!P.ev_done) CUDA_TRY(cudaEventCreateWithFlags(&P.ev_done, cudaEventDisableTiming));
  return GEYE_OK;
}

// wait: the frame's own graph (submit and server slots; the plan's sort level
// count may then adapt); false: a lane of a batch graph, already complete
static geye_status collect_frame(geye_ctx *ctx, geye_result *out, bool wait = true) {
  Plan &P = *ctx->pending;
  if (wait) CUDA_TRY(cudaEventSynchronize(P.ev_done));
  const int n_models = (int)P.models.size();
  const int *h = static_cast<const int *>(P.h_res);
  if (wait) note_sort_levels(ctx, P, h[kSortLevelsUsed], h[kNmsRoundsUsed]);
  geye_status st = GEYE_OK;
  for (int mi = 0; mi < n_models && out; mi++) {
    const int K = h[32 + mi];
    geye_result &r = out[mi];
    memset(&r, 0, sizeof(r));
    r.num = K;
    const size_t k = std::max(K, 1);
    r.point = (int *)malloc(sizeof(int) * 4 * k);
    r.or_point = (int *)malloc(sizeof(int) * 4 * k);
    r.type = (int *)malloc(sizeof(int) * k);
    r.scale = (float *)malloc(sizeof(float) * k);
    r.score = (float *)malloc(sizeof(float) * k);
    if (!r.point || !r.or_point || !r.type || !r.scale || !r.score) {
      set_error("host allocation failed");
      st = GEYE_ERR_NOMEM;
      continue;
    }
    const int *src = h + 64 + (size_t)mi * 11 * kHostRes;
    const int n = std::min(K, kHostRes);
    memcpy(r.point, src, sizeof(int) * 4 * n);
    memcpy(r.or_point, src + 4 * kHostRes, sizeof(int) * 4 * n);
    memcpy(r.type, src + 8 * kHostRes, sizeof(int) * n);
    memcpy(r.scale, src + 9 * kHostRes, sizeof(float) * n);
    memcpy(r.score, src + 10 * kHostRes, sizeof(float) * n);
    if (K > n) {   // more kept boxes than the pinned block holds: the rest straight from the device
      const int *res = P.d_result.as<int>() + (size_t)mi * P.max_cap * 11;
      const size_t rest = (size_t)(K - n);
      CUDA_TRY(cudaMemcpy(r.point + 4 * n, res + 4 * n, sizeof(int) * 4 * rest, cudaMemcpyDeviceToHost));
      CUDA_TRY(cudaMemcpy(r.or_point + 4 * n, res + 4 * (size_t)P.max_cap + 4 * n, sizeof(int) * 4 * rest,
                          cudaMemcpyDeviceToHost));
      CUDA_TRY(cudaMemcpy(r.type + n, res + 8 * (size_t)P.max_cap + n, sizeof(int) * rest, cudaMemcpyDeviceToHost));
      CUDA_TRY(cudaMemcpy(r.scale + n, res + 9 * (size_t)P.max_cap + n, sizeof(float) * rest,
                          cudaMemcpyDeviceToHost));
      CUDA_TRY(cudaMemcpy(r.score + n, res + 10 * (size_t)P.max_cap + n, sizeof(float) * rest,
                          cudaMemcpyDeviceToHost));
    }
  }
  P.last_D.assign(h, h + n_models);
  P.last_K.assign(h + 32, h + 32 + n_models);
  ctx->last_plan = &P;
  ctx->pending = nullptr;
  return st;
}

}  // namespace geye

using namespace geye;

extern "C" {

geye_status geye_detect_submit(geye_ctx *ctx, geye_model *const *models, int n_models, const uint8_t *bgr, int width,
                               int height, int width_step, float thresh, float overlap) {
  ARG_CHECK(ctx && models && bgr && n_models > 0, "null argument");
  ARG_CHECK(width >= 16 && height >= 16 && width_step >= 3 * width, "bad frame size");
  ARG_CHECK(!ctx->pending, "a submitted frame has not been collected");
  for (int i = 0; i < n_models; i++) MODEL_CHECK(models[i], ctx->device);
  CUDA_TRY(cudaSetDevice(ctx->device));
  Plan *P = nullptr;
  GEYE_TRY(frame_plan(ctx, models, n_models, width, height, &P));
  GEYE_TRY(ensure_staging(*P));
  uint8_t *dst = static_cast<uint8_t *>(P->h_bgr);
  for (int y = 0; y < height; y++) memcpy(dst + (size_t)y * 3 * width, bgr + (size_t)y * width_step, (size_t)3 * width);
  return enqueue_frame(ctx, *P, thresh, overlap, nullptr, 0, nullptr, nullptr);
}

geye_status geye_detect_query(geye_ctx *ctx) {
  ARG_CHECK(ctx && ctx->pending, "no submitted frame");
  const cudaError_t e = cudaEventQuery(ctx->pending->ev_done);
  if (e == cudaSuccess) return GEYE_OK;
  if (e == cudaErrorNotReady) return GEYE_BUSY;
  set_error(std::string("detect_query: ") + cudaGetErrorString(e));
  return GEYE_ERR_CUDA;
}

geye_status geye_detect_collect(geye_ctx *ctx, geye_result *out) {
  ARG_CHECK(ctx && ctx->pending && out, "no submitted frame or null output");
  return collect_frame(ctx, out);
}

}  // extern "C"

// ---------------------------------------------------------------------------
// server
// ---------------------------------------------------------------------------
struct geye_server {
  int device = 0;
  std::vector<geye_model *> models;
  geye_conv_mode mode = GEYE_CONV_BF16;
  size_t budget = 0, held = 0;
  int max_slots = 1;
  float thresh = -0.5f, overlap = 0.5f;
  bool track = false;
  struct Slot {
    geye_ctx *ctx = nullptr;
    bool busy = false;
    struct Held {
      size_t bytes;        // device bytes of the plan
      long long used;      // last dispatch to it
    };
    std::map<long long, Held> sizes;   // (w << 32 | h) of each plan the slot holds
    size_t bytes = 0;                  // their sum
    long long ticket = 0, t_submit = 0, t_dispatch = 0;
    int stream = 0;
    cudaEvent_t tracked = nullptr;  // this frame's tracker update
    uint8_t *frame = nullptr;       // the frame's pinned buffer, held until it completes
    size_t frame_bytes = 0;
  };
  std::vector<Slot> slots;
  struct Req {
    long long ticket, t_submit;
    int stream, w, h;
    uint8_t *bgr;   // pinned (pool below), the H2D copy's source
    size_t bytes;
  };
  // pinned frame buffers by size: a submitted frame is copied once, into one of
  // these, and goes to the device from there.  They are carved from slabs of
  // kPinnedSlab bytes (cudaMallocHost is slow and synchronises the device, so
  // it runs once per slab, not once per buffer) and reused, never returned.
  std::map<size_t, std::vector<uint8_t *>> pinned_free;
  std::vector<uint8_t *> pinned_all;   // the slabs
  uint8_t *slab_next = nullptr;
  size_t slab_left = 0;
  std::deque<Req> queue;
  struct Done {
    geye_served info;
    std::vector<geye_result> res;
  };
  std::deque<Done> done;
  long long next_ticket = 1, completed = 0;
  geye::TrackerSet trk;
  std::map<int, cudaEvent_t> last_tracked;   // per stream: the event of its latest dispatched tracker update
  std::map<int, long long> stream_busy;      // per stream: frames dispatched and not finished
  // admission (geye_server_set_admission): queued frames a stream may hold, the
  // longest a frame may wait for a slot; 0 = no limit
  int max_queued = 0;
  long long max_wait_ns = 0;
  long long dropped = 0;
};

namespace {

geye_status new_slot(geye_server *s, int *idx) {
  geye_ctx *c = nullptr;
  GEYE_TRY(geye_ctx_create(s->device, nullptr, &c));
  geye_status st = geye_ctx_set_conv_mode(c, s->mode);
  if (st != GEYE_OK) { geye_ctx_destroy(c); return st; }
  // the quicksort-order pass stays an if node of the slot's frame graph (it runs
  // only when a model of the frame needs it): with 32 hardware queues that beats
  // plain launches that return at once, 16 slots in flight (3384 against 2954
  // frames/s end to end at 640x480)
  geye_server::Slot sl;
  sl.ctx = c;
  if (cudaEventCreateWithFlags(&sl.tracked, cudaEventDisableTiming) != cudaSuccess) {
    geye_ctx_destroy(c);
    set_error("server: event creation failed");
    return GEYE_ERR_CUDA;
  }
  s->slots.push_back(sl);
  *idx = (int)s->slots.size() - 1;
  return GEYE_OK;
}

constexpr size_t kPinnedSlab = 64ull << 20;

geye_status get_pinned(geye_server *s, size_t n, uint8_t **out) {
  auto &v = s->pinned_free[n];
  if (!v.empty()) {
    *out = v.back();
    v.pop_back();
    return GEYE_OK;
  }
  const size_t need = (n + 4095) & ~(size_t)4095;
  if (s->slab_left < need) {
    const size_t bytes = std::max(kPinnedSlab, need);
    void *p = nullptr;
    CUDA_TRY(cudaMallocHost(&p, bytes));
    s->pinned_all.push_back(static_cast<uint8_t *>(p));
    s->slab_next = static_cast<uint8_t *>(p);
    s->slab_left = bytes;
  }
  *out = s->slab_next;
  s->slab_next += need;
  s->slab_left -= need;
  return GEYE_OK;
}

void put_pinned(geye_server *s, size_t n, uint8_t *p) {
  if (p) s->pinned_free[n].push_back(p);
}

// a queued frame that will not run: reported by poll with dropped = 1 and empty results
void drop_request(geye_server *s, const geye_server::Req &r) {
  put_pinned(s, r.bytes, r.bgr);
  geye_server::Done d;
  d.info = geye_served{};
  d.info.ticket = r.ticket;
  d.info.stream = r.stream;
  d.info.queued_ns = now_ns() - r.t_submit;
  d.info.latency_ns = d.info.queued_ns;
  d.info.dropped = 1;
  d.res.assign(s->models.size(), geye_result{});
  s->done.push_back(std::move(d));
  s->dropped++;
}

// dispatch the queue head into a slot; false when nothing fits right now
geye_status dispatch_one(geye_server *s, bool *dispatched) {
  *dispatched = false;
  // frames that waited past the limit are dropped rather than served late
  while (s->max_wait_ns > 0 && !s->queue.empty() && now_ns() - s->queue.front().t_submit > s->max_wait_ns) {
    drop_request(s, s->queue.front());
    s->queue.pop_front();
  }
  if (s->queue.empty()) return GEYE_OK;
  geye_server::Req &r = s->queue.front();
  const long long key = ((long long)r.w << 32) | (unsigned)r.h;
  int pick = -1;
  // a free slot that holds a plan (and its frame graph) for this size
  for (size_t i = 0; i < s->slots.size() && pick < 0; i++)
    if (!s->slots[i].busy && s->slots[i].sizes.count(key)) pick = (int)i;
  // else a new slot while slots and memory last
  if (pick < 0 && (int)s->slots.size() < s->max_slots && s->held < s->budget) GEYE_TRY(new_slot(s, &pick));
  // else any free slot: it keeps its plans for other sizes (so that mixed sizes do
  // not rebuild plans) while the memory held stays within the budget, else drops them
  for (size_t i = 0; i < s->slots.size() && pick < 0; i++)
    if (!s->slots[i].busy) pick = (int)i;
  if (pick < 0) return GEYE_OK;
  geye_server::Slot &sl = s->slots[pick];
  const bool fresh = !sl.sizes.count(key);
  // room for a new plan: the least recently used plans of free slots go while
  // the memory held is at the budget
  while (fresh && (s->held >= s->budget || sl.sizes.size() >= 16)) {
    geye_server::Slot *vs = nullptr;
    long long vk = 0, vt = 0;
    for (auto &o : s->slots) {
      if (o.busy) continue;
      for (auto &kv : o.sizes)
        if (!vs || kv.second.used < vt) { vs = &o; vk = kv.first; vt = kv.second.used; }
    }
    if (!vs) break;
    drop_frame_plans(vs->ctx, (int)(vk >> 32), (int)(vk & 0xffffffff));
    s->held -= vs->sizes[vk].bytes;
    vs->bytes -= vs->sizes[vk].bytes;
    vs->sizes.erase(vk);
  }
  Plan *P = nullptr;
  GEYE_TRY(frame_plan(sl.ctx, s->models.data(), (int)s->models.size(), r.w, r.h, &P));
  GEYE_TRY(ensure_staging(*P));
  if (fresh) {
    const size_t b = plan_device_bytes(*P);
    sl.sizes[key] = geye_server::Slot::Held{b, 0};
    sl.bytes += b;
    s->held += b;
  }
  sl.sizes[key].used = now_ns();
  cudaEvent_t after = nullptr;
  auto it = s->last_tracked.find(r.stream);
  if (it != s->last_tracked.end() && s->stream_busy[r.stream] > 0) after = it->second;
  GEYE_TRY(enqueue_frame(sl.ctx, *P, s->thresh, s->overlap, s->track ? &s->trk : nullptr, r.stream, after,
                         sl.tracked, true, r.bgr));
  sl.frame = r.bgr;
  sl.frame_bytes = r.bytes;
  s->last_tracked[r.stream] = sl.tracked;
  s->stream_busy[r.stream]++;
  sl.busy = true;
  sl.ticket = r.ticket;
  sl.stream = r.stream;
  sl.t_submit = r.t_submit;
  sl.t_dispatch = now_ns();
  s->queue.pop_front();
  *dispatched = true;
  return GEYE_OK;
}

geye_status pump(geye_server *s) {
  // a model whose loading context was destroyed has freed filters: no queued
  // frame can run any more, so every queued frame fails before any launch
  for (geye_model *m : s->models)
    if (!s->queue.empty() && (!m || !m->ctx || m->ctx->device != s->device)) {
      for (const auto &r : s->queue) drop_request(s, r);
      s->queue.clear();
      MODEL_CHECK(m, s->device);
    }
  for (;;) {
    bool d = false;
    GEYE_TRY(dispatch_one(s, &d));
    if (!d) return GEYE_OK;
  }
}

geye_status complete(geye_server *s, geye_server::Slot &sl) {
  geye_server::Done d;
  d.res.resize(s->models.size());
  GEYE_TRY(collect_frame(sl.ctx, d.res.data()));
  const long long t = now_ns();
  d.info = geye_served{};
  d.info.ticket = sl.ticket;
  d.info.stream = sl.stream;
  d.info.queued_ns = sl.t_dispatch - sl.t_submit;
  d.info.latency_ns = t - sl.t_submit;
  d.info.n_tracks = s->track ? tracker_count(s->trk, sl.stream) : 0;
  s->done.push_back(std::move(d));
  s->stream_busy[sl.stream]--;
  put_pinned(s, sl.frame_bytes, sl.frame);
  sl.frame = nullptr;
  sl.busy = false;
  s->completed++;
  return GEYE_OK;
}

geye_status reap(geye_server *s, bool block) {
  for (auto &sl : s->slots) {
    if (!sl.busy) continue;
    const cudaError_t e = block ? cudaEventSynchronize(sl.ctx->pending->ev_done) : cudaEventQuery(sl.ctx->pending->ev_done);
    if (e == cudaErrorNotReady) continue;
    if (e != cudaSuccess) {
      set_error(std::string("server: ") + cudaGetErrorString(e));
      return GEYE_ERR_CUDA;
    }
    GEYE_TRY(complete(s, sl));
  }
  return GEYE_OK;
}

}  // namespace

namespace geye {
size_t plan_device_bytes(const Plan &P) {
  size_t b = P.arena.bytes + P.arena16.bytes + P.d_bgr.bytes + P.d_boxes.bytes + P.d_kept_boxes.bytes +
             P.d_nms_f.bytes + P.d_nms_i.bytes + P.d_small.bytes + P.d_ascore.bytes + P.d_result.bytes;
  b += P.tc.d_bank.bytes + P.tc.d_jobs.bytes + P.tc.d_chunks.bytes + P.tc.d_cols.bytes + P.tc.d_sums.bytes;
  for (auto &mp : P.models)
    b += mp->d_root_jobs.bytes + mp->d_part_jobs.bytes + mp->d_dt_jobs.bytes + mp->d_score_jobs.bytes +
         mp->d_dt_blocks1.bytes + mp->d_dt_blocks2.bytes + mp->d_score_blocks.bytes +
         mp->d_counts.bytes + mp->d_as_col.bytes + mp->d_as_row.bytes;
  return b;
}
}  // namespace geye

extern "C" {

geye_status geye_server_create(int device, geye_model *const *models, int n_models, geye_conv_mode mode,
                               size_t hbm_budget, int max_slots, float thresh, float overlap, int track,
                               geye_server **out) {
  ARG_CHECK(out && models && n_models > 0 && max_slots > 0, "bad argument");
  for (int i = 0; i < n_models; i++) MODEL_CHECK(models[i], device);
  CUDA_TRY(cudaSetDevice(device));
  geye_server *s = new geye_server();
  s->device = device;
  s->models.assign(models, models + n_models);
  s->mode = mode;
  s->budget = hbm_budget;
  s->max_slots = max_slots;
  s->thresh = thresh;
  s->overlap = overlap;
  s->track = track != 0;
  if (s->track) {
    const geye_status st = tracker_init(s->trk, 0x5eed5eedull);
    if (st != GEYE_OK) { delete s; return st; }
  }
  *out = s;
  return GEYE_OK;
}

geye_status geye_server_destroy(geye_server *s) {
  if (!s) return GEYE_OK;
  cudaSetDevice(s->device);
  for (auto &sl : s->slots) {
    if (sl.ctx) cudaStreamSynchronize(sl.ctx->stream);
  }
  for (auto &d : s->done)
    for (auto &r : d.res) geye_result_free(&r);
  for (auto &sl : s->slots) {
    if (sl.tracked) cudaEventDestroy(sl.tracked);
    geye_ctx_destroy(sl.ctx);
  }
  for (uint8_t *p : s->pinned_all) cudaFreeHost(p);
  tracker_free(s->trk);
  delete s;
  return GEYE_OK;
}

geye_status geye_server_submit(geye_server *s, int stream, const uint8_t *bgr, int width, int height, int width_step,
                               long long *ticket) {
  ARG_CHECK(s && bgr && ticket, "null argument");
  ARG_CHECK(width >= 16 && height >= 16 && width_step >= 3 * width, "bad frame size");
  ARG_CHECK(stream >= 0 && stream < kTrackerStreams, "stream id out of range");
  for (geye_model *m : s->models) MODEL_CHECK(m, s->device);
  CUDA_TRY(cudaSetDevice(s->device));
  geye_server::Req r;
  r.ticket = s->next_ticket++;
  r.t_submit = now_ns();
  r.stream = stream;
  r.w = width;
  r.h = height;
  r.bytes = (size_t)3 * width * height;
  GEYE_TRY(get_pinned(s, r.bytes, &r.bgr));
  if (width_step == 3 * width) {
    memcpy(r.bgr, bgr, r.bytes);
  } else {
    for (int y = 0; y < height; y++)
      memcpy(r.bgr + (size_t)y * 3 * width, bgr + (size_t)y * width_step, (size_t)3 * width);
  }
  *ticket = r.ticket;
  s->queue.push_back(std::move(r));
  if (s->max_queued > 0) {   // the stream's oldest queued frames make way for its newest
    int n = 0;
    for (const auto &q : s->queue) n += q.stream == stream;
    for (auto it = s->queue.begin(); n > s->max_queued && it != s->queue.end();) {
      if (it->stream == stream) {
        drop_request(s, *it);
        it = s->queue.erase(it);
        n--;
      } else {
        ++it;
      }
    }
  }
  GEYE_TRY(reap(s, false));
  return pump(s);
}

geye_status geye_server_set_admission(geye_server *s, int max_queued_per_stream, long long max_wait_ns) {
  ARG_CHECK(s && max_queued_per_stream >= 0 && max_wait_ns >= 0, "bad argument");
  s->max_queued = max_queued_per_stream;
  s->max_wait_ns = max_wait_ns;
  return GEYE_OK;
}

geye_status geye_server_poll(geye_server *s, int max, geye_served *info, geye_result *results, int *n) {
  ARG_CHECK(s && n && (max == 0 || info), "null argument");
  CUDA_TRY(cudaSetDevice(s->device));
  GEYE_TRY(reap(s, false));
  GEYE_TRY(pump(s));
  int k = 0;
  while (k < max && !s->done.empty()) {
    geye_server::Done &d = s->done.front();
    info[k] = d.info;
    for (size_t m = 0; m < d.res.size(); m++) {
      if (results) results[(size_t)k * s->models.size() + m] = d.res[m];
      else geye_result_free(&d.res[m]);
    }
    s->done.pop_front();
    k++;
  }
  *n = k;
  return GEYE_OK;
}

geye_status geye_server_drain(geye_server *s) {
  ARG_CHECK(s, "null server");
  CUDA_TRY(cudaSetDevice(s->device));
  for (int guard = 0; guard < 1 << 30; guard++) {
    GEYE_TRY(pump(s));
    bool busy = false;
    for (auto &sl : s->slots) busy |= sl.busy;
    if (!busy && s->queue.empty()) return GEYE_OK;
    GEYE_TRY(reap(s, true));
  }
  set_error("server drain did not finish");
  return GEYE_ERR_TIMEOUT;
}

geye_status geye_server_stats(geye_server *s, long long out[8]) {
  ARG_CHECK(s && out, "null argument");
  long long busy = 0;
  for (auto &sl : s->slots) busy += sl.busy;
  out[0] = (long long)s->slots.size();
  out[1] = busy;
  out[2] = (long long)s->queue.size();
  out[3] = (long long)s->done.size();
  out[4] = (long long)s->held;
  out[5] = s->completed;
  out[6] = s->track ? tracker_streams(s->trk) : 0;
  out[7] = s->dropped;
  return GEYE_OK;
}

geye_status geye_server_tracks(geye_server *s, int stream, int max, float *boxes, int *n) {
  ARG_CHECK(s && n && (max == 0 || boxes), "null argument");
  ARG_CHECK(s->track, "the server was created without trackers");
  ARG_CHECK(stream >= 0 && stream < kTrackerStreams, "stream id out of range");
  for (geye_model *m : s->models) MODEL_CHECK(m, s->device);
  CUDA_TRY(cudaSetDevice(s->device));
  for (auto &sl : s->slots)
    if (sl.ctx) CUDA_TRY(cudaStreamSynchronize(sl.ctx->stream));
  return tracker_read(s->trk, stream, max, boxes, n);
}

}  // extern "C"

// ---------------------------------------------------------------------------
// batch: several frames (any mix of sizes) as one CUDA graph, one lane
// (context, stream, plan per size) per frame, the lanes as parallel branches
// of the graph between a fork and a join on the batch's stream
// ---------------------------------------------------------------------------
struct geye_batch {
  int device = 0;
  std::vector<geye_model *> models;
  geye_conv_mode mode = GEYE_CONV_FP32;
  int max_frames = 0;
  std::vector<geye_ctx *> lanes;
  cudaStream_t stream = nullptr;
  cudaEvent_t fork = nullptr, front_done = nullptr;
  std::vector<cudaEvent_t> joins;
  struct Graph {
    cudaGraphExec_t exec = nullptr;
    int kernels = 0;
    void *d_tables = nullptr;   // the batched front end's frame table and work items (read by the graph)
    size_t frames_bytes = 0;    // the frame table's share of d_tables, items after it
    int n_phases = 0;           // resize phases of the batch's deepest pyramid
    std::vector<int> count, offset;   // items per list (front_list) and their offsets
    std::vector<unsigned long long> plans;   // serials of the lanes' plans the graph was captured with
  };
  std::map<std::string, Graph> graphs;   // by lane sizes, thresh, overlap
  int last_kernels = 0;
  cudaEvent_t t0 = nullptr, t1 = nullptr;   // around the last graph launch
};

namespace {

// The batched front end's tables for one batch key: every frame's plan
// pointers and, per stage, the ragged list of (frame, job, chunk) items,
// in one device buffer that the batch graph reads.  Lists: ingest, vertical
// and horizontal resize per phase, pixels, votes, corner norms, features.
int front_list(int stage, int phase) {   // list index of a stage (resize: per phase)
  if (stage == kBatchIngest) return 0;
  if (stage == kBatchResizeV) return 1 + 2 * phase;
  if (stage == kBatchResizeH) return 2 + 2 * phase;
  return 1 + 2 * kBatchMaxPhases + (stage - kBatchPix);
}

geye_status batch_front_tables(geye_batch *b, const std::vector<Plan *> &plans, geye_batch::Graph &g) {
  const int nf = (int)plans.size();
  const int n_lists = 1 + 2 * kBatchMaxPhases + 4;
  std::vector<std::vector<BatchItem>> L(n_lists);
  std::vector<BatchFrame> fr(nf);
  int max_ph = 0;
  for (int f = 0; f < nf; f++) {
    const Plan &P = *plans[f];
    ARG_CHECK((int)P.vjobs.size() <= kBatchMaxPhases, "batch: too many resize phases");
    BatchFrame &F = fr[f];
    F = BatchFrame{};
    F.bgr = P.d_bgr.as<uint8_t>();
    F.width = P.width;
    F.height = P.height;
    F.width_step = 3 * P.width;
    F.arena = P.arena.as<float>();
    F.arena16 = static_cast<uint8_t *>(P.arena16.p);
    F.img0_off = P.lv[0].img_off;
    F.n_phases = (int)P.vjobs.size();
    for (int ph = 0; ph < F.n_phases; ph++) {
      F.vjobs[ph] = P.d_vjobs[ph].as<ResizeJob>();
      F.hjobs[ph] = P.d_hjobs[ph].as<ResizeJob>();
    }
    F.tap_start = P.d_tap_start.as<int>();
    F.tap_si = P.d_tap_si.as<int>();
    F.tap_alpha = P.d_tap_alpha.as<float>();
    F.pix = P.d_pix_jobs.as<HogPixJob>();
    F.hog = P.d_hog_jobs.as<HogJob>();
    F.vote_blocks = P.d_hog_vote_blocks.as<int2>();
    max_ph = std::max(max_ph, F.n_phases);
    for (int ty = 0; ty < (P.height + 31) / 32; ty++)
      for (int tx = 0; tx < (P.width + 31) / 32; tx++) L[0].push_back(BatchItem{f, tx, ty, 0});
    for (int ph = 0; ph < F.n_phases; ph++)
      for (size_t j = 0; j < P.vjobs[ph].size(); j++) {
        for (int c = 0; c * kBatchColumns < P.vjobs[ph][j].dst_w; c++)
          L[front_list(kBatchResizeV, ph)].push_back(BatchItem{f, (int)j, c, 0});
        for (int c = 0; c * kBatchColumns < P.hjobs[ph][j].dst_w; c++)
          L[front_list(kBatchResizeH, ph)].push_back(BatchItem{f, (int)j, c, 0});
      }
    for (size_t j = 0; j < P.pix_jobs.size(); j++)
      for (int c = 0; 1 + c * kBatchColumns < P.pix_jobs[j].xe; c++)
        L[front_list(kBatchPix, 0)].push_back(BatchItem{f, (int)j, c, 0});
    for (int k = 0; k < P.hog_vote_nblocks; k++) L[front_list(kBatchVote, 0)].push_back(BatchItem{f, k, 0, 0});
    const bool fast = !P.hog_jobs.empty() && P.hog_jobs[0].fast;
    for (size_t j = 0; j < P.hog_jobs.size(); j++) {
      const HogJob &J = P.hog_jobs[j];
      if (!fast)
        for (int c = 0; c * kBatchCells < (J.fs0 + 1) * (J.fs1 + 1); c++)
          L[front_list(kBatchNorm, 0)].push_back(BatchItem{f, (int)j, c, 0});
      for (int c = 0; c * kBatchCells < J.fs0 * J.fs1; c++)
        L[front_list(kBatchFeat, 0)].push_back(BatchItem{f, (int)j, c, 0});
    }
  }
  g.n_phases = max_ph;
  g.frames_bytes = ((sizeof(BatchFrame) * nf + 255) / 256) * 256;
  g.count.clear();
  g.offset.clear();
  size_t items = 0;
  for (auto &l : L) {
    g.offset.push_back((int)items);
    g.count.push_back((int)l.size());
    items += l.size();
  }
  std::vector<uint8_t> host(g.frames_bytes + sizeof(BatchItem) * std::max<size_t>(items, 1));
  memcpy(host.data(), fr.data(), sizeof(BatchFrame) * nf);
  BatchItem *it = reinterpret_cast<BatchItem *>(host.data() + g.frames_bytes);
  for (auto &l : L) {
    if (!l.empty()) memcpy(it, l.data(), sizeof(BatchItem) * l.size());
    it += l.size();
  }
  if (g.d_tables) cudaFree(g.d_tables);
  g.d_tables = nullptr;
  CUDA_TRY(cudaMalloc(&g.d_tables, host.size()));
  CUDA_TRY(cudaMemcpy(g.d_tables, host.data(), host.size(), cudaMemcpyHostToDevice));
  (void)b;
  return GEYE_OK;
}

// the stages in order on the batch stream (inside its capture)
void launch_batch_tables(geye_batch *b, geye_batch::Graph &g) {
  const BatchFrame *frames = static_cast<const BatchFrame *>(g.d_tables);
  const BatchItem *items = reinterpret_cast<const BatchItem *>(static_cast<uint8_t *>(g.d_tables) + g.frames_bytes);
  auto run = [&](int stage, int phase) {
    const int l = front_list(stage, phase);
    launch_batch_front(stage, frames, items + g.offset[l], g.count[l], phase, b->stream);
  };
  run(kBatchIngest, 0);
  for (int ph = 0; ph < g.n_phases; ph++) {
    run(kBatchResizeV, ph);
    run(kBatchResizeH, ph);
  }
  run(kBatchPix, 0);
  run(kBatchVote, 0);
  run(kBatchNorm, 0);
  run(kBatchFeat, 0);
}

}  // namespace

extern "C" {

geye_status geye_batch_create(int device, geye_model *const *models, int n_models, geye_conv_mode mode, int max_frames,
                              geye_batch **out) {
  ARG_CHECK(models && n_models > 0 && n_models <= 16 && out, "bad argument");
  ARG_CHECK(max_frames >= 1 && max_frames <= 256, "max_frames must be in 1..256");
  ARG_CHECK(mode == GEYE_CONV_FP32 || mode == GEYE_CONV_BF16 || mode == GEYE_CONV_FP8, "unknown conv mode");
  for (int i = 0; i < n_models; i++) MODEL_CHECK(models[i], device);
  CUDA_TRY(cudaSetDevice(device));
  auto *b = new geye_batch();
  b->device = device;
  b->models.assign(models, models + n_models);
  b->mode = mode;
  b->max_frames = max_frames;
  cudaError_t e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->front_done, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreate(&b->t0);
  if (e == cudaSuccess) e = cudaEventCreate(&b->t1);
  if (e != cudaSuccess) {
    if (b->t0) cudaEventDestroy(b->t0);
    if (b->front_done) cudaEventDestroy(b->front_done);
    if (b->fork) cudaEventDestroy(b->fork);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
    set_error(std::string("batch: ") + cudaGetErrorString(e));
    return GEYE_ERR_CUDA;
  }
  *out = b;
  return GEYE_OK;
}

geye_status geye_batch_destroy(geye_batch *b) {
  if (!b) return GEYE_OK;
  cudaSetDevice(b->device);
  cudaStreamSynchronize(b->stream);
  for (auto &g : b->graphs) {
    if (g.second.exec) cudaGraphExecDestroy(g.second.exec);
    if (g.second.d_tables) cudaFree(g.second.d_tables);
  }
  for (auto e : b->joins) cudaEventDestroy(e);
  if (b->front_done) cudaEventDestroy(b->front_done);
  for (auto *c : b->lanes) geye_ctx_destroy(c);
  cudaEventDestroy(b->fork);
  cudaEventDestroy(b->t0);
  cudaEventDestroy(b->t1);
  cudaStreamDestroy(b->stream);
  delete b;
  return GEYE_OK;
}

geye_status geye_batch_run(geye_batch *b, int n_frames, const uint8_t *const *bgr, const int *widths,
                           const int *heights, const int *width_steps, float thresh, float overlap,
                           geye_result *results) {
  ARG_CHECK(b && bgr && widths && heights && width_steps && results, "null argument");
  ARG_CHECK(n_frames >= 1 && n_frames <= b->max_frames, "n_frames out of range");
  for (geye_model *m : b->models) MODEL_CHECK(m, b->device);
  CUDA_TRY(cudaSetDevice(b->device));
  const int nm = (int)b->models.size();
  std::string key;
  std::vector<Plan *> plans(n_frames);
  for (int i = 0; i < n_frames; i++) {
    ARG_CHECK(bgr[i] && widths[i] >= 16 && heights[i] >= 16 && width_steps[i] >= 3 * widths[i], "bad frame");
    while ((int)b->lanes.size() <= i) {
      geye_ctx *c = nullptr;
      GEYE_TRY(geye_ctx_create(b->device, nullptr, &c));
      c->nms_if_node = false;   // the batch's other lanes in flight
      b->lanes.push_back(c);
      const geye_status st = geye_ctx_set_conv_mode(c, b->mode);
      if (st != GEYE_OK) return st;
      cudaEvent_t j = nullptr;
      CUDA_TRY(cudaEventCreateWithFlags(&j, cudaEventDisableTiming));
      b->joins.push_back(j);
    }
    GEYE_TRY(frame_plan(b->lanes[i], b->models.data(), nm, widths[i], heights[i], &plans[i]));
    GEYE_TRY(ensure_staging(*plans[i]));
    uint8_t *dst = static_cast<uint8_t *>(plans[i]->h_bgr);
    for (int y = 0; y < heights[i]; y++)
      memcpy(dst + (size_t)y * 3 * widths[i], bgr[i] + (size_t)y * width_steps[i], (size_t)3 * widths[i]);
    key += std::to_string(widths[i]) + "x" + std::to_string(heights[i]) + ",";
  }
  {
    unsigned tb, ob;
    memcpy(&tb, &thresh, 4);
    memcpy(&ob, &overlap, 4);
    key += std::to_string(tb) + ":" + std::to_string(ob);
  }
  geye_batch::Graph &g = b->graphs[key];
  std::vector<unsigned long long> serials(n_frames);
  for (int i = 0; i < n_frames; i++) serials[i] = plans[i]->serial;
  if (g.exec && g.plans != serials) {
    // a lane's plan was rebuilt since the capture (its context dropped its plans): the
    // graph reads the old plan's buffers, so it is captured again
    cudaStreamSynchronize(b->stream);
    cudaGraphExecDestroy(g.exec);
    g.exec = nullptr;
  }
  if (!g.exec) {
    GEYE_TRY(batch_front_tables(b, plans, g));
    g.plans = serials;
    cudaGraph_t graph = nullptr;
    CUDA_TRY(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeRelaxed));
    geye_status st = GEYE_OK;
    cudaError_t e = cudaSuccess;
    // every frame in, then the batched front end: one persistent launch per stage for all frames
    for (int i = 0; i < n_frames && e == cudaSuccess; i++)
      e = cudaMemcpyAsync(plans[i]->d_bgr.p, plans[i]->h_bgr, (size_t)3 * widths[i] * heights[i],
                          cudaMemcpyHostToDevice, b->stream);
    if (e == cudaSuccess) {
      launch_batch_tables(b, g);
      e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaEventRecord(b->front_done, b->stream);
    for (int i = 0; i < n_frames && st == GEYE_OK && e == cudaSuccess; i++) {
      geye_ctx *c = b->lanes[i];
      e = cudaStreamWaitEvent(c->stream, b->front_done, 0);
      if (e != cudaSuccess) break;
      const bool graphs = c->use_graphs;
      c->use_graphs = false;   // the lane's kernels go straight into the batch graph
      c->capturing = true;
      c->front_external = true;
      st = enqueue_frame(c, *plans[i], thresh, overlap, nullptr, 0, nullptr, nullptr, false, nullptr, false);
      c->front_external = false;
      c->capturing = false;
      c->use_graphs = graphs;
      c->pending = nullptr;
      if (st == GEYE_OK) e = cudaEventRecord(b->joins[i], c->stream);
      if (e == cudaSuccess && st == GEYE_OK) e = cudaStreamWaitEvent(b->stream, b->joins[i], 0);
    }
    const cudaError_t ec = cudaStreamEndCapture(b->stream, &graph);
    if (st != GEYE_OK || e != cudaSuccess || ec != cudaSuccess) {
      if (graph) cudaGraphDestroy(graph);
      if (g.d_tables) cudaFree(g.d_tables);
      b->graphs.erase(key);
      if (st != GEYE_OK) return st;
      set_error(std::string("batch graph capture: ") + cudaGetErrorString(e != cudaSuccess ? e : ec));
      return GEYE_ERR_CUDA;
    }
    size_t n = 0;
    cudaGraphGetNodes(graph, nullptr, &n);
    std::vector<cudaGraphNode_t> nodes(n);
    if (n) cudaGraphGetNodes(graph, nodes.data(), &n);
    int kernels = 0;
    for (auto nd : nodes) {
      cudaGraphNodeType t;
      if (cudaGraphNodeGetType(nd, &t) == cudaSuccess && t == cudaGraphNodeTypeKernel) kernels++;
    }
    const cudaError_t ie = cudaGraphInstantiate(&g.exec, graph, 0);
    cudaGraphDestroy(graph);
    if (ie != cudaSuccess) {
      g.exec = nullptr;
      if (g.d_tables) cudaFree(g.d_tables);
      b->graphs.erase(key);
      set_error(std::string("batch graph instantiate: ") + cudaGetErrorString(ie));
      return GEYE_ERR_CUDA;
    }
    g.kernels = kernels;
  }
  CUDA_TRY(cudaEventRecord(b->t0, b->stream));
  CUDA_TRY(cudaGraphLaunch(g.exec, b->stream));
  CUDA_TRY(cudaEventRecord(b->t1, b->stream));
  CUDA_TRY(cudaStreamSynchronize(b->stream));
  b->last_kernels = g.kernels;
  geye_status st = GEYE_OK;
  for (int i = 0; i < n_frames; i++) {
    b->lanes[i]->pending = plans[i];
    const geye_status s = collect_frame(b->lanes[i], results + (size_t)i * nm, false);
    if (st == GEYE_OK) st = s;
  }
  return st;
}

geye_status geye_batch_stats(geye_batch *b, int out[4], float *last_ms) {
  ARG_CHECK(b && out && last_ms, "null argument");
  out[0] = (int)b->lanes.size();
  out[1] = (int)b->graphs.size();
  out[2] = b->last_kernels;
  out[3] = 0;
  *last_ms = 0.f;
  if (b->last_kernels) CUDA_TRY(cudaEventElapsedTime(last_ms, b->t0, b->t1));
  return GEYE_OK;
}

}  // extern "C"
