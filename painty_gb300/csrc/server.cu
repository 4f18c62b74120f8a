// server.cu -- continuous-batching stroke-render server.
//
// Requests (paint these strokes on a new canvas, or continue a canvas an earlier request
// created) arrive at any time. A worker thread runs short steps: each step paints the next
// slice of every admitted request's strokes -- up to `step_stamps` stamps per request -- in
// one batched launch (the painty_paint_batch kernel), so requests that arrive while others
// are on the GPU join at the next step instead of waiting for them to finish. Canvases stay
// resident on the device between requests; admission keeps their bytes under a device-memory
// budget by evicting idle canvases (least recently used first) to pinned host memory and
// restoring them when a later request continues them. A canvas's requests run one after
// another, in submission order; different canvases are independent, so a request's result
// does not depend on what else is in flight.
//
// Each request completes with the KM composite of its canvas (Renderer::compose,
// painty/renderer/Renderer.hxx:26-53) downloaded into the caller's buffer.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "internal.h"

namespace {

double now_s() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch())
    .count();
}

enum ReqState { REQ_PENDING = 0, REQ_ACTIVE = 1, REQ_DONE = 2 };

struct HostBlob {  // pinned host copy of a device allocation
  void* p = nullptr;
  size_t bytes = 0;
  void ensure(size_t n) {
    if (p && bytes >= n) return;
    if (p) cudaFreeHost(p);
    p = nullptr;
    bytes = 0;
    PG_CUDA(cudaMallocHost(&p, n));
    bytes = n;
  }
  ~HostBlob() {
    if (p) cudaFreeHost(p);
  }
};

struct ServerCanvas {
  uint64_t id = 0;
  int32_t rows = 0, cols = 0;
  painty_canvas* cv = nullptr;  // created by the canvas's first request
  painty_brush* brush = nullptr;
  bool resident = false;
  bool busy = false;  // one of its requests is active
  uint64_t last_used = 0;
  size_t bytes = 0;  // device bytes when resident
  std::vector<float> r0;  // substrate until the canvas is created
  std::deque<uint64_t> waiting;  // its unfinished requests, in submission order
  HostBlob save_canvas, save_snapshot;
};

struct ServerRequest {
  uint64_t id = 0, canvas_id = 0;
  std::vector<painty_stroke_desc> strokes;
  std::vector<double> points;
  std::vector<int64_t> stroke_stamps;
  float* out_rgb = nullptr;
  size_t next = 0;  // next stroke to paint
  int state = REQ_PENDING;
  bool cancel = false;
  painty_status status = PAINTY_OK;
  std::string error;
  int64_t stamps = 0;
  double t_submit = 0, t_done = 0;
};

}  // namespace

struct painty_server {
  painty_server_options opt{};
  std::vector<double> footprint;
  int device = 0;
  cudaStream_t stream = nullptr;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<uint64_t> pending;
  std::vector<uint64_t> active;
  std::unordered_map<uint64_t, std::unique_ptr<ServerRequest>> reqs;
  std::unordered_map<uint64_t, std::unique_ptr<ServerCanvas>> canvases;
  size_t resident = 0, peak = 0;
  uint64_t next_req = 1, next_canvas = 1, step = 0;
  painty_server_counters stats{};
  bool stop = false;
  uint64_t gen = 0;  // bumped by submit, cancel and finish: the idle worker waits for a change
  std::string worker_error;
  std::thread worker;
};

namespace {

size_t canvas_device_bytes(const painty_server* s, int32_t rows, int32_t cols) {
  const painty_storage st = s->opt.storage;
  const painty_storage rs = st == PAINTY_STORAGE_F64 ? PAINTY_STORAGE_F64 : PAINTY_STORAGE_F32;
  const size_t pe = static_cast<size_t>(rows) * pg::pitch_for(cols);
  return pg::layer_bytes(rows, cols, st, true) + pg::image_bytes(rows, cols, rs) +
         pe * pg::v_bytes(st) + pg::layer_bytes(rows, cols, st, true) /* snapshot */ +
         (4u << 20) /* pickup map, footprint, scratch */;
}

// Moves a canvas's device state (canvas planes and the brush's snapshot) to
// pinned host memory and frees it on the device.
void evict(painty_server* s, ServerCanvas* c) {
  painty_canvas* cv = c->cv;
  painty_brush* b = c->brush;
  c->save_canvas.ensure(cv->bytes);
  PG_CUDA(cudaMemcpyAsync(c->save_canvas.p, cv->base, cv->bytes, cudaMemcpyDeviceToHost,
                          s->stream));
  if (b->has_snapshot) {
    c->save_snapshot.ensure(b->snapshot.bytes);
    PG_CUDA(cudaMemcpyAsync(c->save_snapshot.p, b->snapshot.base, b->snapshot.bytes,
                            cudaMemcpyDeviceToHost, s->stream));
  }
  PG_CUDA(cudaStreamSynchronize(s->stream));
  pg::device_free(cv->base);
  pg::canvas_relayout(cv, nullptr);
  if (b->has_snapshot) {
    pg::device_free(b->snapshot.base);
    b->snapshot.base = nullptr;
  }
  c->resident = false;
}

void restore(painty_server* s, ServerCanvas* c) {
  painty_canvas* cv = c->cv;
  painty_brush* b = c->brush;
  void* base = pg::device_alloc(cv->bytes);
  PG_CUDA(cudaMemcpyAsync(base, c->save_canvas.p, cv->bytes, cudaMemcpyHostToDevice, s->stream));
  pg::canvas_relayout(cv, base);
  if (b->has_snapshot) {
    void* sb = pg::device_alloc(b->snapshot.bytes);
    PG_CUDA(cudaMemcpyAsync(sb, c->save_snapshot.p, b->snapshot.bytes, cudaMemcpyHostToDevice,
                            s->stream));
    pg::layer_layout(b->snapshot, b->snapshot.rows, b->snapshot.cols, b->snapshot.storage, sb,
                     true);
  }
  PG_CUDA(cudaStreamSynchronize(s->stream));
  c->resident = true;
}

void create(painty_server* s, ServerCanvas* c) {
  painty_canvas* cv = nullptr;
  painty_status st = painty_canvas_create(c->rows, c->cols, s->opt.storage, &cv);
  if (st != PAINTY_OK) pg::fail(st, painty_last_error());
  if (!c->r0.empty())
    pg::upload_planes(cv->r0.R, 3, pg::r_type(cv->r0.storage), c->rows, c->cols, cv->wet.pitch,
                      c->r0.data(), PAINTY_HOST_F32_INTERLEAVED, s->stream);
  cv->version++;
  painty_brush* b = nullptr;
  st = painty_brush_create(8.0, s->footprint.data(), s->opt.footprint_rows,
                           s->opt.footprint_cols, &b);
  if (st != PAINTY_OK) {
    painty_canvas_destroy(cv);
    pg::fail(st, painty_last_error());
  }
  b->pickupRate = s->opt.pickup_rate;
  b->depositionRate = s->opt.deposition_rate;
  c->cv = cv;
  c->brush = b;
  c->resident = true;
  std::vector<float>().swap(c->r0);
}

// Marks a request finished (lock held).
void finish(painty_server* s, ServerRequest* r, painty_status st, const std::string& err) {
  r->status = st;
  r->error = err;
  r->state = REQ_DONE;
  r->t_done = now_s();
  if (st == PAINTY_OK)
    s->stats.completed++;
  else if (st == PAINTY_ERR_CANCELLED)
    s->stats.cancelled++;
  else
    s->stats.failed++;
  ServerCanvas* c = s->canvases[r->canvas_id].get();
  if (!c->waiting.empty() && c->waiting.front() == r->id) c->waiting.pop_front();
  c->busy = false;
  c->last_used = s->step;
  s->gen++;  // requests queued behind this one may be admitted now
}

// One scheduling round: admit what fits, paint one step of every active request, complete
// the requests whose strokes are all painted. Called with the lock held.
void worker_round(painty_server* s, std::unique_lock<std::mutex>& lk) {
  // ---- admission: pending requests in arrival order
  std::vector<ServerCanvas*> prep, evictions;
  for (auto it = s->pending.begin(); it != s->pending.end();) {
    if (static_cast<int32_t>(s->active.size()) >= s->opt.max_active) break;
    ServerRequest* r = s->reqs[*it].get();
    ServerCanvas* c = s->canvases[r->canvas_id].get();
    if (c->busy || c->waiting.empty() || c->waiting.front() != r->id) {
      ++it;  // its canvas is painting an earlier request
      continue;
    }
    if (r->cancel) {
      finish(s, r, PAINTY_ERR_CANCELLED, "cancelled before it ran");
      it = s->pending.erase(it);
      continue;
    }
    const size_t need = c->resident ? 0 : c->bytes;
    if (need > s->opt.budget_bytes) {
      finish(s, r, PAINTY_ERR_BUDGET, "canvas larger than the server's memory budget");
      it = s->pending.erase(it);
      continue;
    }
    while (s->resident + need > s->opt.budget_bytes) {  // evict idle canvases, LRU first
      ServerCanvas* lru = nullptr;
      for (auto& kv : s->canvases) {
        ServerCanvas* x = kv.second.get();
        if (x->resident && !x->busy &&
            std::find(evictions.begin(), evictions.end(), x) == evictions.end() &&
            (!lru || x->last_used < lru->last_used))
          lru = x;
      }
      if (!lru) break;
      evictions.push_back(lru);
      s->resident -= lru->bytes;
    }
    if (s->resident + need > s->opt.budget_bytes) break;  // wait for memory to free up
    s->resident += need;
    s->peak = std::max(s->peak, s->resident);
    c->busy = true;
    r->state = REQ_ACTIVE;
    if (!c->resident) prep.push_back(c);
    s->active.push_back(r->id);
    it = s->pending.erase(it);
  }
  std::vector<ServerRequest*> act;
  for (uint64_t id : s->active) act.push_back(s->reqs[id].get());
  s->step++;
  lk.unlock();

  // ---- device work (only this thread touches device state)
  std::vector<std::pair<ServerRequest*, std::string>> failures;
  std::vector<ServerRequest*> done;
  int64_t step_stamps = 0;
  try {
    for (ServerCanvas* c : evictions) evict(s, c);
    for (ServerCanvas* c : prep) {
      if (!c->cv) {
        create(s, c);
      } else {
        restore(s, c);
        s->stats.restores++;
      }
    }
    s->stats.evictions += static_cast<int64_t>(evictions.size());
    // the next slice of every active request, one batched launch
    std::vector<painty_canvas*> cvs;
    std::vector<painty_brush*> brs;
    std::vector<painty_stroke_desc> descs;
    std::vector<double> pts;
    std::vector<std::pair<ServerRequest*, size_t>> slice;  // request, strokes taken
    for (ServerRequest* r : act) {
      ServerCanvas* c = s->canvases[r->canvas_id].get();
      size_t k = r->next;
      int64_t budget = 0;
      while (k < r->strokes.size() && (k == r->next || budget + r->stroke_stamps[k] <= s->opt.step_stamps)) {
        budget += r->stroke_stamps[k];
        k++;
      }
      const int32_t ci = static_cast<int32_t>(cvs.size());
      if (k > r->next) {
        cvs.push_back(c->cv);
        brs.push_back(c->brush);
        for (size_t j = r->next; j < k; j++) {
          painty_stroke_desc d = r->strokes[j];
          const double* p = r->points.data() + 2 * d.first_point;
          d.canvas = ci;
          d.first_point = static_cast<int64_t>(pts.size() / 2);
          pts.insert(pts.end(), p, p + 2 * d.npoints);
          descs.push_back(d);
        }
      }
      slice.emplace_back(r, k - r->next);
    }
    if (!cvs.empty()) {
      pg::paint_batch(cvs.data(), brs.data(), static_cast<int32_t>(cvs.size()), descs.data(),
                      static_cast<int64_t>(descs.size()), pts.data(),
                      static_cast<int64_t>(pts.size() / 2), &step_stamps, s->stream);
    }
    for (auto& sl : slice) {
      ServerRequest* r = sl.first;
      for (size_t j = r->next; j < r->next + sl.second; j++) r->stamps += r->stroke_stamps[j];
      r->next += sl.second;
      if (r->next == r->strokes.size() || r->cancel) done.push_back(r);
    }
    for (ServerRequest* r : done) {  // composite into the caller's buffer
      if (r->cancel || !r->out_rgb) continue;
      ServerCanvas* c = s->canvases[r->canvas_id].get();
      painty_image* img = nullptr;
      const painty_storage rs =
        s->opt.storage == PAINTY_STORAGE_F64 ? PAINTY_STORAGE_F64 : PAINTY_STORAGE_F32;
      if (painty_image_create(c->rows, c->cols, rs, &img) != PAINTY_OK)
        pg::fail(PAINTY_ERR_OUT_OF_MEMORY, painty_last_error());
      const painty_layer* L[1] = {&c->cv->wet};
      try {
        pg::launch_compose(L, 1, &c->cv->r0, img, s->stream);
        const void* p[3] = {img->R[0], img->R[1], img->R[2]};
        // out_rgb is float RGB whatever the storage (F64 results are rounded to float)
        pg::download_planes(p, 3, pg::r_type(rs), c->rows, c->cols, img->pitch, r->out_rgb,
                            PAINTY_HOST_F32_INTERLEAVED, s->stream);
      } catch (...) {
        painty_image_destroy(img);
        throw;
      }
      painty_image_destroy(img);
    }
  } catch (const std::exception& e) {
    for (ServerRequest* r : act) failures.emplace_back(r, e.what());
  }

  lk.lock();
  s->stats.steps++;
  s->stats.stamps += step_stamps;
  if (!failures.empty()) {
    for (auto& f : failures) {
      finish(s, f.first, PAINTY_ERR_CUDA, f.second);
      s->active.erase(std::find(s->active.begin(), s->active.end(), f.first->id));
    }
  } else {
    for (ServerRequest* r : done) {
      finish(s, r, r->cancel ? PAINTY_ERR_CANCELLED : PAINTY_OK,
             r->cancel ? "cancelled while painting" : "");
      s->active.erase(std::find(s->active.begin(), s->active.end(), r->id));
    }
  }
  s->cv_done.notify_all();
}

void worker_main(painty_server* s) {
  cudaSetDevice(s->device);
  std::unique_lock<std::mutex> lk(s->mu);
  uint64_t idle_gen = ~0ull;
  while (true) {
    s->cv_work.wait(lk, [&] {
      return s->stop || !s->active.empty() || (!s->pending.empty() && s->gen != idle_gen);
    });
    if (s->stop) break;
    const uint64_t g = s->gen;
    worker_round(s, lk);
    // nothing admitted and nothing painting: sleep until a submit or cancel changes things
    idle_gen = s->active.empty() ? g : ~0ull;
  }
  // shutting down: every unfinished request is cancelled
  for (uint64_t id : s->pending) finish(s, s->reqs[id].get(), PAINTY_ERR_CANCELLED, "server shut down");
  for (uint64_t id : s->active) finish(s, s->reqs[id].get(), PAINTY_ERR_CANCELLED, "server shut down");
  s->pending.clear();
  s->active.clear();
  s->cv_done.notify_all();
}

}  // namespace

using pg::guard;

extern "C" {

painty_status painty_server_create(const painty_server_options* opt, painty_server** out) {
  return guard([&] {
    PG_REQUIRE(opt && out, "null argument");
    PG_REQUIRE(pg::valid_storage(opt->storage), "unknown storage format");
    PG_REQUIRE(opt->budget_bytes > 0, "the memory budget must be positive");
    PG_REQUIRE(opt->footprint && opt->footprint_rows > 0 && opt->footprint_cols > 0,
               "footprint image is empty");
    auto s = std::make_unique<painty_server>();
    s->opt = *opt;
    if (s->opt.max_active <= 0) s->opt.max_active = 256;
    if (s->opt.step_stamps <= 0) s->opt.step_stamps = 16384;
    s->footprint.assign(opt->footprint,
                        opt->footprint + static_cast<size_t>(opt->footprint_rows) * opt->footprint_cols);
    s->opt.footprint = nullptr;
    PG_CUDA(cudaGetDevice(&s->device));
    PG_CUDA(cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking));
    painty_server* raw = s.get();
    s->worker = std::thread(worker_main, raw);
    *out = s.release();
  });
}

painty_status painty_server_submit(painty_server* s, const painty_request* req,
                                   uint64_t* request_id, uint64_t* canvas_id) {
  return guard([&] {
    PG_REQUIRE(s && req, "null argument");
    PG_REQUIRE(req->nstrokes >= 0 && (req->nstrokes == 0 || req->strokes), "strokes is null");
    PG_REQUIRE(req->npoints >= 0 && (req->npoints == 0 || req->points), "points is null");
    auto r = std::make_unique<ServerRequest>();
    r->strokes.assign(req->strokes, req->strokes + req->nstrokes);
    r->points.assign(req->points, req->points + 2 * req->npoints);
    for (const auto& d : r->strokes) {
      PG_REQUIRE(d.npoints >= 0 && d.npoints <= 512 && d.first_point >= 0 &&
                   d.first_point + d.npoints <= req->npoints,
                 "stroke points out of range");
      PG_REQUIRE(std::isfinite(d.radius) && d.radius >= 0.0, "radius must be finite and >= 0");
      PG_REQUIRE(std::isfinite(d.spacing) && d.spacing > 0.0, "spacing must be positive");
      r->stroke_stamps.push_back(
        pg::stroke_stamp_count(r->points.data() + 2 * d.first_point, d.npoints, d.spacing));
    }
    for (double v : r->points) PG_REQUIRE(std::isfinite(v), "path coordinates must be finite");
    r->out_rgb = req->out_rgb;
    r->t_submit = now_s();
    std::lock_guard<std::mutex> lk(s->mu);
    PG_REQUIRE(!s->stop, "server is shutting down");
    ServerCanvas* c = nullptr;
    if (req->canvas_id == 0) {
      PG_REQUIRE(req->rows > 0 && req->cols > 0, "a new canvas needs rows and cols");
      auto nc = std::make_unique<ServerCanvas>();
      nc->id = s->next_canvas++;
      nc->rows = req->rows;
      nc->cols = req->cols;
      nc->bytes = canvas_device_bytes(s, req->rows, req->cols);
      if (req->r0)
        nc->r0.assign(req->r0, req->r0 + static_cast<size_t>(req->rows) * req->cols * 3);
      c = nc.get();
      s->canvases.emplace(nc->id, std::move(nc));
    } else {
      auto it = s->canvases.find(req->canvas_id);
      PG_REQUIRE(it != s->canvases.end(), "unknown canvas id");
      c = it->second.get();
    }
    r->id = s->next_req++;
    r->canvas_id = c->id;
    c->waiting.push_back(r->id);
    s->pending.push_back(r->id);
    s->stats.submitted++;
    s->gen++;
    if (request_id) *request_id = r->id;
    if (canvas_id) *canvas_id = c->id;
    s->reqs.emplace(r->id, std::move(r));
    s->cv_work.notify_one();
  });
}

painty_status painty_server_wait(painty_server* s, uint64_t request_id, double timeout_s,
                                 double* latency_s, int64_t* stamps) {
  painty_status result = PAINTY_OK;
  const painty_status st = guard([&] {
    PG_REQUIRE(s != nullptr, "server is null");
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->reqs.find(request_id);
    PG_REQUIRE(it != s->reqs.end(), "unknown request id");
    ServerRequest* r = it->second.get();
    const auto pred = [&] { return r->state == REQ_DONE; };
    if (timeout_s < 0)
      s->cv_done.wait(lk, pred);
    else if (!s->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), pred)) {
      result = PAINTY_ERR_TIMEOUT;
      pg::set_last_error("request not finished within the timeout");
      return;
    }
    if (latency_s) *latency_s = r->t_done - r->t_submit;
    if (stamps) *stamps = r->stamps;
    result = r->status;
    if (r->status != PAINTY_OK) pg::set_last_error(r->error);
  });
  return st != PAINTY_OK ? st : result;
}

painty_status painty_server_cancel(painty_server* s, uint64_t request_id) {
  return guard([&] {
    PG_REQUIRE(s != nullptr, "server is null");
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->reqs.find(request_id);
    PG_REQUIRE(it != s->reqs.end(), "unknown request id");
    ServerRequest* r = it->second.get();
    if (r->state == REQ_DONE) return;
    r->cancel = true;
    s->gen++;
    s->cv_work.notify_one();
  });
}

painty_status painty_server_stats(painty_server* s, painty_server_counters* out) {
  return guard([&] {
    PG_REQUIRE(s && out, "null argument");
    std::lock_guard<std::mutex> lk(s->mu);
    *out = s->stats;
    out->resident_bytes = s->resident;
    out->peak_resident_bytes = s->peak;
    out->active = static_cast<int64_t>(s->active.size());
    out->pending = static_cast<int64_t>(s->pending.size());
    out->canvases = static_cast<int64_t>(s->canvases.size());
  });
}

painty_status painty_server_destroy(painty_server* s) {
  return guard([&] {
    if (!s) return;
    {
      std::lock_guard<std::mutex> lk(s->mu);
      s->stop = true;
    }
    s->cv_work.notify_all();
    if (s->worker.joinable()) s->worker.join();
    for (auto& kv : s->canvases) {
      ServerCanvas* c = kv.second.get();
      if (c->brush) painty_brush_destroy(c->brush);
      if (c->cv) {
        if (c->resident) painty_canvas_destroy(c->cv);
        else delete c->cv;  // evicted: no device memory left to free
      }
    }
    cudaStreamDestroy(s->stream);
    delete s;
  });
}

}  // extern "C"
