// server.cu -- continuous-batching stroke-render server.
//
// Requests (paint these strokes on a new canvas, or continue a canvas an earlier request
// created) arrive at any time. A worker thread admits each one as soon as a slot (a stream
// with its event and status word) and device memory allow, and runs it as a chain of
// stamp-kernel launches on its slot's stream: each launch paints the request's next
// `step_stamps` stamps (whole strokes) with the batched stamp kernel. Launches of different
// requests run concurrently on the device -- nothing waits for a step of the whole server --
// so a request that arrives while others are painting starts as soon as it is admitted. The
// worker polls each slot's completion word, which the slot's last kernel writes into pinned
// host memory: a finished chunk is followed by the next one, a finished request by the KM
// composite of its canvas (Renderer::compose, painty/renderer/Renderer.hxx:26-53) written
// straight into the caller's pinned buffer, or composited and downloaded in the slot's stream
// order when that buffer is pageable.
//
// Canvases stay resident on the device between requests. Their memory (canvas, composite
// image, brush buffers) is carved on the host from one device reservation made when the
// server starts, so creating and dropping canvases calls no CUDA allocator; memory
// is returned only when the GPU has finished with it (a canvas after its last request).
// Admission keeps the resident bytes under a budget by evicting idle canvases (least recently
// used first) to pinned host memory and restoring them when a later request continues them. A canvas's requests run one after another, in
// submission order; different canvases are independent, so a request's result does not
// depend on what else is in flight. painty_server_release drops a canvas once its queued
// requests are done.
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "device_common.cuh"
#include "internal.h"

namespace {

double now_s() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch())
    .count();
}

enum ReqState { REQ_PENDING = 0, REQ_ACTIVE = 1, REQ_DONE = 2 };
enum Phase { PH_PAINT = 0, PH_FINISH = 1 };

struct HostBlob {  // pinned host memory holding an evicted device allocation
  void* p = nullptr;
  size_t bytes = 0;
};

struct ServerCanvas {
  uint64_t id = 0;
  int32_t rows = 0, cols = 0;
  painty_canvas* cv = nullptr;  // created by the canvas's first request
  painty_brush* brush = nullptr;
  painty_image img{};           // the composite of the canvas (resident with it)
  bool resident = false;
  bool busy = false;     // one of its requests is admitted
  bool release = false;  // drop the canvas once its queued requests are done
  bool dropped = false;  // released and freed
  uint64_t last_used = 0;
  size_t bytes = 0;  // device bytes when resident
  std::vector<float> r0;  // substrate until the canvas is created (a copy of pageable memory)
  const float* r0_pinned = nullptr;  // or the caller's pinned substrate
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
  int phase = PH_PAINT;
  int slot = -1;
  bool cancel = false;
  painty_status status = PAINTY_OK;
  std::string error;
  int64_t stamps = 0;
  int64_t total_stamps = 0;  // of all its strokes
  double t_submit = 0, t_done = 0;
  int64_t remaining() const { return total_stamps - stamps; }
};

// A request with more stamps than this left is "long": its serial chain sets the tail latency.
constexpr int64_t kLongRequest = 200000;

// Pinned staging per slot for a launch's descriptors (a chunk of strokes: their descriptors
// and path points); larger chunks are copied from pageable memory.
constexpr size_t kStagingBytes = 128 << 10;

struct Slot {
  cudaStream_t st = nullptr;
  cudaEvent_t ev = nullptr;
  unsigned* status = nullptr;  // pinned: the last launch's kernel status word
  // pinned completion word: the slot's self-signalling kernels store `seq` into it when their
  // results are visible, and the worker polls it (nothing is queued behind those kernels: an
  // item waiting on a long kernel holds back other streams' work in the device's queues)
  unsigned* done = nullptr;
  unsigned* done_dev = nullptr;  // its device address
  unsigned seq = 0;
  double armed_at = 0.0;
  unsigned* d_counter = nullptr;  // device: finish kernel's count of finished blocks
  void* staging = nullptr;     // pinned: the last launch's descriptors (kStagingBytes)
  void* d_desc = nullptr;      // device: the launch's descriptors (kStagingBytes)
  void* d_scratch = nullptr;   // device: the launch's scratch, grown to what launches need
  size_t d_scratch_bytes = 0;
  bool busy = false;
  painty_server* owner = nullptr;
  int index = 0;
};

}  // namespace

struct painty_server {
  painty_server_options opt{};
  std::vector<double> footprint;
  int device = 0;
  int sms = 0;
  cudaStream_t stream = nullptr;  // creation, eviction and restore
  std::unique_ptr<pg::DeviceHeap> heap;  // canvases, images, brush buffers, slot buffers
  std::vector<Slot> slots;
  unsigned* status_words = nullptr;
  unsigned* done_words = nullptr;
  unsigned char* staging = nullptr;  // pinned, kStagingBytes per slot
  std::vector<int> watch;  // slots whose self-signalling launch is in flight (worker only)
  std::multimap<size_t, void*> pinned_free;  // pinned blobs of released canvases, by size
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<uint64_t> pending;
  std::deque<uint64_t> finished;  // completion order, for painty_server_poll
  std::vector<uint64_t> active;
  std::unordered_map<uint64_t, std::unique_ptr<ServerRequest>> reqs;
  std::unordered_map<uint64_t, std::unique_ptr<ServerCanvas>> canvases;
  std::vector<ServerCanvas*> to_drop;  // released canvases waiting for the worker to free them
  std::vector<int> passed;  // slots whose stream reached the end of their last launch
  size_t resident = 0, peak = 0;
  uint64_t next_req = 1, next_canvas = 1, tick = 0;
  painty_server_counters stats{};
  bool stop = false;
  uint64_t gen = 0;  // bumped by submit, cancel, release and finish
  std::thread worker;
};

namespace {

painty_storage image_storage(const painty_server* s) {
  return s->opt.storage == PAINTY_STORAGE_F64 ? PAINTY_STORAGE_F64 : PAINTY_STORAGE_F32;
}

size_t canvas_device_bytes(const painty_server* s, int32_t rows, int32_t cols) {
  const painty_storage st = s->opt.storage;
  const painty_storage rs = image_storage(s);
  const size_t pe = static_cast<size_t>(rows) * pg::pitch_for(cols);
  return pg::layer_bytes(rows, cols, st, true) + 2 * pg::image_bytes(rows, cols, rs) +
         pe * pg::v_bytes(st) + pg::layer_bytes(rows, cols, st, true) /* snapshot */ +
         (4u << 20) /* pickup map, footprint, scratch */;
}

// Pinned host memory for an eviction: a released canvas's blob of at least that size, or a
// new one.
void* pinned_take(painty_server* s, size_t bytes, size_t* got) {
  auto it = s->pinned_free.lower_bound(bytes);
  if (it != s->pinned_free.end() && it->first <= 2 * bytes) {
    void* p = it->second;
    *got = it->first;
    s->pinned_free.erase(it);
    return p;
  }
  void* p = nullptr;
  PG_CUDA(cudaMallocHost(&p, bytes));
  *got = bytes;
  return p;
}

void blob_save(painty_server* s, HostBlob& b, const void* dev, size_t bytes) {
  if (!b.p || b.bytes < bytes) {
    if (b.p) s->pinned_free.emplace(b.bytes, b.p);
    b.p = pinned_take(s, bytes, &b.bytes);
  }
  PG_CUDA(cudaMemcpyAsync(b.p, dev, bytes, cudaMemcpyDeviceToHost, s->stream));
}

// Host callback at the end of a slot's launched work: the worker learns of it without polling.
void CUDART_CB slot_passed(void* p) {
  Slot* sl = static_cast<Slot*>(p);
  painty_server* s = sl->owner;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->passed.push_back(sl->index);
  }
  s->cv_work.notify_one();
}

// Marks the end of the work just queued on a slot: its event and the callback after it.
void mark_slot(Slot& sl) {
  PG_CUDA(cudaEventRecord(sl.ev, sl.st));
  PG_CUDA(cudaLaunchHostFunc(sl.st, slot_passed, &sl));
}

// The next completion value of a slot whose launch signals by itself (worker thread).
unsigned arm_slot(painty_server* s, Slot& sl) {
  sl.seq++;
  sl.armed_at = now_s();
  s->watch.push_back(sl.index);
  return sl.seq;
}

// Slots whose completion word caught up with their launch (worker thread, lock held).
void poll_watched(painty_server* s) {
  for (size_t i = 0; i < s->watch.size();) {
    Slot& sl = s->slots[s->watch[i]];
    bool passed = *reinterpret_cast<volatile unsigned*>(sl.done) == sl.seq;
    if (!passed && now_s() - sl.armed_at > 2.0) {
      // a long launch: make sure the stream has not failed (a failed stream never signals)
      const cudaError_t q = cudaStreamQuery(sl.st);
      if (q != cudaErrorNotReady) {
        if (q != cudaSuccess) *sl.status = 1u << 31;  // reported as an internal error
        passed = true;
      }
      sl.armed_at = now_s();
    }
    if (passed) {
      std::atomic_thread_fence(std::memory_order_acquire);  // then its status and results
      s->passed.push_back(sl.index);
      s->watch[i] = s->watch.back();
      s->watch.pop_back();
    } else {
      i++;
    }
  }
}

template <class TK, class TV>
struct LayerView {
  const TK* K[3];
  const TK* S[3];
  const TV* V;
  int64_t es;  // element stride (8: packed pixel records)
};

// The composite of a canvas (its wet layer over R0, Renderer::compose of one layer,
// painty/renderer/Renderer.hxx:26-53) written as float RGB straight into pinned host memory,
// one grid-stride pass; the last block to finish stores `value` into the completion word.
template <class TK, class TV, class M>
__global__ void finish_kernel(LayerView<TK, TV> w, const M* __restrict__ r0r,
                              const M* __restrict__ r0g, const M* __restrict__ r0b, int32_t rows,
                              int32_t cols, int64_t wpitch, int64_t rpitch,
                              float* __restrict__ out, unsigned* counter, unsigned* done,
                              unsigned value) {
  const int64_t n = static_cast<int64_t>(rows) * cols;
  for (int64_t p = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; p < n;
       p += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int64_t r = p / cols, c = p - r * cols;
    const int64_t j = (r * wpitch + c) * w.es, e = r * rpitch + c;
    const M d = pg::ld_elem<M>(w.V + j);
    const M R[3] = {r0r[e], r0g[e], r0b[e]};
#pragma unroll
    for (int ch = 0; ch < 3; ch++)
      out[p * 3 + ch] = static_cast<float>(
        pg::km_reflectance(pg::ld_elem<M>(w.K[ch] + j), pg::ld_elem<M>(w.S[ch] + j), R[ch], d));
  }
  __threadfence_system();  // this thread's results before the block's count
  __syncthreads();
  if (threadIdx.x == 0 && atomicAdd(counter, 1u) == gridDim.x - 1) {
    __threadfence_system();
    *reinterpret_cast<volatile unsigned*>(done) = value;
    __threadfence_system();
  }
}

void image_alloc(painty_server* s, ServerCanvas* c, cudaStream_t st) {
  const painty_storage rs = image_storage(s);
  void* base = s->heap->alloc(pg::image_bytes(c->rows, c->cols, rs), st);
  pg::image_layout(c->img, c->rows, c->cols, rs, base);
  c->img.owned = false;
}

void image_free(painty_server* s, ServerCanvas* c) {
  s->heap->free(c->img.base, s->stream);
  c->img.base = nullptr;
}

// Moves a canvas's device state (canvas planes and the brush's snapshot) to pinned host
// memory and frees it on the device. Called by the worker for idle canvases only.
void evict(painty_server* s, ServerCanvas* c) {
  painty_canvas* cv = c->cv;
  painty_brush* b = c->brush;
  b->heap_stream = s->stream;
  blob_save(s, c->save_canvas, cv->base, cv->bytes);
  if (b->has_snapshot) blob_save(s, c->save_snapshot, b->snapshot.base, b->snapshot.bytes);
  PG_CUDA(cudaStreamSynchronize(s->stream));
  s->heap->free(cv->base, s->stream);
  pg::canvas_relayout(cv, nullptr);
  if (b->has_snapshot) {
    s->heap->free(b->snapshot.base, s->stream);
    b->snapshot.base = nullptr;
  }
  image_free(s, c);
  c->resident = false;
}

void restore(painty_server* s, ServerCanvas* c) {
  painty_canvas* cv = c->cv;
  painty_brush* b = c->brush;
  b->heap_stream = s->stream;
  void* base = s->heap->alloc(cv->bytes, s->stream);
  PG_CUDA(cudaMemcpyAsync(base, c->save_canvas.p, cv->bytes, cudaMemcpyHostToDevice, s->stream));
  pg::canvas_relayout(cv, base);
  if (b->has_snapshot) {
    void* sb = s->heap->alloc(b->snapshot.bytes, s->stream);
    PG_CUDA(cudaMemcpyAsync(sb, c->save_snapshot.p, b->snapshot.bytes, cudaMemcpyHostToDevice,
                            s->stream));
    pg::layer_layout(b->snapshot, b->snapshot.rows, b->snapshot.cols, b->snapshot.storage, sb,
                     true);
  }
  image_alloc(s, c, s->stream);
  PG_CUDA(cudaStreamSynchronize(s->stream));
  c->resident = true;
}

// A new canvas, its substrate and its brush, all in the order of `st` (the stream of the
// request that creates it; nothing waits).
void create(painty_server* s, ServerCanvas* c, cudaStream_t st) {
  painty_canvas* cv = pg::canvas_create_on(c->rows, c->cols, s->opt.storage, s->heap.get(), st,
                                           false);
  try {
    const float* r0 = c->r0_pinned ? c->r0_pinned : (c->r0.empty() ? nullptr : c->r0.data());
    if (r0)
      pg::upload_planes_async(cv->r0.R, 3, pg::r_type(cv->r0.storage), c->rows, c->cols,
                              cv->wet.pitch, r0, PAINTY_HOST_F32_INTERLEAVED, st);
    cv->version++;
    painty_brush* b = nullptr;
    const painty_status bst = painty_brush_create(8.0, s->footprint.data(),
                                                  s->opt.footprint_rows, s->opt.footprint_cols, &b);
    if (bst != PAINTY_OK) pg::fail(bst, painty_last_error());
    b->pickupRate = s->opt.pickup_rate;
    b->depositionRate = s->opt.deposition_rate;
    b->heap = s->heap.get();
    b->heap_stream = st;
    c->brush = b;
  } catch (...) {
    cudaStreamSynchronize(st);  // its memory is reused at once: let queued work finish
    pg::canvas_destroy_on(cv, s->heap.get(), st);
    throw;
  }
  c->cv = cv;
  image_alloc(s, c, st);
  c->resident = true;
  std::vector<float>().swap(c->r0);  // a pageable source was copied out during the call
}

// Frees a released canvas (worker thread; nothing of it is in flight).
void drop(painty_server* s, ServerCanvas* c) {
  if (c->brush) {
    c->brush->heap_stream = s->stream;
    painty_brush_destroy(c->brush);
  }
  if (c->cv) {
    if (c->resident) {
      image_free(s, c);
      pg::canvas_destroy_on(c->cv, s->heap.get(), s->stream);
    } else {
      delete c->cv;  // evicted: no device memory left to free
    }
  }
  for (HostBlob* b : {&c->save_canvas, &c->save_snapshot}) {
    if (b->p) s->pinned_free.emplace(b->bytes, b->p);
    *b = HostBlob{};
  }
  c->brush = nullptr;
  c->cv = nullptr;
  c->resident = false;
  c->dropped = true;
}

// Marks a request finished (lock held).
void finish(painty_server* s, ServerRequest* r, painty_status st, const std::string& err) {
  r->status = st;
  r->error = err;
  r->state = REQ_DONE;
  r->t_done = now_s();
  s->finished.push_back(r->id);
  if (st == PAINTY_OK)
    s->stats.completed++;
  else if (st == PAINTY_ERR_CANCELLED)
    s->stats.cancelled++;
  else
    s->stats.failed++;
  ServerCanvas* c = s->canvases[r->canvas_id].get();
  if (!c->waiting.empty() && c->waiting.front() == r->id) c->waiting.pop_front();
  c->busy = false;
  c->last_used = s->tick;
  if (r->slot >= 0) s->slots[r->slot].busy = false;
  r->slot = -1;
  if (c->release && c->waiting.empty() && !c->busy) {
    if (c->resident) s->resident -= c->bytes;
    s->to_drop.push_back(c);
  }
  s->gen++;  // requests queued behind this one may be admitted now
}

// Cluster cap for a launch: larger clusters shorten one canvas's chain of stamps, single CTAs
// paint the most canvases at once, so the cap shrinks as more requests are in flight.
int cluster_cap(const painty_server* s) {
  const int inflight = static_cast<int>(s->active.size());
  for (int c : {8, 4, 2})
    if (inflight * c <= s->sms) return c;
  return 1;
}

// Launches the next chunk of a request's strokes (worker thread, lock not held).
void launch_chunk(painty_server* s, ServerRequest* r, ServerCanvas* c, int cap) {
  const double t0 = now_s();
  Slot& sl = s->slots[r->slot];
  size_t k = r->next;
  int64_t budget = 0;
  while (k < r->strokes.size() &&
         (k == r->next || budget + r->stroke_stamps[k] <= s->opt.step_stamps)) {
    budget += r->stroke_stamps[k];
    k++;
  }
  std::vector<painty_stroke_desc> descs;
  std::vector<double> pts;
  for (size_t j = r->next; j < k; j++) {
    painty_stroke_desc d = r->strokes[j];
    const double* p = r->points.data() + 2 * d.first_point;
    d.canvas = 0;
    d.first_point = static_cast<int64_t>(pts.size() / 2);
    pts.insert(pts.end(), p, p + 2 * d.npoints);
    descs.push_back(d);
  }
  *sl.status = 0;
  pg::BatchOptions opt;
  opt.max_cluster = cap;
  opt.status_host = sl.status;
  opt.host_staging = sl.staging;  // the slot's previous launch finished before this one
  opt.host_staging_bytes = kStagingBytes;
  if (!sl.d_desc) sl.d_desc = s->heap->alloc(kStagingBytes, sl.st);
  opt.device_desc = sl.d_desc;
  opt.device_desc_bytes = kStagingBytes;
  opt.device_scratch = sl.d_scratch;
  opt.device_scratch_bytes = sl.d_scratch_bytes;
  size_t scratch_needed = 0;
  opt.scratch_needed = &scratch_needed;
  opt.done_host = sl.done;  // the kernel signals its own completion
  opt.done_value = arm_slot(s, sl);
  c->brush->heap_stream = sl.st;
  int64_t n = 0;
  painty_canvas* cvs[1] = {c->cv};
  painty_brush* brs[1] = {c->brush};
  pg::paint_batch(cvs, brs, 1, descs.data(), static_cast<int64_t>(descs.size()), pts.data(),
                  static_cast<int64_t>(pts.size() / 2), &n, sl.st, &opt);
  if (scratch_needed > sl.d_scratch_bytes) {
    // this launch used a temporary; the slot's buffer (last used by a finished launch) grows
    // for the next one
    s->heap->free(sl.d_scratch, sl.st);
    sl.d_scratch_bytes = (scratch_needed + (64 << 10) - 1) / (64 << 10) * (64 << 10);
    sl.d_scratch = s->heap->alloc(sl.d_scratch_bytes, sl.st);
  }
  r->stamps += budget;
  r->next = k;
  s->stats.worker_launch_us += static_cast<int64_t>((now_s() - t0) * 1e6);
}

template <class TK, class TV, class M>
void launch_finish_kernel(painty_server* s, Slot& sl, ServerCanvas* c, float* out_dev,
                          unsigned value) {
  const painty_layer& wet = c->cv->wet;
  const painty_image& r0 = c->cv->r0;
  LayerView<TK, TV> w{};
  for (int i = 0; i < 3; i++) {
    w.K[i] = static_cast<const TK*>(wet.K[i]);
    w.S[i] = static_cast<const TK*>(wet.S[i]);
  }
  w.V = static_cast<const TV*>(wet.V);
  w.es = wet.estride;
  PG_CUDA(cudaMemsetAsync(sl.d_counter, 0, sizeof(unsigned), sl.st));
  const int64_t n = static_cast<int64_t>(c->rows) * c->cols;
  const int grid = static_cast<int>(std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256,
                                                                          int64_t(s->sms) * 8)));
  finish_kernel<TK, TV, M><<<grid, 256, 0, sl.st>>>(
    w, static_cast<const M*>(r0.R[0]), static_cast<const M*>(r0.R[1]),
    static_cast<const M*>(r0.R[2]), c->rows, c->cols, wet.pitch, r0.pitch, out_dev,
    sl.d_counter, sl.done_dev, value);
  pg::count_launch();
  PG_CUDA(cudaGetLastError());
}

// The composite of a finished request's canvas into the caller's buffer, in the slot's
// stream order (worker thread): computed straight into a pinned buffer by one kernel that
// signals its completion word, or composed on the device and downloaded (pageable buffers).
void launch_finish(painty_server* s, ServerRequest* r, ServerCanvas* c) {
  const double t0 = now_s();
  Slot& sl = s->slots[r->slot];
  // out_rgb is float RGB whatever the storage (F64 results are rounded to float)
  float* out_dev = static_cast<float*>(const_cast<void*>(pg::mapped_host(r->out_rgb)));
  if (out_dev) {
    const unsigned v = arm_slot(s, sl);
    switch (s->opt.storage) {
      case PAINTY_STORAGE_F16: launch_finish_kernel<__half, __half, float>(s, sl, c, out_dev, v); break;
      case PAINTY_STORAGE_BF16:
        launch_finish_kernel<__nv_bfloat16, __half, float>(s, sl, c, out_dev, v);
        break;
      case PAINTY_STORAGE_F64: launch_finish_kernel<double, double, double>(s, sl, c, out_dev, v); break;
      default: launch_finish_kernel<float, float, float>(s, sl, c, out_dev, v); break;
    }
  } else {
    const painty_layer* L[1] = {&c->cv->wet};
    pg::launch_compose(L, 1, &c->cv->r0, &c->img, sl.st);
    const void* p[3] = {c->img.R[0], c->img.R[1], c->img.R[2]};
    pg::download_planes_async(p, 3, pg::r_type(c->img.storage), c->rows, c->cols, c->img.pitch,
                              r->out_rgb, PAINTY_HOST_F32_INTERLEAVED, sl.st);
    mark_slot(sl);
  }
  s->stats.worker_finish_us += static_cast<int64_t>((now_s() - t0) * 1e6);
}

struct Admitted {
  ServerRequest* r;
  ServerCanvas* c;
  bool prep;  // create or restore the canvas first
};

// One pass of the worker: admit what fits, start admitted requests, advance every request
// whose slot's work has finished. Called with the lock held; returns whether anything moved.
bool worker_round(painty_server* s, std::unique_lock<std::mutex>& lk) {
  // ---- drops and admission (lock held): pending requests in arrival order
  std::vector<ServerCanvas*> drops;
  drops.swap(s->to_drop);
  std::vector<ServerCanvas*> evictions;
  std::vector<Admitted> admitted;
  int free_slots = 0;
  for (const Slot& sl : s->slots) free_slots += sl.busy ? 0 : 1;
  for (auto it = s->pending.begin(); it != s->pending.end() && free_slots > 0;) {
    ServerRequest* r = s->reqs[*it].get();
    ServerCanvas* c = s->canvases[r->canvas_id].get();
    if (c->busy || c->waiting.empty() || c->waiting.front() != r->id) {
      ++it;  // its canvas is painting an earlier request
      continue;
    }
    if (std::find(evictions.begin(), evictions.end(), c) != evictions.end()) {
      ++it;  // chosen for eviction in this pass: it is admitted (and restored) in a later one
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
        if (x->resident && !x->busy && !x->release &&
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
    r->phase = PH_PAINT;
    for (int i = 0; i < static_cast<int>(s->slots.size()); i++)
      if (!s->slots[i].busy) {
        s->slots[i].busy = true;
        r->slot = i;
        break;
      }
    free_slots--;
    admitted.push_back({r, c, !c->resident});
    s->active.push_back(r->id);
    it = s->pending.erase(it);
  }
  // requests in flight and their cancel flags, as of now
  struct Running {
    ServerRequest* r;
    ServerCanvas* c;
    bool cancel;
  };
  std::vector<Running> running;
  std::vector<int> passed;
  poll_watched(s);
  passed.swap(s->passed);
  if (!passed.empty()) {
    std::vector<ServerRequest*> by_slot(s->slots.size(), nullptr);
    for (uint64_t id : s->active) {
      ServerRequest* r = s->reqs[id].get();
      if (r->slot >= 0) by_slot[r->slot] = r;
    }
    for (int slot : passed) {
      ServerRequest* r = by_slot[slot];
      bool fresh = false;
      for (const Admitted& a : admitted) fresh = fresh || a.r == r;
      if (r && !fresh) running.push_back({r, s->canvases[r->canvas_id].get(), r->cancel});
    }
  }
  int cap = cluster_cap(s);
  // no queue: the GPU has room, so a long request's chain may take a large cluster (its
  // latency, the server's p99, is that chain); under a backlog throughput comes first
  const int long_cap = s->pending.empty() ? 8 : cap;
  s->tick++;
  lk.unlock();

  // ---- device work (only this thread touches device state)
  const double t_work = now_s();
  std::vector<std::pair<ServerRequest*, std::string>> failures;
  std::vector<ServerRequest*> done;
  bool moved = !admitted.empty() || !drops.empty();
  int64_t chunks = 0;
  for (ServerCanvas* c : drops) drop(s, c);
  try {
    for (ServerCanvas* c : evictions) evict(s, c);
  } catch (const std::exception& e) {  // the canvases stay resident; their bytes count again
    lk.lock();
    for (ServerCanvas* c : evictions)
      if (c->resident) s->resident += c->bytes;
    lk.unlock();
    for (const Admitted& a : admitted) failures.emplace_back(a.r, e.what());
    admitted.clear();
  }
  for (const Admitted& a : admitted) {
    try {
      if (a.prep) {
        if (!a.c->cv) {
          const double t = now_s();
          create(s, a.c, s->slots[a.r->slot].st);
          s->stats.worker_create_us += static_cast<int64_t>((now_s() - t) * 1e6);
        } else {
          restore(s, a.c);
          s->stats.restores++;
        }
      }
      if (a.r->strokes.empty()) {
        a.r->phase = PH_FINISH;
        if (a.r->out_rgb)
          launch_finish(s, a.r, a.c);
        else
          mark_slot(s->slots[a.r->slot]);
      } else {
        launch_chunk(s, a.r, a.c, a.r->remaining() > kLongRequest ? long_cap : cap);
        chunks++;
      }
    } catch (const std::exception& e) {
      failures.emplace_back(a.r, e.what());
    }
  }
  s->stats.evictions += static_cast<int64_t>(evictions.size());
  for (const Running& x : running) {
    ServerRequest* r = x.r;
    const cudaError_t q = cudaEventQuery(s->slots[r->slot].ev);
    if (q == cudaErrorNotReady) continue;
    moved = true;
    try {
      PG_CUDA(q);
      if (r->phase == PH_FINISH) {
        done.push_back(r);
        continue;
      }
      if (*s->slots[r->slot].status != 0)
        pg::fail(PAINTY_ERR_CUDA, "batched stamp kernel reported an internal error");
      if (r->next < r->strokes.size() && !x.cancel) {
        launch_chunk(s, r, x.c, r->remaining() > kLongRequest ? long_cap : cap);
        chunks++;
      } else if (r->out_rgb && !x.cancel) {
        r->phase = PH_FINISH;
        launch_finish(s, r, x.c);
      } else {
        done.push_back(r);
      }
    } catch (const std::exception& e) {
      failures.emplace_back(r, e.what());
    }
  }

  // a failed request's slot is not reused before its stream has drained (its callback takes
  // the lock, so the wait happens here, unlocked)
  for (auto& f : failures)
    if (f.first->slot >= 0) {
      Slot& sl = s->slots[f.first->slot];
      cudaStreamSynchronize(sl.st);
      // any completion value its launches wrote is stale now: the next one starts above it
      s->watch.erase(std::remove(s->watch.begin(), s->watch.end(), sl.index), s->watch.end());
      const unsigned seen = *reinterpret_cast<volatile unsigned*>(sl.done);
      sl.seq = std::max(sl.seq, seen);
    }
  const double busy = now_s() - t_work;
  lk.lock();
  for (ServerCanvas* c : drops) s->canvases.erase(c->id);  // its requests are all finished
  s->stats.steps += chunks;
  s->stats.worker_busy_us += static_cast<int64_t>(busy * 1e6);
  for (auto& f : failures) {
    finish(s, f.first, PAINTY_ERR_CUDA, f.second);
    s->active.erase(std::find(s->active.begin(), s->active.end(), f.first->id));
  }
  for (ServerRequest* r : done) {
    s->stats.stamps += r->stamps;
    const bool cancelled = r->cancel && (r->next < r->strokes.size() || r->out_rgb);
    finish(s, r, cancelled ? PAINTY_ERR_CANCELLED : PAINTY_OK,
           cancelled ? "cancelled while painting" : "");
    s->active.erase(std::find(s->active.begin(), s->active.end(), r->id));
  }
  if (!failures.empty() || !done.empty()) s->cv_done.notify_all();
  return moved;
}

void worker_main(painty_server* s) {
  cudaSetDevice(s->device);
  std::unique_lock<std::mutex> lk(s->mu);
  uint64_t idle_gen = ~0ull;
  while (true) {
    // wake on a finished launch, a drop, or a change to what could be admitted
    // launches that signal through their completion words are polled every 50 us
    const auto wait = s->watch.empty() ? std::chrono::microseconds(50000)
                                       : std::chrono::microseconds(50);
    s->cv_work.wait_for(lk, wait, [&] {
      return s->stop || !s->passed.empty() || !s->to_drop.empty() ||
             (!s->pending.empty() && s->gen != idle_gen);
    });
    poll_watched(s);
    if (s->stop) break;
    const uint64_t g = s->gen;
    worker_round(s, lk);
    idle_gen = g;  // admit again only after a submit, cancel, release or finish
  }
  // shutting down: every request still queued is cancelled; launched work drains first
  std::vector<uint64_t> act = s->active;
  lk.unlock();
  for (const Slot& sl : s->slots) cudaStreamSynchronize(sl.st);
  lk.lock();
  for (uint64_t id : s->pending) finish(s, s->reqs[id].get(), PAINTY_ERR_CANCELLED, "server shut down");
  for (uint64_t id : act) finish(s, s->reqs[id].get(), PAINTY_ERR_CANCELLED, "server shut down");
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
    s->opt.max_active = std::min(s->opt.max_active, 1024);
    if (s->opt.step_stamps <= 0) s->opt.step_stamps = 16384;
    s->footprint.assign(opt->footprint,
                        opt->footprint + static_cast<size_t>(opt->footprint_rows) * opt->footprint_cols);
    s->opt.footprint = nullptr;
    PG_CUDA(cudaGetDevice(&s->device));
    PG_CUDA(cudaDeviceGetAttribute(&s->sms, cudaDevAttrMultiProcessorCount, s->device));
    PG_CUDA(cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking));
    // one reservation for everything the server keeps on the device, carved on the host: the
    // budget's canvases plus the slots' launch buffers
    s->heap = std::make_unique<pg::DeviceHeap>(
      s->opt.budget_bytes + static_cast<size_t>(s->opt.max_active) * (kStagingBytes + (1u << 20)) +
      (size_t(256) << 20));
    PG_CUDA(cudaMallocHost(&s->status_words, sizeof(unsigned) * s->opt.max_active));
    // completion words a cache line apart (the GPU writes them, the worker polls them)
    PG_CUDA(cudaMallocHost(&s->done_words, 64 * static_cast<size_t>(s->opt.max_active)));
    std::memset(s->done_words, 0, 64 * static_cast<size_t>(s->opt.max_active));
    PG_CUDA(cudaMallocHost(&s->staging, kStagingBytes * s->opt.max_active));
    s->slots.resize(static_cast<size_t>(s->opt.max_active));
    for (int i = 0; i < s->opt.max_active; i++) {
      Slot& sl = s->slots[i];
      PG_CUDA(cudaStreamCreateWithFlags(&sl.st, cudaStreamNonBlocking));
      PG_CUDA(cudaEventCreateWithFlags(&sl.ev, cudaEventDisableTiming));
      sl.status = s->status_words + i;
      sl.done = s->done_words + 16 * i;
      sl.done_dev = static_cast<unsigned*>(const_cast<void*>(pg::mapped_host(sl.done)));
      PG_REQUIRE(sl.done_dev != nullptr, "pinned completion words are not mapped");
      sl.d_counter = static_cast<unsigned*>(s->heap->alloc(256, s->stream));
      sl.staging = s->staging + kStagingBytes * i;
      *sl.status = 0;
      sl.owner = s.get();
      sl.index = i;
    }
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
      r->total_stamps += r->stroke_stamps.back();
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
      if (req->r0) {
        // pinned substrates are read in place when the canvas is created; others are copied
        cudaPointerAttributes pa{};
        if (cudaPointerGetAttributes(&pa, req->r0) == cudaSuccess &&
            pa.type == cudaMemoryTypeHost)
          nc->r0_pinned = req->r0;
        else
          nc->r0.assign(req->r0, req->r0 + static_cast<size_t>(req->rows) * req->cols * 3);
        cudaGetLastError();
      }
      c = nc.get();
      s->canvases.emplace(nc->id, std::move(nc));
    } else {
      auto it = s->canvases.find(req->canvas_id);
      PG_REQUIRE(it != s->canvases.end(), "unknown canvas id");
      c = it->second.get();
      PG_REQUIRE(!c->release, "the canvas was released");
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

painty_status painty_server_release(painty_server* s, uint64_t canvas_id) {
  return guard([&] {
    PG_REQUIRE(s != nullptr, "server is null");
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->canvases.find(canvas_id);
    PG_REQUIRE(it != s->canvases.end(), "unknown canvas id");
    ServerCanvas* c = it->second.get();
    if (c->release) return;
    c->release = true;
    if (c->waiting.empty() && !c->busy) {
      if (c->resident) s->resident -= c->bytes;
      s->to_drop.push_back(c);
    }
    s->gen++;
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

painty_status painty_server_poll(painty_server* s, double timeout_s, uint64_t* request_id) {
  painty_status result = PAINTY_OK;
  const painty_status st = guard([&] {
    PG_REQUIRE(s && request_id, "null argument");
    std::unique_lock<std::mutex> lk(s->mu);
    const auto pred = [&] { return !s->finished.empty(); };
    if (timeout_s < 0)
      s->cv_done.wait(lk, pred);
    else if (!s->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), pred)) {
      result = PAINTY_ERR_TIMEOUT;
      pg::set_last_error("no request finished within the timeout");
      return;
    }
    *request_id = s->finished.front();
    s->finished.pop_front();
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
    int64_t live = 0;
    for (auto& kv : s->canvases) live += kv.second->release ? 0 : 1;
    out->canvases = live;
    out->heap_bytes = s->heap->reserved();
    out->heap_fallbacks = s->heap->fallbacks();
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
    for (auto& kv : s->canvases)
      if (!kv.second->dropped) drop(s, kv.second.get());
    cudaStreamSynchronize(s->stream);
    for (auto& kv : s->pinned_free) cudaFreeHost(kv.second);
    for (Slot& sl : s->slots) {
      cudaEventDestroy(sl.ev);
      cudaStreamDestroy(sl.st);
    }
    cudaFreeHost(s->status_words);
    cudaFreeHost(s->done_words);
    cudaFreeHost(s->staging);
    for (Slot& sl : s->slots) {
      s->heap->free(sl.d_desc, s->stream);
      s->heap->free(sl.d_scratch, s->stream);
      s->heap->free(sl.d_counter, s->stream);
    }
    s->heap.reset();
    cudaStreamDestroy(s->stream);
    delete s;
  });
}

}  // extern "C"
