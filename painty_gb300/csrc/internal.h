// internal.h -- host-side definitions shared by the library's translation units.
#pragma once

#include <cuda_runtime.h>

#include <atomic>
#include <cstdint>
#include <map>
#include <memory>
#include <mutex>
#include <utility>
#include <vector>
#include <stdexcept>
#include <string>
#include <unordered_map>
#include <unordered_set>

#include "offset_alloc.h"
#include "painty_gb300.h"

namespace pg {

struct Error : std::runtime_error {
  painty_status status;
  Error(painty_status s, const std::string& m) : std::runtime_error(m), status(s) {}
};

[[noreturn]] void fail(painty_status s, const std::string& msg);
void check_cuda(cudaError_t e, const char* what);
#define PG_CUDA(x) ::pg::check_cuda((x), #x)
#define PG_REQUIRE(cond, msg) \
  do {                        \
    if (!(cond)) ::pg::fail(PAINTY_ERR_INVALID_ARGUMENT, (msg)); \
  } while (0)

void set_last_error(const std::string& msg);
void count_launch(int64_t n = 1);

// Runs fn, converting exceptions to a status code and recording the message.
template <class Fn>
painty_status guard(Fn&& fn) {
  try {
    fn();
    return PAINTY_OK;
  } catch (const Error& e) {
    set_last_error(e.what());
    return e.status;
  } catch (const std::bad_alloc&) {
    set_last_error("host allocation failed");
    return PAINTY_ERR_OUT_OF_MEMORY;
  } catch (const std::exception& e) {
    set_last_error(e.what());
    return PAINTY_ERR_INVALID_ARGUMENT;
  }
}

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

// Element sizes: K/S planes, V (and h) planes, reflectance planes.
size_t ks_bytes(painty_storage s);
size_t v_bytes(painty_storage s);
inline size_t r_bytes(painty_storage s) { return s == PAINTY_STORAGE_F64 ? 8 : 4; }
bool valid_storage(painty_storage s);

// Row pitch in elements: a multiple of 64 elements (>= 128 bytes for every element type), so
// each row starts 128-byte aligned and plane sizes are multiples of 8 elements.
inline int64_t pitch_for(int32_t cols) { return (static_cast<int64_t>(cols) + 63) / 64 * 64; }

void* device_alloc(size_t bytes);
void device_free(void* p);
// Stream-ordered device memory from `pool` (a pool with a retained release threshold): the
// allocation and the release are ordered on `st` and never synchronise the device. For
// objects a long-running owner (the server) creates and drops while kernels run.
void* device_alloc_on(size_t bytes, cudaMemPool_t pool, cudaStream_t st);
void device_free_on(void* p, cudaStream_t st);
// A launch temporary, ordered on `st` (free with cudaFreeAsync on a stream ordered after its
// last use), from the library's own pool that keeps freed memory for reuse.
void* temp_alloc(size_t bytes, cudaStream_t st);
// Pool settings shared by the library's pools (retained memory, no cross-stream reuse waits).
void configure_pool(cudaMemPool_t pool);
// The device address of pinned (page-locked, mapped) host memory, or nullptr for pageable
// memory: kernels read and write such memory in place over the host link.
const void* mapped_host(const void* host);

// One device reservation carved up on the host: allocation and release are host bookkeeping
// (best fit, neighbours merged on release, 256-byte granules), so neither calls into CUDA.
// For an owner that releases memory only once the GPU has finished with it (the server: a
// canvas's memory after its last request completed). A request the reservation cannot hold
// falls back to stream-ordered cudaMallocAsync on the given stream.
class DeviceHeap {
 public:
  explicit DeviceHeap(size_t bytes);  // reserves `bytes`, or what the device has free
  ~DeviceHeap();
  DeviceHeap(const DeviceHeap&) = delete;
  DeviceHeap& operator=(const DeviceHeap&) = delete;
  void* alloc(size_t bytes, cudaStream_t st);
  void free(void* p, cudaStream_t st);
  size_t reserved() const { return size_; }
  int64_t fallbacks() const { return fallbacks_; }

 private:
  std::mutex mu_;
  char* base_ = nullptr;
  size_t size_ = 0;
  OffsetAllocator ranges_;              // the reservation's layout
  std::unordered_set<void*> outside_;  // fallback allocations
  int64_t fallbacks_ = 0;
};

}  // namespace pg

// Opaque handle types of the C ABI.
struct painty_layer {
  int32_t rows = 0, cols = 0;
  int64_t pitch = 0;
  painty_storage storage = PAINTY_STORAGE_F32;
  void* base = nullptr;  // one allocation holding the 7 planes
  size_t bytes = 0;
  void* K[3] = {nullptr, nullptr, nullptr};
  void* S[3] = {nullptr, nullptr, nullptr};
  void* V = nullptr;
  // Elements from one pixel to the next within a plane view: 1 for planar layers (7 planes);
  // 8 for packed layers (one record per pixel: K r,g,b, S r,g,b, V, pad), the layout of
  // canvases and snapshots, whose stamps touch whole pixels.
  int64_t estride = 1;
  bool owned = true;
  // a canvas's wet layer: the canvas's write counter, bumped by every write through the layer
  uint64_t* writes = nullptr;
  void touch() const {
    if (writes) ++*writes;
  }
  int64_t plane_elems() const { return static_cast<int64_t>(rows) * pitch; }
};

struct painty_image {
  int32_t rows = 0, cols = 0;
  int64_t pitch = 0;
  painty_storage storage = PAINTY_STORAGE_F32;  // F32 or F64
  void* base = nullptr;
  size_t bytes = 0;
  void* R[3] = {nullptr, nullptr, nullptr};
  bool owned = true;
  int64_t plane_elems() const { return static_cast<int64_t>(rows) * pitch; }
};

struct painty_canvas {
  painty_layer wet;  // borrowed view: owned = false
  painty_image r0;   // borrowed view: owned = false
  void* h = nullptr;  // height map, V element type
  void* base = nullptr;
  size_t bytes = 0;
  uint64_t id = 0;       // process-unique
  uint64_t version = 0;  // bumped by every write that does not go through a stamp
};

// FootprintBrush<vec3> (painty/renderer/FootprintBrush.hxx:22-502): host copy of the brush
// parameters and the device buffers it owns.
struct painty_brush {
  double radius = 0.0;  // FootprintBrush.hxx:437
  int32_t sizeMap = 0;  // :443
  int32_t F = 0;
  int32_t support2 = 0;  // squared stamp-pixel radius beyond which the footprint is zero
  int32_t width = 0;     // footprint width before padding (2 ceil(r) + 1)
  // footprints built from `full`, by width, shared by every brush of the same footprint image
  // (the process-wide cache of stamp.cu)
  std::shared_ptr<struct FootprintFamily> fp_family;
  std::vector<double> full;
  int32_t fh = 0, fw = 0;
  std::vector<double> footprint;  // F*F
  bool useSnapshot = true;        // :477
  double capacity = 1.0;          // :483
  double pickupRate = 0.9;        // :489
  double depositionRate = 0.05;   // :495
  double paintK[3] = {0, 0, 0};
  double paintS[3] = {0, 0, 0};
  // device state; `math64` is fixed by the first canvas the brush paints
  int bound = -1;  // -1 unbound, 0 FP32 math, 1 FP64 math
  void* d_footprint = nullptr;
  size_t d_footprint_bytes = 0;
  bool footprint_stale = true;
  void* d_pickup = nullptr;  // 7 planes of S*S
  size_t d_pickup_bytes = 0;
  bool pickup_clear = true;
  void* d_owner = nullptr;
  size_t d_owner_bytes = 0;
  void* d_cellmap = nullptr;  // cell maps of large stamps (2 F*F ints per CTA)
  size_t d_cellmap_bytes = 0;
  // snapshot (FootprintBrush.hxx:471): canvas-sized layer, allocated at first use
  painty_layer snapshot;
  bool has_snapshot = false;
  // snapshot-ring state on the device (box and grown box of the last stamp painted with the
  // snapshot) and the canvas state it describes; ring_pending: a reset mode for the next run
  // (-1 none)
  uint64_t ring_canvas = 0;
  uint64_t ring_version = 0;
  int ring_pending = -1;
  void* d_stamps = nullptr;
  size_t d_stamps_bytes = 0;
  // device memory from an owner's heap (released only after the brush's work finished; the
  // heap's fallback is ordered on heap_stream), instead of cudaMalloc / cudaFree
  pg::DeviceHeap* heap = nullptr;
  cudaStream_t heap_stream = nullptr;
  unsigned* d_status = nullptr;  // 16 words: [0] kernel status, [2] stamps applied (rounding
                                 // seed), [8..15] the ring state
  int* d_ring() const { return reinterpret_cast<int*>(d_status) + 8; }
};

namespace pg {
// Layout helpers (defined in core.cu).
void layer_layout(painty_layer& L, int32_t rows, int32_t cols, painty_storage s, void* base,
                  bool packed = false);
size_t layer_bytes(int32_t rows, int32_t cols, painty_storage s, bool packed = false);
void image_layout(painty_image& I, int32_t rows, int32_t cols, painty_storage s, void* base);
size_t image_bytes(int32_t rows, int32_t cols, painty_storage s);
// Points a canvas's plane views into a new device allocation of the canvas layout (nullptr:
// no allocation, as for a canvas whose state was moved to host memory).
void canvas_relayout(painty_canvas* c, void* base);
// A canvas (as painty_canvas_create) in heap memory, initialised in `st`'s order (with
// `sync`, returns after `st` has finished that). Free with canvas_destroy_on once the GPU
// has finished with it.
painty_canvas* canvas_create_on(int32_t rows, int32_t cols, painty_storage storage,
                                DeviceHeap* heap, cudaStream_t st, bool sync = true);
void canvas_destroy_on(painty_canvas* c, DeviceHeap* heap, cudaStream_t st);

// Plane transfer between a host buffer and `nch` device planes of element type `dev_type`
// (0 f32, 1 f16, 2 bf16, 3 f64) with the given pitch and element stride (1 planar, 8 packed).
// Synchronous w.r.t. the host buffer.
enum DevType { DT_F32 = 0, DT_F16 = 1, DT_BF16 = 2, DT_F64 = 3 };
DevType ks_type(painty_storage s);
DevType v_type(painty_storage s);
DevType r_type(painty_storage s);
void upload_planes(void* const* planes, int nch, DevType dt, int32_t rows, int32_t cols,
                   int64_t pitch, const void* host, painty_host_format fmt, cudaStream_t st,
                   int64_t estride = 1);
// The same ordered on `st` without waiting (a pinned host buffer must stay valid until the
// stream passes the copy; pageable memory is copied out before the call returns).
void upload_planes_async(void* const* planes, int nch, DevType dt, int32_t rows, int32_t cols,
                         int64_t pitch, const void* host, painty_host_format fmt,
                         cudaStream_t st, int64_t estride = 1);
void download_planes(const void* const* planes, int nch, DevType dt, int32_t rows,
                     int32_t cols, int64_t pitch, void* host, painty_host_format fmt,
                     cudaStream_t st, int64_t estride = 1);
// The same without waiting: the copy is ordered on `st` (the host buffer is written once the
// stream passes it; pinned host memory keeps the call from blocking).
void download_planes_async(const void* const* planes, int nch, DevType dt, int32_t rows,
                           int32_t cols, int64_t pitch, void* host, painty_host_format fmt,
                           cudaStream_t st, int64_t estride = 1);
void fill_planes(void* const* planes, int nch, DevType dt, int64_t elems, const double* values,
                 cudaStream_t st, int64_t estride = 1);
// Copies a layer's 7 planes into another of the same size and storage (any layouts).
void copy_layer(const painty_layer& src, painty_layer& dst, cudaStream_t st);
void copy_planes_async(void* const* dst, const void* const* src, int nch, size_t plane_bytes,
                       cudaStream_t st);

// Batched painting (stamp.cu): painty_paint_batch after argument checks.
// BatchOptions (NULL: the defaults): max_cluster caps the CTAs per canvas the cost model may
// choose (1, 2, 4 or 8). With status_host set (pinned host memory) the call returns right
// after the launch: the kernel's status word is copied there in stream order, temporaries
// are freed in stream order, and the caller checks the word once the stream has passed the
// launch (nonzero: the kernel reported an internal error).
struct BatchOptions {
  int max_cluster = 8;
  int threads = 0;  // CTA size: 512 or 1024, 0 = chosen by the cost model
  unsigned* status_host = nullptr;
  // pinned host memory the launch's descriptors are staged in when they fit (the caller
  // guarantees no earlier copy from it is still pending); otherwise a pageable copy
  void* host_staging = nullptr;
  size_t host_staging_bytes = 0;
  // device buffers for the launch's descriptors and scratch, used when large enough (the
  // caller guarantees no earlier launch still uses them); otherwise launch temporaries.
  // *_needed (when set) receive the sizes this launch wanted.
  void* device_desc = nullptr;
  size_t device_desc_bytes = 0;
  void* device_scratch = nullptr;
  size_t device_scratch_bytes = 0;
  size_t* desc_needed = nullptr;
  size_t* scratch_needed = nullptr;
  // pinned host word the kernel sets to done_value once the launch's results (and the status
  // word) are visible to the host; such a launch is never split
  unsigned* done_host = nullptr;
  unsigned done_value = 0;
};
void paint_batch(painty_canvas* const* canvases, painty_brush* const* brushes, int32_t nc,
                 const painty_stroke_desc* strokes, int64_t ns, const double* points,
                 int64_t npoints, int64_t* stamps_out, cudaStream_t st,
                 const BatchOptions* opt = nullptr);
// Stamps painty's paintStroke puts on a path at the given chord spacing (host count).
int64_t stroke_stamp_count(const double* path, int32_t n, double spacing);

// KM composite launcher (core.cu). layers: L pointers; r0 and out may alias.
void launch_compose(const painty_layer* const* layers, int32_t L, const painty_image* r0,
                    painty_image* out, cudaStream_t st);
}  // namespace pg
