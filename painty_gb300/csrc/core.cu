// core.cu -- library plumbing, layers / images / canvases, plane transfers, and the fused
// multi-layer Kubelka-Munk composite and drying kernels.
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <mutex>
#include <string>
#include <type_traits>
#include <vector>

#include "device_common.cuh"
#include "internal.h"

namespace pg {

// Set by a kernel whose shared-memory pipeline stalled beyond its wait limit (the kernel
// then writes NaN where it stopped and returns); read and cleared by
// painty_take_device_faults.
__device__ unsigned int g_pipeline_fault = 0;

namespace {
thread_local std::string g_last_error;
std::atomic<int64_t> g_launches{0};
std::atomic<uint64_t> g_canvas_ids{1};
}  // namespace

void set_last_error(const std::string& msg) { g_last_error = msg; }
void count_launch(int64_t n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

[[noreturn]] void fail(painty_status s, const std::string& msg) { throw Error(s, msg); }

void check_cuda(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return;
  if (e == cudaErrorMemoryAllocation) {
    cudaGetLastError();
    fail(PAINTY_ERR_OUT_OF_MEMORY, std::string(what) + ": " + cudaGetErrorString(e));
  }
  fail(PAINTY_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

bool valid_storage(painty_storage s) {
  return s == PAINTY_STORAGE_F32 || s == PAINTY_STORAGE_F16 || s == PAINTY_STORAGE_BF16 ||
         s == PAINTY_STORAGE_F64;
}
size_t ks_bytes(painty_storage s) {
  switch (s) {
    case PAINTY_STORAGE_F16:
    case PAINTY_STORAGE_BF16: return 2;
    case PAINTY_STORAGE_F64: return 8;
    default: return 4;
  }
}
size_t v_bytes(painty_storage s) { return ks_bytes(s); }  // F16 and BF16 keep V in FP16
DevType ks_type(painty_storage s) {
  switch (s) {
    case PAINTY_STORAGE_F16: return DT_F16;
    case PAINTY_STORAGE_BF16: return DT_BF16;
    case PAINTY_STORAGE_F64: return DT_F64;
    default: return DT_F32;
  }
}
DevType v_type(painty_storage s) {
  switch (s) {
    case PAINTY_STORAGE_F16:
    case PAINTY_STORAGE_BF16: return DT_F16;
    case PAINTY_STORAGE_F64: return DT_F64;
    default: return DT_F32;
  }
}
DevType r_type(painty_storage s) { return s == PAINTY_STORAGE_F64 ? DT_F64 : DT_F32; }

static size_t dt_size(DevType t) { return t == DT_F64 ? 8 : (t == DT_F32 ? 4 : 2); }
static size_t align256(size_t x) { return (x + 255) / 256 * 256; }

void* device_alloc(size_t bytes) {
  void* p = nullptr;
  if (bytes == 0) return nullptr;
  PG_CUDA(cudaMalloc(&p, bytes));
  return p;
}
void device_free(void* p) {
  if (p) cudaFree(p);
}
void* device_alloc_on(size_t bytes, cudaMemPool_t pool, cudaStream_t st) {
  void* p = nullptr;
  if (bytes == 0) return nullptr;
  const cudaError_t e = cudaMallocFromPoolAsync(&p, bytes, pool, st);
  if (e == cudaErrorMemoryAllocation) {
    cudaGetLastError();
    fail(PAINTY_ERR_OUT_OF_MEMORY, "device memory exhausted (pool allocation)");
  }
  PG_CUDA(e);
  return p;
}
void device_free_on(void* p, cudaStream_t st) {
  if (p) cudaFreeAsync(p, st);
}

// Settings of the library's stream-ordered pools: freed memory is kept for reuse, and memory
// freed on one stream is not handed to another by making the second wait for the first (that
// reuse would chain independent streams, e.g. a server's requests, into one).
void configure_pool(cudaMemPool_t pool) {
  uint64_t keep = ~0ull;
  PG_CUDA(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep));
  int no = 0;
  PG_CUDA(cudaMemPoolSetAttribute(pool, cudaMemPoolReuseAllowInternalDependencies, &no));
}

// The library's pool for launch temporaries, one per device, keeping freed memory for reuse:
// the default pool returns memory at every synchronisation, and mapping it again on the next
// allocation costs more than the launches it serves.
void* temp_alloc(size_t bytes, cudaStream_t st) {
  static std::mutex mu;
  static cudaMemPool_t pools[64] = {};
  int dev = 0;
  PG_CUDA(cudaGetDevice(&dev));
  PG_REQUIRE(dev >= 0 && dev < 64, "device ordinal out of range");
  cudaMemPool_t pool = nullptr;
  {
    std::lock_guard<std::mutex> lk(mu);
    if (!pools[dev]) {
      cudaMemPoolProps props{};
      props.allocType = cudaMemAllocationTypePinned;
      props.location.type = cudaMemLocationTypeDevice;
      props.location.id = dev;
      PG_CUDA(cudaMemPoolCreate(&pools[dev], &props));
      configure_pool(pools[dev]);
    }
    pool = pools[dev];
  }
  return device_alloc_on(std::max<size_t>(bytes, 16), pool, st);
}

// Planar: 7 planes, each 256-byte aligned. Packed: one record of 8 elements per pixel (K and
// S, V of the same size in every storage format).
size_t layer_bytes(int32_t rows, int32_t cols, painty_storage s, bool packed) {
  const size_t pe = static_cast<size_t>(rows) * pitch_for(cols);
  if (packed) return align256(pe * 8 * ks_bytes(s));
  return 6 * align256(pe * ks_bytes(s)) + align256(pe * v_bytes(s));
}
void layer_layout(painty_layer& L, int32_t rows, int32_t cols, painty_storage s, void* base,
                  bool packed) {
  L.rows = rows;
  L.cols = cols;
  L.pitch = pitch_for(cols);
  L.storage = s;
  L.base = base;
  L.bytes = layer_bytes(rows, cols, s, packed);
  char* p = static_cast<char*>(base);
  if (packed) {
    const size_t es = ks_bytes(s);
    for (int c = 0; c < 3; c++) L.K[c] = p + c * es;
    for (int c = 0; c < 3; c++) L.S[c] = p + (3 + c) * es;
    L.V = p + 6 * es;
    L.estride = 8;
    return;
  }
  const size_t ksb = align256(static_cast<size_t>(L.plane_elems()) * ks_bytes(s));
  for (int c = 0; c < 3; c++) L.K[c] = p + c * ksb;
  for (int c = 0; c < 3; c++) L.S[c] = p + (3 + c) * ksb;
  L.V = p + 6 * ksb;
  L.estride = 1;
}
size_t image_bytes(int32_t rows, int32_t cols, painty_storage s) {
  const size_t pe = static_cast<size_t>(rows) * pitch_for(cols);
  return 3 * align256(pe * r_bytes(s));
}
void image_layout(painty_image& I, int32_t rows, int32_t cols, painty_storage s, void* base) {
  I.rows = rows;
  I.cols = cols;
  I.pitch = pitch_for(cols);
  I.storage = s;
  I.base = base;
  I.bytes = image_bytes(rows, cols, s);
  const size_t rb = align256(static_cast<size_t>(I.plane_elems()) * r_bytes(s));
  for (int c = 0; c < 3; c++) I.R[c] = static_cast<char*>(base) + c * rb;
}

void canvas_relayout(painty_canvas* c, void* base) {
  const int32_t rows = c->wet.rows, cols = c->wet.cols;
  const painty_storage st = c->wet.storage;
  const painty_storage rs = c->r0.storage;
  c->base = base;
  if (!base) {  // evicted: views point nowhere until the canvas is restored
    for (int i = 0; i < 3; i++) c->wet.K[i] = c->wet.S[i] = c->r0.R[i] = nullptr;
    c->wet.V = c->h = c->wet.base = c->r0.base = nullptr;
    return;
  }
  const size_t lb = layer_bytes(rows, cols, st, true);
  const size_t ib = image_bytes(rows, cols, rs);
  layer_layout(c->wet, rows, cols, st, base, true);
  c->wet.owned = false;
  c->wet.writes = &c->version;
  image_layout(c->r0, rows, cols, rs, static_cast<char*>(base) + lb);
  c->r0.owned = false;
  c->h = static_cast<char*>(base) + lb + ib;
}

painty_canvas* canvas_create_on(int32_t rows, int32_t cols, painty_storage storage,
                                DeviceHeap* heap, cudaStream_t st, bool sync) {
  PG_REQUIRE(rows > 0 && cols > 0, "rows and cols must be positive");
  PG_REQUIRE(valid_storage(storage), "unknown storage format");
  PG_REQUIRE(heap != nullptr, "no heap");
  auto* c = new painty_canvas();
  const painty_storage rs = storage == PAINTY_STORAGE_F64 ? PAINTY_STORAGE_F64 : PAINTY_STORAGE_F32;
  const size_t lb = layer_bytes(rows, cols, storage, true);
  const size_t ib = image_bytes(rows, cols, rs);
  const size_t hb = static_cast<size_t>(rows) * pitch_for(cols) * v_bytes(storage);
  try {
    c->wet.rows = rows;
    c->wet.cols = cols;
    c->wet.storage = storage;
    c->r0.storage = rs;
    c->bytes = lb + ib + align256(hb);
    canvas_relayout(c, heap->alloc(c->bytes, st));
    c->id = g_canvas_ids.fetch_add(1);
    PG_CUDA(cudaMemsetAsync(c->base, 0, c->bytes, st));
    const double one[3] = {1.0, 1.0, 1.0};  // Canvas.hxx:33 background
    fill_planes(c->r0.R, 3, r_type(rs), c->r0.plane_elems(), one, st);
    if (sync) PG_CUDA(cudaStreamSynchronize(st));
  } catch (...) {
    if (c->base) {
      cudaStreamSynchronize(st);  // the memory is reused at once: let queued work finish
      heap->free(c->base, st);
    }
    delete c;
    throw;
  }
  return c;
}

void canvas_destroy_on(painty_canvas* c, DeviceHeap* heap, cudaStream_t st) {
  if (!c) return;
  heap->free(c->base, st);
  delete c;
}

// ------------------------------------------------------------------ device heap
DeviceHeap::DeviceHeap(size_t bytes) {
  bytes = (bytes + 255) / 256 * 256;
  void* p = nullptr;
  if (bytes > 0 && cudaMalloc(&p, bytes) != cudaSuccess) {
    cudaGetLastError();
    size_t free_b = 0, total_b = 0;
    p = nullptr;
    if (cudaMemGetInfo(&free_b, &total_b) == cudaSuccess && free_b > (size_t(1) << 30)) {
      bytes = (free_b - (size_t(1) << 30)) / 256 * 256;  // leave 1 GB to everything else
      if (cudaMalloc(&p, bytes) != cudaSuccess) {
        cudaGetLastError();
        p = nullptr;
      }
    }
    if (!p) bytes = 0;
  }
  base_ = static_cast<char*>(p);
  size_ = p ? bytes : 0;
  ranges_.reset(size_);
}

DeviceHeap::~DeviceHeap() {
  if (base_) cudaFree(base_);
  for (void* p : outside_) cudaFree(p);
}

void* DeviceHeap::alloc(size_t bytes, cudaStream_t st) {
  const size_t len = (std::max<size_t>(bytes, 1) + 255) / 256 * 256;
  {
    std::lock_guard<std::mutex> lk(mu_);
    size_t off = 0;
    if (ranges_.alloc(len, &off)) return base_ + off;  // best fit
    fallbacks_++;
  }
  void* p = nullptr;
  const cudaError_t e = cudaMallocAsync(&p, len, st);
  if (e == cudaErrorMemoryAllocation) {
    cudaGetLastError();
    fail(PAINTY_ERR_OUT_OF_MEMORY, "device memory exhausted (heap fallback)");
  }
  PG_CUDA(e);
  std::lock_guard<std::mutex> lk(mu_);
  outside_.insert(p);
  return p;
}

void DeviceHeap::free(void* p, cudaStream_t st) {
  if (!p) return;
  std::lock_guard<std::mutex> lk(mu_);
  char* c = static_cast<char*>(p);
  if (base_ && c >= base_ && c < base_ + size_) {
    ranges_.release(static_cast<size_t>(c - base_));  // false: not an allocation of this heap
    return;
  }
  if (outside_.erase(p)) cudaFreeAsync(p, st);
}

// ------------------------------------------------------------------ transfer kernels
namespace {

struct PlanePtrs {
  void* p[3];
};
struct LayerPtrs {  // K r,g,b, S r,g,b, V
  void* p[7];
};

template <class TD, class TS>
__device__ __forceinline__ TD convert(TS v);
template <> __device__ __forceinline__ float convert<float, float>(float v) { return v; }
template <> __device__ __forceinline__ float convert<float, double>(double v) { return static_cast<float>(v); }
template <> __device__ __forceinline__ double convert<double, double>(double v) { return v; }
template <> __device__ __forceinline__ double convert<double, float>(float v) { return v; }
template <> __device__ __forceinline__ __half convert<__half, float>(float v) { return __float2half_rn(v); }
template <> __device__ __forceinline__ __half convert<__half, double>(double v) { return __double2half(v); }
template <> __device__ __forceinline__ __nv_bfloat16 convert<__nv_bfloat16, float>(float v) { return __float2bfloat16_rn(v); }
template <> __device__ __forceinline__ __nv_bfloat16 convert<__nv_bfloat16, double>(double v) { return __double2bfloat16(v); }
template <> __device__ __forceinline__ float convert<float, __half>(__half v) { return __half2float(v); }
template <> __device__ __forceinline__ double convert<double, __half>(__half v) { return __half2float(v); }
template <> __device__ __forceinline__ float convert<float, __nv_bfloat16>(__nv_bfloat16 v) { return __bfloat162float(v); }
template <> __device__ __forceinline__ double convert<double, __nv_bfloat16>(__nv_bfloat16 v) { return __bfloat162float(v); }

// staging (host layout, contiguous) -> pitched planes
template <class TD, class TS>
__global__ void scatter_kernel(const TS* __restrict__ src, PlanePtrs dst, int nch,
                               int interleaved, int32_t rows, int32_t cols, int64_t pitch,
                               int64_t es) {
  const int64_t n = static_cast<int64_t>(rows) * cols;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n * nch;
       i += (int64_t)gridDim.x * blockDim.x) {
    int64_t p, c;
    if (interleaved) {
      p = i / nch;
      c = i - p * nch;
    } else {
      c = i / n;
      p = i - c * n;
    }
    const int64_t r = p / cols, col = p - r * cols;
    static_cast<TD*>(dst.p[c])[(r * pitch + col) * es] = convert<TD, TS>(src[i]);
  }
}

// pitched planes -> staging (host layout)
template <class TD, class TS>
__global__ void gather_kernel(PlanePtrs src, TD* __restrict__ dst, int nch, int interleaved,
                              int32_t rows, int32_t cols, int64_t pitch, int64_t es) {
  const int64_t n = static_cast<int64_t>(rows) * cols;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n * nch;
       i += (int64_t)gridDim.x * blockDim.x) {
    int64_t p, c;
    if (interleaved) {
      p = i / nch;
      c = i - p * nch;
    } else {
      c = i / n;
      p = i - c * n;
    }
    const int64_t r = p / cols, col = p - r * cols;
    dst[i] = convert<TD, TS>(static_cast<const TS*>(src.p[c])[(r * pitch + col) * es]);
  }
}

template <class T>
__global__ void fill_kernel(PlanePtrs dst, int nch, int64_t elems, double v0, double v1,
                            double v2, int64_t es) {
  const double v[3] = {v0, v1, v2};
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < elems * nch;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t c = i / elems;
    static_cast<T*>(dst.p[c])[(i - c * elems) * es] = convert<T, double>(v[c]);
  }
}

// PaintLayer::set(i, j, k, s, v) for n cells in order: cell m writes its 7 values (K, S as
// triples, V) at (rows[m], cols[m]). Later cells win where cells repeat, as successive set()
// calls do.
template <class TK, class TV>
__global__ void set_cells_kernel(LayerPtrs dst, int64_t pitch, int64_t es, const int32_t* rc,
                                 const double* vals, int64_t n) {
  for (int64_t m = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; m < n;
       m += (int64_t)gridDim.x * blockDim.x) {
    const int64_t at = (static_cast<int64_t>(rc[2 * m]) * pitch + rc[2 * m + 1]) * es;
    // a later cell at the same position takes precedence
    bool later = false;
    for (int64_t q = m + 1; q < n && !later; q++)
      later = rc[2 * q] == rc[2 * m] && rc[2 * q + 1] == rc[2 * m + 1];
    if (later) continue;
#pragma unroll
    for (int c = 0; c < 6; c++) static_cast<TK*>(dst.p[c])[at] = convert<TK, double>(vals[7 * m + c]);
    static_cast<TV*>(dst.p[6])[at] = convert<TV, double>(vals[7 * m + 6]);
  }
}

// Layer copy between any layouts: the 7 values of each pixel, src element stride -> dst.
template <class TK, class TV>
__global__ void copy_layer_kernel(LayerPtrs src, LayerPtrs dst, int64_t elems, int64_t ses,
                                  int64_t des) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < elems;
       i += (int64_t)gridDim.x * blockDim.x) {
#pragma unroll
    for (int c = 0; c < 6; c++)
      static_cast<TK*>(dst.p[c])[i * des] = static_cast<const TK*>(src.p[c])[i * ses];
    static_cast<TV*>(dst.p[6])[i * des] = static_cast<const TV*>(src.p[6])[i * ses];
  }
}

int grid_for(int64_t n, int block) {
  const int64_t g = (n + block - 1) / block;
  return static_cast<int>(std::max<int64_t>(1, std::min<int64_t>(g, 152 * 32)));
}

bool host_is_f64(painty_host_format f) {
  return f == PAINTY_HOST_F64_INTERLEAVED || f == PAINTY_HOST_F64_PLANAR;
}
bool host_is_interleaved(painty_host_format f) {
  return f == PAINTY_HOST_F64_INTERLEAVED || f == PAINTY_HOST_F32_INTERLEAVED;
}

template <class TS>
void launch_scatter(DevType dt, const TS* src, PlanePtrs dst, int nch, int il, int32_t rows,
                    int32_t cols, int64_t pitch, int64_t es, cudaStream_t st) {
  const int64_t n = static_cast<int64_t>(rows) * cols * nch;
  const int g = grid_for(n, 256);
  switch (dt) {
    case DT_F32: scatter_kernel<float, TS><<<g, 256, 0, st>>>(src, dst, nch, il, rows, cols, pitch, es); break;
    case DT_F16: scatter_kernel<__half, TS><<<g, 256, 0, st>>>(src, dst, nch, il, rows, cols, pitch, es); break;
    case DT_BF16: scatter_kernel<__nv_bfloat16, TS><<<g, 256, 0, st>>>(src, dst, nch, il, rows, cols, pitch, es); break;
    case DT_F64: scatter_kernel<double, TS><<<g, 256, 0, st>>>(src, dst, nch, il, rows, cols, pitch, es); break;
  }
  count_launch();
  PG_CUDA(cudaGetLastError());
}

template <class TD>
void launch_gather(DevType dt, PlanePtrs src, TD* dst, int nch, int il, int32_t rows,
                   int32_t cols, int64_t pitch, int64_t es, cudaStream_t st) {
  const int64_t n = static_cast<int64_t>(rows) * cols * nch;
  const int g = grid_for(n, 256);
  switch (dt) {
    case DT_F32: gather_kernel<TD, float><<<g, 256, 0, st>>>(src, dst, nch, il, rows, cols, pitch, es); break;
    case DT_F16: gather_kernel<TD, __half><<<g, 256, 0, st>>>(src, dst, nch, il, rows, cols, pitch, es); break;
    case DT_BF16: gather_kernel<TD, __nv_bfloat16><<<g, 256, 0, st>>>(src, dst, nch, il, rows, cols, pitch, es); break;
    case DT_F64: gather_kernel<TD, double><<<g, 256, 0, st>>>(src, dst, nch, il, rows, cols, pitch, es); break;
  }
  count_launch();
  PG_CUDA(cudaGetLastError());
}

}  // namespace

void upload_planes(void* const* planes, int nch, DevType dt, int32_t rows, int32_t cols,
                   int64_t pitch, const void* host, painty_host_format fmt, cudaStream_t st,
                   int64_t estride) {
  upload_planes_async(planes, nch, dt, rows, cols, pitch, host, fmt, st, estride);
  PG_CUDA(cudaStreamSynchronize(st));
}

// The device address of pinned (page-locked, mapped) host memory, or nullptr for pageable
// memory. Kernels read and write such memory in place over the host link.
const void* mapped_host(const void* host) {
  cudaPointerAttributes pa{};
  if (cudaPointerGetAttributes(&pa, host) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return pa.type == cudaMemoryTypeHost ? pa.devicePointer : nullptr;
}

void upload_planes_async(void* const* planes, int nch, DevType dt, int32_t rows, int32_t cols,
                         int64_t pitch, const void* host, painty_host_format fmt,
                         cudaStream_t st, int64_t estride) {
  PG_REQUIRE(host != nullptr, "host buffer is null");
  PG_REQUIRE(fmt >= PAINTY_HOST_F64_INTERLEAVED && fmt <= PAINTY_HOST_F32_PLANAR,
             "unknown host format");
  const bool f64 = host_is_f64(fmt);
  const size_t hes = f64 ? 8 : 4;
  const size_t n = static_cast<size_t>(rows) * cols;
  // Fast path: planar host data of the device element type into planar device planes -> one
  // 2D copy per plane.
  if ((!host_is_interleaved(fmt) || nch == 1) && estride == 1) {
    if ((dt == DT_F32 && !f64) || (dt == DT_F64 && f64)) {
      for (int c = 0; c < nch; c++)
        PG_CUDA(cudaMemcpy2DAsync(planes[c], pitch * hes,
                                  static_cast<const char*>(host) + c * n * hes, cols * hes,
                                  cols * hes, rows, cudaMemcpyHostToDevice, st));
      return;
    }
  }
  // pinned host memory is read in place by the scatter kernel; pageable memory goes through
  // a device staging copy
  const void* mapped = mapped_host(host);
  void* staging = nullptr;
  if (!mapped) {
    staging = temp_alloc(n * nch * hes, st);
    PG_CUDA(cudaMemcpyAsync(staging, host, n * nch * hes, cudaMemcpyHostToDevice, st));
  }
  const void* src = mapped ? mapped : staging;
  PlanePtrs pp{{planes[0], nch > 1 ? planes[1] : nullptr, nch > 2 ? planes[2] : nullptr}};
  const int il = host_is_interleaved(fmt) ? 1 : 0;
  if (f64)
    launch_scatter<double>(dt, static_cast<const double*>(src), pp, nch, il, rows, cols, pitch,
                           estride, st);
  else
    launch_scatter<float>(dt, static_cast<const float*>(src), pp, nch, il, rows, cols, pitch,
                          estride, st);
  if (staging) PG_CUDA(cudaFreeAsync(staging, st));
}

void download_planes(const void* const* planes, int nch, DevType dt, int32_t rows,
                     int32_t cols, int64_t pitch, void* host, painty_host_format fmt,
                     cudaStream_t st, int64_t estride) {
  download_planes_async(planes, nch, dt, rows, cols, pitch, host, fmt, st, estride);
  PG_CUDA(cudaStreamSynchronize(st));
}

void download_planes_async(const void* const* planes, int nch, DevType dt, int32_t rows,
                           int32_t cols, int64_t pitch, void* host, painty_host_format fmt,
                           cudaStream_t st, int64_t estride) {
  PG_REQUIRE(host != nullptr, "host buffer is null");
  PG_REQUIRE(fmt >= PAINTY_HOST_F64_INTERLEAVED && fmt <= PAINTY_HOST_F32_PLANAR,
             "unknown host format");
  const bool f64 = host_is_f64(fmt);
  const size_t hes = f64 ? 8 : 4;
  const size_t n = static_cast<size_t>(rows) * cols;
  if ((!host_is_interleaved(fmt) || nch == 1) && estride == 1) {
    if ((dt == DT_F32 && !f64) || (dt == DT_F64 && f64)) {
      for (int c = 0; c < nch; c++)
        PG_CUDA(cudaMemcpy2DAsync(static_cast<char*>(host) + c * n * hes, cols * hes,
                                  planes[c], pitch * hes, cols * hes, rows,
                                  cudaMemcpyDeviceToHost, st));
      return;
    }
  }
  // pinned host memory is written in place by the gather kernel; pageable memory through a
  // device staging copy
  void* mapped = const_cast<void*>(mapped_host(host));
  void* staging = mapped ? nullptr : temp_alloc(n * nch * hes, st);
  void* dst = mapped ? mapped : staging;
  PlanePtrs pp{{const_cast<void*>(planes[0]), nch > 1 ? const_cast<void*>(planes[1]) : nullptr,
                nch > 2 ? const_cast<void*>(planes[2]) : nullptr}};
  const int il = host_is_interleaved(fmt) ? 1 : 0;
  if (f64)
    launch_gather<double>(dt, pp, static_cast<double*>(dst), nch, il, rows, cols, pitch,
                          estride, st);
  else
    launch_gather<float>(dt, pp, static_cast<float*>(dst), nch, il, rows, cols, pitch, estride,
                         st);
  if (staging) {
    PG_CUDA(cudaMemcpyAsync(host, staging, n * nch * hes, cudaMemcpyDeviceToHost, st));
    PG_CUDA(cudaFreeAsync(staging, st));
  }
}

void fill_planes(void* const* planes, int nch, DevType dt, int64_t elems, const double* v,
                 cudaStream_t st, int64_t estride) {
  PlanePtrs pp{{planes[0], nch > 1 ? planes[1] : nullptr, nch > 2 ? planes[2] : nullptr}};
  const int g = grid_for(elems * nch, 256);
  const double v0 = v[0], v1 = nch > 1 ? v[1] : 0.0, v2 = nch > 2 ? v[2] : 0.0;
  switch (dt) {
    case DT_F32: fill_kernel<float><<<g, 256, 0, st>>>(pp, nch, elems, v0, v1, v2, estride); break;
    case DT_F16: fill_kernel<__half><<<g, 256, 0, st>>>(pp, nch, elems, v0, v1, v2, estride); break;
    case DT_BF16: fill_kernel<__nv_bfloat16><<<g, 256, 0, st>>>(pp, nch, elems, v0, v1, v2, estride); break;
    case DT_F64: fill_kernel<double><<<g, 256, 0, st>>>(pp, nch, elems, v0, v1, v2, estride); break;
  }
  count_launch();
  PG_CUDA(cudaGetLastError());
}

void copy_layer(const painty_layer& src, painty_layer& dst, cudaStream_t st) {
  PG_REQUIRE(src.rows == dst.rows && src.cols == dst.cols && src.storage == dst.storage,
             "layers differ in size or storage");
  if (src.estride == dst.estride) {
    PG_CUDA(cudaMemcpyAsync(dst.base, src.base, src.bytes, cudaMemcpyDeviceToDevice, st));
    return;
  }
  LayerPtrs s{{src.K[0], src.K[1], src.K[2], src.S[0], src.S[1], src.S[2], src.V}};
  LayerPtrs d{{dst.K[0], dst.K[1], dst.K[2], dst.S[0], dst.S[1], dst.S[2], dst.V}};
  const int64_t elems = src.plane_elems();
  const int g = grid_for(elems, 256);
  switch (src.storage) {
    case PAINTY_STORAGE_F32:
      copy_layer_kernel<float, float><<<g, 256, 0, st>>>(s, d, elems, src.estride, dst.estride);
      break;
    case PAINTY_STORAGE_F16:
      copy_layer_kernel<__half, __half><<<g, 256, 0, st>>>(s, d, elems, src.estride, dst.estride);
      break;
    case PAINTY_STORAGE_BF16:
      copy_layer_kernel<__nv_bfloat16, __half><<<g, 256, 0, st>>>(s, d, elems, src.estride,
                                                                    dst.estride);
      break;
    case PAINTY_STORAGE_F64:
      copy_layer_kernel<double, double><<<g, 256, 0, st>>>(s, d, elems, src.estride, dst.estride);
      break;
  }
  count_launch();
  PG_CUDA(cudaGetLastError());
}

void copy_planes_async(void* const* dst, const void* const* src, int nch, size_t plane_bytes,
                       cudaStream_t st) {
  for (int c = 0; c < nch; c++)
    PG_CUDA(cudaMemcpyAsync(dst[c], src[c], plane_bytes, cudaMemcpyDeviceToDevice, st));
}

// ------------------------------------------------------------------ composite kernel
namespace {

constexpr int kMaxLayersPerLaunch = 16;

template <class TK, class TV, class TR>
struct ComposeArgs {
  const TK* K[kMaxLayersPerLaunch][3];
  const TK* S[kMaxLayersPerLaunch][3];
  const TV* V[kMaxLayersPerLaunch];
  const TR* r0[3];
  TR* out[3];
  int32_t L;
  int64_t groups;  // plane elements / 8
};

// One thread owns PIX consecutive pixels, PIX = 16 bytes of the K/S element type (4 for F32,
// 8 for F16/BF16, 2 for F64): 16-byte streaming loads of each layer's 7 planes, the KM
// recurrence R <- KM(K_l, S_l, R, V_l) through all L layers in registers, one streaming store
// of R. Per pixel this reads 7 L + 3 planes and writes 3, each exactly once. The grid is one
// wave of resident blocks walking the planes with a grid stride.
template <class TK, class TV, class TR>
__global__ void __launch_bounds__(256) km_composite_kernel(
  const __grid_constant__ ComposeArgs<TK, TV, TR> a) {
  using M = typename MathOf<TR>::type;
  constexpr int PIX = 16 / sizeof(TK);
  const int64_t groups = a.groups;
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t g = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; g < groups;
       g += stride) {
    const int64_t e = g * PIX;
    M r[3][PIX];
#pragma unroll
    for (int c = 0; c < 3; c++) {
      TR t[PIX];
      load_vec<PIX>(a.r0[c] + e, t);
#pragma unroll
      for (int i = 0; i < PIX; i++) r[c][i] = static_cast<M>(t[i]);
    }
    for (int l = 0; l < a.L; l++) {
      TV v[PIX];
      TK k[3][PIX], s[3][PIX];
      load_vec<PIX>(a.V[l] + e, v);
#pragma unroll
      for (int c = 0; c < 3; c++) {
        load_vec<PIX>(a.K[l][c] + e, k[c]);
        load_vec<PIX>(a.S[l][c] + e, s[c]);
      }
#pragma unroll
      for (int c = 0; c < 3; c++)
#pragma unroll
        for (int i = 0; i < PIX; i++)
          r[c][i] = km_reflectance(ld_elem<M>(&k[c][i]), ld_elem<M>(&s[c][i]), r[c][i],
                                   ld_elem<M>(&v[i]));
    }
#pragma unroll
    for (int c = 0; c < 3; c++) {
      TR t[PIX];
#pragma unroll
      for (int i = 0; i < PIX; i++) t[i] = static_cast<TR>(r[c][i]);
      store_vec<PIX>(a.out[c] + e, t);
    }
  }
}

// Composite over layers of any layout (a canvas's packed wet layer, or mixed stacks): one
// thread per pixel, each layer's values read with its element stride.
// 16-bit layer storage (FP16 / BF16 K and S, FP16 V): 4 pixels per thread, each plane read
// as one 8-byte vector, and the next layer's 7 vectors loaded before this layer is computed,
// so a thread keeps a layer's loads in flight while its KM arithmetic runs (FP32 math, R0 and
// the result in FP32).
template <class TK, class TV>
struct Compose16Args {
  const TK* K[kMaxLayersPerLaunch][3];
  const TK* S[kMaxLayersPerLaunch][3];
  const TV* V[kMaxLayersPerLaunch];
  const float* r0[3];
  float* out[3];
  int32_t L;
  int64_t groups;  // plane elements / 4
};
struct Layer16 {  // one layer's 4 pixels: K r,g,b, S r,g,b, V as packed 16-bit pairs
  uint2 k[3], s[3], v;
};
template <class T>
__device__ __forceinline__ float elem16(const uint2& w, int i) {
  const uint32_t word = i < 2 ? w.x : w.y;
  if constexpr (std::is_same<T, __nv_bfloat16>::value) {
    // BF16 is the top half of an FP32: place the half in the high bits (bit operations only)
    return __uint_as_float((i & 1) ? (word & 0xffff0000u) : (word << 16));
  } else {
    const unsigned short h = static_cast<unsigned short>((i & 1) ? word >> 16 : word & 0xffffu);
    T t;
    memcpy(&t, &h, 2);
    return to_f(t);
  }
}
template <class TK, class TV>
__device__ __forceinline__ void load_layer16(const Compose16Args<TK, TV>& a, int l, int64_t e,
                                             Layer16& o) {
#pragma unroll
  for (int c = 0; c < 3; c++) {
    o.k[c] = ld_stream_u2(a.K[l][c] + e);
    o.s[c] = ld_stream_u2(a.S[l][c] + e);
  }
  o.v = ld_stream_u2(a.V[l] + e);
}
template <class TK, class TV>
__global__ void __launch_bounds__(256, 4) km_composite16_kernel(
  const __grid_constant__ Compose16Args<TK, TV> a) {
  const int64_t groups = a.groups;
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t g = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; g < groups;
       g += stride) {
    const int64_t e = g * 4;
    float r[3][4];
#pragma unroll
    for (int c = 0; c < 3; c++) {
      const uint4 t = ld_stream_u4(a.r0[c] + e);
      r[c][0] = __uint_as_float(t.x);
      r[c][1] = __uint_as_float(t.y);
      r[c][2] = __uint_as_float(t.z);
      r[c][3] = __uint_as_float(t.w);
    }
    Layer16 cur, nxt;
    load_layer16(a, 0, e, cur);
    for (int l = 0; l < a.L; l++) {
      if (l + 1 < a.L) load_layer16(a, l + 1, e, nxt);
#pragma unroll
      for (int i = 0; i < 4; i += 2) {  // pixel pairs on the packed FP32 pipe
        const float2 d = f2(elem16<TV>(cur.v, i), elem16<TV>(cur.v, i + 1));
        float2 K[3], S[3], R[3];
#pragma unroll
        for (int c = 0; c < 3; c++) {
          K[c] = f2(elem16<TK>(cur.k[c], i), elem16<TK>(cur.k[c], i + 1));
          S[c] = f2(elem16<TK>(cur.s[c], i), elem16<TK>(cur.s[c], i + 1));
          R[c] = f2(r[c][i], r[c][i + 1]);
        }
        km_reflectance2x3(K, S, R, d);
#pragma unroll
        for (int c = 0; c < 3; c++) {
          r[c][i] = R[c].x;
          r[c][i + 1] = R[c].y;
        }
      }
      cur = nxt;
    }
#pragma unroll
    for (int c = 0; c < 3; c++)
      st_stream_u4(a.out[c] + e, make_uint4(__float_as_uint(r[c][0]), __float_as_uint(r[c][1]),
                                            __float_as_uint(r[c][2]), __float_as_uint(r[c][3])));
  }
}

// ---- bulk-copy pipeline primitives (mbarrier + cp.async.bulk, PTX ISA 8.0+)
__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint64_t* b, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(b)), "r"(count)
               : "memory");
}
__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* b) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(b)) : "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* b, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(b)),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* b, uint32_t parity) {
  uint32_t ok;
  asm volatile(
    "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
    "selp.u32 %0, 1, 0, p;\n\t}"
    : "=r"(ok)
    : "r"(smem_addr(b)), "r"(parity)
    : "memory");
  return ok != 0;
}
__device__ __forceinline__ uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
// Waits for the completion of the barrier's phase of `parity`. Gives up -- recording the
// fault in g_pipeline_fault and raising the block's abort flag -- after one second, or at
// once when another thread of the block has given up already (abort flag set).
__device__ __forceinline__ bool mbar_wait(uint64_t* b, uint32_t parity,
                                          volatile int* abort_flag) {
  if (mbar_try_wait(b, parity)) return true;
  const uint64_t t0 = global_ns();
  for (;;) {
    if (mbar_try_wait(b, parity)) return true;
    if (abort_flag && *abort_flag) return false;
    if (global_ns() - t0 > 1000000000ull) {
      atomicExch(&g_pipeline_fault, 1u);
      if (abort_flag) *abort_flag = 1;
      return false;
    }
  }
}
// Global -> shared bulk copy completing on `bar` (16-byte aligned addresses, size a multiple
// of 16).
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes,
                                         uint64_t* bar) {
  asm volatile(
    "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
    ::"r"(smem_addr(dst)), "l"(src), "r"(bytes), "r"(smem_addr(bar))
    : "memory");
}

// 16-bit composite fed by bulk copies. The register-fed kernel above keeps only two layers'
// loads in flight per thread and its occupancy is limited by the KM arithmetic's registers,
// so HBM waits on latency. Here one thread per block streams the planes into shared memory
// with cp.async.bulk (a 5-deep ring of stages, one stage = one layer's 7 planes of a tile of
// 1024 pixels, plus the tile's R0 planes with its first layer), and eight warps compute
// from shared memory: ~70 KB in flight per block, two blocks per SM, whatever the registers.
// Each consumer thread owns 4 consecutive pixels of the tile and carries R through the
// layers in registers; the result is stored straight from registers.
constexpr int kBulkTile = 1024;     // pixels per tile
constexpr int kBulkStages = 5;      // ring depth
constexpr int kBulkConsumers = 8;   // consumer warps (4 pixels per thread)
constexpr size_t kBulkStageBytes = size_t(7) * kBulkTile * 2;
constexpr size_t kBulkR0Bytes = size_t(3) * kBulkTile * 4;
constexpr size_t kBulkSmem = kBulkStages * kBulkStageBytes + 2 * kBulkR0Bytes + 256;

template <class TK, class TV>
__global__ void __launch_bounds__(32 * (kBulkConsumers + 1), 2) km_composite16_bulk_kernel(
  const __grid_constant__ Compose16Args<TK, TV> a) {
  extern __shared__ __align__(128) unsigned char smem[];
  uint16_t* stages = reinterpret_cast<uint16_t*>(smem);
  float* r0buf = reinterpret_cast<float*>(smem + kBulkStages * kBulkStageBytes);
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + kBulkStages * kBulkStageBytes +
                                               2 * kBulkR0Bytes);
  uint64_t* full = bars;                      // [kBulkStages], one arrival + the bytes
  uint64_t* empty = bars + kBulkStages;       // [kBulkStages], one arrival per consumer warp
  uint64_t* r0free = bars + 2 * kBulkStages;  // [2], one arrival per consumer warp
  volatile int* abort_flag = reinterpret_cast<volatile int*>(bars + 2 * kBulkStages + 2);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    for (int i = 0; i < kBulkStages; i++) {
      mbar_init(&full[i], 1);
      mbar_init(&empty[i], kBulkConsumers);
    }
    mbar_init(&r0free[0], kBulkConsumers);
    mbar_init(&r0free[1], kBulkConsumers);
    *abort_flag = 0;
    fence_mbar_init();
  }
  __syncthreads();

  const int64_t elems = a.groups * 4;
  const int64_t ntiles = (elems + kBulkTile - 1) / kBulkTile;
  const int L = a.L;

  if (warp == kBulkConsumers) {  // producer
    if (lane != 0) return;
    uint32_t q = 0, slot = 0, use = 0, tl = 0;
    bool ok = true;
    for (int64_t tile = blockIdx.x; ok && tile < ntiles; tile += gridDim.x, tl++) {
      const int64_t base = tile * kBulkTile;
      const int64_t rest = elems - base;
      const uint32_t n = static_cast<uint32_t>(rest < kBulkTile ? rest : kBulkTile);
      for (int l = 0; l < L; l++) {
        if (use > 0 && !mbar_wait(&empty[slot], (use - 1) & 1, abort_flag)) {
          ok = false;
          break;
        }
        if (l == 0 && tl >= 2 && !mbar_wait(&r0free[tl & 1], ((tl >> 1) - 1) & 1, abort_flag)) {
          ok = false;
          break;
        }
        const uint32_t pb = n * 2;
        mbar_arrive_expect_tx(&full[slot], 7 * pb + (l == 0 ? 3 * n * 4 : 0));
        uint16_t* sb = stages + slot * (7 * kBulkTile);
#pragma unroll
        for (int c = 0; c < 3; c++) {
          bulk_g2s(sb + c * kBulkTile, a.K[l][c] + base, pb, &full[slot]);
          bulk_g2s(sb + (3 + c) * kBulkTile, a.S[l][c] + base, pb, &full[slot]);
        }
        bulk_g2s(sb + 6 * kBulkTile, a.V[l] + base, pb, &full[slot]);
        if (l == 0) {
          float* rb = r0buf + (tl & 1) * (3 * kBulkTile);
#pragma unroll
          for (int c = 0; c < 3; c++) bulk_g2s(rb + c * kBulkTile, a.r0[c] + base, n * 4, &full[slot]);
        }
        q++;
        if (++slot == kBulkStages) {
          slot = 0;
          use++;
        }
      }
    }
    if (!ok) {  // the consumers gave up: let the copies in flight land before the block exits
      for (uint32_t k = q > kBulkStages ? q - kBulkStages : 0; k < q; k++)
        mbar_wait(&full[k % kBulkStages], (k / kBulkStages) & 1, nullptr);
    }
    return;
  }

  // consumers
  const int p0 = threadIdx.x * 4;
  uint32_t slot = 0, use = 0, tl = 0;
  for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x, tl++) {
    const int64_t base = tile * kBulkTile;
    const bool act = base + p0 < elems;
    float r[3][4];
    for (int l = 0; l < L; l++) {
      if (!mbar_wait(&full[slot], use & 1, abort_flag)) {
        if (act) {  // a stalled pipeline leaves NaN, never a plausible image
#pragma unroll
          for (int c = 0; c < 3; c++)
            st_stream_u4(a.out[c] + base + p0, make_uint4(0x7fc00000u, 0x7fc00000u,
                                                           0x7fc00000u, 0x7fc00000u));
        }
        return;
      }
      if (l == 0) {
        const float* rb = r0buf + (tl & 1) * (3 * kBulkTile);
#pragma unroll
        for (int c = 0; c < 3; c++) {
          const float4 t = *reinterpret_cast<const float4*>(rb + c * kBulkTile + p0);
          r[c][0] = t.x;
          r[c][1] = t.y;
          r[c][2] = t.z;
          r[c][3] = t.w;
        }
        __syncwarp();
        if (lane == 0) mbar_arrive(&r0free[tl & 1]);
      }
      const uint16_t* sb = stages + slot * (7 * kBulkTile) + p0;
      Layer16 cur;
#pragma unroll
      for (int c = 0; c < 3; c++) {
        cur.k[c] = *reinterpret_cast<const uint2*>(sb + c * kBulkTile);
        cur.s[c] = *reinterpret_cast<const uint2*>(sb + (3 + c) * kBulkTile);
      }
      cur.v = *reinterpret_cast<const uint2*>(sb + 6 * kBulkTile);
      __syncwarp();
      if (lane == 0) mbar_arrive(&empty[slot]);
      if (++slot == kBulkStages) {
        slot = 0;
        use++;
      }
#pragma unroll
      for (int i = 0; i < 4; i += 2) {
        const float2 d = f2(elem16<TV>(cur.v, i), elem16<TV>(cur.v, i + 1));
        float2 K[3], S[3], R[3];
#pragma unroll
        for (int c = 0; c < 3; c++) {
          K[c] = f2(elem16<TK>(cur.k[c], i), elem16<TK>(cur.k[c], i + 1));
          S[c] = f2(elem16<TK>(cur.s[c], i), elem16<TK>(cur.s[c], i + 1));
          R[c] = f2(r[c][i], r[c][i + 1]);
        }
        km_reflectance2x3<false>(K, S, R, d);  // 16-bit layers: no guards needed
#pragma unroll
        for (int c = 0; c < 3; c++) {
          r[c][i] = R[c].x;
          r[c][i + 1] = R[c].y;
        }
      }
    }
    if (act) {
#pragma unroll
      for (int c = 0; c < 3; c++)
        st_stream_u4(a.out[c] + base + p0,
                     make_uint4(__float_as_uint(r[c][0]), __float_as_uint(r[c][1]),
                                __float_as_uint(r[c][2]), __float_as_uint(r[c][3])));
    }
  }
}

template <class TK, class TV, class TR>
struct ComposeStridedArgs {
  const TK* K[kMaxLayersPerLaunch][3];
  const TK* S[kMaxLayersPerLaunch][3];
  const TV* V[kMaxLayersPerLaunch];
  int64_t es[kMaxLayersPerLaunch];
  const TR* r0[3];
  TR* out[3];
  int32_t L;
  int64_t elems;
};
template <class TK, class TV, class TR>
__global__ void __launch_bounds__(256) km_composite_strided_kernel(
  const __grid_constant__ ComposeStridedArgs<TK, TV, TR> a) {
  using M = typename MathOf<TR>::type;
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < a.elems;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    M r[3];
#pragma unroll
    for (int c = 0; c < 3; c++) r[c] = static_cast<M>(a.r0[c][i]);
    for (int l = 0; l < a.L; l++) {
      const int64_t j = i * a.es[l];
      const M v = ld_elem<M>(a.V[l] + j);
#pragma unroll
      for (int c = 0; c < 3; c++)
        r[c] = km_reflectance(ld_elem<M>(a.K[l][c] + j), ld_elem<M>(a.S[l][c] + j), r[c], v);
    }
#pragma unroll
    for (int c = 0; c < 3; c++) a.out[c][i] = static_cast<TR>(r[c]);
  }
}

template <class Kern>
int resident_grid(Kern kern, int block) {
  static int cached[64] = {0};
  int dev = 0;
  PG_CUDA(cudaGetDevice(&dev));
  if (dev < 64 && cached[dev] > 0) return cached[dev];
  int sms = 0, per_sm = 0;
  PG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  PG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, block, 0));
  const int g = std::max(1, sms * std::max(1, per_sm));
  if (dev < 64) cached[dev] = g;
  return g;
}

template <class TK, class TV, class TR>
void compose_strided(const painty_layer* const* layers, int32_t L, const painty_image* r0,
                     painty_image* out, cudaStream_t st) {
  const int64_t elems = r0->plane_elems();
  auto kern = km_composite_strided_kernel<TK, TV, TR>;
  const int wave = resident_grid(kern, 256);
  for (int32_t l0 = 0; l0 < L; l0 += kMaxLayersPerLaunch) {
    ComposeStridedArgs<TK, TV, TR> a{};
    const int32_t n = std::min<int32_t>(kMaxLayersPerLaunch, L - l0);
    for (int32_t i = 0; i < n; i++) {
      const painty_layer* ly = layers[l0 + i];
      for (int c = 0; c < 3; c++) {
        a.K[i][c] = static_cast<const TK*>(ly->K[c]);
        a.S[i][c] = static_cast<const TK*>(ly->S[c]);
      }
      a.V[i] = static_cast<const TV*>(ly->V);
      a.es[i] = ly->estride;
    }
    const painty_image* src = l0 == 0 ? r0 : out;
    for (int c = 0; c < 3; c++) {
      a.r0[c] = static_cast<const TR*>(src->R[c]);
      a.out[c] = static_cast<TR*>(out->R[c]);
    }
    a.L = n;
    a.elems = elems;
    const int grid = static_cast<int>(std::min<int64_t>((elems + 255) / 256, wave));
    kern<<<std::max(grid, 1), 256, 0, st>>>(a);
    count_launch();
    PG_CUDA(cudaGetLastError());
  }
}

template <class TK, class TV>
int bulk_grid() {
  static int cached[64] = {0};
  int dev = 0;
  PG_CUDA(cudaGetDevice(&dev));
  if (dev < 64 && cached[dev] > 0) return cached[dev];
  auto kern = km_composite16_bulk_kernel<TK, TV>;
  PG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               static_cast<int>(kBulkSmem)));
  int sms = 0, per_sm = 0;
  PG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  PG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 32 * (kBulkConsumers + 1),
                                                        kBulkSmem));
  const int g = std::max(1, sms * std::max(1, per_sm));
  if (dev < 64) cached[dev] = g;
  return g;
}

bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15) == 0; }

template <class TK, class TV>
void compose16(const painty_layer* const* layers, int32_t L, const painty_image* r0,
               painty_image* out, cudaStream_t st) {
  const int64_t elems = r0->plane_elems();  // a multiple of 64 elements
  bool bulk = true;  // every plane 16-byte aligned: the bulk-copy kernel
  for (int32_t l = 0; l < L; l++) {
    for (int c = 0; c < 3; c++)
      bulk = bulk && aligned16(layers[l]->K[c]) && aligned16(layers[l]->S[c]);
    bulk = bulk && aligned16(layers[l]->V);
  }
  for (int c = 0; c < 3; c++) bulk = bulk && aligned16(r0->R[c]) && aligned16(out->R[c]);
  auto kern = bulk ? km_composite16_bulk_kernel<TK, TV> : km_composite16_kernel<TK, TV>;
  const int block = bulk ? 32 * (kBulkConsumers + 1) : 256;
  const size_t smem = bulk ? kBulkSmem : 0;
  const int wave = bulk ? bulk_grid<TK, TV>() : resident_grid(kern, 256);
  for (int32_t l0 = 0; l0 < L; l0 += kMaxLayersPerLaunch) {
    Compose16Args<TK, TV> a{};
    const int32_t n = std::min<int32_t>(kMaxLayersPerLaunch, L - l0);
    for (int32_t i = 0; i < n; i++) {
      const painty_layer* ly = layers[l0 + i];
      for (int c = 0; c < 3; c++) {
        a.K[i][c] = static_cast<const TK*>(ly->K[c]);
        a.S[i][c] = static_cast<const TK*>(ly->S[c]);
      }
      a.V[i] = static_cast<const TV*>(ly->V);
    }
    const painty_image* src = l0 == 0 ? r0 : out;
    for (int c = 0; c < 3; c++) {
      a.r0[c] = static_cast<const float*>(src->R[c]);
      a.out[c] = static_cast<float*>(out->R[c]);
    }
    a.L = n;
    a.groups = elems / 4;
    const int64_t blocks_needed =
      bulk ? (elems + kBulkTile - 1) / kBulkTile : (a.groups + 255) / 256;
    const int grid = static_cast<int>(std::min<int64_t>(blocks_needed, wave));
    kern<<<std::max(grid, 1), block, smem, st>>>(a);
    count_launch();
    PG_CUDA(cudaGetLastError());
  }
}

template <class TK, class TV, class TR>
void compose_typed(const painty_layer* const* layers, int32_t L, const painty_image* r0,
                   painty_image* out, cudaStream_t st) {
  for (int32_t l = 0; l < L; l++)
    if (layers[l]->estride != 1) {
      compose_strided<TK, TV, TR>(layers, L, r0, out, st);
      return;
    }
  if constexpr (sizeof(TK) == 2) {
    compose16<TK, TV>(layers, L, r0, out, st);
  } else {
  constexpr int PIX = 16 / sizeof(TK);
  const int64_t elems = r0->plane_elems();  // a multiple of 64 elements
  auto kern = km_composite_kernel<TK, TV, TR>;
  const int wave = resident_grid(kern, 256);
  for (int32_t l0 = 0; l0 < L; l0 += kMaxLayersPerLaunch) {
    ComposeArgs<TK, TV, TR> a{};
    const int32_t n = std::min<int32_t>(kMaxLayersPerLaunch, L - l0);
    for (int32_t i = 0; i < n; i++) {
      const painty_layer* ly = layers[l0 + i];
      for (int c = 0; c < 3; c++) {
        a.K[i][c] = static_cast<const TK*>(ly->K[c]);
        a.S[i][c] = static_cast<const TK*>(ly->S[c]);
      }
      a.V[i] = static_cast<const TV*>(ly->V);
    }
    const painty_image* src = l0 == 0 ? r0 : out;
    for (int c = 0; c < 3; c++) {
      a.r0[c] = static_cast<const TR*>(src->R[c]);
      a.out[c] = static_cast<TR*>(out->R[c]);
    }
    a.L = n;
    a.groups = elems / PIX;
    const int64_t blocks_needed = (a.groups + 255) / 256;
    const int grid = static_cast<int>(std::min<int64_t>(blocks_needed, wave));
    kern<<<std::max(grid, 1), 256, 0, st>>>(a);
    count_launch();
    PG_CUDA(cudaGetLastError());
  }
  }
}

}  // namespace

void launch_compose(const painty_layer* const* layers, int32_t L, const painty_image* r0,
                    painty_image* out, cudaStream_t st) {
  PG_REQUIRE(r0 && out, "null image");
  PG_REQUIRE(L >= 0, "negative layer count");
  PG_REQUIRE(r0->rows == out->rows && r0->cols == out->cols, "image sizes differ");
  PG_REQUIRE(r0->storage == out->storage, "image storages differ");
  const painty_storage s = L > 0 ? layers[0]->storage : PAINTY_STORAGE_F32;
  for (int32_t l = 0; l < L; l++) {
    PG_REQUIRE(layers[l] != nullptr, "null layer");
    PG_REQUIRE(layers[l]->rows == r0->rows && layers[l]->cols == r0->cols,
               "layer size differs from the substrate (painty reallocates R0 here; pass an "
               "image of the layer's size)");
    PG_REQUIRE(layers[l]->storage == s, "layers have different storage formats");
  }
  if (L == 0) {
    if (out != r0) {
      const void* src[3] = {r0->R[0], r0->R[1], r0->R[2]};
      copy_planes_async(out->R, src, 3, r0->plane_elems() * r_bytes(r0->storage), st);
    }
    return;
  }
  if (s == PAINTY_STORAGE_F64) {
    PG_REQUIRE(r0->storage == PAINTY_STORAGE_F64, "F64 layers compose onto an F64 image");
    compose_typed<double, double, double>(layers, L, r0, out, st);
    return;
  }
  PG_REQUIRE(r0->storage == PAINTY_STORAGE_F32, "F32/F16/BF16 layers compose onto an F32 image");
  switch (s) {
    case PAINTY_STORAGE_F32: compose_typed<float, float, float>(layers, L, r0, out, st); break;
    case PAINTY_STORAGE_F16: compose_typed<__half, __half, float>(layers, L, r0, out, st); break;
    case PAINTY_STORAGE_BF16:
      compose_typed<__nv_bfloat16, __half, float>(layers, L, r0, out, st);
      break;
    default: fail(PAINTY_ERR_INVALID_ARGUMENT, "bad storage");
  }
}

// ------------------------------------------------------------------ drying kernel
namespace {
// Canvas::dryCanvas (painty/renderer/Canvas.hxx:105-121): h += V; R0 = KM(K, S, R0, V);
// K = S = V = 0. One pass over the wet layer, R0 and h.
struct PtrTriple {
  void* p[3];
};

template <class TK, class TV, class TR>
__global__ void __launch_bounds__(256) km_dry_kernel(PtrTriple wk, PtrTriple ws, TV* v, TV* h,
                                                       PtrTriple r0, int64_t elems, int64_t es) {
  using M = typename MathOf<TR>::type;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < elems;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t j = i * es;  // the wet layer's element (packed or planar)
    const M vol = ld_elem<M>(v + j);
    st_elem<M>(h + i, ld_elem<M>(h + i) + vol);
#pragma unroll
    for (int c = 0; c < 3; c++) {
      TK* kp = static_cast<TK*>(wk.p[c]);
      TK* sp = static_cast<TK*>(ws.p[c]);
      TR* rp = static_cast<TR*>(r0.p[c]);
      const M r = km_reflectance(ld_elem<M>(kp + j), ld_elem<M>(sp + j), ld_elem<M>(rp + i), vol);
      st_elem<M>(rp + i, r);
      st_elem<M>(kp + j, M(0));
      st_elem<M>(sp + j, M(0));
    }
    st_elem<M>(v + j, M(0));
  }
}

template <class TK, class TV, class TR>
void dry_typed(painty_canvas* c, cudaStream_t st) {
  const int64_t elems = c->wet.plane_elems();
  PtrTriple wk{{c->wet.K[0], c->wet.K[1], c->wet.K[2]}};
  PtrTriple ws{{c->wet.S[0], c->wet.S[1], c->wet.S[2]}};
  PtrTriple r0{{c->r0.R[0], c->r0.R[1], c->r0.R[2]}};
  const int g = grid_for(elems, 256);
  km_dry_kernel<TK, TV, TR><<<g, 256, 0, st>>>(wk, ws, static_cast<TV*>(c->wet.V),
                                                 static_cast<TV*>(c->h), r0, elems,
                                                 c->wet.estride);
  count_launch();
  PG_CUDA(cudaGetLastError());
}
}  // namespace

}  // namespace pg

// ====================================================================== C ABI
using pg::guard;

extern "C" {

int32_t painty_abi_version(void) { return PAINTY_GB300_ABI_VERSION; }

const char* painty_status_string(painty_status s) {
  switch (s) {
    case PAINTY_OK: return "ok";
    case PAINTY_ERR_INVALID_ARGUMENT: return "invalid argument";
    case PAINTY_ERR_OUT_OF_MEMORY: return "out of memory";
    case PAINTY_ERR_CUDA: return "CUDA error";
    case PAINTY_ERR_UNSUPPORTED: return "unsupported";
    case PAINTY_ERR_BUDGET: return "over memory budget";
    case PAINTY_ERR_TIMEOUT: return "device wait timed out";
    case PAINTY_ERR_CANCELLED: return "cancelled";
    case PAINTY_ERR_STATE: return "invalid state";
  }
  return "unknown status";
}

const char* painty_last_error(void) { return pg::g_last_error.c_str(); }

int64_t painty_kernel_launch_count(void) { return pg::g_launches.load(); }

painty_status painty_take_device_faults(uint32_t* faults) {
  return guard([&] {
    PG_REQUIRE(faults != nullptr, "faults is null");
    unsigned int v = 0, zero = 0;
    PG_CUDA(cudaDeviceSynchronize());
    PG_CUDA(cudaMemcpyFromSymbol(&v, pg::g_pipeline_fault, sizeof(v)));
    PG_CUDA(cudaMemcpyToSymbol(pg::g_pipeline_fault, &zero, sizeof(zero)));
    *faults = v;
  });
}

// ---------------------------------------------------------------- layers
painty_status painty_layer_create(int32_t rows, int32_t cols, painty_storage storage,
                                  painty_layer** out) {
  return guard([&] {
    PG_REQUIRE(out != nullptr, "out is null");
    PG_REQUIRE(rows > 0 && cols > 0, "rows and cols must be positive");
    PG_REQUIRE(pg::valid_storage(storage), "unknown storage format");
    auto* L = new painty_layer();
    try {
      void* base = pg::device_alloc(pg::layer_bytes(rows, cols, storage));
      pg::layer_layout(*L, rows, cols, storage, base);
      PG_CUDA(cudaMemset(base, 0, L->bytes));
    } catch (...) {
      if (L->base) pg::device_free(L->base);
      delete L;
      throw;
    }
    *out = L;
  });
}

painty_status painty_layer_destroy(painty_layer* layer) {
  return guard([&] {
    if (!layer) return;
    PG_REQUIRE(layer->owned, "borrowed layer handles are not destroyed");
    pg::device_free(layer->base);
    delete layer;
  });
}

painty_status painty_layer_clear(painty_layer* layer, void* stream) {
  return guard([&] {
    PG_REQUIRE(layer != nullptr, "layer is null");
    PG_CUDA(cudaMemsetAsync(layer->base, 0, layer->bytes, pg::as_stream(stream)));
    layer->touch();
  });
}

static void layer_plane_ptrs(const painty_layer* L, painty_plane plane, void** p, int* nch,
                             pg::DevType* dt) {
  switch (plane) {
    case PAINTY_PLANE_K:
      for (int c = 0; c < 3; c++) p[c] = L->K[c];
      *nch = 3;
      *dt = pg::ks_type(L->storage);
      return;
    case PAINTY_PLANE_S:
      for (int c = 0; c < 3; c++) p[c] = L->S[c];
      *nch = 3;
      *dt = pg::ks_type(L->storage);
      return;
    case PAINTY_PLANE_V:
      p[0] = L->V;
      *nch = 1;
      *dt = pg::v_type(L->storage);
      return;
    default: pg::fail(PAINTY_ERR_INVALID_ARGUMENT, "a layer has planes K, S and V");
  }
}

painty_status painty_layer_upload(painty_layer* layer, painty_plane plane, const void* host,
                                  painty_host_format fmt, void* stream) {
  return guard([&] {
    PG_REQUIRE(layer != nullptr, "layer is null");
    void* p[3] = {nullptr, nullptr, nullptr};
    int nch = 0;
    pg::DevType dt;
    layer_plane_ptrs(layer, plane, p, &nch, &dt);
    pg::upload_planes(p, nch, dt, layer->rows, layer->cols, layer->pitch, host, fmt,
                      pg::as_stream(stream), layer->estride);
    layer->touch();
  });
}

painty_status painty_layer_download(const painty_layer* layer, painty_plane plane, void* host,
                                    painty_host_format fmt, void* stream) {
  return guard([&] {
    PG_REQUIRE(layer != nullptr, "layer is null");
    void* p[3] = {nullptr, nullptr, nullptr};
    int nch = 0;
    pg::DevType dt;
    layer_plane_ptrs(layer, plane, p, &nch, &dt);
    const void* cp[3] = {p[0], p[1], p[2]};
    pg::download_planes(cp, nch, dt, layer->rows, layer->cols, layer->pitch, host, fmt,
                        pg::as_stream(stream), layer->estride);
  });
}

painty_status painty_layer_copy(const painty_layer* src, painty_layer* dst, void* stream) {
  return guard([&] {
    PG_REQUIRE(src && dst, "layer is null");
    pg::copy_layer(*src, *dst, pg::as_stream(stream));
    dst->touch();
  });
}

painty_status painty_layer_set_cells(painty_layer* layer, int64_t n, const int32_t* rows_cols,
                                     const double* K, const double* S, const double* V,
                                     void* stream) {
  return guard([&] {
    PG_REQUIRE(layer != nullptr, "layer is null");
    PG_REQUIRE(n >= 0 && n <= (int64_t(1) << 24), "n must be in [0, 2^24]");
    if (n == 0) return;
    PG_REQUIRE(rows_cols && K && S && V, "null argument");
    std::vector<double> vals(static_cast<size_t>(n) * 7);
    for (int64_t m = 0; m < n; m++) {
      const int32_t r = rows_cols[2 * m], c = rows_cols[2 * m + 1];
      PG_REQUIRE(r >= 0 && r < layer->rows && c >= 0 && c < layer->cols,
                 "cell outside the layer");
      for (int q = 0; q < 3; q++) {
        vals[7 * m + q] = K[3 * m + q];
        vals[7 * m + 3 + q] = S[3 * m + q];
      }
      vals[7 * m + 6] = V[m];
    }
    const cudaStream_t st = pg::as_stream(stream);
    char* d = nullptr;
    const size_t brc = static_cast<size_t>(n) * 2 * sizeof(int32_t);
    const size_t bv = vals.size() * sizeof(double);
    d = static_cast<decltype(d)>(pg::temp_alloc(brc + bv + 16, st));
    char* dv = d + (brc + 15) / 16 * 16;
    PG_CUDA(cudaMemcpyAsync(d, rows_cols, brc, cudaMemcpyHostToDevice, st));
    PG_CUDA(cudaMemcpyAsync(dv, vals.data(), bv, cudaMemcpyHostToDevice, st));
    pg::LayerPtrs lp{};
    for (int c = 0; c < 3; c++) {
      lp.p[c] = layer->K[c];
      lp.p[3 + c] = layer->S[c];
    }
    lp.p[6] = layer->V;
    for (int64_t b0 = 0; b0 < n; b0 += 4096) {
      const int64_t nb = std::min<int64_t>(4096, n - b0);
      const auto* rc = reinterpret_cast<const int32_t*>(d) + 2 * b0;
      const auto* v = reinterpret_cast<const double*>(dv) + 7 * b0;
      const int g = static_cast<int>((nb + 255) / 256);
      switch (layer->storage) {
        case PAINTY_STORAGE_F32:
          pg::set_cells_kernel<float, float><<<g, 256, 0, st>>>(lp, layer->pitch, layer->estride, rc, v, nb);
          break;
        case PAINTY_STORAGE_F16:
          pg::set_cells_kernel<__half, __half><<<g, 256, 0, st>>>(lp, layer->pitch, layer->estride, rc, v, nb);
          break;
        case PAINTY_STORAGE_BF16:
          pg::set_cells_kernel<__nv_bfloat16, __half><<<g, 256, 0, st>>>(lp, layer->pitch, layer->estride, rc, v, nb);
          break;
        case PAINTY_STORAGE_F64:
          pg::set_cells_kernel<double, double><<<g, 256, 0, st>>>(lp, layer->pitch, layer->estride, rc, v, nb);
          break;
      }
      pg::count_launch();
      PG_CUDA(cudaGetLastError());
    }
    PG_CUDA(cudaFreeAsync(d, st));
    PG_CUDA(cudaStreamSynchronize(st));
    layer->touch();
  });
}

painty_status painty_layer_info(const painty_layer* layer, int32_t* rows, int32_t* cols,
                                painty_storage* storage) {
  return guard([&] {
    PG_REQUIRE(layer != nullptr, "layer is null");
    if (rows) *rows = layer->rows;
    if (cols) *cols = layer->cols;
    if (storage) *storage = layer->storage;
  });
}

// ---------------------------------------------------------------- images
painty_status painty_image_create(int32_t rows, int32_t cols, painty_storage storage,
                                  painty_image** out) {
  return guard([&] {
    PG_REQUIRE(out != nullptr, "out is null");
    PG_REQUIRE(rows > 0 && cols > 0, "rows and cols must be positive");
    PG_REQUIRE(storage == PAINTY_STORAGE_F32 || storage == PAINTY_STORAGE_F64,
               "images are F32 or F64");
    auto* I = new painty_image();
    try {
      void* base = pg::device_alloc(pg::image_bytes(rows, cols, storage));
      pg::image_layout(*I, rows, cols, storage, base);
      PG_CUDA(cudaMemset(base, 0, I->bytes));
    } catch (...) {
      if (I->base) pg::device_free(I->base);
      delete I;
      throw;
    }
    *out = I;
  });
}

painty_status painty_image_destroy(painty_image* img) {
  return guard([&] {
    if (!img) return;
    PG_REQUIRE(img->owned, "borrowed image handles are not destroyed");
    pg::device_free(img->base);
    delete img;
  });
}

painty_status painty_image_fill(painty_image* img, double r, double g, double b, void* stream) {
  return guard([&] {
    PG_REQUIRE(img != nullptr, "image is null");
    const double v[3] = {r, g, b};
    pg::fill_planes(img->R, 3, pg::r_type(img->storage), img->plane_elems(), v,
                    pg::as_stream(stream));
  });
}

painty_status painty_image_upload(painty_image* img, const void* host, painty_host_format fmt,
                                  void* stream) {
  return guard([&] {
    PG_REQUIRE(img != nullptr, "image is null");
    pg::upload_planes(img->R, 3, pg::r_type(img->storage), img->rows, img->cols, img->pitch,
                      host, fmt, pg::as_stream(stream));
  });
}

painty_status painty_image_download(const painty_image* img, void* host, painty_host_format fmt,
                                    void* stream) {
  return guard([&] {
    PG_REQUIRE(img != nullptr, "image is null");
    const void* p[3] = {img->R[0], img->R[1], img->R[2]};
    pg::download_planes(p, 3, pg::r_type(img->storage), img->rows, img->cols, img->pitch, host,
                        fmt, pg::as_stream(stream));
  });
}

// ---------------------------------------------------------------- composite
painty_status painty_compose_layers(const painty_layer* const* layers, int32_t L,
                                    const painty_image* r0, painty_image* out, void* stream) {
  return guard([&] {
    PG_REQUIRE(L == 0 || layers != nullptr, "layers is null");
    pg::launch_compose(layers, L, r0, out, pg::as_stream(stream));
  });
}

painty_status painty_compose_layers_unfused(const painty_layer* const* layers, int32_t L,
                                            const painty_image* r0, painty_image* out,
                                            void* stream) {
  return guard([&] {
    PG_REQUIRE(L == 0 || layers != nullptr, "layers is null");
    if (L == 0) {
      pg::launch_compose(layers, 0, r0, out, pg::as_stream(stream));
      return;
    }
    pg::launch_compose(layers, 1, r0, out, pg::as_stream(stream));
    for (int32_t l = 1; l < L; l++) pg::launch_compose(layers + l, 1, out, out, pg::as_stream(stream));
  });
}

painty_status painty_compose_layers_host(const float* K, const float* S, const float* V,
                                         int32_t L, const float* R0, float* out, int32_t rows,
                                         int32_t cols, void* stream) {
  return guard([&] {
    PG_REQUIRE(rows > 0 && cols > 0, "rows and cols must be positive");
    PG_REQUIRE(L >= 0 && (L == 0 || (K && S && V)), "layer planes are null");
    PG_REQUIRE(R0 && out, "R0 or out is null");
    const int64_t npix = static_cast<int64_t>(rows) * cols;
    // Pinned host buffers are mapped into the device's address space (and on Grace-Blackwell
    // read coherently over NVLink-C2C): the fused composite then reads the layer stacks and
    // writes the image where they lie, streaming at the host link's rate with no staging.
    // Planes must start on 16 bytes and hold a multiple of 4 pixels for its vector accesses.
    {
      const float* hp[5] = {K, S, V, R0, out};
      const float* dp[5] = {};
      bool mapped = npix % 4 == 0;
      for (int i = 0; i < 5 && mapped; i++) {
        if (!hp[i]) continue;  // no layers
        cudaPointerAttributes pa{};
        if (cudaPointerGetAttributes(&pa, hp[i]) != cudaSuccess || pa.type != cudaMemoryTypeHost ||
            !pa.devicePointer || (reinterpret_cast<uintptr_t>(pa.devicePointer) & 15) != 0) {
          cudaGetLastError();
          mapped = false;
          break;
        }
        dp[i] = static_cast<const float*>(pa.devicePointer);
      }
      if (mapped) {
        const cudaStream_t st = pg::as_stream(stream);
        std::vector<painty_layer> views(static_cast<size_t>(L));
        std::vector<const painty_layer*> lp(static_cast<size_t>(L));
        for (int32_t l = 0; l < L; l++) {
          painty_layer& ly = views[l];
          ly.rows = rows;
          ly.cols = cols;
          ly.pitch = cols;  // npix, a multiple of 4, is the plane's extent
          ly.storage = PAINTY_STORAGE_F32;
          for (int c = 0; c < 3; c++) {
            ly.K[c] = const_cast<float*>(dp[0]) + (3 * static_cast<int64_t>(l) + c) * npix;
            ly.S[c] = const_cast<float*>(dp[1]) + (3 * static_cast<int64_t>(l) + c) * npix;
          }
          ly.V = const_cast<float*>(dp[2]) + static_cast<int64_t>(l) * npix;
          ly.owned = false;
          lp[l] = &ly;
        }
        painty_image ir{}, io{};
        ir.rows = io.rows = rows;
        ir.cols = io.cols = cols;
        ir.pitch = io.pitch = cols;
        ir.storage = io.storage = PAINTY_STORAGE_F32;
        ir.owned = io.owned = false;
        for (int c = 0; c < 3; c++) {
          ir.R[c] = const_cast<float*>(dp[3]) + c * npix;
          io.R[c] = const_cast<float*>(dp[4]) + c * npix;
        }
        pg::launch_compose(lp.data(), L, &ir, &io, st);
        PG_CUDA(cudaStreamSynchronize(st));
        return;
      }
    }
    constexpr int kStreams = 3;
    const int64_t pitch = pg::pitch_for(cols);
    // bands of about 16 MB of layer data each
    const int64_t row_bytes = static_cast<int64_t>(7 * L + 6) * pitch * 4;
    const int32_t band = static_cast<int32_t>(
      std::max<int64_t>(1, std::min<int64_t>(rows, (int64_t(16) << 20) / row_bytes)));
    const int64_t plane = static_cast<int64_t>(band) * pitch;  // device plane of one band
    const int64_t nplanes = 7 * static_cast<int64_t>(L) + 6;   // K, S, V, R0, out
    PG_CUDA(cudaStreamSynchronize(pg::as_stream(stream)));
    cudaStream_t st[kStreams] = {};
    void* buf[kStreams] = {};
    auto cleanup = [&] {
      for (int i = 0; i < kStreams; i++) {
        if (buf[i]) cudaFreeAsync(buf[i], st[i]);
        if (st[i]) {
          cudaStreamSynchronize(st[i]);
          cudaStreamDestroy(st[i]);
        }
      }
    };
    try {
      for (int i = 0; i < kStreams; i++) {
        PG_CUDA(cudaStreamCreateWithFlags(&st[i], cudaStreamNonBlocking));
        buf[i] = pg::temp_alloc(static_cast<size_t>(nplanes * plane) * 4, st[i]);
        // the pitch padding is computed on but never copied out: start it at zero
        PG_CUDA(cudaMemsetAsync(buf[i], 0, static_cast<size_t>(nplanes * plane) * 4, st[i]));
      }
      // host planes [n][rows][cols] <-> device planes [n][band][pitch], rows r0 .. r0 + h
      auto copy3d = [&](const float* hbase, float* dbase, int n, int32_t r0, int32_t h,
                        bool up, cudaStream_t s) {
        cudaMemcpy3DParms m{};
        cudaPitchedPtr hp = make_cudaPitchedPtr(const_cast<float*>(hbase), cols * 4, cols, rows);
        cudaPitchedPtr dp = make_cudaPitchedPtr(dbase, pitch * 4, pitch, band);
        m.extent = make_cudaExtent(static_cast<size_t>(cols) * 4, h, n);
        if (up) {
          m.srcPtr = hp;
          m.srcPos = make_cudaPos(0, r0, 0);
          m.dstPtr = dp;
          m.kind = cudaMemcpyHostToDevice;
        } else {
          m.srcPtr = dp;
          m.dstPtr = hp;
          m.dstPos = make_cudaPos(0, r0, 0);
          m.kind = cudaMemcpyDeviceToHost;
        }
        PG_CUDA(cudaMemcpy3DAsync(&m, s));
      };
      std::vector<painty_layer> views(static_cast<size_t>(L));
      std::vector<const painty_layer*> lp(static_cast<size_t>(L));
      int b = 0;
      for (int32_t r0 = 0; r0 < rows; r0 += band, b++) {
        const int32_t h = std::min(band, rows - r0);
        cudaStream_t s = st[b % kStreams];
        float* d = static_cast<float*>(buf[b % kStreams]);
        float* dK = d;
        float* dS = dK + 3 * static_cast<int64_t>(L) * plane;
        float* dV = dS + 3 * static_cast<int64_t>(L) * plane;
        float* dR = dV + static_cast<int64_t>(L) * plane;
        float* dO = dR + 3 * plane;
        if (L > 0) {
          copy3d(K, dK, 3 * L, r0, h, true, s);
          copy3d(S, dS, 3 * L, r0, h, true, s);
          copy3d(V, dV, L, r0, h, true, s);
        }
        copy3d(R0, dR, 3, r0, h, true, s);
        for (int32_t l = 0; l < L; l++) {
          painty_layer& ly = views[l];
          ly.rows = h;
          ly.cols = cols;
          ly.pitch = pitch;
          ly.storage = PAINTY_STORAGE_F32;
          for (int c = 0; c < 3; c++) {
            ly.K[c] = dK + (3 * static_cast<int64_t>(l) + c) * plane;
            ly.S[c] = dS + (3 * static_cast<int64_t>(l) + c) * plane;
          }
          ly.V = dV + static_cast<int64_t>(l) * plane;
          ly.owned = false;
          lp[l] = &ly;
        }
        painty_image ir{}, io{};
        ir.rows = io.rows = h;
        ir.cols = io.cols = cols;
        ir.pitch = io.pitch = pitch;
        ir.storage = io.storage = PAINTY_STORAGE_F32;
        ir.owned = io.owned = false;
        for (int c = 0; c < 3; c++) {
          ir.R[c] = dR + c * plane;
          io.R[c] = dO + c * plane;
        }
        pg::launch_compose(lp.data(), L, &ir, &io, s);
        copy3d(out, dO, 3, r0, h, false, s);
      }
    } catch (...) {
      cleanup();
      throw;
    }
    cleanup();
  });
}

// ---------------------------------------------------------------- canvas
painty_status painty_canvas_create(int32_t rows, int32_t cols, painty_storage storage,
                                   painty_canvas** out) {
  return guard([&] {
    PG_REQUIRE(out != nullptr, "out is null");
    PG_REQUIRE(rows > 0 && cols > 0, "rows and cols must be positive");
    PG_REQUIRE(pg::valid_storage(storage), "unknown storage format");
    auto* c = new painty_canvas();
    const painty_storage rs = storage == PAINTY_STORAGE_F64 ? PAINTY_STORAGE_F64 : PAINTY_STORAGE_F32;
    const size_t lb = pg::layer_bytes(rows, cols, storage, true);
    const size_t ib = pg::image_bytes(rows, cols, rs);
    const size_t hb = static_cast<size_t>(rows) * pg::pitch_for(cols) * pg::v_bytes(storage);
    try {
      c->bytes = lb + ib + (hb + 255) / 256 * 256;
      c->base = pg::device_alloc(c->bytes);
      pg::layer_layout(c->wet, rows, cols, storage, c->base, true);
      c->wet.owned = false;
      c->wet.writes = &c->version;
      pg::image_layout(c->r0, rows, cols, rs, static_cast<char*>(c->base) + lb);
      c->r0.owned = false;
      c->h = static_cast<char*>(c->base) + lb + ib;
      c->id = pg::g_canvas_ids.fetch_add(1);
      PG_CUDA(cudaMemset(c->base, 0, c->bytes));
      const double one[3] = {1.0, 1.0, 1.0};  // Canvas.hxx:33 background
      pg::fill_planes(c->r0.R, 3, pg::r_type(rs), c->r0.plane_elems(), one, nullptr);
      PG_CUDA(cudaStreamSynchronize(nullptr));
    } catch (...) {
      if (c->base) pg::device_free(c->base);
      delete c;
      throw;
    }
    *out = c;
  });
}

painty_status painty_canvas_destroy(painty_canvas* c) {
  return guard([&] {
    if (!c) return;
    pg::device_free(c->base);
    delete c;
  });
}

painty_status painty_canvas_clear(painty_canvas* c, void* stream) {
  return guard([&] {
    PG_REQUIRE(c != nullptr, "canvas is null");
    const cudaStream_t st = pg::as_stream(stream);
    PG_CUDA(cudaMemsetAsync(c->wet.base, 0, c->wet.bytes, st));
    const size_t hb = static_cast<size_t>(c->wet.plane_elems()) * pg::v_bytes(c->wet.storage);
    PG_CUDA(cudaMemsetAsync(c->h, 0, hb, st));
    const double one[3] = {1.0, 1.0, 1.0};
    pg::fill_planes(c->r0.R, 3, pg::r_type(c->r0.storage), c->r0.plane_elems(), one, st);
    c->version++;
  });
}

painty_status painty_canvas_upload(painty_canvas* c, painty_plane plane, const void* host,
                                   painty_host_format fmt, void* stream) {
  return guard([&] {
    PG_REQUIRE(c != nullptr, "canvas is null");
    const cudaStream_t st = pg::as_stream(stream);
    c->version++;
    if (plane == PAINTY_PLANE_R0) {
      pg::upload_planes(c->r0.R, 3, pg::r_type(c->r0.storage), c->wet.rows, c->wet.cols,
                        c->wet.pitch, host, fmt, st);
    } else if (plane == PAINTY_PLANE_H) {
      void* p[1] = {c->h};
      pg::upload_planes(p, 1, pg::v_type(c->wet.storage), c->wet.rows, c->wet.cols,
                        c->wet.pitch, host, fmt, st);
    } else if (plane == PAINTY_PLANE_VL) {
      void* p[1] = {static_cast<char*>(c->wet.V) + pg::v_bytes(c->wet.storage)};
      pg::upload_planes(p, 1, pg::v_type(c->wet.storage), c->wet.rows, c->wet.cols,
                        c->wet.pitch, host, fmt, st, c->wet.estride);
    } else {
      void* p[3] = {nullptr, nullptr, nullptr};
      int nch = 0;
      pg::DevType dt;
      layer_plane_ptrs(&c->wet, plane, p, &nch, &dt);
      pg::upload_planes(p, nch, dt, c->wet.rows, c->wet.cols, c->wet.pitch, host, fmt, st,
                        c->wet.estride);
    }
  });
}

painty_status painty_canvas_download(const painty_canvas* c, painty_plane plane, void* host,
                                     painty_host_format fmt, void* stream) {
  return guard([&] {
    PG_REQUIRE(c != nullptr, "canvas is null");
    const cudaStream_t st = pg::as_stream(stream);
    if (plane == PAINTY_PLANE_R0) {
      const void* p[3] = {c->r0.R[0], c->r0.R[1], c->r0.R[2]};
      pg::download_planes(p, 3, pg::r_type(c->r0.storage), c->wet.rows, c->wet.cols,
                          c->wet.pitch, host, fmt, st);
    } else if (plane == PAINTY_PLANE_H) {
      const void* p[1] = {c->h};
      pg::download_planes(p, 1, pg::v_type(c->wet.storage), c->wet.rows, c->wet.cols,
                          c->wet.pitch, host, fmt, st);
    } else if (plane == PAINTY_PLANE_VL) {
      const void* p[1] = {static_cast<const char*>(c->wet.V) + pg::v_bytes(c->wet.storage)};
      pg::download_planes(p, 1, pg::v_type(c->wet.storage), c->wet.rows, c->wet.cols,
                          c->wet.pitch, host, fmt, st, c->wet.estride);
    } else {
      void* p[3] = {nullptr, nullptr, nullptr};
      int nch = 0;
      pg::DevType dt;
      layer_plane_ptrs(&c->wet, plane, p, &nch, &dt);
      const void* cp[3] = {p[0], p[1], p[2]};
      pg::download_planes(cp, nch, dt, c->wet.rows, c->wet.cols, c->wet.pitch, host, fmt, st,
                          c->wet.estride);
    }
  });
}

painty_status painty_canvas_layer(painty_canvas* c, painty_layer** out) {
  return guard([&] {
    PG_REQUIRE(c && out, "null argument");
    *out = &c->wet;
  });
}

painty_status painty_canvas_r0(painty_canvas* c, painty_image** out) {
  return guard([&] {
    PG_REQUIRE(c && out, "null argument");
    *out = &c->r0;
  });
}

painty_status painty_canvas_info(const painty_canvas* c, int32_t* rows, int32_t* cols,
                                 painty_storage* storage) {
  return guard([&] {
    PG_REQUIRE(c != nullptr, "canvas is null");
    if (rows) *rows = c->wet.rows;
    if (cols) *cols = c->wet.cols;
    if (storage) *storage = c->wet.storage;
  });
}

painty_status painty_canvas_compose(const painty_canvas* c, painty_image* out, void* stream) {
  return guard([&] {
    PG_REQUIRE(c != nullptr, "canvas is null");
    const painty_layer* L[1] = {&c->wet};
    pg::launch_compose(L, 1, &c->r0, out, pg::as_stream(stream));
  });
}

painty_status painty_canvas_dry(painty_canvas* c, void* stream) {
  return guard([&] {
    PG_REQUIRE(c != nullptr, "canvas is null");
    const cudaStream_t st = pg::as_stream(stream);
    c->version++;
    switch (c->wet.storage) {
      case PAINTY_STORAGE_F32: pg::dry_typed<float, float, float>(c, st); break;
      case PAINTY_STORAGE_F16: pg::dry_typed<__half, __half, float>(c, st); break;
      case PAINTY_STORAGE_BF16: pg::dry_typed<__nv_bfloat16, __half, float>(c, st); break;
      case PAINTY_STORAGE_F64: pg::dry_typed<double, double, double>(c, st); break;
    }
  });
}

// ---------------------------------------------------------------- mixing
painty_status painty_mix_paint(const double* w, int32_t n, const double* palK,
                               const double* palS, double K[3], double S[3]) {
  return guard([&] {
    PG_REQUIRE(w && palK && palS && K && S, "null argument");
    PG_REQUIRE(n > 0, "palette size must be positive");
    // PaintMixer.cxx:327-355: normalise when |sum w - 1| >= 10e-6, then K,S = sum w_i K_i,S_i
    double norm = 1.0, wsum = 0.0;
    for (int i = 0; i < n; i++) wsum += w[i];
    if (!(std::fabs(wsum - 1.0) < 10e-6)) norm = 1. / wsum;
    for (int i = 0; i < 3; i++) {
      K[i] = 0.0;
      S[i] = 0.0;
    }
    for (int l = 0; l < n; l++)
      for (int i = 0; i < 3; i++) {
        K[i] += norm * w[l] * palK[l * 3 + i];
        S[i] += norm * w[l] * palS[l * 3 + i];
      }
  });
}

}  // extern "C"
