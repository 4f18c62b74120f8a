// stamp.cu -- the imprint brush: in-order stamp deposition with pickup/deposit mixing.
//
// Semantics are painty's FootprintBrush (painty/renderer/FootprintBrush.hxx):
//   imprint (:73-143)       for the F x F box around the centre, in row-major order:
//                             canvas pixel = trunc(col + cx, row + cy)  (double)
//                             map cell     = round(R(-theta) (col, row)) + (wr, hr)  (double)
//                           skip if either is outside, then pickupPaint, depositPaint
//   updateSnapshot (:278-319) before each stamp, copy canvas -> snapshot over the box grown by
//                           the radius, except the box's strict interior
//   pickupPaint (:349-384), depositPaint (:393-431), blend (:331-340)
//
// Parallel execution inside a stamp. The sequential loop touches, per pixel p, one pickup-map
// cell m(p) and one canvas pixel c(p) (snapshot and canvas planes at c(p)). Pixels that share
// neither commute, so a stamp runs in waves: in each wave every remaining pixel that holds
// the lowest remaining row-major index for its map cell (an atomicMin owner table in shared
// memory) and whose earlier pixels on the same canvas pixel are done is processed. Each
// resource therefore sees its pixels in row-major order, which reproduces the sequential
// result exactly; the globally lowest remaining pixel always qualifies, so every wave makes
// progress (a cap on the wave count guards the loop regardless).
// Two pixels share a map cell when the rounded rotation is not injective (common: pairs).
// Two pixels share a canvas pixel only at the left/top edge, where trunc() sends both
// col + cx in (-1, 0) and in [0, 1) to column 0; the earlier pixels there are the left, upper,
// upper-left and upper-right neighbours, tracked with done flags for the first of the two
// duplicated columns / rows.
//
// Map coordinates: the reference evaluates round(fl(fl(col*c - row*s) + wr)) in double. The
// kernel evaluates the same expression in FP32 (error below 4e-5 for |col|, |row| <= 127)
// and uses it when it is at least 2e-4 away from a rounding tie; otherwise it repeats the
// reference's double operations (__dmul_rn/__dadd_rn, no contraction), so the chosen cell is
// always the reference's. cos(-theta), sin(-theta) come from the host's libm for host-given
// stamps, as in the reference.
//
// Arithmetic: storage F64 uses the reference's double operations in the reference's order
// without contraction (bit-identical results); F32/F16/BF16 use FP32 arithmetic on values
// stored in those types.
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "device_common.cuh"
#include "internal.h"

namespace pg {

struct StampRec {
  double cx, cy, c, s;  // centre, cos(-theta), sin(-theta)
};

namespace {

constexpr int kStampThreads = 1024;
constexpr int kMaxPixelsPerThread = 64;  // F*F <= 64 * 1024
constexpr int kMaxWaves = 64;
constexpr unsigned kStatusWaveCap = 1u;

template <class M>
struct Arith;
template <>
struct Arith<float> {
  static __device__ __forceinline__ float mul(float a, float b) { return a * b; }
  static __device__ __forceinline__ float add(float a, float b) { return a + b; }
  static __device__ __forceinline__ float sub(float a, float b) { return a - b; }
  static __device__ __forceinline__ float div(float a, float b) { return __fdiv_rn(a, b); }
};
template <>
struct Arith<double> {
  static __device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
  static __device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
  static __device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }
  static __device__ __forceinline__ double div(double a, double b) { return __ddiv_rn(a, b); }
};

template <class TK, class TV>
struct StampArgs {
  using M = typename MathOf<TK>::type;
  TK* cK[3];
  TK* cS[3];
  TV* cV;
  TK* sK[3];  // pickup source: snapshot planes, or the canvas planes without a snapshot
  TK* sS[3];
  TV* sV;
  M* pK[3];  // pickup map, S*S per plane
  M* pS[3];
  M* pV;
  const M* footprint;  // F*F
  const StampRec* stamps;
  int64_t n;
  int32_t rows, cols;
  int64_t pitch;
  int32_t F, S, wr;
  double radius;
  M pickupRate, depositionRate, capacity;
  M paintK[3], paintS[3];
  int32_t use_snapshot;
  int* owner_global;  // S*S ints when the owner table does not fit in shared memory
  unsigned* status;
};

struct StampShared {
  double cx, cy, c, s;
  float cf, sf;
  int tl[2], br[2], tla[2], bra[2];
  int c0, r0;  // first index of the duplicated column / row, -1 if none
};

// Reference map coordinate round(fl(fl(u*c - v*s) + w)) (sgn = +1) or
// round(fl(fl(u*s + v*c) + w)) style, given as a = u*ca, b = v*cb in the caller's order.
__device__ __forceinline__ int map_coord(float fast, int u, double ca, int v, double cb,
                                         bool minus, int w) {
  const float fr = fast - floorf(fast);
  if (fabsf(fr - 0.5f) > 2e-4f) return __float2int_rn(fast);
  const double p1 = __dmul_rn(static_cast<double>(u), ca);
  const double p2 = __dmul_rn(static_cast<double>(v), cb);
  const double r = minus ? __dsub_rn(p1, p2) : __dadd_rn(p1, p2);
  return static_cast<int>(round(__dadd_rn(r, static_cast<double>(w))));
}

template <class M>
__device__ __forceinline__ void blend3(M va, const M (&a)[3], M vb, const M (&b)[3], M (&r)[3]) {
  using A = Arith<M>;
  const M tot = A::add(va, vb);
  if (tot > M(0.001)) {
#pragma unroll
    for (int i = 0; i < 3; i++) r[i] = A::div(A::add(A::mul(va, a[i]), A::mul(vb, b[i])), tot);
  } else {
#pragma unroll
    for (int i = 0; i < 3; i++) r[i] = a[i];
  }
}

// pickupPaint then depositPaint for one stamp pixel (FootprintBrush.hxx:349-431)
template <class TK, class TV>
__device__ __forceinline__ void process_pixel(const StampArgs<TK, TV>& a, int xc, int yc, int mx,
                                              int my) {
  using M = typename MathOf<TK>::type;
  using A = Arith<M>;
  const M fp = (my < a.F && mx < a.F) ? a.footprint[my * a.F + mx] : M(0);
  if (!(fp > M(0))) return;
  const int64_t c = static_cast<int64_t>(yc) * a.pitch + xc;
  const int m = my * a.S + mx;
  M vp = a.pV[m];
  M kp[3], sp[3];
#pragma unroll
  for (int i = 0; i < 3; i++) {
    kp[i] = a.pK[i][m];
    sp[i] = a.pS[i][m];
  }
  // pickupPaint
  const M vsrc = ld_elem<M>(a.sV + c);
  const M vleave = A::mul(A::mul(a.pickupRate, vsrc), fp);
  bool pk_changed = false;
  if (vleave > M(0.001)) {
    st_elem<M>(a.sV + c, A::sub(vsrc, vleave));
    M ks[3], ss[3], nk[3], ns[3];
#pragma unroll
    for (int i = 0; i < 3; i++) {
      ks[i] = ld_elem<M>(a.sK[i] + c);
      ss[i] = ld_elem<M>(a.sS[i] + c);
    }
    blend3(vp, kp, vleave, ks, nk);
    blend3(vp, sp, vleave, ss, ns);
#pragma unroll
    for (int i = 0; i < 3; i++) {
      kp[i] = nk[i];
      sp[i] = ns[i];
    }
    vp = A::add(vp, vleave);
    pk_changed = true;
  }
  // depositPaint
  const M dfree = A::sub(a.capacity, vp);
  const M vfree = (M(0) < dfree) ? dfree : M(0);  // std::max(0.0, x)
  M ksrc[3], ssrc[3];
  blend3(vp, kp, vfree, a.paintK, ksrc);
  blend3(vp, sp, vfree, a.paintS, ssrc);
  const M pleave = A::mul(A::mul(a.depositionRate, vp), fp);
  a.pV[m] = A::sub(vp, pleave);
  if (pk_changed) {
#pragma unroll
    for (int i = 0; i < 3; i++) {
      a.pK[i][m] = kp[i];
      a.pS[i][m] = sp[i];
    }
  }
  const M vcan = ld_elem<M>(a.cV + c);
  const M vb = A::mul(a.capacity, fp);
  M ck[3], cs[3], nk[3], ns[3];
#pragma unroll
  for (int i = 0; i < 3; i++) {
    ck[i] = ld_elem<M>(a.cK[i] + c);
    cs[i] = ld_elem<M>(a.cS[i] + c);
  }
  blend3(vb, ksrc, vcan, ck, nk);
  blend3(vb, ssrc, vcan, cs, ns);
#pragma unroll
  for (int i = 0; i < 3; i++) {
    st_elem<M>(a.cK[i] + c, nk[i]);
    st_elem<M>(a.cS[i] + c, ns[i]);
  }
  st_elem<M>(a.cV + c, A::add(vb, vcan));
}

struct PixelInfo {
  int xc, yc, mx, my;
  bool valid;
};

template <class TK, class TV>
__device__ __forceinline__ PixelInfo pixel_info(const StampArgs<TK, TV>& a,
                                                const StampShared& sh, const int* xs,
                                                const int* ys, int idx) {
  PixelInfo p;
  const int row = idx / a.F, col = idx - (idx / a.F) * a.F;
  const int dr = row - a.wr, dc = col - a.wr;
  p.xc = xs[col];
  p.yc = ys[row];
  const float dcf = static_cast<float>(dc), drf = static_cast<float>(dr);
  const float wrf = static_cast<float>(a.wr);
  const float fx = fmaf(-drf, sh.sf, dcf * sh.cf) + wrf;  // col*cos - row*sin + wr
  const float fy = fmaf(drf, sh.cf, dcf * sh.sf) + wrf;   // col*sin + row*cos + hr
  p.mx = map_coord(fx, dc, sh.c, dr, sh.s, true, a.wr);
  p.my = map_coord(fy, dc, sh.s, dr, sh.c, false, a.wr);
  p.valid = p.yc >= 0 && p.xc >= 0 && p.xc < a.cols && p.yc < a.rows && p.my >= 0 &&
            p.mx >= 0 && p.mx < a.S && p.my < a.S;
  return p;
}

// Earlier pixels on the same canvas pixel must be done (left/top edge duplicates).
__device__ __forceinline__ bool canvas_ready(const StampShared& sh, const uint8_t* done_c0,
                                             const uint8_t* done_r0, int row, int col) {
  bool ok = true;
  if (sh.c0 >= 0 && col == sh.c0 + 1) ok = ok && done_c0[row];
  if (sh.r0 >= 0 && row == sh.r0 + 1) {
    ok = ok && done_r0[col];
    if (sh.c0 >= 0 && col == sh.c0) ok = ok && done_r0[sh.c0 + 1];
    if (sh.c0 >= 0 && col == sh.c0 + 1) ok = ok && done_r0[sh.c0];
  }
  return ok;
}

template <class TK, class TV>
__global__ void __launch_bounds__(kStampThreads, 1) stamp_kernel(const __grid_constant__ StampArgs<TK, TV> a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ StampShared sh;
  const int tid = threadIdx.x;
  const int T = blockDim.x;
  const int F = a.F, S = a.S;
  const int npix = F * F;
  int* own = a.owner_global ? a.owner_global : reinterpret_cast<int*>(smem_raw);
  const size_t own_bytes = a.owner_global ? 0 : static_cast<size_t>(S) * S * sizeof(int);
  int* xs = reinterpret_cast<int*>(smem_raw + own_bytes);
  int* ys = xs + F;
  uint8_t* done_c0 = reinterpret_cast<uint8_t*>(ys + F);
  uint8_t* done_r0 = done_c0 + F;

  for (int64_t k = 0; k < a.n; k++) {
    if (tid == 0) {
      const StampRec st = a.stamps[k];
      sh.cx = st.cx;
      sh.cy = st.cy;
      sh.c = st.c;
      sh.s = st.s;
      sh.cf = static_cast<float>(st.c);
      sh.sf = static_cast<float>(st.s);
      const double w = a.wr;
      // FootprintBrush.hxx:291-305
      sh.tl[0] = static_cast<int>(__dsub_rn(st.cx, w));
      sh.tl[1] = static_cast<int>(__dsub_rn(st.cy, w));
      sh.br[0] = static_cast<int>(__dadd_rn(st.cx, w));
      sh.br[1] = static_cast<int>(__dadd_rn(st.cy, w));
      sh.tla[0] = max(static_cast<int>(__dsub_rn(__dsub_rn(st.cx, w), a.radius)), 0);
      sh.tla[1] = max(static_cast<int>(__dsub_rn(__dsub_rn(st.cy, w), a.radius)), 0);
      sh.bra[0] = min(static_cast<int>(__dadd_rn(__dadd_rn(st.cx, w), a.radius)), a.cols - 1);
      sh.bra[1] = min(static_cast<int>(__dadd_rn(__dadd_rn(st.cy, w), a.radius)), a.rows - 1);
      sh.c0 = -1;
      sh.r0 = -1;
    }
    __syncthreads();
    // canvas coordinates per column / row; owner table reset; done flags reset
    for (int i = tid; i < F; i += T) {
      xs[i] = static_cast<int>(__dadd_rn(static_cast<double>(i - a.wr), sh.cx));
      ys[i] = static_cast<int>(__dadd_rn(static_cast<double>(i - a.wr), sh.cy));
      done_c0[i] = 0;
      done_r0[i] = 0;
    }
    for (int i = tid; i < S * S; i += T) own[i] = INT_MAX;
    // snapshot refresh around the footprint box (FootprintBrush.hxx:307-318)
    if (a.use_snapshot) {
      const int w = sh.bra[0] - sh.tla[0] + 1, h = sh.bra[1] - sh.tla[1] + 1;
      if (w > 0 && h > 0) {
        const int total = w * h;
        for (int i = tid; i < total; i += T) {
          const int row = sh.tla[1] + i / w, col = sh.tla[0] + i % w;
          if (row > sh.tl[1] && row < sh.br[1] && col > sh.tl[0] && col < sh.br[0]) continue;
          const int64_t o = static_cast<int64_t>(row) * a.pitch + col;
#pragma unroll
          for (int ch = 0; ch < 3; ch++) {
            a.sK[ch][o] = a.cK[ch][o];
            a.sS[ch][o] = a.cS[ch][o];
          }
          a.sV[o] = a.cV[o];
        }
      }
    }
    __syncthreads();
    for (int i = tid; i + 1 < F; i += T) {
      if (xs[i] == xs[i + 1]) sh.c0 = i;
      if (ys[i] == ys[i + 1]) sh.r0 = i;
    }
    __syncthreads();
    // first claim: every valid pixel bids for its map cell
    uint64_t rem = 0;
    for (int j = 0; j < kMaxPixelsPerThread; j++) {
      const int idx = j * T + tid;
      if (idx >= npix) break;
      const PixelInfo p = pixel_info(a, sh, xs, ys, idx);
      const int row = idx / F, col = idx - row * F;
      if (p.valid) {
        rem |= (1ull << j);
        atomicMin(&own[p.my * S + p.mx], idx);
      } else {
        if (col == sh.c0) done_c0[row] = 1;
        if (row == sh.r0) done_r0[col] = 1;
      }
    }
    __syncthreads();
    for (int wave = 0;; wave++) {
      uint64_t processed = 0;
      for (uint64_t bits = rem; bits; bits &= bits - 1) {
        const int j = __ffsll(static_cast<long long>(bits)) - 1;
        const int idx = j * T + tid;
        const PixelInfo p = pixel_info(a, sh, xs, ys, idx);
        const int row = idx / F, col = idx - row * F;
        if (own[p.my * S + p.mx] == idx && canvas_ready(sh, done_c0, done_r0, row, col)) {
          process_pixel(a, p.xc, p.yc, p.mx, p.my);
          processed |= (1ull << j);
        }
      }
      __syncthreads();
      rem &= ~processed;
      for (uint64_t bits = processed; bits; bits &= bits - 1) {
        const int j = __ffsll(static_cast<long long>(bits)) - 1;
        const int idx = j * T + tid;
        const int row = idx / F, col = idx - row * F;
        if (col == sh.c0) done_c0[row] = 1;
        if (row == sh.r0) done_r0[col] = 1;
      }
      for (uint64_t bits = rem; bits; bits &= bits - 1) {
        const int j = __ffsll(static_cast<long long>(bits)) - 1;
        const PixelInfo p = pixel_info(a, sh, xs, ys, j * T + tid);
        own[p.my * S + p.mx] = INT_MAX;
      }
      const int any = __syncthreads_or(rem != 0);
      if (!any) break;
      if (wave + 1 >= kMaxWaves) {  // cannot happen; guards the loop bound
        if (tid == 0) atomicOr(a.status, kStatusWaveCap);
        break;
      }
      for (uint64_t bits = rem; bits; bits &= bits - 1) {
        const int j = __ffsll(static_cast<long long>(bits)) - 1;
        const int idx = j * T + tid;
        const PixelInfo p = pixel_info(a, sh, xs, ys, idx);
        atomicMin(&own[p.my * S + p.mx], idx);
      }
      __syncthreads();
    }
  }
}

}  // namespace
}  // namespace pg

// ====================================================================== brush
struct painty_brush {
  double radius = 0.0;  // FootprintBrush.hxx:437
  int32_t sizeMap = 0;  // :443
  int32_t F = 0;
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
  // snapshot (FootprintBrush.hxx:471): canvas-sized layer, allocated at first use
  painty_layer snapshot;
  bool has_snapshot = false;
  void* d_stamps = nullptr;
  size_t d_stamps_bytes = 0;
  unsigned* d_status = nullptr;
};

namespace pg {
namespace {

// OpenCV's BORDER_REFLECT ("fedcba|abcdefgh|hgfedcb") for the footprint resample
int reflect_index(int p, int len) {
  if (len == 1) return 0;
  while (p < 0 || p >= len) p = p < 0 ? -p - 1 : len - 1 - (p - len);
  return p;
}

// painty::Interpolate (painty/image/Mat.hxx:68-103), single channel
double interpolate(const double* in, int rows, int cols, double px, double py) {
  const int x = static_cast<int>(std::floor(px));
  const int y = static_cast<int>(std::floor(py));
  const int x0 = reflect_index(x, cols), x1 = reflect_index(x + 1, cols);
  const int y0 = reflect_index(y, rows), y1 = reflect_index(y + 1, rows);
  const double a = px - static_cast<double>(x);
  const double c = py - static_cast<double>(y);
  return (in[y0 * cols + x0] * (1.0 - a) + in[y0 * cols + x1] * a) * (1.0 - c) +
         (in[y1 * cols + x0] * (1.0 - a) + in[y1 * cols + x1] * a) * c;
}

// FootprintBrush::setRadius (FootprintBrush.hxx:46-63). The footprint image is resampled to
// width x width by a pixel-centre aligned bilinear resample (in place of OpenCV's
// Lanczos-4 resize) and zero-padded by (sizeMap - width) / 2 on each side.
void set_radius(painty_brush* b, double radius) {
  if (std::fabs(b->radius - radius) < 0.5) return;
  b->radius = radius;
  const int width = static_cast<int>(2.0 * std::ceil(radius) + 1.0);
  b->sizeMap = static_cast<int>(std::ceil(std::sqrt(2.0) * width));
  const int pad = (b->sizeMap - width) / 2;
  b->F = width + 2 * pad;
  b->footprint.assign(static_cast<size_t>(b->F) * b->F, 0.0);
  const double sy = static_cast<double>(b->fh) / width, sx = static_cast<double>(b->fw) / width;
  for (int i = 0; i < width; i++)
    for (int j = 0; j < width; j++)
      b->footprint[static_cast<size_t>(i + pad) * b->F + (j + pad)] =
        interpolate(b->full.data(), b->fh, b->fw, (static_cast<double>(j) + 0.5) * sx - 0.5,
                    (static_cast<double>(i) + 0.5) * sy - 0.5);
  b->footprint_stale = true;
  b->pickup_clear = true;
}

void ensure(void** p, size_t* cap, size_t bytes) {
  if (*cap >= bytes && *p) return;
  if (*p) device_free(*p);
  *p = nullptr;
  *cap = 0;
  *p = device_alloc(bytes);
  *cap = bytes;
}

int max_dyn_smem() {
  int dev = 0, v = 0;
  PG_CUDA(cudaGetDevice(&dev));
  PG_CUDA(cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  return v;
}

template <class TK, class TV>
void launch_stamps(painty_canvas* c, painty_brush* b, const StampRec* d_stamps, int64_t n,
                   cudaStream_t st) {
  using M = typename MathOf<TK>::type;
  StampArgs<TK, TV> a{};
  for (int i = 0; i < 3; i++) {
    a.cK[i] = static_cast<TK*>(c->wet.K[i]);
    a.cS[i] = static_cast<TK*>(c->wet.S[i]);
    const painty_layer& src = b->useSnapshot ? b->snapshot : c->wet;
    a.sK[i] = static_cast<TK*>(src.K[i]);
    a.sS[i] = static_cast<TK*>(src.S[i]);
  }
  a.cV = static_cast<TV*>(c->wet.V);
  a.sV = static_cast<TV*>(b->useSnapshot ? b->snapshot.V : c->wet.V);
  const size_t cells = static_cast<size_t>(b->sizeMap) * b->sizeMap;
  M* pk = static_cast<M*>(b->d_pickup);
  for (int i = 0; i < 3; i++) {
    a.pK[i] = pk + i * cells;
    a.pS[i] = pk + (3 + i) * cells;
  }
  a.pV = pk + 6 * cells;
  a.footprint = static_cast<const M*>(b->d_footprint);
  a.stamps = d_stamps;
  a.n = n;
  a.rows = c->wet.rows;
  a.cols = c->wet.cols;
  a.pitch = c->wet.pitch;
  a.F = b->F;
  a.S = b->sizeMap;
  a.wr = (b->F - 1) / 2;
  a.radius = b->radius;
  a.pickupRate = static_cast<M>(b->pickupRate);
  a.depositionRate = static_cast<M>(b->depositionRate);
  a.capacity = static_cast<M>(b->capacity);
  for (int i = 0; i < 3; i++) {
    a.paintK[i] = static_cast<M>(b->paintK[i]);
    a.paintS[i] = static_cast<M>(b->paintS[i]);
  }
  a.use_snapshot = b->useSnapshot ? 1 : 0;
  a.status = b->d_status;
  const size_t small = static_cast<size_t>(b->F) * (2 * sizeof(int) + 2);
  const size_t own = cells * sizeof(int);
  const int limit = max_dyn_smem() - static_cast<int>(sizeof(StampShared)) - 1024;
  size_t dyn = small + own;
  if (dyn > static_cast<size_t>(limit)) {
    ensure(&b->d_owner, &b->d_owner_bytes, own);
    a.owner_global = static_cast<int*>(b->d_owner);
    dyn = small;
  }
  auto kern = stamp_kernel<TK, TV>;
  PG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               static_cast<int>(dyn)));
  kern<<<1, kStampThreads, dyn, st>>>(a);
  count_launch();
  PG_CUDA(cudaGetLastError());
}

// Prepares device state and runs n stamps (host records) on the canvas.
void run_stamps(painty_canvas* c, painty_brush* b, const std::vector<StampRec>& recs,
                cudaStream_t st) {
  PG_REQUIRE(c && b, "null handle");
  if (recs.empty()) return;
  PG_REQUIRE(b->sizeMap > 0 && b->F > 0, "brush radius gives an empty footprint");
  PG_REQUIRE(static_cast<int64_t>(b->F) * b->F <= int64_t(kMaxPixelsPerThread) * kStampThreads,
             "brush radius above the supported maximum (footprint side 256)");
  const bool f64 = c->wet.storage == PAINTY_STORAGE_F64;
  const int mode = f64 ? 1 : 0;
  if (b->bound < 0) b->bound = mode;
  PG_REQUIRE(b->bound == mode,
             "a brush paints either F64 canvases or F32/F16/BF16 canvases, not both");
  const size_t msz = f64 ? 8 : 4;
  // footprint
  const size_t fp_bytes = static_cast<size_t>(b->F) * b->F * msz;
  if (b->footprint_stale || b->d_footprint_bytes < fp_bytes) {
    ensure(&b->d_footprint, &b->d_footprint_bytes, fp_bytes);
    if (f64) {
      PG_CUDA(cudaMemcpyAsync(b->d_footprint, b->footprint.data(), fp_bytes,
                              cudaMemcpyHostToDevice, st));
    } else {
      std::vector<float> f(b->footprint.begin(), b->footprint.end());
      PG_CUDA(cudaMemcpyAsync(b->d_footprint, f.data(), fp_bytes, cudaMemcpyHostToDevice, st));
      PG_CUDA(cudaStreamSynchronize(st));
    }
    b->footprint_stale = false;
  }
  // pickup map
  const size_t pk_bytes = static_cast<size_t>(b->sizeMap) * b->sizeMap * 7 * msz;
  if (b->d_pickup_bytes < pk_bytes) {
    ensure(&b->d_pickup, &b->d_pickup_bytes, pk_bytes);
    b->pickup_clear = true;
  }
  if (b->pickup_clear) {
    PG_CUDA(cudaMemsetAsync(b->d_pickup, 0, pk_bytes, st));
    b->pickup_clear = false;
  }
  if (!b->d_status) {
    b->d_status = static_cast<unsigned*>(device_alloc(sizeof(unsigned)));
    PG_CUDA(cudaMemsetAsync(b->d_status, 0, sizeof(unsigned), st));
  }
  // snapshot (FootprintBrush.hxx:280-284: full copy when the sizes differ)
  if (b->useSnapshot) {
    if (!b->has_snapshot || b->snapshot.rows != c->wet.rows || b->snapshot.cols != c->wet.cols ||
        b->snapshot.storage != c->wet.storage) {
      if (b->has_snapshot) device_free(b->snapshot.base);
      b->has_snapshot = false;
      void* base = device_alloc(layer_bytes(c->wet.rows, c->wet.cols, c->wet.storage));
      layer_layout(b->snapshot, c->wet.rows, c->wet.cols, c->wet.storage, base);
      b->has_snapshot = true;
      PG_CUDA(cudaMemcpyAsync(b->snapshot.base, c->wet.base, c->wet.bytes,
                              cudaMemcpyDeviceToDevice, st));
    }
  }
  // stamps
  const size_t sbytes = recs.size() * sizeof(StampRec);
  ensure(&b->d_stamps, &b->d_stamps_bytes, sbytes);
  PG_CUDA(cudaMemcpyAsync(b->d_stamps, recs.data(), sbytes, cudaMemcpyHostToDevice, st));
  const auto* ds = static_cast<const StampRec*>(b->d_stamps);
  const int64_t n = static_cast<int64_t>(recs.size());
  switch (c->wet.storage) {
    case PAINTY_STORAGE_F32: launch_stamps<float, float>(c, b, ds, n, st); break;
    case PAINTY_STORAGE_F16: launch_stamps<__half, __half>(c, b, ds, n, st); break;
    case PAINTY_STORAGE_BF16: launch_stamps<__nv_bfloat16, __half>(c, b, ds, n, st); break;
    case PAINTY_STORAGE_F64: launch_stamps<double, double>(c, b, ds, n, st); break;
  }
  // the stamp records live in a reused buffer: finish before returning
  unsigned status = 0;
  PG_CUDA(cudaMemcpyAsync(&status, b->d_status, sizeof(unsigned), cudaMemcpyDeviceToHost, st));
  PG_CUDA(cudaStreamSynchronize(st));
  if (status != 0) fail(PAINTY_ERR_CUDA, "stamp kernel reported an internal error");
}

StampRec make_rec(double cx, double cy, double theta) {
  PG_REQUIRE(std::isfinite(cx) && std::isfinite(cy) && std::isfinite(theta),
             "stamp centre and angle must be finite");
  PG_REQUIRE(std::fabs(cx) < 1e9 && std::fabs(cy) < 1e9, "stamp centre out of range");
  return StampRec{cx, cy, std::cos(-theta), std::sin(-theta)};
}

// Spline.hxx:27-73 in the reference's operation order
double catmull_rom(double p_1, double p0, double p1, double p2, double t) {
  constexpr double tau = 0.5;
  const double t2 = t * t;
  const double t3 = t2 * t;
  const double b1 = -tau * t + 2.0 * tau * t2 - tau * t3;
  const double b2 = 1.0 + (tau - 3.0) * t2 + (2.0 - tau) * t3;
  const double b3 = tau * t + (3.0 - 2.0 * tau) * t2 + (tau - 2.0) * t3;
  const double b4 = -tau * t2 + tau * t3;
  return p_1 * b1 + p0 * b2 + p1 * b3 + p2 * b4;
}
double catmull_rom_deriv(double p_1, double p0, double p1, double p2, double t) {
  constexpr double tau = 0.5;
  const double t2 = t * t;
  const double b1 = tau * (-3.0 * t2 + 4.0 * t - 1.0);
  const double b2 = -t * (-2.0 * tau + 3.0 * (tau - 2.0) * t + 6.0);
  const double b3 = (t - 1.0) * (3.0 * (tau - 2.0) * t - tau);
  const double b4 = tau * t * (3.0 * t - 2.0);
  return p_1 * b1 + p0 * b2 + p1 * b3 + p2 * b4;
}

}  // namespace

// FootprintBrush::paintStroke (FootprintBrush.hxx:251-267), spacing 1.0 = the reference.
// The predecessor of the first segment is path[0] (the reference's std::max(i - 1UL, 0UL)
// wraps around at i = 0).
void expand_stroke(const double* path, int32_t n, double spacing, std::vector<StampRec>& out) {
  if (n < 2) return;
  for (int i = 0; i < n - 1; i++) {
    const int ipre = i == 0 ? 0 : i - 1;
    const int inext = std::min(i + 2, n - 1);
    const double* pp = path + 2 * ipre;
    const double* p0 = path + 2 * i;
    const double* p1 = path + 2 * (i + 1);
    const double* pn = path + 2 * inext;
    const double dx = p1[0] - p0[0], dy = p1[1] - p0[1];
    const double dist = std::sqrt(dx * dx + dy * dy);
    const int steps = static_cast<int>(dist / spacing);
    for (int pd = 1; pd <= steps; pd++) {
      const double t = static_cast<double>(pd) * spacing / dist;
      const double dirx = catmull_rom_deriv(pp[0], p0[0], p1[0], pn[0], t);
      const double diry = catmull_rom_deriv(pp[1], p0[1], p1[1], pn[1], t);
      out.push_back(make_rec(catmull_rom(pp[0], p0[0], p1[0], pn[0], t),
                             catmull_rom(pp[1], p0[1], p1[1], pn[1], t), std::atan2(diry, dirx)));
    }
  }
}

}  // namespace pg

// ====================================================================== allocation-free stamping
// Scratch of painty_stamps_f32_noalloc: the per-stamp owner table (map_side^2 ints, up to
// 257^2) followed by one status word. Every GPU that loads this library holds it (about
// 258 KB) until the process exits. All calls share it; calls that overlap on the GPU race.
constexpr int kNoAllocMaxMapSide = 257;
constexpr int kNoAllocOwnerCells = kNoAllocMaxMapSide * kNoAllocMaxMapSide;
static __device__ __align__(256) int g_noalloc_scratch[kNoAllocOwnerCells + 64];

namespace pg {
namespace {
constexpr int kNoAllocMaxDevices = 64;
std::mutex g_noalloc_mu;
void* g_noalloc_addr[kNoAllocMaxDevices] = {};

// Device address of the scratch array on the current device. The host-side symbol is only a
// stand-in, so the address is looked up once per device, with that device current.
int* noalloc_scratch() {
  int dev = 0;
  PG_CUDA(cudaGetDevice(&dev));
  PG_REQUIRE(dev >= 0 && dev < kNoAllocMaxDevices, "device ordinal out of range");
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (!g_noalloc_addr[dev]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || p == nullptr) {
      cudaGetLastError();
      fail(PAINTY_ERR_CUDA, std::string("cudaGetSymbolAddress(no-alloc scratch): ") +
                              cudaGetErrorString(e));
    }
    g_noalloc_addr[dev] = p;
  }
  return static_cast<int*>(g_noalloc_addr[dev]);
}
}  // namespace
}  // namespace pg

using pg::guard;

extern "C" {

painty_status painty_brush_create(double radius, const double* footprint, int32_t fh,
                                  int32_t fw, painty_brush** out) {
  return guard([&] {
    PG_REQUIRE(out != nullptr, "out is null");
    PG_REQUIRE(footprint != nullptr && fh > 0 && fw > 0, "footprint image is empty");
    PG_REQUIRE(std::isfinite(radius) && radius >= 0.0, "radius must be finite and >= 0");
    auto* b = new painty_brush();
    b->full.assign(footprint, footprint + static_cast<size_t>(fh) * fw);
    b->fh = fh;
    b->fw = fw;
    pg::set_radius(b, radius);
    *out = b;
  });
}

painty_status painty_brush_destroy(painty_brush* b) {
  return guard([&] {
    if (!b) return;
    pg::device_free(b->d_footprint);
    pg::device_free(b->d_pickup);
    pg::device_free(b->d_owner);
    pg::device_free(b->d_stamps);
    pg::device_free(b->d_status);
    if (b->has_snapshot) pg::device_free(b->snapshot.base);
    delete b;
  });
}

painty_status painty_brush_set_radius(painty_brush* b, double radius) {
  return guard([&] {
    PG_REQUIRE(b != nullptr, "brush is null");
    PG_REQUIRE(std::isfinite(radius) && radius >= 0.0, "radius must be finite and >= 0");
    pg::set_radius(b, radius);
  });
}

painty_status painty_brush_set_rates(painty_brush* b, double pickup, double deposition) {
  return guard([&] {
    PG_REQUIRE(b != nullptr, "brush is null");
    PG_REQUIRE(std::isfinite(pickup) && std::isfinite(deposition), "rates must be finite");
    b->pickupRate = pickup;
    b->depositionRate = deposition;
  });
}

painty_status painty_brush_get_rates(const painty_brush* b, double* pickup, double* deposition) {
  return guard([&] {
    PG_REQUIRE(b != nullptr, "brush is null");
    if (pickup) *pickup = b->pickupRate;
    if (deposition) *deposition = b->depositionRate;
  });
}

painty_status painty_brush_set_snapshot(painty_brush* b, int32_t use) {
  return guard([&] {
    PG_REQUIRE(b != nullptr, "brush is null");
    b->useSnapshot = use != 0;
  });
}

painty_status painty_brush_dip(painty_brush* b, const double K[3], const double S[3],
                               void* stream) {
  return guard([&] {
    PG_REQUIRE(b && K && S, "null argument");
    (void)stream;
    b->pickup_clear = true;  // clean() (FootprintBrush.hxx:160-166), applied before the next stamp
    for (int i = 0; i < 3; i++) {
      b->paintK[i] = K[i];
      b->paintS[i] = S[i];
    }
  });
}

painty_status painty_brush_update_snapshot(painty_brush* b, const painty_canvas* c,
                                           void* stream) {
  return guard([&] {
    PG_REQUIRE(b && c, "null argument");
    const cudaStream_t st = pg::as_stream(stream);
    if (!b->has_snapshot || b->snapshot.rows != c->wet.rows || b->snapshot.cols != c->wet.cols ||
        b->snapshot.storage != c->wet.storage) {
      if (b->has_snapshot) pg::device_free(b->snapshot.base);
      b->has_snapshot = false;
      void* base = pg::device_alloc(pg::layer_bytes(c->wet.rows, c->wet.cols, c->wet.storage));
      pg::layer_layout(b->snapshot, c->wet.rows, c->wet.cols, c->wet.storage, base);
      b->has_snapshot = true;
    }
    PG_CUDA(cudaMemcpyAsync(b->snapshot.base, c->wet.base, c->wet.bytes,
                            cudaMemcpyDeviceToDevice, st));
    PG_CUDA(cudaStreamSynchronize(st));
  });
}

painty_status painty_brush_info(const painty_brush* b, double* radius, int32_t* F, int32_t* S) {
  return guard([&] {
    PG_REQUIRE(b != nullptr, "brush is null");
    if (radius) *radius = b->radius;
    if (F) *F = b->F;
    if (S) *S = b->sizeMap;
  });
}

painty_status painty_brush_footprint(const painty_brush* b, double* host) {
  return guard([&] {
    PG_REQUIRE(b && host, "null argument");
    std::memcpy(host, b->footprint.data(), b->footprint.size() * sizeof(double));
  });
}

painty_status painty_brush_download_pickup(const painty_brush* b, painty_plane plane, void* host,
                                           painty_host_format fmt, void* stream) {
  return guard([&] {
    PG_REQUIRE(b && host, "null argument");
    const int S = b->sizeMap;
    const size_t cells = static_cast<size_t>(S) * S;
    const bool f64 = b->bound == 1;
    const size_t msz = f64 ? 8 : 4;
    const pg::DevType dt = f64 ? pg::DT_F64 : pg::DT_F32;
    if (b->bound < 0 || !b->d_pickup || b->pickup_clear) {
      // never painted, or cleaned: the map is zero
      const size_t nvals = plane == PAINTY_PLANE_V ? cells : cells * 3;
      const bool host64 = fmt == PAINTY_HOST_F64_INTERLEAVED || fmt == PAINTY_HOST_F64_PLANAR;
      std::memset(host, 0, nvals * (host64 ? 8 : 4));
      return;
    }
    char* base = static_cast<char*>(b->d_pickup);
    if (plane == PAINTY_PLANE_V) {
      const void* p[1] = {base + 6 * cells * msz};
      pg::download_planes(p, 1, dt, S, S, S, host, fmt, pg::as_stream(stream));
    } else {
      PG_REQUIRE(plane == PAINTY_PLANE_K || plane == PAINTY_PLANE_S, "pickup planes are K, S, V");
      const int off = plane == PAINTY_PLANE_K ? 0 : 3;
      const void* p[3] = {base + (off + 0) * cells * msz, base + (off + 1) * cells * msz,
                          base + (off + 2) * cells * msz};
      pg::download_planes(p, 3, dt, S, S, S, host, fmt, pg::as_stream(stream));
    }
  });
}

painty_status painty_imprint(painty_canvas* c, painty_brush* b, double cx, double cy,
                             double theta, void* stream) {
  return guard([&] {
    std::vector<pg::StampRec> r{pg::make_rec(cx, cy, theta)};
    pg::run_stamps(c, b, r, pg::as_stream(stream));
  });
}

painty_status painty_stamps(painty_canvas* c, painty_brush* b, const double* s, int64_t n,
                            void* stream) {
  return guard([&] {
    PG_REQUIRE(n >= 0, "negative stamp count");
    PG_REQUIRE(n == 0 || s != nullptr, "stamps is null");
    std::vector<pg::StampRec> r;
    r.reserve(static_cast<size_t>(n));
    for (int64_t i = 0; i < n; i++) r.push_back(pg::make_rec(s[3 * i], s[3 * i + 1], s[3 * i + 2]));
    pg::run_stamps(c, b, r, pg::as_stream(stream));
  });
}

painty_status painty_stroke(painty_canvas* c, painty_brush* b, const double* path, int32_t n,
                            double spacing, int64_t* stamps_out, void* stream) {
  return guard([&] {
    PG_REQUIRE(n >= 0, "negative path length");
    PG_REQUIRE(n == 0 || path != nullptr, "path is null");
    PG_REQUIRE(std::isfinite(spacing) && spacing > 0.0, "spacing must be positive");
    for (int32_t i = 0; i < 2 * n; i++)
      PG_REQUIRE(std::isfinite(path[i]), "path coordinates must be finite");
    std::vector<pg::StampRec> r;
    pg::expand_stroke(path, n, spacing, r);
    if (stamps_out) *stamps_out = static_cast<int64_t>(r.size());
    pg::run_stamps(c, b, r, pg::as_stream(stream));
  });
}

// Runs the stamp kernel on caller-owned buffers without allocating: the owner table and the
// status word live in g_noalloc_scratch. The first call on a device looks up the scratch
// address (make it before any stream capture). Synchronous: returns after the stamps ran.
painty_status painty_stamps_f32_noalloc(const painty_stamp_buffers_f32* b, void* stream) {
  return guard([&] {
    PG_REQUIRE(b != nullptr, "buffers is null");
    PG_REQUIRE(b->n >= 0, "negative stamp count");
    PG_REQUIRE(b->rows > 0 && b->cols > 0 && b->pitch >= b->cols, "bad canvas geometry");
    PG_REQUIRE(b->footprint_side > 0 && (b->footprint_side & 1) == 1,
               "footprint side must be odd and positive");
    PG_REQUIRE(b->map_side >= b->footprint_side && b->map_side <= b->footprint_side + 1,
               "map side must be the footprint side or one more");
    PG_REQUIRE(b->map_side <= kNoAllocMaxMapSide,
               "pickup map side above the allocation-free maximum of 257 (radius about 90)");
    PG_REQUIRE(static_cast<int64_t>(b->footprint_side) * b->footprint_side <=
                 int64_t(pg::kMaxPixelsPerThread) * pg::kStampThreads,
               "footprint side above 256");
    for (int i = 0; i < 3; i++)
      PG_REQUIRE(b->canvas_K[i] && b->canvas_S[i] && b->pickup_K[i] && b->pickup_S[i],
                 "null plane");
    PG_REQUIRE(b->canvas_V && b->pickup_V && b->footprint, "null plane");
    const bool snap = b->snapshot_V != nullptr;
    if (snap)
      for (int i = 0; i < 3; i++)
        PG_REQUIRE(b->snapshot_K[i] && b->snapshot_S[i], "partial snapshot planes");
    if (b->n == 0) return;
    PG_REQUIRE(b->stamps != nullptr, "stamps is null");
    const cudaStream_t st = pg::as_stream(stream);
    int* scratch = pg::noalloc_scratch();
    unsigned* status = reinterpret_cast<unsigned*>(scratch + kNoAllocOwnerCells);
    PG_CUDA(cudaMemsetAsync(status, 0, sizeof(unsigned), st));
    pg::StampArgs<float, float> a{};
    for (int i = 0; i < 3; i++) {
      a.cK[i] = b->canvas_K[i];
      a.cS[i] = b->canvas_S[i];
      a.sK[i] = snap ? b->snapshot_K[i] : b->canvas_K[i];
      a.sS[i] = snap ? b->snapshot_S[i] : b->canvas_S[i];
      a.pK[i] = b->pickup_K[i];
      a.pS[i] = b->pickup_S[i];
      a.paintK[i] = static_cast<float>(b->paint_K[i]);
      a.paintS[i] = static_cast<float>(b->paint_S[i]);
    }
    a.cV = b->canvas_V;
    a.sV = snap ? b->snapshot_V : b->canvas_V;
    a.pV = b->pickup_V;
    a.footprint = b->footprint;
    a.stamps = reinterpret_cast<const pg::StampRec*>(b->stamps);
    a.n = b->n;
    a.rows = b->rows;
    a.cols = b->cols;
    a.pitch = b->pitch;
    a.F = b->footprint_side;
    a.S = b->map_side;
    a.wr = (b->footprint_side - 1) / 2;
    a.radius = b->radius;
    a.pickupRate = static_cast<float>(b->pickup_rate);
    a.depositionRate = static_cast<float>(b->deposition_rate);
    a.capacity = static_cast<float>(b->capacity);
    a.use_snapshot = snap ? 1 : 0;
    a.owner_global = scratch;
    a.status = status;
    const size_t dyn = static_cast<size_t>(b->footprint_side) * (2 * sizeof(int) + 2);
    auto kern = pg::stamp_kernel<float, float>;
    PG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 static_cast<int>(dyn)));
    kern<<<1, pg::kStampThreads, dyn, st>>>(a);
    pg::count_launch();
    PG_CUDA(cudaGetLastError());
    unsigned hs = 0;
    PG_CUDA(cudaMemcpyAsync(&hs, status, sizeof(unsigned), cudaMemcpyDeviceToHost, st));
    PG_CUDA(cudaStreamSynchronize(st));
    if (hs != 0) pg::fail(PAINTY_ERR_CUDA, "stamp kernel reported an internal error");
  });
}

}  // extern "C"
