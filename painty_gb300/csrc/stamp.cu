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
#include <map>
#include <type_traits>
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
  M* pK[3];  // pickup map in global memory, S*S per plane (the brush's state)
  M* pS[3];
  M* pV;
  const M* footprint;  // F*F
  const StampRec* stamps;
  int64_t n;
  int32_t rows, cols;
  int64_t pitch;
  int32_t F, S, wr;
  // Stamp pixels with dc^2 + dr^2 > support2 map to cells whose footprint is 0 (the rotated
  // and rounded cell lies within 0.71 px of the rotated point) and change nothing.
  int32_t support2;
  double radius;
  M pickupRate, depositionRate, capacity;
  M paintK[3], paintS[3];
  int32_t use_snapshot;
  // Snapshot dirty map (rows x pitch bytes): 1 where the snapshot may differ from the canvas.
  // The ring refresh copies only dirty pixels (copying an equal pixel is a no-op); pixels a
  // stamp changes are marked. NULL: refresh the whole ring.
  uint8_t* dirty;
  int32_t pickup_zero;    // the map starts cleared (a dip or new radius since the last run)
  int32_t pickup_smem;    // stage the pickup map in shared memory for the launch
  int32_t footprint_smem; // stage the footprint in shared memory
  int* owner_global;      // S*S ints when the owner table does not fit in shared memory
  unsigned* status;
};

constexpr int kParamChunk = 32;  // stamps whose parameters are derived together

struct StampParams {
  double cx, cy, c, s;
  float cf, sf;
  int tl[2], br[2], tla[2], bra[2];
};

// Reference map coordinate round(fl(fl(u*ca -/+ v*cb) + w)): the FP32 value `fast` decides
// unless it lies within 2e-4 of a rounding tie (its error is below 4e-5), then the
// reference's double operations are repeated.
__device__ __forceinline__ int map_coord(float fast, int u, double ca, int v, double cb,
                                         bool minus, int w) {
  const float fr = fast - floorf(fast);
  if (fabsf(fr - 0.5f) > 2e-4f) return __float2int_rn(fast);
  const double p1 = __dmul_rn(static_cast<double>(u), ca);
  const double p2 = __dmul_rn(static_cast<double>(v), cb);
  const double r = minus ? __dsub_rn(p1, p2) : __dadd_rn(p1, p2);
  return static_cast<int>(round(__dadd_rn(r, static_cast<double>(w))));
}

// blend (FootprintBrush.hxx:331-340): (va a + vb b) / (va + vb) when va + vb > MinVolume.
// FP64 divides as the reference; FP32 multiplies by the correctly rounded reciprocal.
__device__ __forceinline__ void blend3(double va, const double (&a)[3], double vb,
                                       const double (&b)[3], double (&r)[3]) {
  const double tot = __dadd_rn(va, vb);
  if (tot > 0.001) {
#pragma unroll
    for (int i = 0; i < 3; i++)
      r[i] = __ddiv_rn(__dadd_rn(__dmul_rn(va, a[i]), __dmul_rn(vb, b[i])), tot);
  } else {
#pragma unroll
    for (int i = 0; i < 3; i++) r[i] = a[i];
  }
}
__device__ __forceinline__ void blend3(float va, const float (&a)[3], float vb,
                                       const float (&b)[3], float (&r)[3]) {
  const float tot = va + vb;
  if (tot > 0.001f) {
    const float inv = __frcp_rn(tot);
#pragma unroll
    for (int i = 0; i < 3; i++) r[i] = fmaf(va, a[i], vb * b[i]) * inv;
  } else {
#pragma unroll
    for (int i = 0; i < 3; i++) r[i] = a[i];
  }
}

// Plane p (K r,g,b, S r,g,b, V) of the pickup map in global memory.
template <class TK, class TV, class M>
__device__ __forceinline__ M* pickup_plane(const StampArgs<TK, TV>& a, int p) {
  return p < 3 ? a.pK[p] : (p < 6 ? a.pS[p - 3] : a.pV);
}

// pickupPaint then depositPaint for one stamp pixel (FootprintBrush.hxx:349-431); fp > 0.
// PS: the pickup map is staged in shared memory at `pbase` (7 planes `cells` apart).
template <bool PS, class TK, class TV, class M>
__device__ __forceinline__ void process_pixel(const StampArgs<TK, TV>& a, M* pbase, int cells,
                                              M fp, int64_t c, int m) {
  using A = Arith<M>;
  auto cell = [&](int p) -> M& {
    if constexpr (PS) return pbase[p * cells + m];
    else return pickup_plane<TK, TV, M>(a, p)[m];
  };
  // independent loads first: pickup cell, pickup source, canvas pixel
  M vp = cell(6);
  M kp[3], sp[3], ck[3], cs[3];
#pragma unroll
  for (int i = 0; i < 3; i++) {
    kp[i] = cell(i);
    sp[i] = cell(3 + i);
    ck[i] = ld_elem<M>(a.cK[i] + c);
    cs[i] = ld_elem<M>(a.cS[i] + c);
  }
  const M vsrc = ld_elem<M>(a.sV + c);
  M vcan = ld_elem<M>(a.cV + c);
  // pickupPaint
  const M vleave = A::mul(A::mul(a.pickupRate, vsrc), fp);
  bool pk_changed = false;
  if (vleave > M(0.001)) {
    st_elem<M>(a.sV + c, A::sub(vsrc, vleave));
    M ks[3], ss[3], nk[3], ns[3];
    if (a.use_snapshot) {
#pragma unroll
      for (int i = 0; i < 3; i++) {
        ks[i] = ld_elem<M>(a.sK[i] + c);
        ss[i] = ld_elem<M>(a.sS[i] + c);
      }
    } else {  // the pickup source is the canvas itself
#pragma unroll
      for (int i = 0; i < 3; i++) {
        ks[i] = ck[i];
        ss[i] = cs[i];
      }
      vcan = ld_elem<M>(a.cV + c);  // the stored remainder
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
  cell(6) = A::sub(vp, pleave);
  if (pk_changed) {
#pragma unroll
    for (int i = 0; i < 3; i++) {
      cell(i) = kp[i];
      cell(3 + i) = sp[i];
    }
  }
  const M vb = A::mul(a.capacity, fp);
  M nk[3], ns[3];
  blend3(vb, ksrc, vcan, ck, nk);
  blend3(vb, ssrc, vcan, cs, ns);
#pragma unroll
  for (int i = 0; i < 3; i++) {
    st_elem<M>(a.cK[i] + c, nk[i]);
    st_elem<M>(a.cS[i] + c, ns[i]);
  }
  st_elem<M>(a.cV + c, A::add(vb, vcan));
  if (a.dirty) a.dirty[c] = 1;
}

struct PixelInfo {
  int xc, yc, mx, my;
  bool live;  // inside canvas and map, and a positive footprint: the pixel changes state
};

// Stamp pixel (row, col) of the F x F box: canvas pixel, pickup-map cell, footprint height.
template <class TK, class TV, class M>
__device__ __forceinline__ PixelInfo pixel_info(const StampArgs<TK, TV>& a, const StampParams& sp,
                                                const int* xs, const int* ys, const M* fps,
                                                int row, int col, M* fp_out) {
  PixelInfo p;
  const int dr = row - a.wr, dc = col - a.wr;
  p.xc = xs[col];
  p.yc = ys[row];
  const float dcf = static_cast<float>(dc), drf = static_cast<float>(dr);
  const float wrf = static_cast<float>(a.wr);
  const float fx = fmaf(-drf, sp.sf, dcf * sp.cf) + wrf;  // col*cos - row*sin + wr
  const float fy = fmaf(drf, sp.cf, dcf * sp.sf) + wrf;   // col*sin + row*cos + hr
  p.mx = map_coord(fx, dc, sp.c, dr, sp.s, true, a.wr);
  p.my = map_coord(fy, dc, sp.s, dr, sp.c, false, a.wr);
  const bool inside = p.yc >= 0 && p.xc >= 0 && p.xc < a.cols && p.yc < a.rows && p.my >= 0 &&
                      p.mx >= 0 && p.mx < a.S && p.my < a.S;
  M fp = M(0);
  if (inside && p.mx < a.F && p.my < a.F) fp = fps[p.my * a.F + p.mx];
  *fp_out = fp;
  p.live = inside && fp > M(0);
  return p;
}

// Earlier pixels on the same canvas pixel (left/top edge duplicates) finished in an earlier
// wave. done_c[row] / done_r[col] hold the 1-based wave in which pixel (c0, row) / (col, r0)
// finished (c0, r0: the first of the duplicated column / row), 0 while pending.
__device__ __forceinline__ bool canvas_ready(const int* xs, const int* ys, int F,
                                             const uint16_t* done_c, const uint16_t* done_r,
                                             int row, int col, int wave) {
  auto fin = [wave](uint16_t d) { return d != 0 && d <= wave; };
  const bool dupx_prev = col > 0 && xs[col - 1] == xs[col];  // col == c0 + 1
  const bool dupy_prev = row > 0 && ys[row - 1] == ys[row];  // row == r0 + 1
  bool ok = true;
  if (dupx_prev) ok = ok && fin(done_c[row]);
  if (dupy_prev) {
    ok = ok && fin(done_r[col]);
    if (col + 1 < F && xs[col] == xs[col + 1]) ok = ok && fin(done_r[col + 1]);  // up-right
    if (dupx_prev) ok = ok && fin(done_r[col - 1]);                                // up-left
  }
  return ok;
}

__device__ __forceinline__ void mark_done(const int* xs, const int* ys, int F, uint16_t* done_c,
                                          uint16_t* done_r, int row, int col, uint16_t v) {
  if (col + 1 < F && xs[col] == xs[col + 1]) done_c[row] = v;
  if (row + 1 < F && ys[row] == ys[row + 1]) done_r[col] = v;
}

// FootprintBrush.hxx:291-305 box and snapshot-ring bounds, in the reference's double ops
__device__ __forceinline__ StampParams derive_params(const StampRec& st, int wr, double radius,
                                                     int rows, int cols) {
  StampParams p;
  p.cx = st.cx;
  p.cy = st.cy;
  p.c = st.c;
  p.s = st.s;
  p.cf = static_cast<float>(st.c);
  p.sf = static_cast<float>(st.s);
  const double w = wr;
  p.tl[0] = static_cast<int>(__dsub_rn(st.cx, w));
  p.tl[1] = static_cast<int>(__dsub_rn(st.cy, w));
  p.br[0] = static_cast<int>(__dadd_rn(st.cx, w));
  p.br[1] = static_cast<int>(__dadd_rn(st.cy, w));
  p.tla[0] = max(static_cast<int>(__dsub_rn(__dsub_rn(st.cx, w), radius)), 0);
  p.tla[1] = max(static_cast<int>(__dsub_rn(__dsub_rn(st.cy, w), radius)), 0);
  p.bra[0] = min(static_cast<int>(__dadd_rn(__dadd_rn(st.cx, w), radius)), cols - 1);
  p.bra[1] = min(static_cast<int>(__dadd_rn(__dadd_rn(st.cy, w), radius)), rows - 1);
  return p;
}

__host__ __device__ constexpr size_t align_up(size_t x, size_t a) {
  return (x + a - 1) / a * a;
}

// Dynamic shared memory layout of stamp_kernel (all offsets 16-byte aligned).
struct StampSmem {
  size_t fp, pick, own, xs, ys, done_c, done_r, queue, total;
};
constexpr int kRefreshQueue = 2048;  // snapshot-refresh queue entries (canvas offsets)
template <class M>
__host__ __device__ inline StampSmem stamp_smem_layout(int F, int S, bool fp_smem,
                                                       bool pick_smem, bool own_smem) {
  StampSmem L{};
  size_t o = 0;
  L.fp = o;
  if (fp_smem) o = align_up(o + size_t(F) * F * sizeof(M), 16);
  L.pick = o;
  if (pick_smem) o = align_up(o + size_t(7) * S * S * sizeof(M), 16);
  L.own = o;
  if (own_smem) o = align_up(o + size_t(S) * S * sizeof(int), 16);
  L.xs = o;
  o = align_up(o + size_t(F) * sizeof(int), 16);
  L.ys = o;
  o = align_up(o + size_t(F) * sizeof(int), 16);
  L.done_c = o;
  o = align_up(o + size_t(F) * sizeof(uint16_t), 16);
  L.done_r = o;
  o = align_up(o + size_t(F) * sizeof(uint16_t), 16);
  L.queue = o;
  o = align_up(o + size_t(kRefreshQueue) * sizeof(int), 16);
  L.total = o;
  return L;
}

constexpr int kEpochMax = 32767;  // owner keys: ((kEpochMax - epoch) << 16) | pixel index
constexpr int kWarps = kStampThreads / 32;

// Snapshot refresh, pass 1: scan the dirty bytes of ring row segment [lo, hi] four at a
// time (one 32-bit word per lane) and queue the dirty pixels (canvas offsets) in shared
// memory; a pixel's dirty byte is cleared only once it is queued, so entries past the queue's
// end stay dirty (and flag an overflow) for the next scan. Requires a dirty map.
template <class TK, class TV>
__device__ __forceinline__ void scan_segment(const StampArgs<TK, TV>& a, int row, int lo, int hi,
                                             int lane, int* queue, int* qcount, int* qover) {
  const int64_t rb = static_cast<int64_t>(row) * a.pitch;
  for (int w0 = (lo & ~3); w0 <= hi; w0 += 4 * 32) {
    const int w = w0 + 4 * lane;
    uint32_t word = 0, take = 0;
    if (w <= hi) {
      word = *reinterpret_cast<const uint32_t*>(a.dirty + rb + w);
#pragma unroll
      for (int b = 0; b < 4; b++) {
        const int col = w + b;
        if (col >= lo && col <= hi && ((word >> (8 * b)) & 0xffu)) take |= 1u << b;
      }
    }
    const int n = __popc(take);
    int incl = n;  // warp inclusive prefix sum of the counts
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const int v = __shfl_up_sync(0xffffffffu, incl, d);
      if (lane >= d) incl += v;
    }
    const int total = __shfl_sync(0xffffffffu, incl, 31);
    int base = 0;
    if (lane == 31 && total > 0) base = atomicAdd(qcount, total);
    base = __shfl_sync(0xffffffffu, base, 31);
    int slot = base + incl - n;
    uint32_t cleared = word;
    for (int b = 0; b < 4; b++) {
      if (!((take >> b) & 1u)) continue;
      if (slot < kRefreshQueue) {
        queue[slot] = static_cast<int>(rb + w + b);
        cleared &= ~(0xffu << (8 * b));
      } else {
        *qover = 1;
      }
      slot++;
    }
    if (take && cleared != word) *reinterpret_cast<uint32_t*>(a.dirty + rb + w) = cleared;
  }
}

// Snapshot refresh without a dirty map: copy every pixel of the segment.
template <class TK, class TV>
__device__ __forceinline__ void copy_segment(const StampArgs<TK, TV>& a, int row, int lo, int hi,
                                             int lane) {
  const int64_t rb = static_cast<int64_t>(row) * a.pitch;
  for (int col = lo + lane; col <= hi; col += 32) {
    const int64_t o = rb + col;
#pragma unroll
    for (int ch = 0; ch < 3; ch++) {
      a.sK[ch][o] = a.cK[ch][o];
      a.sS[ch][o] = a.cS[ch][o];
    }
    a.sV[o] = a.cV[o];
  }
}

// Snapshot refresh, pass 2: copy the queued pixels canvas -> snapshot (7 planes).
template <class TK, class TV>
__device__ __forceinline__ void copy_queued(const StampArgs<TK, TV>& a, const int* queue,
                                            int count, int tid, int T) {
  for (int q = tid; q < count; q += T) {
    const int64_t o = queue[q];
    TK k[3], s[3];
#pragma unroll
    for (int ch = 0; ch < 3; ch++) {
      k[ch] = a.cK[ch][o];
      s[ch] = a.cS[ch][o];
    }
    const TV v = a.cV[o];
#pragma unroll
    for (int ch = 0; ch < 3; ch++) {
      a.sK[ch][o] = k[ch];
      a.sS[ch][o] = s[ch];
    }
    a.sV[o] = v;
  }
}

// The ring of a stamp: rows of the grown box, the strict interior of the box excepted
// (FootprintBrush.hxx:307-318); one warp per row. With a dirty map the dirty pixels are
// queued (copied by copy_queued); without one every ring pixel is copied here.
template <class TK, class TV>
__device__ __forceinline__ void scan_ring(const StampArgs<TK, TV>& a, const StampParams& sp,
                                          int warp, int lane, int nwarps, int* queue,
                                          int* qcount, int* qover) {
  for (int row = sp.tla[1] + warp; row <= sp.bra[1]; row += nwarps) {
    const bool interior_row = row > sp.tl[1] && row < sp.br[1];
    const int lo0 = sp.tla[0], hi0 = interior_row ? min(sp.tl[0], sp.bra[0]) : sp.bra[0];
    const int lo1 = max(sp.br[0], sp.tla[0]), hi1 = interior_row ? sp.bra[0] : -1;
    if (a.dirty) {
      scan_segment(a, row, lo0, hi0, lane, queue, qcount, qover);
      scan_segment(a, row, lo1, hi1, lane, queue, qcount, qover);
    } else {
      copy_segment(a, row, lo0, hi0, lane);
      copy_segment(a, row, lo1, hi1, lane);
    }
  }
}

// One CTA applies the stamps in order. Pixel slots: warp w owns box rows w, w+32, ...; lane l
// owns columns l, l+32, ...; slot j = jr * NC + jc (jr-th row, jc-th column of the thread).
// Stamps of a host-built record list (imprint / painty_stamps / painty_stroke).
struct RecordSource {
  const StampRec* recs;
  int64_t n;
  __device__ __forceinline__ int64_t count() const { return n; }
  __device__ __forceinline__ StampRec get(int64_t k) const { return recs[k]; }
};

// One stroke's stamps applied in order by the whole CTA (the kernel body shared by the
// single-canvas and the batched kernels). `a` may live in shared or parameter memory.
template <bool PS, bool BIG, class TK, class TV, class Src>
__device__ __forceinline__ void run_stroke(const StampArgs<TK, TV>& a, const Src& src,
                                           unsigned char* smem_raw, StampParams* sparams,
                                           int* s_q) {
  using M = typename MathOf<TK>::type;
  int& s_qcount = s_q[0];
  int& s_qover = s_q[1];
  const int64_t nstamps = src.count();
  const int tid = threadIdx.x;
  const int T = blockDim.x;
  const int warp = tid >> 5, lane = tid & 31;
  const int F = a.F, S = a.S;
  const int npix = F * F;
  const int cells = S * S;
  const int NC = (F + 31) / 32;
  const StampSmem L = stamp_smem_layout<M>(F, S, !BIG, PS, !BIG);
  const M* fps = !BIG ? reinterpret_cast<M*>(smem_raw + L.fp) : a.footprint;
  M* pbase = PS ? reinterpret_cast<M*>(smem_raw + L.pick) : nullptr;
  int* own = BIG ? a.owner_global : reinterpret_cast<int*>(smem_raw + L.own);
  int* xs = reinterpret_cast<int*>(smem_raw + L.xs);
  int* ys = reinterpret_cast<int*>(smem_raw + L.ys);
  uint16_t* done_c = reinterpret_cast<uint16_t*>(smem_raw + L.done_c);
  uint16_t* done_r = reinterpret_cast<uint16_t*>(smem_raw + L.done_r);
  int* queue = reinterpret_cast<int*>(smem_raw + L.queue);

  // launch prologue: footprint and pickup map staged, owner table reset
  if (!BIG) {
    M* f = reinterpret_cast<M*>(smem_raw + L.fp);
    for (int i = tid; i < npix; i += T) f[i] = a.footprint[i];
  }
  for (int i = tid; i < 7 * cells; i += T) {
    const int p = i / cells, m = i - p * cells;
    if (PS)
      pbase[i] = a.pickup_zero ? M(0) : pickup_plane<TK, TV, M>(a, p)[m];
    else if (a.pickup_zero)
      pickup_plane<TK, TV, M>(a, p)[m] = M(0);
  }
  for (int i = tid; i < cells; i += T) own[i] = INT_MAX;
  if (tid == 0) {
    s_qcount = 0;
    s_qover = 0;
  }
  int epoch = 0;

  for (int64_t k = 0; k < nstamps; k++) {
    const int slot = static_cast<int>(k % kParamChunk);
    if (slot == 0) {  // derive the next chunk of stamp parameters in parallel
      __syncthreads();
      const int64_t j = k + tid;
      if (tid < kParamChunk && j < nstamps)
        sparams[tid] = derive_params(src.get(j), a.wr, a.radius, a.rows, a.cols);
      if (epoch > kEpochMax - 2 * kMaxWaves) {  // owner keys about to wrap: reset
        for (int i = tid; i < cells; i += T) own[i] = INT_MAX;
        epoch = 0;
      }
      __syncthreads();
    }
    const StampParams& sp = sparams[slot];
    // phase A: per column / row canvas coordinates (double, as the reference), done flags
    // reset, snapshot ring scanned for dirty pixels
    for (int i = tid; i < F; i += T) {
      xs[i] = static_cast<int>(__dadd_rn(static_cast<double>(i - a.wr), sp.cx));
      ys[i] = static_cast<int>(__dadd_rn(static_cast<double>(i - a.wr), sp.cy));
      done_c[i] = 0;
      done_r[i] = 0;
    }
    if (a.use_snapshot) scan_ring(a, sp, warp, lane, kWarps, queue, &s_qcount, &s_qover);
    __syncthreads();
    // phase B: queued snapshot copies; live pixels (inside the support disc, canvas and map,
    // positive footprint) classified and bidding for their map cells (wave 1)
    if (a.use_snapshot) copy_queued(a, queue, min(s_qcount, kRefreshQueue), tid, T);
    int wave = 1;
    int key_hi = (kEpochMax - epoch) << 16;
    epoch++;
    uint64_t rem = 0;
    for (int row = warp, jr = 0; row < F; row += kWarps, jr++) {
      const int dr = row - a.wr;
      for (int col = lane, jc = 0; col < F; col += 32, jc++) {
        const int dc = col - a.wr;
        bool live = false;
        if (dc * dc + dr * dr <= a.support2) {
          M fp;
          const PixelInfo p = pixel_info(a, sp, xs, ys, fps, row, col, &fp);
          if (p.live) {
            live = true;
            atomicMin(&own[p.my * S + p.mx], key_hi | (row * F + col));
          }
        }
        if (live)
          rem |= 1ull << (jr * NC + jc);
        else
          mark_done(xs, ys, F, done_c, done_r, row, col, 1);  // done "before" wave 1
      }
    }
    __syncthreads();
    // The refresh queue overflowed: drain the rest before painting. Each round clears the
    // dirty bytes of the pixels it queued, so the rounds end; the cap only guards the loop.
    for (int round = 0; s_qover; round++) {
      if (round > (sp.bra[1] - sp.tla[1] + 2) * (sp.bra[0] - sp.tla[0] + 2) / kRefreshQueue + 2) {
        if (tid == 0) atomicOr(a.status, kStatusWaveCap);
        break;
      }
      __syncthreads();
      if (tid == 0) {
        s_qcount = 0;
        s_qover = 0;
      }
      __syncthreads();
      scan_ring(a, sp, warp, lane, kWarps, queue, &s_qcount, &s_qover);
      __syncthreads();
      copy_queued(a, queue, min(s_qcount, kRefreshQueue), tid, T);
      __syncthreads();
    }
    if (tid == 0) s_qcount = 0;
    for (;;) {
      for (uint64_t bits = rem; bits; bits &= bits - 1) {
        const int j = __ffsll(static_cast<long long>(bits)) - 1;
        const int row = warp + kWarps * (j / NC), col = lane + 32 * (j % NC);
        M fp;
        const PixelInfo p = pixel_info(a, sp, xs, ys, fps, row, col, &fp);
        if (own[p.my * S + p.mx] == (key_hi | (row * F + col)) &&
            canvas_ready(xs, ys, F, done_c, done_r, row, col, wave)) {
          process_pixel<PS, TK, TV, M>(a, pbase, cells, fp,
                                       static_cast<int64_t>(p.yc) * a.pitch + p.xc,
                                       p.my * S + p.mx);
          rem &= ~(1ull << j);
          mark_done(xs, ys, F, done_c, done_r, row, col, static_cast<uint16_t>(wave + 1));
        }
      }
      const int any = __syncthreads_or(rem != 0);
      if (!any) break;
      if (wave >= kMaxWaves) {  // cannot happen: the lowest remaining pixel always runs
        if (tid == 0) atomicOr(a.status, kStatusWaveCap);
        break;
      }
      wave++;
      key_hi = (kEpochMax - epoch) << 16;
      epoch++;
      for (uint64_t bits = rem; bits; bits &= bits - 1) {  // bid for the map cell
        const int j = __ffsll(static_cast<long long>(bits)) - 1;
        const int row = warp + kWarps * (j / NC), col = lane + 32 * (j % NC);
        M fp;
        const PixelInfo p = pixel_info(a, sp, xs, ys, fps, row, col, &fp);
        atomicMin(&own[p.my * S + p.mx], key_hi | (row * F + col));
      }
      __syncthreads();
    }
  }
  // epilogue: the brush keeps its pickup map
  __syncthreads();
  if (PS) {
    for (int i = tid; i < 7 * cells; i += T) {
      const int p = i / cells, m = i - p * cells;
      pickup_plane<TK, TV, M>(a, p)[m] = pbase[i];
    }
    __syncthreads();
  }
}

// PS: pickup map staged in shared memory. BIG: footprint and owner table in global memory
// (maps too large for shared memory); otherwise both are in shared memory.
template <bool PS, bool BIG, class TK, class TV>
__global__ void __launch_bounds__(kStampThreads, 1) stamp_kernel(const __grid_constant__ StampArgs<TK, TV> a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ StampParams sparams[kParamChunk];
  __shared__ int s_q[2];
  run_stroke<PS, BIG>(a, RecordSource{a.stamps, a.n}, smem_raw, sparams, s_q);
}

// ---------------------------------------------------------------------- batched painting
constexpr int kMaxPathPoints = 512;  // control points per stroke in the batched kernel

// Spline.hxx:27-73 in painty's operation order, without contraction (device side).
__device__ __forceinline__ double cr_pos(double p_1, double p0, double p1, double p2, double t) {
  const double t2 = __dmul_rn(t, t), t3 = __dmul_rn(t2, t);
  const double b1 = __dsub_rn(__dadd_rn(__dmul_rn(-0.5, t), __dmul_rn(1.0, t2)), __dmul_rn(0.5, t3));
  const double b2 = __dadd_rn(__dadd_rn(1.0, __dmul_rn(-2.5, t2)), __dmul_rn(1.5, t3));
  const double b3 = __dadd_rn(__dadd_rn(__dmul_rn(0.5, t), __dmul_rn(2.0, t2)), __dmul_rn(-1.5, t3));
  const double b4 = __dadd_rn(__dmul_rn(-0.5, t2), __dmul_rn(0.5, t3));
  return __dadd_rn(__dadd_rn(__dadd_rn(__dmul_rn(p_1, b1), __dmul_rn(p0, b2)), __dmul_rn(p1, b3)),
                   __dmul_rn(p2, b4));
}
__device__ __forceinline__ double cr_deriv(double p_1, double p0, double p1, double p2, double t) {
  const double t2 = __dmul_rn(t, t);
  const double b1 = __dmul_rn(0.5, __dsub_rn(__dadd_rn(__dmul_rn(-3.0, t2), __dmul_rn(4.0, t)), 1.0));
  const double b2 = __dmul_rn(-t, __dadd_rn(__dadd_rn(-1.0, __dmul_rn(-4.5, t)), 6.0));
  const double b3 = __dmul_rn(__dsub_rn(t, 1.0), __dsub_rn(__dmul_rn(-4.5, t), 0.5));
  const double b4 = __dmul_rn(__dmul_rn(0.5, t), __dsub_rn(__dmul_rn(3.0, t), 2.0));
  return __dadd_rn(__dadd_rn(__dadd_rn(__dmul_rn(p_1, b1), __dmul_rn(p0, b2)), __dmul_rn(p1, b3)),
                   __dmul_rn(p2, b4));
}

// Stamps of FootprintBrush::paintStroke (FootprintBrush.hxx:251-267) over a path with chord
// spacing `spacing`, generated on the device: stamp pd of segment i sits at t = pd*spacing/dist.
// The angle's atan2 / cos / sin are the device's double functions (within 1-2 ulp of libm's).
struct PathSource {
  const double* pts;  // (x, y) pairs
  int npts;
  double spacing;
  const int64_t* seg_end;  // inclusive prefix sums of the per-segment stamp counts
  int64_t n;
  __device__ __forceinline__ int64_t count() const { return n; }
  __device__ __forceinline__ StampRec get(int64_t k) const {
    int lo = 0, hi = npts - 2;
    while (lo < hi) {
      const int mid = (lo + hi) >> 1;
      if (seg_end[mid] > k) hi = mid; else lo = mid + 1;
    }
    const int i = lo;
    const int64_t pd = k - (i > 0 ? seg_end[i - 1] : 0) + 1;
    const double* pp = pts + 2 * (i > 0 ? i - 1 : 0);
    const double* p0 = pts + 2 * i;
    const double* p1 = pts + 2 * (i + 1);
    const double* pn = pts + 2 * min(i + 2, npts - 1);
    const double dx = __dsub_rn(p1[0], p0[0]), dy = __dsub_rn(p1[1], p0[1]);
    const double dist = __dsqrt_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)));
    const double t = __ddiv_rn(__dmul_rn(static_cast<double>(pd), spacing), dist);
    const double dirx = cr_deriv(pp[0], p0[0], p1[0], pn[0], t);
    const double diry = cr_deriv(pp[1], p0[1], p1[1], pn[1], t);
    const double theta = atan2(diry, dirx);
    StampRec r;
    r.cx = cr_pos(pp[0], p0[0], p1[0], pn[0], t);
    r.cy = cr_pos(pp[1], p0[1], p1[1], pn[1], t);
    r.c = cos(-theta);
    r.s = sin(-theta);
    return r;
  }
};

template <class TK, class TV>
struct BatchCanvas {
  TK* cK[3];
  TK* cS[3];
  TV* cV;
  TK* sK[3];
  TK* sS[3];
  TV* sV;
  uint8_t* dirty;
  int32_t rows, cols;
  int64_t pitch;
  int32_t use_snapshot;
  int32_t nstrokes;
  int64_t first_stroke;
  double pickup_rate, deposition_rate, capacity;
  void* brush_pickup;  // the brush's own pickup map: the canvas's last stroke paints into it
};

struct BatchStroke {
  int64_t first_point;
  int32_t npoints;
  int32_t F, S, wr, support2;
  int32_t plan;  // bit 0: pickup map in shared memory; bit 1: footprint and owners global
  int64_t fp_offset;
  double radius, spacing;
  double K[3], Sc[3];
};

template <class TK, class TV>
struct BatchArgs {
  using M = typename MathOf<TK>::type;
  const BatchCanvas<TK, TV>* canvases;
  const BatchStroke* strokes;
  const double* points;
  const M* footprints;
  const int32_t* order;  // canvases, heaviest first
  int32_t ncanvas;
  int* counter;
  M* scratch_pickup;  // per CTA: 7 planes of Smax^2
  int* scratch_owner; // per CTA: Smax^2
  int64_t pickup_stride, owner_stride;
  unsigned* status;
};

// Persistent batched painting: each CTA claims canvases (heaviest first) and applies their
// strokes in order, each as setRadius + dip + paintStroke on the canvas's brush.
template <class TK, class TV>
__global__ void __launch_bounds__(kStampThreads, 1) batch_kernel(const __grid_constant__ BatchArgs<TK, TV> b) {
  using M = typename MathOf<TK>::type;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ StampParams sparams[kParamChunk];
  __shared__ int s_q[2];
  __shared__ StampArgs<TK, TV> sa;
  __shared__ int s_item;
  __shared__ int64_t seg_end[kMaxPathPoints];
  const int tid = threadIdx.x, T = blockDim.x;
  for (;;) {
    __syncthreads();
    if (tid == 0) {
      const int i = atomicAdd(b.counter, 1);
      s_item = i < b.ncanvas ? b.order[i] : -1;
    }
    __syncthreads();
    const int ci = s_item;
    if (ci < 0) return;
    const BatchCanvas<TK, TV>& cv = b.canvases[ci];
    for (int32_t k = 0; k < cv.nstrokes; k++) {
      const BatchStroke& st = b.strokes[cv.first_stroke + k];
      const int nseg = st.npoints - 1;
      __syncthreads();
      if (tid == 0) {
        const bool last = k + 1 == cv.nstrokes;
        const int64_t cells = static_cast<int64_t>(st.S) * st.S;
        M* pk = last ? static_cast<M*>(cv.brush_pickup)
                     : b.scratch_pickup + static_cast<int64_t>(blockIdx.x) * b.pickup_stride;
        for (int i = 0; i < 3; i++) {
          sa.cK[i] = cv.cK[i];
          sa.cS[i] = cv.cS[i];
          sa.sK[i] = cv.sK[i];
          sa.sS[i] = cv.sS[i];
          sa.pK[i] = pk + i * cells;
          sa.pS[i] = pk + (3 + i) * cells;
          sa.paintK[i] = static_cast<M>(st.K[i]);
          sa.paintS[i] = static_cast<M>(st.Sc[i]);
        }
        sa.cV = cv.cV;
        sa.sV = cv.sV;
        sa.pV = pk + 6 * cells;
        sa.footprint = b.footprints + st.fp_offset;
        sa.stamps = nullptr;
        sa.n = 0;
        sa.rows = cv.rows;
        sa.cols = cv.cols;
        sa.pitch = cv.pitch;
        sa.F = st.F;
        sa.S = st.S;
        sa.wr = st.wr;
        sa.support2 = st.support2;
        sa.radius = st.radius;
        sa.pickupRate = static_cast<M>(cv.pickup_rate);
        sa.depositionRate = static_cast<M>(cv.deposition_rate);
        sa.capacity = static_cast<M>(cv.capacity);
        sa.use_snapshot = cv.use_snapshot;
        sa.dirty = cv.use_snapshot ? cv.dirty : nullptr;
        sa.pickup_zero = 1;  // dip: the pickup map starts clean
        sa.pickup_smem = st.plan & 1;
        sa.footprint_smem = (st.plan & 2) ? 0 : 1;
        sa.owner_global = (st.plan & 2)
                            ? b.scratch_owner + static_cast<int64_t>(blockIdx.x) * b.owner_stride
                            : nullptr;
        sa.status = b.status;
      }
      const double* pts = b.points + 2 * st.first_point;
      for (int i = tid; i < nseg; i += T) {  // stamps per segment (paintStroke's loop bound)
        const double dx = __dsub_rn(pts[2 * (i + 1)], pts[2 * i]);
        const double dy = __dsub_rn(pts[2 * (i + 1) + 1], pts[2 * i + 1]);
        const double dist = __dsqrt_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)));
        seg_end[i] = static_cast<int64_t>(static_cast<int>(__ddiv_rn(dist, st.spacing)));
      }
      __syncthreads();
      if (tid == 0)
        for (int i = 1; i < nseg; i++) seg_end[i] += seg_end[i - 1];
      __syncthreads();
      const int64_t n = nseg > 0 ? seg_end[nseg - 1] : 0;
      if (n == 0) continue;
      const PathSource src{pts, st.npoints, st.spacing, seg_end, n};
      switch (st.plan) {
        case 0: run_stroke<false, false>(sa, src, smem_raw, sparams, s_q); break;
        case 1: run_stroke<true, false>(sa, src, smem_raw, sparams, s_q); break;
        case 2: run_stroke<false, true>(sa, src, smem_raw, sparams, s_q); break;
        default: run_stroke<true, true>(sa, src, smem_raw, sparams, s_q); break;
      }
    }
  }
}

}  // namespace
}  // namespace pg

// ====================================================================== brush

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

// Squared radius bound (in stamp pixels) of the footprint's support: a stamp pixel at
// distance d from the centre maps to a cell at distance >= d - sqrt(0.5) (rotation keeps d,
// rounding moves each coordinate by <= 0.5), so pixels with d > R + 0.71 see a zero footprint.
int32_t support_radius2(const double* fp, int F) {
  const int wr = (F - 1) / 2;
  double R = -1.0;
  for (int i = 0; i < F; i++)
    for (int j = 0; j < F; j++)
      if (fp[static_cast<size_t>(i) * F + j] > 0.0)
        R = std::max(R, std::sqrt(double((i - wr) * (i - wr) + (j - wr) * (j - wr))));
  if (R < 0.0) return -1;  // an all-zero footprint: every stamp pixel is a no-op
  const double b = R + 0.7072;
  return static_cast<int32_t>(std::floor(b * b)) + 1;
}

// FootprintBrush::setRadius (FootprintBrush.hxx:46-63). The footprint image is resampled to
// width x width by a pixel-centre aligned bilinear resample (in place of OpenCV's
// Lanczos-4 resize) and zero-padded by (sizeMap - width) / 2 on each side.
// The padded footprint of a brush width (cached per width: the resample depends on it only).
const std::pair<std::vector<double>, int32_t>& footprint_for(painty_brush* b, int width) {
  auto it = b->fp_cache.find(width);
  if (it != b->fp_cache.end()) return it->second;
  const int sizeMap = static_cast<int>(std::ceil(std::sqrt(2.0) * width));
  const int pad = (sizeMap - width) / 2;
  const int F = width + 2 * pad;
  std::vector<double> fp(static_cast<size_t>(F) * F, 0.0);
  const double sy = static_cast<double>(b->fh) / width, sx = static_cast<double>(b->fw) / width;
  for (int i = 0; i < width; i++)
    for (int j = 0; j < width; j++)
      fp[static_cast<size_t>(i + pad) * F + (j + pad)] =
        interpolate(b->full.data(), b->fh, b->fw, (static_cast<double>(j) + 0.5) * sx - 0.5,
                    (static_cast<double>(i) + 0.5) * sy - 0.5);
  const int32_t s2 = support_radius2(fp.data(), F);
  return b->fp_cache.emplace(width, std::make_pair(std::move(fp), s2)).first->second;
}

void set_radius(painty_brush* b, double radius) {
  if (std::fabs(b->radius - radius) < 0.5) return;
  b->radius = radius;
  const int width = static_cast<int>(2.0 * std::ceil(radius) + 1.0);
  b->width = width;
  b->sizeMap = static_cast<int>(std::ceil(std::sqrt(2.0) * width));
  const int pad = (b->sizeMap - width) / 2;
  b->F = width + 2 * pad;
  const auto& fp = footprint_for(b, width);
  b->footprint = fp.first;
  b->support2 = fp.second;
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
  static int cached[64] = {0};
  int dev = 0;
  PG_CUDA(cudaGetDevice(&dev));
  if (dev < 64 && cached[dev] > 0) return cached[dev];
  int v = 0;
  PG_CUDA(cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  if (dev < 64) cached[dev] = v;
  return v;
}

// Shared-memory plan for a launch. The small variant keeps the footprint and the owner table
// in shared memory (BIG = false); maps too large for that keep both in global memory. The
// pickup map (7 planes) is staged in shared memory when it fits beside them.
struct SmemPlan {
  bool big, pick;
  StampSmem layout;
};
template <class M>
SmemPlan plan_smem_limit(int F, int S, size_t limit, bool allow_small = true) {
  const bool cand[4][2] = {{false, true}, {false, false}, {true, true}, {true, false}};
  for (const auto& c : cand) {
    const bool big = c[0], pick = c[1];
    if (!big && !allow_small) continue;
    const StampSmem L = stamp_smem_layout<M>(F, S, !big, pick, !big);
    if (L.total <= limit) return SmemPlan{big, pick, L};
  }
  fail(PAINTY_ERR_UNSUPPORTED, "stamp kernel shared memory plan failed");
}

template <class M>
SmemPlan plan_smem(int F, int S, bool allow_small) {
  const size_t limit = static_cast<size_t>(max_dyn_smem()) - sizeof(StampParams) * kParamChunk - 512;
  return plan_smem_limit<M>(F, S, limit, allow_small);
}

template <class TK, class TV>
void launch_stamps(painty_canvas* c, painty_brush* b, const StampRec* d_stamps, int64_t n,
                   bool pickup_zero, cudaStream_t st) {
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
  a.dirty = b->useSnapshot ? static_cast<uint8_t*>(b->d_dirty) : nullptr;
  a.pickup_zero = pickup_zero ? 1 : 0;
  a.status = b->d_status;
  a.support2 = b->support2;
  const SmemPlan plan = plan_smem<M>(b->F, b->sizeMap, true);
  const bool big = plan.big;
  if (big) {
    ensure(&b->d_owner, &b->d_owner_bytes, cells * sizeof(int));
    a.owner_global = static_cast<int*>(b->d_owner);
  }
  a.footprint_smem = big ? 0 : 1;
  a.pickup_smem = plan.pick ? 1 : 0;
  auto kern = plan.pick ? (big ? stamp_kernel<true, true, TK, TV> : stamp_kernel<true, false, TK, TV>)
                        : (big ? stamp_kernel<false, true, TK, TV> : stamp_kernel<false, false, TK, TV>);
  const StampSmem Lk = plan.layout;
  PG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               static_cast<int>(Lk.total)));
  kern<<<1, kStampThreads, Lk.total, st>>>(a);
  count_launch();
  PG_CUDA(cudaGetLastError());
}

// Snapshot buffer for painting canvas c with brush b (FootprintBrush.hxx:280-284: a full copy
// when the sizes differ) and its dirty map: clean after a full copy; all dirty when the canvas
// changed outside this brush's stamps since its last run, or another canvas was painted.
void prepare_snapshot(painty_canvas* c, painty_brush* b, cudaStream_t st) {
  if (!b->useSnapshot) return;
  if (!b->has_snapshot || b->snapshot.rows != c->wet.rows || b->snapshot.cols != c->wet.cols ||
      b->snapshot.storage != c->wet.storage) {
    if (b->has_snapshot) device_free(b->snapshot.base);
    b->has_snapshot = false;
    void* base = device_alloc(layer_bytes(c->wet.rows, c->wet.cols, c->wet.storage));
    layer_layout(b->snapshot, c->wet.rows, c->wet.cols, c->wet.storage, base);
    b->has_snapshot = true;
    PG_CUDA(cudaMemcpyAsync(b->snapshot.base, c->wet.base, c->wet.bytes,
                            cudaMemcpyDeviceToDevice, st));
    ensure(&b->d_dirty, &b->d_dirty_bytes, static_cast<size_t>(c->wet.plane_elems()));
    PG_CUDA(cudaMemsetAsync(b->d_dirty, 0, c->wet.plane_elems(), st));
    b->dirty_canvas = c->id;
    b->dirty_version = c->version;
  }
  if (b->dirty_canvas != c->id || b->dirty_version != c->version) {
    ensure(&b->d_dirty, &b->d_dirty_bytes, static_cast<size_t>(c->wet.plane_elems()));
    PG_CUDA(cudaMemsetAsync(b->d_dirty, 1, c->wet.plane_elems(), st));
  }
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
  // pickup map: cleared by the kernel itself when a dip / new radius is pending
  const size_t pk_bytes = static_cast<size_t>(b->sizeMap) * b->sizeMap * 7 * msz;
  if (b->d_pickup_bytes < pk_bytes) {
    ensure(&b->d_pickup, &b->d_pickup_bytes, pk_bytes);
    b->pickup_clear = true;
  }
  const bool pickup_zero = b->pickup_clear;
  b->pickup_clear = false;
  if (!b->d_status) {
    b->d_status = static_cast<unsigned*>(device_alloc(sizeof(unsigned)));
    PG_CUDA(cudaMemsetAsync(b->d_status, 0, sizeof(unsigned), st));
  }
  prepare_snapshot(c, b, st);
  // stamps
  const size_t sbytes = recs.size() * sizeof(StampRec);
  ensure(&b->d_stamps, &b->d_stamps_bytes, sbytes);
  PG_CUDA(cudaMemcpyAsync(b->d_stamps, recs.data(), sbytes, cudaMemcpyHostToDevice, st));
  const auto* ds = static_cast<const StampRec*>(b->d_stamps);
  const int64_t n = static_cast<int64_t>(recs.size());
  switch (c->wet.storage) {
    case PAINTY_STORAGE_F32: launch_stamps<float, float>(c, b, ds, n, pickup_zero, st); break;
    case PAINTY_STORAGE_F16: launch_stamps<__half, __half>(c, b, ds, n, pickup_zero, st); break;
    case PAINTY_STORAGE_BF16:
      launch_stamps<__nv_bfloat16, __half>(c, b, ds, n, pickup_zero, st);
      break;
    case PAINTY_STORAGE_F64: launch_stamps<double, double>(c, b, ds, n, pickup_zero, st); break;
  }
  // other writers of this canvas must invalidate this brush's snapshot bookkeeping
  c->version++;
  b->dirty_canvas = c->id;
  b->dirty_version = c->version;
  // the stamp records live in a reused buffer: finish before returning
  unsigned status = 0;
  PG_CUDA(cudaMemcpyAsync(&status, b->d_status, sizeof(unsigned), cudaMemcpyDeviceToHost, st));
  PG_CUDA(cudaStreamSynchronize(st));
  if (status != 0) fail(PAINTY_ERR_CUDA, "stamp kernel reported an internal error");
}


// ---------------------------------------------------------------------- batched painting (host)
template <class TK, class TV>
void run_batch_typed(painty_canvas* const* canvases, painty_brush* const* brushes, int32_t nc,
                     const painty_stroke_desc* strokes, int64_t ns, const double* points,
                     int64_t npoints, int64_t* stamps_out, cudaStream_t st) {
  using M = typename MathOf<TK>::type;
  const bool f64 = std::is_same<M, double>::value;
  const size_t msz = sizeof(M);
  // strokes grouped by canvas, in order
  std::vector<std::vector<int64_t>> per(nc);
  for (int64_t i = 0; i < ns; i++) per[strokes[i].canvas].push_back(i);
  // launch shared-memory budget: the opt-in maximum minus the kernel's static shared memory
  cudaFuncAttributes fa{};
  PG_CUDA(cudaFuncGetAttributes(&fa, batch_kernel<TK, TV>));
  const size_t limit = static_cast<size_t>(max_dyn_smem()) - fa.sharedSizeBytes - 256;
  std::vector<BatchStroke> bs;
  bs.reserve(static_cast<size_t>(ns));
  std::vector<M> fptable;
  std::map<std::pair<const painty_brush*, int32_t>, int64_t> fp_off;
  std::vector<double> work(nc, 0.0);
  int32_t smax = 1;
  size_t dyn = 0;
  int64_t total_stamps = 0;
  std::vector<int64_t> first(nc, 0);
  for (int32_t c = 0; c < nc; c++) {
    painty_brush* b = brushes[c];
    first[c] = static_cast<int64_t>(bs.size());
    for (int64_t si : per[c]) {
      const painty_stroke_desc& sk = strokes[si];
      set_radius(b, sk.radius);  // FootprintBrush::setRadius: new footprint only on a 0.5 change
      PG_REQUIRE(b->sizeMap > 0 && b->F > 0, "brush radius gives an empty footprint");
      PG_REQUIRE(static_cast<int64_t>(b->F) * b->F <= int64_t(kMaxPixelsPerThread) * kStampThreads,
                 "brush radius above the supported maximum (footprint side 256)");
      const auto key = std::make_pair(static_cast<const painty_brush*>(b), b->width);
      auto it = fp_off.find(key);
      if (it == fp_off.end()) {
        it = fp_off.emplace(key, static_cast<int64_t>(fptable.size())).first;
        for (double v : b->footprint) fptable.push_back(static_cast<M>(v));
      }
      BatchStroke x{};
      x.first_point = sk.first_point;
      x.npoints = sk.npoints;
      x.F = b->F;
      x.S = b->sizeMap;
      x.wr = (b->F - 1) / 2;
      x.support2 = b->support2;
      x.fp_offset = it->second;
      x.radius = b->radius;
      x.spacing = sk.spacing;
      for (int i = 0; i < 3; i++) {
        x.K[i] = sk.K[i];
        x.Sc[i] = sk.S[i];
      }
      const SmemPlan plan = plan_smem_limit<M>(b->F, b->sizeMap, limit);
      x.plan = (plan.pick ? 1 : 0) | (plan.big ? 2 : 0);
      dyn = std::max(dyn, plan.layout.total);
      smax = std::max(smax, b->sizeMap);
      // stamp count (paintStroke's loop bounds) and a work estimate for the ordering
      const int64_t n = stroke_stamp_count(points + 2 * sk.first_point, sk.npoints, sk.spacing);
      total_stamps += n;
      work[c] += static_cast<double>(n) * (0.4 * b->F * b->F + 4.0 * b->F * (b->radius + 1));
      bs.push_back(x);
      for (int i = 0; i < 3; i++) {  // dip
        b->paintK[i] = sk.K[i];
        b->paintS[i] = sk.S[i];
      }
    }
  }
  if (stamps_out) *stamps_out = total_stamps;
  // canvases, brushes' device state
  std::vector<BatchCanvas<TK, TV>> bc(nc);
  for (int32_t c = 0; c < nc; c++) {
    painty_canvas* cv = canvases[c];
    painty_brush* b = brushes[c];
    const int mode = f64 ? 1 : 0;
    if (b->bound < 0) b->bound = mode;
    PG_REQUIRE(b->bound == mode,
               "a brush paints either F64 canvases or F32/F16/BF16 canvases, not both");
    if (!b->d_status) {
      b->d_status = static_cast<unsigned*>(device_alloc(sizeof(unsigned)));
      PG_CUDA(cudaMemsetAsync(b->d_status, 0, sizeof(unsigned), st));
    }
    const size_t pk_bytes = static_cast<size_t>(b->sizeMap) * b->sizeMap * 7 * msz;
    ensure(&b->d_pickup, &b->d_pickup_bytes, pk_bytes);
    if (!per[c].empty()) prepare_snapshot(cv, b, st);
    BatchCanvas<TK, TV>& x = bc[c];
    for (int i = 0; i < 3; i++) {
      x.cK[i] = static_cast<TK*>(cv->wet.K[i]);
      x.cS[i] = static_cast<TK*>(cv->wet.S[i]);
      const painty_layer& src = b->useSnapshot ? b->snapshot : cv->wet;
      x.sK[i] = static_cast<TK*>(src.K[i]);
      x.sS[i] = static_cast<TK*>(src.S[i]);
    }
    x.cV = static_cast<TV*>(cv->wet.V);
    x.sV = static_cast<TV*>(b->useSnapshot ? b->snapshot.V : cv->wet.V);
    x.dirty = b->useSnapshot ? static_cast<uint8_t*>(b->d_dirty) : nullptr;
    x.rows = cv->wet.rows;
    x.cols = cv->wet.cols;
    x.pitch = cv->wet.pitch;
    x.use_snapshot = b->useSnapshot ? 1 : 0;
    x.nstrokes = static_cast<int32_t>(per[c].size());
    x.first_stroke = first[c];
    x.pickup_rate = b->pickupRate;
    x.deposition_rate = b->depositionRate;
    x.capacity = b->capacity;
    x.brush_pickup = b->d_pickup;
  }
  // heaviest canvases first
  std::vector<int32_t> order(nc);
  for (int32_t c = 0; c < nc; c++) order[c] = c;
  std::stable_sort(order.begin(), order.end(),
                   [&](int32_t a, int32_t b2) { return work[a] > work[b2]; });
  // device copies of the descriptors (stream-ordered, freed after the launch)
  int dev = 0, sms = 0;
  PG_CUDA(cudaGetDevice(&dev));
  PG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const int grid = std::max(1, std::min(sms, nc));
  auto upload = [&](const void* h, size_t bytes) -> void* {
    void* d = nullptr;
    PG_CUDA(cudaMallocAsync(&d, std::max<size_t>(bytes, 16), st));
    if (bytes) PG_CUDA(cudaMemcpyAsync(d, h, bytes, cudaMemcpyHostToDevice, st));
    return d;
  };
  void* d_canvas = upload(bc.data(), bc.size() * sizeof(bc[0]));
  void* d_strokes = upload(bs.data(), bs.size() * sizeof(BatchStroke));
  void* d_points = upload(points, static_cast<size_t>(npoints) * 2 * sizeof(double));
  void* d_fp = upload(fptable.data(), fptable.size() * sizeof(M));
  void* d_order = upload(order.data(), order.size() * sizeof(int32_t));
  const int64_t pstride = static_cast<int64_t>(7) * smax * smax;
  const int64_t ostride = static_cast<int64_t>(smax) * smax;
  void* d_scratch_p = nullptr;
  void* d_scratch_o = nullptr;
  void* d_counter = nullptr;
  PG_CUDA(cudaMallocAsync(&d_scratch_p, grid * pstride * msz, st));
  PG_CUDA(cudaMallocAsync(&d_scratch_o, grid * ostride * sizeof(int), st));
  PG_CUDA(cudaMallocAsync(&d_counter, sizeof(int) + sizeof(unsigned), st));
  PG_CUDA(cudaMemsetAsync(d_counter, 0, sizeof(int) + sizeof(unsigned), st));
  BatchArgs<TK, TV> a{};
  a.canvases = static_cast<const BatchCanvas<TK, TV>*>(d_canvas);
  a.strokes = static_cast<const BatchStroke*>(d_strokes);
  a.points = static_cast<const double*>(d_points);
  a.footprints = static_cast<const M*>(d_fp);
  a.order = static_cast<const int32_t*>(d_order);
  a.ncanvas = nc;
  a.counter = static_cast<int*>(d_counter);
  a.status = reinterpret_cast<unsigned*>(static_cast<int*>(d_counter) + 1);
  a.scratch_pickup = static_cast<M*>(d_scratch_p);
  a.scratch_owner = static_cast<int*>(d_scratch_o);
  a.pickup_stride = pstride;
  a.owner_stride = ostride;
  auto kern = batch_kernel<TK, TV>;
  PG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               static_cast<int>(dyn)));
  kern<<<grid, kStampThreads, dyn, st>>>(a);
  count_launch();
  PG_CUDA(cudaGetLastError());
  unsigned status = 0;
  PG_CUDA(cudaMemcpyAsync(&status, a.status, sizeof(unsigned), cudaMemcpyDeviceToHost, st));
  for (void* d : {d_canvas, d_strokes, d_points, d_fp, d_order, d_scratch_p, d_scratch_o, d_counter})
    PG_CUDA(cudaFreeAsync(d, st));
  PG_CUDA(cudaStreamSynchronize(st));
  for (int32_t c = 0; c < nc; c++) {
    if (per[c].empty()) continue;
    painty_brush* b = brushes[c];
    canvases[c]->version++;
    b->dirty_canvas = canvases[c]->id;
    b->dirty_version = canvases[c]->version;
    b->pickup_clear = false;  // the last stroke's pickup map is in the brush's buffer
  }
  if (status != 0) fail(PAINTY_ERR_CUDA, "batched stamp kernel reported an internal error");
}

}  // namespace

int64_t stroke_stamp_count(const double* p, int32_t npts, double spacing) {
  int64_t n = 0;
  for (int32_t i = 0; i + 1 < npts; i++) {
    const double dx = p[2 * (i + 1)] - p[2 * i], dy = p[2 * (i + 1) + 1] - p[2 * i + 1];
    n += static_cast<int>(std::sqrt(dx * dx + dy * dy) / spacing);
  }
  return n;
}

void paint_batch(painty_canvas* const* canvases, painty_brush* const* brushes, int32_t ncanvas,
                 const painty_stroke_desc* strokes, int64_t nstrokes, const double* points,
                 int64_t npoints, int64_t* stamps_out, cudaStream_t st) {
  PG_REQUIRE(ncanvas > 0 && canvases && brushes, "no canvases");
  PG_REQUIRE(nstrokes >= 0 && (nstrokes == 0 || strokes), "strokes is null");
  PG_REQUIRE(npoints >= 0 && (npoints == 0 || points), "points is null");
  const painty_storage storage = canvases[0] ? canvases[0]->wet.storage : PAINTY_STORAGE_F32;
  for (int32_t c = 0; c < ncanvas; c++) {
    PG_REQUIRE(canvases[c] && brushes[c], "null canvas or brush");
    PG_REQUIRE(canvases[c]->wet.storage == storage, "canvases of one batch share a storage format");
    PG_REQUIRE(static_cast<int64_t>(canvases[c]->wet.rows) * canvases[c]->wet.pitch < (int64_t(1) << 31),
               "canvas too large for the batched kernel");
  }
  {
    std::vector<const void*> seen_c(canvases, canvases + ncanvas), seen_b(brushes, brushes + ncanvas);
    std::sort(seen_c.begin(), seen_c.end());
    std::sort(seen_b.begin(), seen_b.end());
    PG_REQUIRE(std::adjacent_find(seen_c.begin(), seen_c.end()) == seen_c.end() &&
                 std::adjacent_find(seen_b.begin(), seen_b.end()) == seen_b.end(),
               "each canvas of a batch has its own brush");
  }
  for (int64_t i = 0; i < 2 * npoints; i++)
    PG_REQUIRE(std::isfinite(points[i]), "path coordinates must be finite");
  for (int64_t i = 0; i < nstrokes; i++) {
    const painty_stroke_desc& s = strokes[i];
    PG_REQUIRE(s.canvas >= 0 && s.canvas < ncanvas, "stroke canvas index out of range");
    PG_REQUIRE(s.npoints >= 0 && s.npoints <= kMaxPathPoints,
               "stroke paths hold at most 512 points in a batch");
    PG_REQUIRE(s.first_point >= 0 && s.first_point + s.npoints <= npoints,
               "stroke points out of range");
    PG_REQUIRE(std::isfinite(s.radius) && s.radius >= 0.0, "radius must be finite and >= 0");
    PG_REQUIRE(std::isfinite(s.spacing) && s.spacing > 0.0, "spacing must be positive");
  }
  switch (storage) {
    case PAINTY_STORAGE_F32:
      run_batch_typed<float, float>(canvases, brushes, ncanvas, strokes, nstrokes, points, npoints, stamps_out, st);
      break;
    case PAINTY_STORAGE_F16:
      run_batch_typed<__half, __half>(canvases, brushes, ncanvas, strokes, nstrokes, points, npoints, stamps_out, st);
      break;
    case PAINTY_STORAGE_BF16:
      run_batch_typed<__nv_bfloat16, __half>(canvases, brushes, ncanvas, strokes, nstrokes, points, npoints, stamps_out, st);
      break;
    case PAINTY_STORAGE_F64:
      run_batch_typed<double, double>(canvases, brushes, ncanvas, strokes, nstrokes, points, npoints, stamps_out, st);
      break;
  }
}

namespace {

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
    pg::device_free(b->d_dirty);
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
    pg::ensure(&b->d_dirty, &b->d_dirty_bytes, static_cast<size_t>(c->wet.plane_elems()));
    PG_CUDA(cudaMemsetAsync(b->d_dirty, 0, c->wet.plane_elems(), st));
    b->dirty_canvas = c->id;
    b->dirty_version = c->version;
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
    a.dirty = nullptr;  // no dirty map: the whole ring is refreshed, as painty does
    a.pickup_zero = 0;
    a.owner_global = scratch;
    a.status = status;
    const pg::SmemPlan plan = pg::plan_smem<float>(b->footprint_side, b->map_side, false);
    a.pickup_smem = plan.pick ? 1 : 0;
    a.footprint_smem = 0;
    a.support2 = 2 * b->footprint_side * b->footprint_side;  // no cull: every box pixel
    a.footprint = b->footprint;  // global: the owner table is the scratch array
    auto kern = a.pickup_smem ? pg::stamp_kernel<true, true, float, float>
                              : pg::stamp_kernel<false, true, float, float>;
    const pg::StampSmem Lk = pg::stamp_smem_layout<float>(b->footprint_side, b->map_side,
                                                          false, a.pickup_smem != 0, false);
    PG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 static_cast<int>(Lk.total)));
    kern<<<1, pg::kStampThreads, Lk.total, st>>>(a);
    pg::count_launch();
    PG_CUDA(cudaGetLastError());
    unsigned hs = 0;
    PG_CUDA(cudaMemcpyAsync(&hs, status, sizeof(unsigned), cudaMemcpyDeviceToHost, st));
    PG_CUDA(cudaStreamSynchronize(st));
    if (hs != 0) pg::fail(PAINTY_ERR_CUDA, "stamp kernel reported an internal error");
  });
}

painty_status painty_paint_batch(painty_canvas* const* canvases, painty_brush* const* brushes,
                                 int32_t ncanvas, const painty_stroke_desc* strokes, int64_t nstrokes,
                                 const double* points, int64_t npoints, int64_t* stamps_out,
                                 void* stream) {
  return guard([&] {
    pg::paint_batch(canvases, brushes, ncanvas, strokes, nstrokes, points, npoints, stamps_out,
                    pg::as_stream(stream));
  });
}

}  // extern "C"
