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
#include <cstdlib>
#include <cstdio>
#include <map>
#include <tuple>
#include <queue>
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

#ifdef PAINTY_PHASE_TIMERS
constexpr bool kPhaseTimers = true;
#else
constexpr bool kPhaseTimers = false;
#endif
// per phase of the stamp loop: warp cycles summed over warps and stamps (phase-timing build)
__device__ unsigned long long g_phase_cycles[16];

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
  // Packed layers (the PK kernels): pixel records of the canvas and of the pickup source
  void* crec;
  void* srec;
  M* pK[3];  // pickup map in global memory, S*S per plane (the brush's state)
  M* pS[3];
  M* pV;
  M* prec;   // PK kernels: the pickup map as cell records of 8 values (K r,g,b, S r,g,b, V, pad)
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
  // Snapshot-ring state (8 ints in device memory, may be NULL): the box and the grown box of
  // the last stamp this brush applied with a snapshot, read before the first stamp and
  // written after the last. ring_reset overrides it: kRingKeep uses it, kRingUnknown
  // refreshes the whole first ring, kRingClean treats the snapshot as equal to the canvas.
  int* ring;
  int32_t ring_reset;
  // stamps applied to the canvas so far (device counter, may be NULL): seeds the stochastic
  // rounding of 16-bit storage
  unsigned* stamp_count;
  // Box pixels inside the support disc, listed (row-major) in shared memory for the launch,
  // with a per-stamp cell map of the box; 0: no list, every stamp paints in waves
  int32_t ndisc;
  int32_t pickup_zero;    // the map starts cleared (a dip or new radius since the last run)
  int32_t pickup_smem;    // stage the pickup map in shared memory for the launch
  int32_t footprint_smem; // stage the footprint in shared memory
  int* owner_global;      // S*S ints when the owner table does not fit in shared memory
  // 2 F*F ints per CTA of the cluster when the cell maps do not fit in shared memory beside
  // the support-disc list (large stamps); NULL: in shared memory
  int* cellmap_global;
  unsigned* status;
};

constexpr int kParamChunk = 32;               // stamps whose parameters are derived together
constexpr int kParamRing = 2 * kParamChunk;   // parameter slots: the current and the next chunk

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

// blend (FootprintBrush.hxx:331-340) of the K and S triples together (same volumes):
// (va a + vb b) / (va + vb) when va + vb > MinVolume, else a. FP64 divides as the reference;
// FP32 multiplies by the hardware reciprocal (relative error ~1e-7), branch-free.
__device__ __forceinline__ void blend6(double va, const double (&a)[6], double vb,
                                       const double (&b)[6], double (&r)[6]) {
  const double tot = __dadd_rn(va, vb);
  if (tot > 0.001) {
#pragma unroll
    for (int i = 0; i < 6; i++)
      r[i] = __ddiv_rn(__dadd_rn(__dmul_rn(va, a[i]), __dmul_rn(vb, b[i])), tot);
  } else {
#pragma unroll
    for (int i = 0; i < 6; i++) r[i] = a[i];
  }
}
__device__ __forceinline__ void blend6(float va, const float (&a)[6], float vb,
                                       const float (&b)[6], float (&r)[6]) {
  const float tot = va + vb;
  const bool mix = tot > 0.001f;
  const float inv = rcp_approx(tot);
#pragma unroll
  for (int i = 0; i < 6; i++) r[i] = mix ? fmaf(va, a[i], vb * b[i]) * inv : a[i];
}

// Plane p (K r,g,b, S r,g,b, V) of the pickup map in global memory.
template <class TK, class TV, class M>
__device__ __forceinline__ M* pickup_plane(const StampArgs<TK, TV>& a, int p) {
  return p < 3 ? a.pK[p] : (p < 6 ? a.pS[p - 3] : a.pV);
}

// A pickup-map cell record (K r,g,b, S r,g,b, V, pad) as 16-byte words.
template <class M>
union CellRec {
  static constexpr int kWords = 8 * sizeof(M) / 16;
  uint4 w[kWords];
  M v[8];
};

// pickupPaint then depositPaint for one stamp pixel (FootprintBrush.hxx:349-431); fp > 0.
// PS: the pickup map is staged in shared memory at `pbase` (7 planes `cells` apart). CG:
// global loads from L2 only (other CTAs of a cluster write the same planes). snap: the next
// stamp's ring refresh of this pixel, done here -- the snapshot receives the values just stored.
// PK: packed layers (pixel records); otherwise planar planes. Triples are handled as K r,g,b
// then S r,g,b.
template <bool PS, bool CG, bool PK, class TK, class TV, class M>
__device__ __forceinline__ void process_pixel(const StampArgs<TK, TV>& a, M* pbase, int cells,
                                              M fp, int c, int m, uint32_t seed, bool snap) {
  using A = Arith<M>;
  if (!in_bounds(a.status, kBoundsCanvas, c, static_cast<int64_t>(a.rows) * a.pitch) ||
      !in_bounds(a.status, kBoundsCell, m, static_cast<int64_t>(a.S) * a.S))
    return;
  // 16-bit storage rounds its stores stochastically (bits from the canvas's stamp count and
  // the pixel; independent of how stamps are grouped into launches)
  constexpr bool kSR = sizeof(TK) == 2;
  uint32_t h0 = 0, h1 = 0, h2 = 0, h3 = 0;
  if constexpr (kSR) {
    h0 = hash32(seed ^ (static_cast<uint32_t>(c) * 0x9e3779b1u));
    h1 = hash32(h0 + 0x632be5abu);
    h2 = hash32(h1 + 0x632be5abu);
    h3 = hash32(h2 + 0x632be5abu);
  }
  // the pickup cell: planar planes (!PK) or a cell record (PK), in shared (PS) or global memory
  auto cell = [&](int p) -> M& {
    if constexpr (PS) return pbase[p * cells + m];
    else return pickup_plane<TK, TV, M>(a, p)[m];
  };
  CellRec<M> crec_{};
  M* const cell_rec = PK ? (PS ? pbase : a.prec) + static_cast<int64_t>(m) * 8 : nullptr;
  // every load first (one round trip): pickup cell, canvas pixel, snapshot pixel; global
  // loads from L2 (another CTA of a cluster may have written them)
  M vp;
  M pk[6], cn[6], sn[6];
  M vsrc, vcan;
  if constexpr (PK) {
    const uint4* w = reinterpret_cast<const uint4*>(cell_rec);
#pragma unroll
    for (int i = 0; i < CellRec<M>::kWords; i++) {
      if constexpr (PS || !CG) crec_.w[i] = w[i];
      else crec_.w[i] = __ldcg(w + i);
    }
#pragma unroll
    for (int i = 0; i < 6; i++) pk[i] = crec_.v[i];
    vp = crec_.v[6];
  } else {
    auto pick = [&](int p) -> M {
      if constexpr (PS) return pbase[p * cells + m];
      else return ld_sel<CG, M>(pickup_plane<TK, TV, M>(a, p) + m);
    };
    vp = pick(6);
#pragma unroll
    for (int i = 0; i < 6; i++) pk[i] = pick(i);
  }
  if constexpr (PK) {
    const PixRec<TK, TV> cr = load_rec<CG, TK, TV>(a.crec, c);
#pragma unroll
    for (int i = 0; i < 6; i++) cn[i] = ld_elem<M>(&cr.k[i]);
    vcan = ld_elem<M>(&cr.v[6]);
    if (a.use_snapshot) {
      const PixRec<TK, TV> sr = load_rec<CG, TK, TV>(a.srec, c);
#pragma unroll
      for (int i = 0; i < 6; i++) sn[i] = ld_elem<M>(&sr.k[i]);
      vsrc = ld_elem<M>(&sr.v[6]);
    } else {  // the pickup source is the canvas itself
#pragma unroll
      for (int i = 0; i < 6; i++) sn[i] = cn[i];
      vsrc = vcan;
    }
  } else {
#pragma unroll
    for (int i = 0; i < 3; i++) {
      cn[i] = ld_sel<CG, M>(a.cK[i] + c);
      cn[3 + i] = ld_sel<CG, M>(a.cS[i] + c);
    }
    vsrc = ld_sel<CG, M>(a.sV + c);
    vcan = ld_sel<CG, M>(a.cV + c);
    if (a.use_snapshot) {
#pragma unroll
      for (int i = 0; i < 3; i++) {
        sn[i] = ld_sel<CG, M>(a.sK[i] + c);
        sn[3 + i] = ld_sel<CG, M>(a.sS[i] + c);
      }
    } else {  // the pickup source is the canvas itself
#pragma unroll
      for (int i = 0; i < 6; i++) sn[i] = cn[i];
    }
  }
  // pickupPaint
  const M vleave = A::mul(A::mul(a.pickupRate, vsrc), fp);
  if (vleave > M(0.001)) {
    const TV left = to_store_sr<TV>(A::sub(vsrc, vleave), h3 >> 16);
    if constexpr (PK)
      *rec_v<TK, TV>(a.srec, c) = left;
    else
      a.sV[c] = left;
    if (!a.use_snapshot) vcan = ld_elem<M>(&left);  // the stored remainder
    M np[6];
    blend6(vp, pk, vleave, sn, np);
#pragma unroll
    for (int i = 0; i < 6; i++) {
      pk[i] = np[i];
      if constexpr (!PK) cell(i) = np[i];
    }
    vp = A::add(vp, vleave);
  }
  // depositPaint
  const M dfree = A::sub(a.capacity, vp);
  const M vfree = (M(0) < dfree) ? dfree : M(0);  // std::max(0.0, x)
  M paint[6], src[6];
#pragma unroll
  for (int i = 0; i < 3; i++) {
    paint[i] = a.paintK[i];
    paint[3 + i] = a.paintS[i];
  }
  blend6(vp, pk, vfree, paint, src);
  const M pleave = A::mul(A::mul(a.depositionRate, vp), fp);
  if constexpr (PK) {
#pragma unroll
    for (int i = 0; i < 6; i++) crec_.v[i] = pk[i];
    crec_.v[6] = A::sub(vp, pleave);
    uint4* w = reinterpret_cast<uint4*>(cell_rec);
#pragma unroll
    for (int i = 0; i < CellRec<M>::kWords; i++) w[i] = crec_.w[i];
  } else {
    cell(6) = A::sub(vp, pleave);
  }
  const M vb = A::mul(a.capacity, fp);
  M out[6];
  blend6(vb, src, vcan, cn, out);
  const uint32_t rb[7] = {h0, h0 >> 16, h1, h1 >> 16, h2, h2 >> 16, h3};
  if constexpr (PK) {
    PixRec<TK, TV> r;
#pragma unroll
    for (int i = 0; i < PixRec<TK, TV>::kWords; i++) r.w[i] = make_uint4(0u, 0u, 0u, 0u);
#pragma unroll
    for (int i = 0; i < 6; i++) r.k[i] = to_store_sr<TK>(out[i], rb[i]);
    r.v[6] = to_store_sr<TV>(A::add(vb, vcan), rb[6]);
    store_rec<TK, TV>(a.crec, c, r);
    if (snap) store_rec<TK, TV>(a.srec, c, r);
  } else {
#pragma unroll
    for (int i = 0; i < 3; i++) {
      const TK k = to_store_sr<TK>(out[i], rb[i]);
      const TK s = to_store_sr<TK>(out[3 + i], rb[3 + i]);
      a.cK[i][c] = k;
      a.cS[i][c] = s;
      if (snap) {
        a.sK[i][c] = k;
        a.sS[i][c] = s;
      }
    }
    const TV v = to_store_sr<TV>(A::add(vb, vcan), rb[6]);
    a.cV[c] = v;
    if (snap) a.sV[c] = v;
  }
}

struct PixelInfo {
  int xc, yc, mx, my;
  bool live;  // inside canvas and map, and a positive footprint: the pixel changes state
};

// Pickup-map cell of stamp pixel (dc, dr) (offsets from the box centre): the reference's
// round(R(-theta) (dc, dr)) + wr, through map_coord.
__device__ __forceinline__ void map_cell(const StampParams& sp, int dc, int dr, int wr, int* mx,
                                         int* my) {
  const float dcf = static_cast<float>(dc), drf = static_cast<float>(dr);
  const float wrf = static_cast<float>(wr);
  const float fx = fmaf(-drf, sp.sf, dcf * sp.cf) + wrf;  // col*cos - row*sin + wr
  const float fy = fmaf(drf, sp.cf, dcf * sp.sf) + wrf;   // col*sin + row*cos + hr
  *mx = map_coord(fx, dc, sp.c, dr, sp.s, true, wr);
  *my = map_coord(fy, dc, sp.s, dr, sp.c, false, wr);
}

// Stamp pixel (row, col) of the F x F box: canvas pixel, pickup-map cell, footprint height.
template <class TK, class TV, class M>
__device__ __forceinline__ PixelInfo pixel_info(const StampArgs<TK, TV>& a, const StampParams& sp,
                                                const int* xs, const int* ys, const M* fps,
                                                int row, int col, M* fp_out) {
  PixelInfo p;
  p.xc = xs[col];
  p.yc = ys[row];
  map_cell(sp, col - a.wr, row - a.wr, a.wr, &p.mx, &p.my);
  const bool inside = p.yc >= 0 && p.xc >= 0 && p.xc < a.cols && p.yc < a.rows && p.my >= 0 &&
                      p.mx >= 0 && p.mx < a.S && p.my < a.S;
  M fp = M(0);
  if (inside && p.mx < a.F && p.my < a.F &&
      in_bounds(a.status, kBoundsFootprint, p.my * a.F + p.mx, static_cast<int64_t>(a.F) * a.F))
    fp = fps[p.my * a.F + p.mx];
  *fp_out = fp;
  p.live = inside && fp > M(0);
  return p;
}

// pixel_info of a pixel the first wave pass found live, from its cached map cell (the same
// canvas pixel, cell and footprint height; recomputed when there is no cache).
template <class TK, class TV, class M>
__device__ __forceinline__ PixelInfo cached_pixel(const StampArgs<TK, TV>& a,
                                                  const StampParams& sp, const int* xs,
                                                  const int* ys, const M* fps, int row, int col,
                                                  M* fp_out, const int* cache) {
  if (!cache) return pixel_info(a, sp, xs, ys, fps, row, col, fp_out);
  const int code = cache[row * a.F + col];
  PixelInfo p;
  p.xc = xs[col];
  p.yc = ys[row];
  p.mx = code & 0xffff;
  p.my = code >> 16;
  *fp_out = fps[p.my * a.F + p.mx];
  p.live = true;
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

// Dynamic shared memory layout of stamp_kernel (all offsets 16-byte aligned). The per-stamp
// arrays (canvas columns / rows of the box, edge-duplicate flags) have kStampBufs buffers and
// the cell map two: while stamp k is painted, stamp k+1 is classified and stamp k+2 set up.
constexpr int kStampBufs = 3;
struct StampSmem {
  size_t fp, pick, own, xs, ys, done_c, done_r, disc, cellmap, total;
};
template <class M>
__host__ __device__ inline StampSmem stamp_smem_layout(int F, int S, int ndisc, bool fp_smem,
                                                       bool pick_smem, bool own_smem,
                                                       int pick_vals = 8, bool cm_smem = true) {
  StampSmem L{};
  size_t o = 0;
  L.fp = o;
  if (fp_smem) o = align_up(o + size_t(F) * F * sizeof(M), 16);
  L.pick = o;
  if (pick_smem) o = align_up(o + size_t(pick_vals) * S * S * sizeof(M), 16);
  L.own = o;
  if (own_smem) o = align_up(o + size_t(S) * S * sizeof(int), 16);
  L.xs = o;
  o = align_up(o + size_t(kStampBufs) * F * sizeof(int), 16);
  L.ys = o;
  o = align_up(o + size_t(kStampBufs) * F * sizeof(int), 16);
  L.done_c = o;
  o = align_up(o + size_t(kStampBufs) * F * sizeof(uint16_t), 16);
  L.done_r = o;
  o = align_up(o + size_t(kStampBufs) * F * sizeof(uint16_t), 16);
  L.disc = o;
  if (ndisc > 0) o = align_up(o + size_t(ndisc) * sizeof(uint32_t), 16);
  L.cellmap = o;
  if (ndisc > 0 && cm_smem) o = align_up(o + size_t(2) * F * F * sizeof(int), 16);
  L.total = o;
  return L;
}

constexpr int kEpochMax = 32767;  // owner keys: ((kEpochMax - epoch) << 16) | pixel index
// Whether paint_waves' per-thread pixel mask (128 bits: rows per warp x 32-column groups)
// covers an F x F box with `threads` threads (every box up to side 255 with 512 threads).
__host__ __device__ constexpr bool waves_fit(int F, int threads) {
  return ((F + threads / 32 - 1) / (threads / 32)) * ((F + 31) / 32) <= 128;
}
// Clusters take 512-thread CTAs for boxes up to this side: there a stamp's fixed costs
// dominate and half-size CTAs win (plain workload, sides 43-91: 188k -> 198k stamps/s);
// larger boxes are painted faster by 1024 threads (the batch's heaviest canvases, sides up
// to 183, ran at 80k instead of 135k stamps/s on 512-thread CTAs).
constexpr int kMax512Side = 127;

// ---------------------------------------------------------------------- snapshot ring
// painty refreshes the snapshot from the canvas over a ring around every stamp: the box grown
// by the radius, the strict interior of the box excepted (FootprintBrush.hxx:291-318). Only
// part of a ring can differ from the snapshot. A pixel of ring j outside box j-1 that was
// inside grown box j-1 lay in ring j-1 (the grown box minus an interior inside the box), so
// it was refreshed by stamp j-1 and not written since (a stamp writes canvas and snapshot
// only inside its box). Ring j therefore needs copying only where it meets box j-1 or leaves
// grown box j-1; the rest would be a copy of equal values. The two parts are disjoint (box
// j-1 within the canvas lies inside grown box j-1) and are cut into at most 20 rectangles.
constexpr int kRingKeep = 0, kRingUnknown = 1, kRingClean = 2;
constexpr int kRefreshRects = 20;

struct IRect {
  int x0, y0, x1, y1;  // inclusive; empty when x0 > x1 or y0 > y1
};

struct RefreshList {
  int4 rect[kRefreshRects];
  int pre[kRefreshRects + 1];  // prefix sums of the rectangle areas
};

// Static shared state of the stamp loop.
struct StampShared {
  RefreshList rl[2];  // double-buffered with the per-stamp arrays
  int prev[8];        // box, grown box of the stamp before the current parameter chunk
  unsigned seed0;     // the canvas's stamp count at launch
};

__device__ __forceinline__ bool rect_empty(const IRect& r) { return r.x0 > r.x1 || r.y0 > r.y1; }

// Piece i (0 top, 1 bottom, 2 left, 3 right) of X with H cut out; X itself as piece 0 when
// H misses X.
__device__ __forceinline__ IRect rect_piece(const IRect& X, const IRect& H, int i) {
  const IRect none{0, 0, -1, -1};
  if (rect_empty(X)) return none;
  const int hx0 = max(H.x0, X.x0), hx1 = min(H.x1, X.x1);
  const int hy0 = max(H.y0, X.y0), hy1 = min(H.y1, X.y1);
  if (hx0 > hx1 || hy0 > hy1) return i == 0 ? X : none;
  switch (i) {
    case 0: return IRect{X.x0, X.y0, X.x1, hy0 - 1};
    case 1: return IRect{X.x0, hy1 + 1, X.x1, X.y1};
    case 2: return IRect{X.x0, hy0, hx0 - 1, hy1};
    default: return IRect{hx1 + 1, hy0, X.x1, hy1};
  }
}

// Box (canvas pixels a stamp may write) and grown box (clipped) of a stamp as 8 ints.
__device__ __forceinline__ void stamp_rects(const StampParams& sp, int* out) {
  out[0] = sp.tl[0];
  out[1] = sp.tl[1];
  out[2] = sp.br[0];
  out[3] = sp.br[1];
  out[4] = sp.tla[0];
  out[5] = sp.tla[1];
  out[6] = sp.bra[0];
  out[7] = sp.bra[1];
}

// Warp 0: the rectangles of ring pixels to copy for the stamp `sp`, given the previous
// stamp's box and grown box (prev[0..7]).
__device__ __forceinline__ void build_refresh(const StampParams& sp, const int* prev, int lane,
                                              RefreshList* rl) {
  const IRect G{sp.tla[0], sp.tla[1], sp.bra[0], sp.bra[1]};
  const IRect I{sp.tl[0] + 1, sp.tl[1] + 1, sp.br[0] - 1, sp.br[1] - 1};
  const IRect Bp{prev[0], prev[1], prev[2], prev[3]};
  const IRect Gp{prev[4], prev[5], prev[6], prev[7]};
  IRect r{0, 0, -1, -1};
  if (lane < 4) {  // ring pixels inside the previous box
    const IRect X{max(Bp.x0, G.x0), max(Bp.y0, G.y0), min(Bp.x1, G.x1), min(Bp.y1, G.y1)};
    r = rect_piece(X, I, lane);
  } else if (lane < kRefreshRects) {  // ring pixels outside the previous grown box
    const IRect X = rect_piece(G, Gp, (lane - 4) >> 2);
    r = rect_piece(X, I, (lane - 4) & 3);
  }
  const int area = rect_empty(r) ? 0 : (r.x1 - r.x0 + 1) * (r.y1 - r.y0 + 1);
  int incl = area;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const int v = __shfl_up_sync(0xffffffffu, incl, d);
    if (lane >= d) incl += v;
  }
  if (lane < kRefreshRects) {
    rl->rect[lane] = make_int4(r.x0, r.y0, r.x1, r.y1);
    rl->pre[lane + 1] = incl;
  }
  if (lane == 0) rl->pre[0] = 0;
}

// All threads of a CTA: copy its share (of the cluster's 2^lg_csize CTAs) of the listed ring
// pixels canvas -> snapshot (7 planes), two pixels per thread in flight. `rt` is the thread's
// index counted from the CTA's last thread: the copy falls on the high warps, painting on the
// low ones. `skip` (may be NULL): the current stamp's cell map, its box starting at canvas
// (x0, y0); pixels it paints (cell >= 0) are copied by their painter instead, and the rest of
// the list is not touched by the stamp, so the copy runs beside its painting.
template <bool CG, bool PK, class TK, class TV>
__device__ __forceinline__ void refresh_ring(const StampArgs<TK, TV>& a, const RefreshList& rl,
                                             int rt, int T, int crank, int lg_csize,
                                             const int* skip, int x0, int y0) {
  const int all = rl.pre[kRefreshRects];  // < 2^22 pixels: the products below fit 32 bits
  const int first = (all * crank) >> lg_csize;
  const int total = (all * (crank + 1)) >> lg_csize;
  const int F = a.F;
  constexpr int U = 2;
  for (int base = first; base < total; base += U * T) {
    int64_t off[U];
#pragma unroll
    for (int u = 0; u < U; u++) {
      const int idx = base + u * T + rt;
      off[u] = -1;
      if (idx < total) {
        int r = 0;  // the rectangle holding idx: pre[r] <= idx < pre[r + 1] (binary search)
#pragma unroll
        for (int step = 16; step > 0; step >>= 1)
          if (r + step < kRefreshRects && idx >= rl.pre[r + step]) r += step;
        const int4 R = rl.rect[r];
        const int w = R.z - R.x + 1;
        const int local = idx - rl.pre[r];
        // local / w through a float reciprocal (local < 2^22), corrected to the exact quotient
        int dy = static_cast<int>(static_cast<float>(local) * __frcp_rn(static_cast<float>(w)));
        if (dy * w > local) dy--;
        if ((dy + 1) * w <= local) dy++;
        const int y = R.y + dy, x = R.x + local - dy * w;
        bool take = true;
        if (skip) {
          const int bx = x - x0, by = y - y0;
          take = !(bx >= 0 && by >= 0 && bx < F && by < F && skip[by * F + bx] >= 0);
        }
        if (take && in_bounds(a.status, kBoundsCanvas, static_cast<int64_t>(y) * a.pitch + x,
                              static_cast<int64_t>(a.rows) * a.pitch))
          off[u] = static_cast<int64_t>(y) * a.pitch + x;
      }
    }
    if constexpr (PK) {  // whole pixel records
      PixRec<TK, TV> r[U];
#pragma unroll
      for (int u = 0; u < U; u++)
        if (off[u] >= 0) r[u] = load_rec<CG, TK, TV>(a.crec, static_cast<int>(off[u]));
#pragma unroll
      for (int u = 0; u < U; u++)
        if (off[u] >= 0) store_rec<TK, TV>(a.srec, static_cast<int>(off[u]), r[u]);
      continue;
    }
    TK k[U][3], s[U][3];
    TV v[U];
#pragma unroll
    for (int u = 0; u < U; u++) {
      if (off[u] < 0) continue;
#pragma unroll
      for (int ch = 0; ch < 3; ch++) {
        if constexpr (CG) {
          k[u][ch] = __ldcg(a.cK[ch] + off[u]);
          s[u][ch] = __ldcg(a.cS[ch] + off[u]);
        } else {
          k[u][ch] = a.cK[ch][off[u]];
          s[u][ch] = a.cS[ch][off[u]];
        }
      }
      if constexpr (CG)
        v[u] = __ldcg(a.cV + off[u]);
      else
        v[u] = a.cV[off[u]];
    }
#pragma unroll
    for (int u = 0; u < U; u++) {
      if (off[u] < 0) continue;
#pragma unroll
      for (int ch = 0; ch < 3; ch++) {
        a.sK[ch][off[u]] = k[u][ch];
        a.sS[ch][off[u]] = s[u][ch];
      }
      a.sV[off[u]] = v[u];
    }
  }
}

// Stamps of a host-built record list (imprint / painty_stamps / painty_stroke).
struct RecordSource {
  const StampRec* recs;
  int64_t n;
  __device__ __forceinline__ int64_t count() const { return n; }
  __device__ __forceinline__ StampRec get(int64_t k) const { return recs[k]; }
};

// Painting of a stamp without edge duplicates. A stamp pixel changes state only through its
// pickup-map cell (where the footprint is positive) and its canvas pixel. Canvas pixels of
// different stamp pixels differ unless truncation maps two box columns (rows) at the canvas's
// left (top) edge to one (`dup` stamps, painted in waves). Otherwise stamp pixels conflict
// only through cells, and the pixels of one cell lie within sqrt(2) of each other (each lies
// within sqrt(1/2) of the cell's rotated centre: rounding moves a map coordinate by at most
// 1/2), so they are 8-neighbours. Each cell's first pixel in painty's row-major order
// (no earlier neighbour maps to the cell) paints itself and then its later neighbours that
// map to the cell, in row-major order; cells are independent.
//
// Pass 1: cell of every support-disc pixel (packed my << 16 | mx; -1 when the pixel changes
// nothing: outside the canvas or the map, or a zero footprint).
//
// In a cluster whose maps are in shared memory, each CTA classifies its own share of the disc
// [first, last) and stores each entry into every CTA's map: `peers` holds the other CTAs' maps
// for this stamp (shared::cluster addresses), `npeers` of them. The cluster barrier that ends
// the phase makes the stores visible; the maps written here were last read in the phase
// before it.
struct PeerMaps {
  unsigned smem[16];  // shared::cluster addresses of the other CTAs' maps
};
__device__ __forceinline__ unsigned dsmem_map_u32(unsigned local, unsigned rank) {
  unsigned r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(local), "r"(rank));
  return r;
}
__device__ __forceinline__ void dsmem_st(unsigned addr, int v) {
  asm volatile("st.shared::cluster.u32 [%0], %1;" ::"r"(addr), "r"(v) : "memory");
}
template <class TK, class TV, class M>
__device__ __forceinline__ void classify_disc(const StampArgs<TK, TV>& a, const StampParams& sp,
                                              const int* xs, const int* ys, const M* fps,
                                              const uint32_t* disc, int first, int last,
                                              int* cellmap, int rt, int T,
                                              const PeerMaps* peers, int npeers) {
  const int F = a.F;
  for (int i = first + rt; i < last; i += T) {  // rt: counted from the last thread (high warps)
    const uint32_t e = disc[i];
    const int row = static_cast<int>(e >> 16), col = static_cast<int>(e & 0xffffu);
    M fp;
    const PixelInfo p = pixel_info(a, sp, xs, ys, fps, row, col, &fp);
    if (in_bounds(a.status, kBoundsCellMap, row * F + col, static_cast<int64_t>(F) * F)) {
      const int v = p.live ? ((p.my << 16) | p.mx) : -1;
      const int idx = row * F + col;
      cellmap[idx] = v;
      for (int q = 0; q < npeers; q++) dsmem_st(peers->smem[q] + 4u * static_cast<unsigned>(idx), v);
    }
  }
}

// Pass 2: first pixels paint their cell's pixels (this CTA's share of the disc). `nxt`: the
// next stamp's parameters, or NULL for the last stamp -- painted pixels inside the next ring
// are refreshed into the snapshot as they are written (the next refresh would copy exactly
// these values).
template <bool PS, bool CG, bool PK, class TK, class TV, class M>
__device__ __forceinline__ void paint_disc(const StampArgs<TK, TV>& a, const int* xs, const int* ys,
                                        const M* fps, M* pbase, const uint32_t* disc, int first,
                                        int last, const int* cellmap, uint32_t seed, int tid,
                                        int T, const StampParams* nxt) {
  const int F = a.F, S = a.S;
  const int cells = S * S;
  const int pitch32 = static_cast<int>(a.pitch);  // planes hold fewer than 2^31 elements
  const bool snapping = nxt != nullptr && a.use_snapshot;
  // canvas pixel (x, y) lies in the next stamp's ring: its grown box minus the box's interior
  // (this CTA paints disc entries [first, last))
  auto in_ring = [&](int x, int y) -> bool {
    if (!snapping) return false;
    const bool g = x >= nxt->tla[0] && x <= nxt->bra[0] && y >= nxt->tla[1] && y <= nxt->bra[1];
    const bool i = x > nxt->tl[0] && x < nxt->br[0] && y > nxt->tl[1] && y < nxt->br[1];
    return g && !i;
  };
  for (int i = first + tid; i < last; i += T) {
    const uint32_t e = disc[i];
    const int row = static_cast<int>(e >> 16), col = static_cast<int>(e & 0xffffu);
    if (!in_bounds(a.status, kBoundsCellMap, row * F + col, static_cast<int64_t>(F) * F))
      continue;
    const int* cm = cellmap + row * F + col;
    const int m = cm[0];
    if (m < 0) continue;
    const bool l = col > 0, r = col + 1 < F, u = row > 0, d = row + 1 < F;
    if ((l && cm[-1] == m) || (u && cm[-F] == m) || (u && l && cm[-F - 1] == m) ||
        (u && r && cm[-F + 1] == m))
      continue;  // a later pixel of its cell
    // later pixels of the cell, row-major: right, down-left, down, down-right
    unsigned follow = 0;
    if (r && cm[1] == m) follow |= 1u;
    if (d && l && cm[F - 1] == m) follow |= 2u;
    if (d && cm[F] == m) follow |= 4u;
    if (d && r && cm[F + 1] == m) follow |= 8u;
    const int mx = m & 0xffff, my = m >> 16;
    if (!in_bounds(a.status, kBoundsFootprint, my * F + mx, static_cast<int64_t>(F) * F)) continue;
    const M fp = fps[my * F + mx];
    const int cell = my * S + mx;
    process_pixel<PS, CG, PK, TK, TV, M>(a, pbase, cells, fp, ys[row] * pitch32 + xs[col], cell,
                                         seed, in_ring(xs[col], ys[row]));
    for (; follow; follow &= follow - 1) {
      const int q = __ffs(follow) - 1;
      const int rr = row + (q == 0 ? 0 : 1);
      const int cc = col + (q == 0 ? 1 : q - 2);
      process_pixel<PS, CG, PK, TK, TV, M>(a, pbase, cells, fp, ys[rr] * pitch32 + xs[cc],
                                           cell, seed, in_ring(xs[cc], ys[rr]));
    }
  }
}

// Painting of a stamp with edge duplicates, in waves: live pixels bid (atomicMin on
// epoch-tagged row-major indices) for their cells and run when they hold their cell's lowest
// remaining index and their earlier duplicates (done_c / done_r) finished. Called by the
// whole CTA; returns the next epoch. Out of line: rare, and it keeps the cell path's
// registers free.
template <bool PS, bool CG, bool PK, class TK, class TV, class M>
//
// `cache` (F*F ints, or null): where the first pass keeps each live pixel's map cell, so the
// waves after it skip the rotation (the stamp's own cell map, free while it paints in waves).
__device__ __noinline__ int paint_waves(const StampArgs<TK, TV>& a, const StampParams& sp,
                                        const int* xs, const int* ys, uint16_t* done_c,
                                        uint16_t* done_r, const M* fps, M* pbase, int* own,
                                        int epoch, uint32_t seed, int* cache) {
  const int tid = threadIdx.x;
  const int warp = tid >> 5, lane = tid & 31;
  const int F = a.F, S = a.S;
  const int cells = S * S;
  const int NC = (F + 31) / 32;
  const int kWarps = static_cast<int>(blockDim.x) >> 5;
  if (epoch > kEpochMax - 2 * kMaxWaves) {  // owner keys about to wrap: reset the table
    for (int i = tid; i < cells; i += blockDim.x) own[i] = INT_MAX;
    epoch = 0;
    __syncthreads();
  }
  uint64_t rem[2] = {0, 0};  // this thread's pixels still to paint (bit j: slot j)
  int wave = 1;
  int key_hi = (kEpochMax - epoch) << 16;
  epoch++;
  for (int row = warp, jr = 0; row < F; row += kWarps, jr++) {
    const int dr = row - a.wr;
    for (int col = lane, jc = 0; col < F; col += 32, jc++) {
      const int dc = col - a.wr;
      bool lv = false;
      if (dc * dc + dr * dr <= a.support2) {
        M fp;
        const PixelInfo p = pixel_info(a, sp, xs, ys, fps, row, col, &fp);
        if (p.live && in_bounds(a.status, kBoundsOwner, p.my * S + p.mx, cells)) {
          lv = true;
          atomicMin(&own[p.my * S + p.mx], key_hi | (row * F + col));
          if (cache) cache[row * F + col] = (p.my << 16) | p.mx;
        }
      }
      if (lv) {
        const int j = jr * NC + jc;
        rem[j >> 6] |= 1ull << (j & 63);
      } else
        mark_done(xs, ys, F, done_c, done_r, row, col, 1);  // done "before" wave 1
    }
  }
  __syncthreads();
  for (;;) {
    for (int wd = 0; wd < 2; wd++)
    for (uint64_t bits = rem[wd]; bits; bits &= bits - 1) {
      const int j = 64 * wd + __ffsll(static_cast<long long>(bits)) - 1;
      const int row = warp + kWarps * (j / NC), col = lane + 32 * (j % NC);
      M fp;
      const PixelInfo p = cached_pixel(a, sp, xs, ys, fps, row, col, &fp, cache);
      if (own[p.my * S + p.mx] == (key_hi | (row * F + col)) &&
          canvas_ready(xs, ys, F, done_c, done_r, row, col, wave)) {
        process_pixel<PS, CG, PK, TK, TV, M>(a, pbase, cells, fp,
                                             p.yc * static_cast<int>(a.pitch) + p.xc,
                                             p.my * S + p.mx, seed, false);
        rem[wd] &= ~(1ull << (j & 63));
        mark_done(xs, ys, F, done_c, done_r, row, col, static_cast<uint16_t>(wave + 1));
      }
    }
    const int any = __syncthreads_or((rem[0] | rem[1]) != 0);
    if (!any) break;
    if (wave >= kMaxWaves) {  // cannot happen: the lowest remaining pixel always runs
      if (tid == 0) atomicOr(a.status, kStatusWaveCap);
      break;
    }
    wave++;
    key_hi = (kEpochMax - epoch) << 16;
    epoch++;
    for (int wd = 0; wd < 2; wd++)
    for (uint64_t bits = rem[wd]; bits; bits &= bits - 1) {  // bid for the map cell
      const int j = 64 * wd + __ffsll(static_cast<long long>(bits)) - 1;
      const int row = warp + kWarps * (j / NC), col = lane + 32 * (j % NC);
      M fp;
      const PixelInfo p = cached_pixel(a, sp, xs, ys, fps, row, col, &fp, cache);
      atomicMin(&own[p.my * S + p.mx], key_hi | (row * F + col));
    }
    __syncthreads();
  }
  return epoch;
}

// Per-stamp setup of a stamp: canvas columns / rows of the box (double, as the reference),
// duplicate flags reset, the ring rectangles (warp 0) given the previous stamp's box and
// grown box `prev`. Returns whether this thread saw an edge duplicate.
template <class TK, class TV, class Prev>
__device__ __forceinline__ int setup_stamp(const StampArgs<TK, TV>& a, const StampParams& sp,
                                           const Prev& prev_of, int* xs, int* ys,
                                           uint16_t* done_c, uint16_t* done_r, RefreshList* rl,
                                           int rt, int T) {
  const int F = a.F;
  int dup = 0;
  for (int i = rt; i < F; i += T) {  // rt: counted from the last thread (high warps)
    const int x = static_cast<int>(__dadd_rn(static_cast<double>(i - a.wr), sp.cx));
    const int y = static_cast<int>(__dadd_rn(static_cast<double>(i - a.wr), sp.cy));
    xs[i] = x;
    ys[i] = y;
    done_c[i] = 0;
    done_r[i] = 0;
    if (i + 1 < F) {
      const int x1 = static_cast<int>(__dadd_rn(static_cast<double>(i + 1 - a.wr), sp.cx));
      const int y1 = static_cast<int>(__dadd_rn(static_cast<double>(i + 1 - a.wr), sp.cy));
      dup |= (x == x1) | (y == y1);
    }
  }
  if (a.use_snapshot && (rt >> 5) == 0) {  // the last warp
    int prev[8];
    prev_of(prev);
    build_refresh(sp, prev, 31 - (rt & 31), rl);
  }
  return dup;
}

// One stroke's stamps applied in order by the whole CTA -- or by a cluster of CTAs, each
// painting and refreshing its share (the pickup map is then in global memory: PS false, CG
// true). The kernel body shared by the single-canvas and the batched kernels; `a` may live in
// shared or parameter memory.
//
// One barrier per stamp. Phase k paints stamp k (by cells, or in waves when it has edge
// duplicates), refreshes stamp k+1's ring beside it (the pixels stamp k paints are refreshed
// by their painter), classifies stamp k+1's support disc and sets up stamp k+2. After a wave-
// painted stamp the next ring is refreshed in a phase of its own.
template <bool PS, bool BIG, bool CG, bool PK, class TK, class TV, class Src>
__device__ __forceinline__ void run_stroke(const StampArgs<TK, TV>& a, const Src& src,
                                           unsigned char* smem_raw, StampParams* sparams,
                                           StampShared* sh) {
  using M = typename MathOf<TK>::type;
  const int64_t nstamps = src.count();
  const int tid = threadIdx.x;
  const int T = blockDim.x;
  const int lane = tid & 31;
  auto warp_id = [tid]() { return tid >> 5; };
  const int F = a.F, S = a.S;
  const int npix = F * F;
  const int cells = S * S;
  const StampSmem L = stamp_smem_layout<M>(F, S, a.ndisc, !BIG, PS, !BIG, PK ? 8 : 7,
                                           a.cellmap_global == nullptr);
  const M* fps = !BIG ? reinterpret_cast<M*>(smem_raw + L.fp) : a.footprint;
  M* pbase = PS ? reinterpret_cast<M*>(smem_raw + L.pick) : nullptr;
  int* own = BIG ? a.owner_global : reinterpret_cast<int*>(smem_raw + L.own);
  int* xs_b = reinterpret_cast<int*>(smem_raw + L.xs);
  int* ys_b = reinterpret_cast<int*>(smem_raw + L.ys);
  uint16_t* dc_b = reinterpret_cast<uint16_t*>(smem_raw + L.done_c);
  uint16_t* dr_b = reinterpret_cast<uint16_t*>(smem_raw + L.done_r);
  uint32_t* disc = reinterpret_cast<uint32_t*>(smem_raw + L.disc);
  const int ndisc = a.ndisc;
  const int crank = static_cast<int>(cluster_rank()), csize = static_cast<int>(cluster_size());
  // each CTA keeps its own pair of cell maps, as in shared memory
  int* cm_b = a.cellmap_global ? a.cellmap_global + static_cast<int64_t>(crank) * 2 * npix
                               : reinterpret_cast<int*>(smem_raw + L.cellmap);
  auto csync = [csize]() {
    if (csize > 1)
      cluster_barrier();
    else
      __syncthreads();
  };
  if (tid == 0 && (PS || !CG) && csize > 1) atomicOr(a.status, kStatusWaveCap);  // host bug
  // Work split inside the CTA: painting takes disc entries from the first thread up; the ring
  // copy, classification and per-stamp setup count threads from the last one (rt), so they
  // fall on the warps that paint least.
  const int rt = T - 1 - tid;
  const int lg_csize = 31 - __clz(csize);  // cluster sizes are powers of two
  const int ns = static_cast<int>(nstamps);  // < 2^31 stamps per launch (checked by the host)
  const int dfirst = (ndisc * crank) >> lg_csize, dlast = (ndisc * (crank + 1)) >> lg_csize;
  static_assert((kParamRing & (kParamRing - 1)) == 0, "parameter ring size is a power of two");
  auto par = [&](int k) -> StampParams& { return sparams[k & (kParamRing - 1)]; };
  // stamp k's per-stamp arrays sit in slot k mod 3 (columns, rows, duplicate flags) and its
  // cell map and ring list in slot k mod 2
  auto xs_at = [&](int slot) { return xs_b + slot * F; };
  auto ys_at = [&](int slot) { return ys_b + slot * F; };
  auto dc_at = [&](int slot) { return dc_b + slot * F; };
  auto dr_at = [&](int slot) { return dr_b + slot * F; };
  auto cm_of = [&](int k) { return cm_b + (k & 1) * npix; };
  // classification in a cluster: each CTA its share of the disc, stored into every CTA's map
  // through distributed shared memory. Only for maps in shared memory: a map in global memory
  // is read with L1-cached loads, which could return a line from before a peer's store.
  __shared__ PeerMaps peer_maps[2];
  const bool peer_smem = a.cellmap_global == nullptr;
  const int npeers = csize > 1 && peer_smem ? csize - 1 : 0;
  const int cfirst = npeers > 0 ? dfirst : 0, clast = npeers > 0 ? dlast : ndisc;
  auto rl_of = [&](int k) { return &sh->rl[k & 1]; };
  auto next_slot = [](int slot) { return slot == kStampBufs - 1 ? 0 : slot + 1; };
  // rectangles of stamp k - 1 (the brush's ring state before the first stamp)
  auto prev_of = [&](int k, int* out) {
    if (k == 0)
      for (int i = 0; i < 8; i++) out[i] = sh->prev[i];
    else
      stamp_rects(par(k - 1), out);
  };
  // parameters of stamps k0 .. k0 + 31 (one warp in the middle of the CTA)
  const int dtid = tid - (T >> 1);
  auto derive_chunk = [&](int k0) {
    const int j = k0 + dtid;
    if (dtid >= 0 && dtid < kParamChunk && j < ns)
      par(j) = derive_params(src.get(j), a.wr, a.radius, a.rows, a.cols);
  };
  auto setup = [&](int k, int slot) -> int {
    return setup_stamp(a, par(k), [&](int* out) { prev_of(k, out); }, xs_at(slot), ys_at(slot),
                       dc_at(slot), dr_at(slot), rl_of(k), rt, T);
  };

  // launch prologue: footprint and pickup map staged, owner table reset, ring state
  if (!BIG) {
    M* f = reinterpret_cast<M*>(smem_raw + L.fp);
    for (int i = tid; i < npix; i += T) f[i] = a.footprint[i];
  }
  if constexpr (PK) {  // cell records
    for (int i = tid + crank * T; i < 8 * cells; i += T * csize) {
      if (PS)
        pbase[i] = a.pickup_zero ? M(0) : a.prec[i];
      else if (a.pickup_zero)
        a.prec[i] = M(0);
    }
  } else {
    for (int i = tid + crank * T; i < 7 * cells; i += T * csize) {
      const int p = i / cells, m = i - p * cells;
      if (PS)
        pbase[i] = a.pickup_zero ? M(0) : pickup_plane<TK, TV, M>(a, p)[m];
      else if (a.pickup_zero)
        pickup_plane<TK, TV, M>(a, p)[m] = M(0);
    }
  }
  if (!BIG || crank == 0)
    for (int i = tid; i < cells; i += T) own[i] = INT_MAX;
  if (tid < 2 * npeers) {  // the other CTAs' maps, per stamp parity
    const int par_k = tid / npeers, q = tid - par_k * npeers;
    const int rank = q < crank ? q : q + 1;
    const unsigned local = static_cast<unsigned>(__cvta_generic_to_shared(cm_b + par_k * npix));
    peer_maps[par_k].smem[q] = dsmem_map_u32(local, static_cast<unsigned>(rank));
  }
  if (tid == 0) {  // the stamp before the first: from the brush's ring state or the reset mode
    const int big = 1 << 30;
    const int unknown[8] = {0, 0, -1, -1, 0, 0, -1, -1};
    const int clean[8] = {0, 0, -1, -1, -big, -big, big, big};
    for (int i = 0; i < 8; i++)
      sh->prev[i] = (a.ring_reset == kRingKeep && a.ring) ? __ldcg(a.ring + i)
                    : a.ring_reset == kRingClean          ? clean[i]
                                                          : unknown[i];
    sh->seed0 = a.stamp_count ? __ldcg(a.stamp_count) : 0u;
  }
  // support-disc pixels, row-major (warp 0: per-row column intervals, prefix sums), and cell
  // maps whose pixels outside the disc read as "changes nothing"
  if (ndisc > 0) {
    for (int i = tid; i < 2 * npix; i += T) cm_b[i] = -1;
    if (warp_id() == 0) {
      int base = 0;
      for (int r0 = 0; r0 < F; r0 += 32) {
        const int row = r0 + lane;
        int lo = 0, n = 0;
        if (row < F) {
          const int dr = row - a.wr;
          const int rem2 = a.support2 - dr * dr;
          if (rem2 >= 0) {
            int h = static_cast<int>(sqrtf(static_cast<float>(rem2)));
            while ((h + 1) * (h + 1) <= rem2) h++;
            while (h > 0 && h * h > rem2) h--;
            lo = max(a.wr - h, 0);
            n = min(a.wr + h, F - 1) - lo + 1;
          }
        }
        int incl = n;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
          const int v = __shfl_up_sync(0xffffffffu, incl, d);
          if (lane >= d) incl += v;
        }
        const int start = base + incl - n;
        for (int j = 0; j < n && start + j < ndisc; j++)
          disc[start + j] = (static_cast<uint32_t>(row) << 16) | static_cast<uint32_t>(lo + j);
        base += __shfl_sync(0xffffffffu, incl, 31);
      }
      if (lane == 0 && base != ndisc) atomicOr(a.status, kStatusWaveCap);
    }
  }
  derive_chunk(0);
  csync();  // parameters, disc list; a cleared pickup map is visible to the whole cluster
  // stamps 0 and 1 set up, stamp 0's ring refreshed and its disc classified
  int dup0 = 0, dup1 = 0;
  int s0 = 0;  // slot of the stamp being painted (k mod 3)
  if (ns > 0) dup0 = __syncthreads_or(setup(0, 0));
  if (ns > 1) dup1 = __syncthreads_or(setup(1, 1));
  if (ns > 0) {
    if (a.use_snapshot)
      refresh_ring<CG, PK>(a, *rl_of(0), rt, T, crank, lg_csize, nullptr, 0, 0);
    if (!dup0 && ndisc > 0)
      classify_disc(a, par(0), xs_at(0), ys_at(0), fps, disc, cfirst, clast, cm_of(0), rt, T,
                    &peer_maps[0], npeers);
  }
  csync();
  int epoch = 0;
  // phase timers (phase-timing build): each thread's clock between the loop's phase marks
  unsigned long long acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  long long t_mark = kPhaseTimers ? clock64() : 0;
  auto lap = [&](int i) {
    if constexpr (kPhaseTimers) {
      const long long t = clock64();
      acc[i] += static_cast<unsigned long long>(t - t_mark);
      t_mark = t;
    }
  };
  for (int k = 0; k < ns; k++) {
    const StampParams& sp = par(k);
    const bool has_next = k + 1 < ns;
    const int s1 = next_slot(s0), s2 = next_slot(s1);
    const uint32_t seed = hash32(sh->seed0 + static_cast<uint32_t>(k));
    if (!dup0 && ndisc > 0) {
      paint_disc<PS, CG, PK, TK, TV, M>(a, xs_at(s0), ys_at(s0), fps, pbase, disc, dfirst, dlast,
                                        cm_of(k), seed, tid, T,
                                        has_next ? &par(k + 1) : nullptr);
      lap(0);
      if (has_next && a.use_snapshot)
        refresh_ring<CG, PK>(a, *rl_of(k + 1), rt, T, crank, lg_csize, cm_of(k), xs_at(s0)[0],
                             ys_at(s0)[0]);
      lap(1);
    } else {
      if (crank == 0)  // edge duplicates: the first CTA alone, in waves
        epoch = paint_waves<PS, CG, PK, TK, TV, M>(a, sp, xs_at(s0), ys_at(s0), dc_at(s0),
                                                   dr_at(s0), fps, pbase, own, epoch, seed,
                                                   ndisc > 0 ? cm_of(k) : nullptr);
      csync();
      if (has_next && a.use_snapshot)
        refresh_ring<CG, PK>(a, *rl_of(k + 1), rt, T, crank, lg_csize, nullptr, 0, 0);
      lap(7);
    }
    if (has_next && !dup1 && ndisc > 0)
      classify_disc(a, par(k + 1), xs_at(s1), ys_at(s1), fps, disc, cfirst, clast, cm_of(k + 1),
                    rt, T, &peer_maps[(k + 1) & 1], npeers);
    lap(2);
    if (((k + 3) & (kParamChunk - 1)) == 0) derive_chunk(k + 3);  // read from phase k + 1 on
    lap(3);
    int nd = 0;
    if (k + 2 < ns) nd = setup(k + 2, s2);
    lap(4);
    nd = __syncthreads_or(nd);
    lap(5);
    if (csize > 1) cluster_barrier();  // this phase's writes before the next phase's reads
    lap(6);
    dup0 = dup1;
    dup1 = nd;
    s0 = s1;
  }
  if constexpr (kPhaseTimers) {
    if ((tid & 31) == 0) {  // lane 0 stands for its warp
      for (int i = 0; i < 8; i++) atomicAdd(&g_phase_cycles[i], acc[i]);
      if (tid == 0) {
        atomicAdd(&g_phase_cycles[8], static_cast<unsigned long long>(ns));
        atomicAdd(&g_phase_cycles[9], static_cast<unsigned long long>(ns) * (T >> 5));
      }
    }
  }
  // epilogue: the brush keeps its pickup map and the ring state
  if (tid == 0 && crank == 0 && a.stamp_count)
    *a.stamp_count = sh->seed0 + static_cast<unsigned>(ns);
  if (tid == 0 && crank == 0 && a.ring && a.use_snapshot) {
    if (ns > 0)
      stamp_rects(par(ns - 1), a.ring);
    else
      for (int i = 0; i < 8; i++) a.ring[i] = sh->prev[i];
  }
  if (PS) {
    if constexpr (PK) {
      for (int i = tid; i < 8 * cells; i += T) a.prec[i] = pbase[i];
    } else {
      for (int i = tid; i < 7 * cells; i += T) {
        const int p = i / cells, m = i - p * cells;
        pickup_plane<TK, TV, M>(a, p)[m] = pbase[i];
      }
    }
  }
  csync();  // the ring state and pickup map are written before any CTA reads them again
}

// PS: pickup map staged in shared memory. BIG: footprint and owner table in global memory
// (maps too large for shared memory); otherwise both are in shared memory. CG: a cluster
// launch (global loads from L2).
// NT threads per CTA: 1024, or 512 for clusters (each CTA then holds 128 registers per thread;
// measured 188k -> 198k stamps/s on the plain workload).
template <bool PS, bool BIG, bool CG, bool PK, class TK, class TV, int NT = kStampThreads>
__global__ void __launch_bounds__(NT, 1) stamp_kernel(const __grid_constant__ StampArgs<TK, TV> a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ StampParams sparams[kParamRing];
  __shared__ StampShared sh;
  run_stroke<PS, BIG, CG, PK>(a, RecordSource{a.stamps, a.n}, smem_raw, sparams, &sh);
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
  void* crec;          // packed canvas and pickup-source records
  void* srec;
  int* ring;           // the brush's snapshot-ring state
  unsigned* stamp_count;
  int32_t ring_reset;  // for the canvas's first stroke with stamps
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
  int32_t ndisc;  // support-disc list length (0: waves only)
  int32_t plan;  // bit 0: pickup map in shared memory; bit 1: footprint and owners global;
                 // bit 2: cell maps global
  int32_t fp_len;         // elements of the footprint array (F^2)
  const void* footprint;  // the width's padded footprint in the math type, device-resident
  double radius, spacing;
  double K[3], Sc[3];
};

template <class TK, class TV>
struct BatchArgs {
  using M = typename MathOf<TK>::type;
  const BatchCanvas<TK, TV>* canvases;
  const BatchStroke* strokes;
  const double* points;
  const int32_t* order;  // this launch's queue of canvases, heaviest first
  int32_t norder;        // its length
  int32_t ncanvas;       // canvases of the batch (indices in the queue are below it)
  int* counter;
  int* claims;        // per cluster: the canvas it claimed last
  M* scratch_pickup;  // per cluster: Smax^2 cell records
  int* scratch_owner; // per cluster: Smax^2
  int* scratch_cellmap;  // per cluster: CTAs x 2 Fmax^2 (strokes whose cell maps are global)
  int64_t pickup_stride, owner_stride, cellmap_stride;
  unsigned* status;
  // extents of the descriptor arrays and the scratch, for the bounds-checked build
  int64_t nstrokes, npoints;
  int32_t nslots;
  unsigned* status_host;  // device address of pinned host memory for the final status, or null
  unsigned* done_host;    // device address of a pinned completion word, or null
  unsigned done_value;    // written there once everything above is visible to the host
};

// Persistent batched painting: each CTA claims canvases (heaviest first) and applies their
// strokes in order, each as setRadius + dip + paintStroke on the canvas's brush. NT threads
// per CTA, one CTA per SM: 1024 (64 registers per thread), or 512 for clusters (128 registers:
// the stamps a cluster shares run faster on half-size CTAs).
template <class TK, class TV, int NT>
__global__ void __launch_bounds__(NT, 1) batch_kernel(const __grid_constant__ BatchArgs<TK, TV> b) {
  using M = typename MathOf<TK>::type;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ StampParams sparams[kParamRing];
  __shared__ StampShared sh;
  __shared__ StampArgs<TK, TV> sa;
  __shared__ int s_item;
  __shared__ int64_t seg_end[kMaxPathPoints];
  const int tid = threadIdx.x, T = blockDim.x;
  // a cluster (or a lone CTA) paints one canvas at a time; its first CTA claims the canvas
  const int crank = static_cast<int>(cluster_rank()), csize = static_cast<int>(cluster_size());
  const int cid = static_cast<int>(blockIdx.x) / csize;
  for (;;) {
    __syncthreads();
    if (tid == 0 && crank == 0) {
      const int i = atomicAdd(b.counter, 1);
      b.claims[cid] = i < b.norder ? b.order[i] : -1;
    }
    if (csize > 1) cluster_barrier();
    if (tid == 0) s_item = __ldcg(b.claims + cid);
    if (csize > 1)
      cluster_barrier();  // every CTA has the claim before the next one overwrites it
    else
      __syncthreads();
    const int ci = s_item;
    if (ci < 0) break;
    if (!in_bounds(b.status, kBoundsDescriptor, ci, b.ncanvas) ||
        !in_bounds(b.status, kBoundsDescriptor, cid, b.nslots))
      break;
    const BatchCanvas<TK, TV>& cv = b.canvases[ci];
    if (!in_bounds(b.status, kBoundsDescriptor, cv.first_stroke + cv.nstrokes - 1,
                   b.nstrokes + (cv.nstrokes == 0 ? 1 : 0)))
      continue;
    bool ran = false;  // a stroke with stamps has run on this canvas (uniform over the CTA)
    for (int32_t k = 0; k < cv.nstrokes; k++) {
      const BatchStroke& st = b.strokes[cv.first_stroke + k];
      const int nseg = st.npoints - 1;
      if (!in_bounds(b.status, kBoundsDescriptor, st.first_point + st.npoints - 1,
                     b.npoints + (st.npoints == 0 ? 1 : 0)) ||
          !in_bounds(b.status, kBoundsDescriptor, int64_t(st.F) * st.F - 1,
                     st.footprint ? st.fp_len : 0) ||
          !in_bounds(b.status, kBoundsDescriptor, nseg, kMaxPathPoints))
        continue;
      __syncthreads();
      if (tid == 0) {
        const bool last = k + 1 == cv.nstrokes;
        const int64_t cells = static_cast<int64_t>(st.S) * st.S;
        M* pk = last ? static_cast<M*>(cv.brush_pickup)
                     : b.scratch_pickup + static_cast<int64_t>(cid) * b.pickup_stride;
        for (int i = 0; i < 3; i++) {
          sa.cK[i] = cv.cK[i];
          sa.cS[i] = cv.cS[i];
          sa.sK[i] = cv.sK[i];
          sa.sS[i] = cv.sS[i];
          sa.pK[i] = nullptr;
          sa.pS[i] = nullptr;
          sa.paintK[i] = static_cast<M>(st.K[i]);
          sa.paintS[i] = static_cast<M>(st.Sc[i]);
        }
        sa.cV = cv.cV;
        sa.sV = cv.sV;
        sa.crec = cv.crec;
        sa.srec = cv.srec;
        sa.pV = nullptr;
        sa.prec = pk;
        (void)cells;
        sa.footprint = static_cast<const M*>(st.footprint);
        sa.stamps = nullptr;
        sa.n = 0;
        sa.rows = cv.rows;
        sa.cols = cv.cols;
        sa.pitch = cv.pitch;
        sa.F = st.F;
        sa.S = st.S;
        sa.wr = st.wr;
        sa.support2 = st.support2;
        sa.ndisc = st.ndisc;
        sa.radius = st.radius;
        sa.pickupRate = static_cast<M>(cv.pickup_rate);
        sa.depositionRate = static_cast<M>(cv.deposition_rate);
        sa.capacity = static_cast<M>(cv.capacity);
        sa.use_snapshot = cv.use_snapshot;
        sa.ring = cv.ring;
        sa.stamp_count = cv.stamp_count;
        sa.ring_reset = ran ? kRingKeep : cv.ring_reset;
        sa.pickup_zero = 1;  // dip: the pickup map starts clean
        sa.pickup_smem = st.plan & 1;
        sa.footprint_smem = (st.plan & 2) ? 0 : 1;
        sa.owner_global = (st.plan & 2)
                            ? b.scratch_owner + static_cast<int64_t>(cid) * b.owner_stride
                            : nullptr;
        sa.cellmap_global = (st.plan & 4) ? b.scratch_cellmap + static_cast<int64_t>(cid) * b.cellmap_stride
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
      if (n == 0) {  // no stamps: a last stroke still leaves the brush a clean pickup map
        if (k + 1 == cv.nstrokes && crank == 0) {
          const int64_t pc = static_cast<int64_t>(7) * st.S * st.S;
          for (int64_t i = tid; i < pc; i += T) static_cast<M*>(cv.brush_pickup)[i] = M(0);
        }
        continue;
      }
      const PathSource src{pts, st.npoints, st.spacing, seg_end, n};
      if (csize > 1) {  // clusters: the pickup map in global memory, loads from L2
        if (st.plan & 2)
          run_stroke<false, true, true, true>(sa, src, smem_raw, sparams, &sh);
        else
          run_stroke<false, false, true, true>(sa, src, smem_raw, sparams, &sh);
      } else {
        switch (st.plan & 3) {  // bit 2 (global cell maps) travels in sa.cellmap_global
          case 0: run_stroke<false, false, false, true>(sa, src, smem_raw, sparams, &sh); break;
          case 1: run_stroke<true, false, false, true>(sa, src, smem_raw, sparams, &sh); break;
          case 2: run_stroke<false, true, false, true>(sa, src, smem_raw, sparams, &sh); break;
          default: run_stroke<true, true, false, true>(sa, src, smem_raw, sparams, &sh); break;
        }
      }
      ran = true;
    }
  }
  // the last CTA to finish stores the launch's status word into the caller's pinned memory
  // (status_host: its device address), so no copy has to follow the kernel on the stream
  // and then the completion word: a host thread polling it learns the launch is over without
  // anything queued behind the kernel
  if ((b.status_host || b.done_host) && tid == 0) {
    __threadfence_system();  // this CTA's canvas and brush writes
    if (atomicAdd(b.counter + 7, 1) == static_cast<int>(gridDim.x) - 1) {
      __threadfence_system();
      if (b.status_host)
        *reinterpret_cast<volatile unsigned*>(b.status_host) = atomicOr(b.status, 0u);
      __threadfence_system();
      if (b.done_host) *reinterpret_cast<volatile unsigned*>(b.done_host) = b.done_value;
      __threadfence_system();
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

}  // namespace
}  // namespace pg

// The padded footprints of one footprint image, by brush width: (footprint, support2). Brushes
// made from equal images share one family, so a new brush (a server's new canvas) finds the
// resampled footprints already built.
struct FootprintFamily {
  std::mutex mu;
  std::vector<double> image;
  int32_t fh = 0, fw = 0;
  std::map<int32_t, std::pair<std::vector<double>, int32_t>> by_width;
  // device copies of the padded footprints by (device, width, element bytes): uploaded once,
  // then shared by every launch that paints with the width
  std::map<std::tuple<int, int32_t, int>, void*> on_device;
};

namespace pg {
namespace {

std::mutex g_family_mu;
// every family ever made, for the life of the process: a family's device footprints may be
// read by launches still in flight when its last brush is destroyed, and the next brush of
// the same image finds them ready
std::map<uint64_t, std::vector<std::shared_ptr<FootprintFamily>>> g_families;

// The family of a footprint image (FNV-1a of its bytes, then compared value for value).
std::shared_ptr<FootprintFamily> footprint_family(const std::vector<double>& img, int32_t fh,
                                                  int32_t fw) {
  uint64_t h = 1469598103934665603ull;
  auto mix = [&h](const void* p, size_t n) {
    const unsigned char* c = static_cast<const unsigned char*>(p);
    for (size_t i = 0; i < n; i++) h = (h ^ c[i]) * 1099511628211ull;
  };
  mix(&fh, sizeof(fh));
  mix(&fw, sizeof(fw));
  mix(img.data(), img.size() * sizeof(double));
  std::lock_guard<std::mutex> lk(g_family_mu);
  auto& list = g_families[h];
  for (const auto& f : list)
    if (f->fh == fh && f->fw == fw && f->image == img) return f;
  auto f = std::make_shared<FootprintFamily>();
  f->image = img;
  f->fh = fh;
  f->fw = fw;
  list.push_back(f);
  return f;
}

// FootprintBrush::setRadius (FootprintBrush.hxx:46-63). The footprint image is resampled to
// width x width by a pixel-centre aligned bilinear resample (in place of OpenCV's
// Lanczos-4 resize) and zero-padded by (sizeMap - width) / 2 on each side.
// The padded footprint of a brush width (cached per width: the resample depends on it only).
const std::pair<std::vector<double>, int32_t>& footprint_for(painty_brush* b, int width) {
  if (!b->fp_family) b->fp_family = footprint_family(b->full, b->fh, b->fw);
  FootprintFamily& fam = *b->fp_family;
  std::lock_guard<std::mutex> lk(fam.mu);  // entries are never erased: references stay valid
  auto it = fam.by_width.find(width);
  if (it != fam.by_width.end()) return it->second;
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
  return fam.by_width.emplace(width, std::make_pair(std::move(fp), s2)).first->second;
}

// The device copy of a width's padded footprint in the math type M, uploaded on first use
// (synchronously, on a stream of its own) and reused by every later launch on the device.
template <class M>
const M* device_footprint(painty_brush* b, int width) {
  const std::vector<double>& fp = footprint_for(b, width).first;
  FootprintFamily& fam = *b->fp_family;
  int dev = 0;
  PG_CUDA(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lk(fam.mu);
  const auto key = std::make_tuple(dev, static_cast<int32_t>(width), static_cast<int>(sizeof(M)));
  auto it = fam.on_device.find(key);
  if (it != fam.on_device.end()) return static_cast<const M*>(it->second);
  const std::vector<M> h(fp.begin(), fp.end());
  void* d = nullptr;
  PG_CUDA(cudaMalloc(&d, h.size() * sizeof(M)));
  cudaStream_t s = nullptr;
  PG_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
  const cudaError_t e1 = cudaMemcpyAsync(d, h.data(), h.size() * sizeof(M),
                                         cudaMemcpyHostToDevice, s);
  const cudaError_t e2 = cudaStreamSynchronize(s);
  cudaStreamDestroy(s);
  if (e1 != cudaSuccess || e2 != cudaSuccess) {
    cudaFree(d);
    PG_CUDA(e1 != cudaSuccess ? e1 : e2);
  }
  fam.on_device.emplace(key, d);
  return static_cast<const M*>(d);
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

// Device memory of a brush: cudaMalloc / cudaFree, or from its owner's heap.
void* brush_alloc(const painty_brush* b, size_t bytes) {
  return b->heap ? b->heap->alloc(bytes, b->heap_stream) : device_alloc(bytes);
}
void brush_free(const painty_brush* b, void* p) {
  if (b->heap)
    b->heap->free(p, b->heap_stream);
  else
    device_free(p);
}

void ensure(const painty_brush* b, void** p, size_t* cap, size_t bytes) {
  if (*cap >= bytes && *p) return;
  if (*p) brush_free(b, *p);
  *p = nullptr;
  *cap = 0;
  *p = brush_alloc(b, bytes);
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
// The support-disc list and cell map (ndisc > 0) are kept when some variant fits with them.
// cm_global: the cell maps live in global memory (allow_cm_global; the support-disc list stays
// in shared memory), which keeps the disc painting for stamps too large for both.
struct SmemPlan {
  bool big, pick;
  int ndisc;
  StampSmem layout;
  bool cm_global = false;
};
template <class M>
SmemPlan plan_smem_limit(int F, int S, int ndisc, size_t limit, bool allow_small = true,
                         bool allow_pick = true, bool allow_cm_global = false,
                         int pick_vals = 8) {
  const bool cand[4][2] = {{false, true}, {false, false}, {true, true}, {true, false}};
  for (int pass = 0; pass < 3; pass++) {
    // pass 0: the disc list and cell maps in shared memory; 1: the cell maps in global
    // memory; 2: no disc list (every stamp paints in waves)
    const int nd = pass == 2 ? 0 : ndisc;
    const bool cm_smem = pass != 1;
    if (pass == 1 && (!allow_cm_global || ndisc == 0)) continue;
    for (const auto& c : cand) {
      const bool big = c[0], pick = c[1];
      if (!big && !allow_small) continue;
      if (pick && !allow_pick) continue;
      const StampSmem L = stamp_smem_layout<M>(F, S, nd, !big, pick, !big, pick_vals, cm_smem);
      if (L.total <= limit) return SmemPlan{big, pick, nd, L, !cm_smem};
    }
    if (ndisc == 0) break;
  }
  fail(PAINTY_ERR_UNSUPPORTED, "stamp kernel shared memory plan failed");
}

// pick_vals: values per staged pickup cell -- 8 for the packed kernels' cell records, 7 for
// the planar kernel's planes.
template <class M>
SmemPlan plan_smem(int F, int S, int ndisc, bool allow_small, bool allow_pick = true,
                   bool allow_cm_global = false, int pick_vals = 8) {
  const size_t limit = static_cast<size_t>(max_dyn_smem()) - sizeof(StampParams) * kParamRing -
                       sizeof(StampShared) - 512;
  return plan_smem_limit<M>(F, S, ndisc, limit, allow_small, allow_pick, allow_cm_global,
                            pick_vals);
}

// Launch of a stamp-path kernel with `cluster` CTAs per thread-block cluster (1: a plain
// launch).
template <class Arg>
void launch_clustered(void (*kern)(Arg), int grid, int cluster, size_t smem, cudaStream_t st,
                      const Arg& arg, int threads = kStampThreads) {
  if (cluster <= 1) {
    kern<<<grid, threads, smem, st>>>(arg);
    return;
  }
  cudaLaunchConfig_t cfg{};
  cfg.gridDim = dim3(static_cast<unsigned>(grid));
  cfg.blockDim = dim3(static_cast<unsigned>(threads));
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = static_cast<unsigned>(cluster);
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  PG_CUDA(cudaLaunchKernelEx(&cfg, kern, arg));
}

// Clusters of `cluster` stamp CTAs (smem bytes each) that fit on the device at once.
template <class Arg>
int max_clusters(void (*kern)(Arg), int cluster, size_t smem, int threads = kStampThreads) {
  cudaLaunchConfig_t cfg{};
  cfg.gridDim = dim3(static_cast<unsigned>(cluster));
  cfg.blockDim = dim3(static_cast<unsigned>(threads));
  cfg.dynamicSmemBytes = smem;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = static_cast<unsigned>(cluster);
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  int n = 0;
  if (cudaOccupancyMaxActiveClusters(&n, kern, &cfg) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return n;
}

// Cluster size from the environment (PAINTY_STAMP_CLUSTER / PAINTY_BATCH_CLUSTER), 0 if unset.
int env_cluster(const char* name, int max_cluster = 8) {
  const char* v = std::getenv(name);
  if (!v || !*v) return 0;
  const int n = std::atoi(v);
  return (n == 1 || n == 2 || n == 4 || n == 8 || n == 16) && n <= max_cluster ? n : 0;
}

// Box pixels (F x F, centre wr) with dc^2 + dr^2 <= support2: the kernel's support-disc list.
int32_t disc_count(int F, int32_t support2) {
  const int wr = (F - 1) / 2;
  int32_t n = 0;
  for (int r = 0; r < F; r++)
    for (int c = 0; c < F; c++)
      n += (c - wr) * (c - wr) + (r - wr) * (r - wr) <= support2 ? 1 : 0;
  return n;
}

template <class TK, class TV>
void launch_stamps(painty_canvas* c, painty_brush* b, const StampRec* d_stamps, int64_t n,
                   bool pickup_zero, int ring_reset, cudaStream_t st) {
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
  a.crec = c->wet.base;
  a.srec = b->useSnapshot ? b->snapshot.base : c->wet.base;
  const size_t cells = static_cast<size_t>(b->sizeMap) * b->sizeMap;
  a.prec = static_cast<M*>(b->d_pickup);  // cell records
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
  a.ring = b->d_ring();
  a.ring_reset = ring_reset;
  a.stamp_count = b->d_status + 2;
  a.pickup_zero = pickup_zero ? 1 : 0;
  a.status = b->d_status;
  a.support2 = b->support2;
  // one canvas: a cluster of CTAs shares each stamp (the pickup map is then in global memory);
  // a lone CTA stages it in shared memory. Measured on GB300 with 512-thread cluster CTAs
  // (12 strokes across a 1024 x 768 FP32 canvas, stamps/s, clusters 1 / 8 / 16): F = 21
  // 320k / 305k; F = 27 287k / 296k; F = 29 264k / 293k / 292k; F = 39 197k / 288k / 288k;
  // F = 47 155k / 278k / 284k; F = 57 109k / 262k / 273k; F = 87 48k / 180k / 242k. Clusters
  // of 2 or 4 are never the fastest. 16 needs a non-portable cluster, else 8 is used.
  // Clusters run 512-thread CTAs when the stamp's box fits their edge-duplicate masks.
  const int nd = disc_count(b->F, b->support2);
  int cl = env_cluster("PAINTY_STAMP_CLUSTER", 16);
  if (cl == 0) cl = nd >= 1400 ? 16 : nd >= 450 ? 8 : 1;
  SmemPlan plan{};
  void (*kern)(StampArgs<TK, TV>) = nullptr;
  int nt = kStampThreads;
  for (;;) {
    plan = plan_smem<M>(b->F, b->sizeMap, nd, true, cl == 1, true);
    nt = cl > 1 && b->F <= kMax512Side ? 512 : kStampThreads;
    if (cl > 1 && nt == 512)
      kern = plan.big ? stamp_kernel<false, true, true, true, TK, TV, 512>
                      : stamp_kernel<false, false, true, true, TK, TV, 512>;
    else if (cl > 1)
      kern = plan.big ? stamp_kernel<false, true, true, true, TK, TV>
                      : stamp_kernel<false, false, true, true, TK, TV>;
    else
      kern = plan.pick ? (plan.big ? stamp_kernel<true, true, false, true, TK, TV>
                                   : stamp_kernel<true, false, false, true, TK, TV>)
                       : (plan.big ? stamp_kernel<false, true, false, true, TK, TV>
                                   : stamp_kernel<false, false, false, true, TK, TV>);
    PG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 static_cast<int>(plan.layout.total)));
    if (cl > 8 &&
        cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) !=
          cudaSuccess) {
      cudaGetLastError();
      cl = 8;
      continue;
    }
    if (cl == 1 || max_clusters(kern, cl, plan.layout.total, nt) >= 1) break;
    cl /= 2;
  }
  a.ndisc = plan.ndisc;
  if (plan.big) {
    ensure(b, &b->d_owner, &b->d_owner_bytes, cells * sizeof(int));
    a.owner_global = static_cast<int*>(b->d_owner);
  }
  a.cellmap_global = nullptr;
  if (plan.cm_global) {
    ensure(b, &b->d_cellmap, &b->d_cellmap_bytes,
           static_cast<size_t>(cl) * 2 * static_cast<size_t>(b->F) * b->F * sizeof(int));
    a.cellmap_global = static_cast<int*>(b->d_cellmap);
  }
  a.footprint_smem = plan.big ? 0 : 1;
  a.pickup_smem = plan.pick ? 1 : 0;
  const StampSmem Lk = plan.layout;
  launch_clustered(kern, cl, cl, Lk.total, st, a, nt);
  count_launch();
  PG_CUDA(cudaGetLastError());
}

// Snapshot buffer for painting canvas c with brush b (FootprintBrush.hxx:280-284: a full copy
// when the sizes differ) and the ring reset mode of the run: clean after a full copy; unknown
// when the canvas changed outside this brush's snapshot runs since its last one, or another
// canvas was painted; otherwise the device ring state carries over.
int prepare_snapshot(painty_canvas* c, painty_brush* b, cudaStream_t st) {
  if (!b->useSnapshot) return kRingUnknown;
  int mode = kRingKeep;
  if (!b->has_snapshot || b->snapshot.rows != c->wet.rows || b->snapshot.cols != c->wet.cols ||
      b->snapshot.storage != c->wet.storage) {
    if (b->has_snapshot) brush_free(b, b->snapshot.base);
    b->has_snapshot = false;
    void* base = brush_alloc(b, layer_bytes(c->wet.rows, c->wet.cols, c->wet.storage, true));
    layer_layout(b->snapshot, c->wet.rows, c->wet.cols, c->wet.storage, base, true);
    b->has_snapshot = true;
    PG_CUDA(cudaMemcpyAsync(b->snapshot.base, c->wet.base, c->wet.bytes,
                            cudaMemcpyDeviceToDevice, st));
    mode = kRingClean;
  } else if (b->ring_canvas != c->id || b->ring_version != c->version) {
    mode = kRingUnknown;
  } else if (b->ring_pending >= 0) {
    mode = b->ring_pending;
  }
  b->ring_pending = -1;
  return mode;
}

// A stamp launch's status words (0: status bits, 4 and 5: the first out-of-range access of a
// bounds-checked build) as an error.
void check_stamp_status(const unsigned* w, const char* what) {
  if (w[0] == 0) return;
  if (w[0] & kStatusBounds)
    fail(PAINTY_ERR_CUDA, std::string(what) + ": bounds check: access kind " +
                            std::to_string(w[4]) + " at index " +
                            std::to_string(static_cast<int32_t>(w[5])) + " out of range");
  fail(PAINTY_ERR_CUDA, std::string(what) + " reported an internal error");
}

// Device status word and ring state of a brush.
void ensure_status(painty_brush* b, cudaStream_t st) {
  if (b->d_status) return;
  b->d_status = static_cast<unsigned*>(brush_alloc(b, 16 * sizeof(unsigned)));
  PG_CUDA(cudaMemsetAsync(b->d_status, 0, 16 * sizeof(unsigned), st));
  b->ring_canvas = 0;  // the ring state holds nothing yet
}

// Prepares device state and runs n stamps (host records) on the canvas.
void run_stamps(painty_canvas* c, painty_brush* b, const std::vector<StampRec>& recs,
                cudaStream_t st) {
  PG_REQUIRE(c && b, "null handle");
  if (recs.empty()) return;
  PG_REQUIRE(recs.size() < static_cast<size_t>(INT_MAX), "at most 2^31 - 1 stamps per call");
  PG_REQUIRE(b->sizeMap > 0 && b->F > 0, "brush radius gives an empty footprint");
  PG_REQUIRE(static_cast<int64_t>(b->F) * b->F <= int64_t(kMaxPixelsPerThread) * kStampThreads,
             "brush radius above the supported maximum (footprint side 256)");
  PG_REQUIRE(static_cast<int64_t>(c->wet.rows) * c->wet.pitch < (int64_t(1) << 31),
             "canvas too large for stamping (a plane holds 2^31 elements or more)");
  const bool f64 = c->wet.storage == PAINTY_STORAGE_F64;
  const int mode = f64 ? 1 : 0;
  if (b->bound < 0) b->bound = mode;
  PG_REQUIRE(b->bound == mode,
             "a brush paints either F64 canvases or F32/F16/BF16 canvases, not both");
  const size_t msz = f64 ? 8 : 4;
  // footprint
  const size_t fp_bytes = static_cast<size_t>(b->F) * b->F * msz;
  if (b->footprint_stale || b->d_footprint_bytes < fp_bytes) {
    ensure(b, &b->d_footprint, &b->d_footprint_bytes, fp_bytes);
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
  const size_t pk_bytes = static_cast<size_t>(b->sizeMap) * b->sizeMap * 8 * msz;
  if (b->d_pickup_bytes < pk_bytes) {
    ensure(b, &b->d_pickup, &b->d_pickup_bytes, pk_bytes);
    b->pickup_clear = true;
  }
  const bool pickup_zero = b->pickup_clear;
  b->pickup_clear = false;
  ensure_status(b, st);
  const int ring_reset = prepare_snapshot(c, b, st);
  // stamps
  const size_t sbytes = recs.size() * sizeof(StampRec);
  ensure(b, &b->d_stamps, &b->d_stamps_bytes, sbytes);
  PG_CUDA(cudaMemcpyAsync(b->d_stamps, recs.data(), sbytes, cudaMemcpyHostToDevice, st));
  const auto* ds = static_cast<const StampRec*>(b->d_stamps);
  const int64_t n = static_cast<int64_t>(recs.size());
  switch (c->wet.storage) {
    case PAINTY_STORAGE_F32:
      launch_stamps<float, float>(c, b, ds, n, pickup_zero, ring_reset, st);
      break;
    case PAINTY_STORAGE_F16:
      launch_stamps<__half, __half>(c, b, ds, n, pickup_zero, ring_reset, st);
      break;
    case PAINTY_STORAGE_BF16:
      launch_stamps<__nv_bfloat16, __half>(c, b, ds, n, pickup_zero, ring_reset, st);
      break;
    case PAINTY_STORAGE_F64:
      launch_stamps<double, double>(c, b, ds, n, pickup_zero, ring_reset, st);
      break;
  }
  // other writers of this canvas (including this brush without its snapshot) invalidate the
  // ring state
  c->version++;
  if (b->useSnapshot) {
    b->ring_canvas = c->id;
    b->ring_version = c->version;
  }
  // the stamp records live in a reused buffer: finish before returning
  unsigned status[6] = {};
  PG_CUDA(cudaMemcpyAsync(status, b->d_status, sizeof(status), cudaMemcpyDeviceToHost, st));
  PG_CUDA(cudaStreamSynchronize(st));
  check_stamp_status(status, "stamp kernel");
}


// ---------------------------------------------------------------------- batched painting (host)
// Stamp cost model for choosing the cluster size of a batch (GB300, 1024-thread CTAs, SM
// cycles per stamp): kStampFixed + kStampPerPixel * disc / cluster, plus kClusterSync when a
// cluster of CTAs shares each stamp (two cluster barriers and the split's imbalance).
constexpr double kStampFixed = 7000.0;
constexpr double kStampPerPixel = 12.0;
constexpr double kClusterSync = 1500.0;
// 512-thread CTAs in clusters: the stamp time relative to 1024-thread CTAs (measured on the
// plain workload's clusters: 188k -> 198k stamps/s); a lone 512-thread CTA paints at about the
// speed of a 1024-thread one (111k vs 114k)
constexpr double kHalfCluster = 0.95;
constexpr double kHalfSingle = 1.03;

// cluster size, clusters, threads of the batch's main launch; cluster size and clusters of its
// launch for the heaviest canvases (0: none)
thread_local int32_t g_last_batch_shape[5] = {0, 0, 0, 0, 0};

// A side stream of the calling thread (per device) with fork and join events, for a batch's
// second launch.
struct SideStream {
  cudaStream_t st = nullptr;
  cudaEvent_t fork = nullptr, join = nullptr;
};
SideStream& side_stream() {
  thread_local std::map<int, SideStream> by_dev;
  int dev = 0;
  PG_CUDA(cudaGetDevice(&dev));
  SideStream& s = by_dev[dev];
  if (!s.st) {
    PG_CUDA(cudaStreamCreateWithFlags(&s.st, cudaStreamNonBlocking));
    PG_CUDA(cudaEventCreateWithFlags(&s.fork, cudaEventDisableTiming));
    PG_CUDA(cudaEventCreateWithFlags(&s.join, cudaEventDisableTiming));
  }
  return s;
}

// Makespan of painting canvases with loads (stamps N, stamp-pixels P) on `slots` clusters of
// `cl` CTAs, heaviest canvas first onto the least-loaded cluster (the kernel's claim order).
double batch_makespan(const std::vector<double>& N, const std::vector<double>& P,
                      const std::vector<int32_t>& order, int slots, int cl, int threads) {
  if (slots < 1) return 1e300;
  std::priority_queue<double, std::vector<double>, std::greater<double>> q;
  for (int i = 0; i < slots; i++) q.push(0.0);
  double span = 0.0;
  const double scale = threads == 512 ? (cl > 1 ? kHalfCluster : kHalfSingle) : 1.0;
  for (int32_t c : order) {
    const double t =
      scale * (N[c] * (kStampFixed + (cl > 1 ? kClusterSync : 0.0)) + kStampPerPixel * P[c] / cl);
    const double end = q.top() + t;
    q.pop();
    q.push(end);
    span = std::max(span, end);
  }
  return span;
}

// Per-process facts about a batch kernel instance, looked up once: its static shared memory,
// the dynamic shared memory it is allowed (raised as launches need more), and how many
// clusters of each size fit on the device for a given dynamic size.
struct BatchKernelInfo {
  std::mutex mu;
  int threads = kStampThreads;
  size_t static_smem = 0;
  size_t allowed = 0;
  std::map<std::pair<int, size_t>, int> fit;
  template <class K>
  void allow_smem(K kern, size_t bytes) {
    std::lock_guard<std::mutex> lk(mu);
    if (bytes <= allowed) return;
    PG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 static_cast<int>(bytes)));
    allowed = bytes;
  }
  template <class K>
  int fits(K kern, int cluster, size_t bytes) {
    std::lock_guard<std::mutex> lk(mu);
    const auto key = std::make_pair(cluster, bytes);
    auto it = fit.find(key);
    if (it != fit.end()) return it->second;
    const int n = max_clusters(kern, cluster, key.second, threads);
    fit.emplace(key, n);
    return n;
  }
};
template <class TK, class TV, int NT>
BatchKernelInfo& batch_kernel_info() {
  static BatchKernelInfo* info = [] {
    auto* i = new BatchKernelInfo();
    cudaFuncAttributes fa{};
    PG_CUDA(cudaFuncGetAttributes(&fa, batch_kernel<TK, TV, NT>));
    i->static_smem = fa.sharedSizeBytes;
    i->threads = NT;
    return i;
  }();
  return *info;
}


// Thread count from the environment (PAINTY_BATCH_THREADS: 512 or 1024), 0 if unset.
int env_threads(const char* name) {
  const char* v = std::getenv(name);
  if (!v || !*v) return 0;
  const int n = std::atoi(v);
  return n == 512 || n == 1024 ? n : 0;
}

template <class TK, class TV>
void run_batch_typed(painty_canvas* const* canvases, painty_brush* const* brushes, int32_t nc,
                     const painty_stroke_desc* strokes, int64_t ns, const double* points,
                     int64_t npoints, int64_t* stamps_out, cudaStream_t st,
                     const BatchOptions& opt) {
  using M = typename MathOf<TK>::type;
  const bool f64 = std::is_same<M, double>::value;
  const size_t msz = sizeof(M);
  // strokes grouped by canvas, in order
  std::vector<std::vector<int64_t>> per(nc);
  for (int64_t i = 0; i < ns; i++) per[strokes[i].canvas].push_back(i);
  // launch shared-memory budget: the opt-in maximum minus the kernel's static shared memory
  BatchKernelInfo& info1k = batch_kernel_info<TK, TV, 1024>();
  BatchKernelInfo& info512 = batch_kernel_info<TK, TV, 512>();
  // shared-memory budgets: the opt-in maximum less the kernel's static shared memory
  const size_t limit1k = static_cast<size_t>(max_dyn_smem()) - info1k.static_smem - 256;
  const size_t limit512 = static_cast<size_t>(max_dyn_smem()) - info512.static_smem - 256;
  std::vector<BatchStroke> bs;
  bs.reserve(static_cast<size_t>(ns));
  std::vector<double> work(nc, 0.0), loadN(nc, 0.0), loadP(nc, 0.0);
  std::vector<int32_t> disc_of;  // per stroke: support-disc pixels
  disc_of.reserve(static_cast<size_t>(ns));
  std::map<std::pair<int32_t, int32_t>, int32_t> disc_cache;
  int32_t smax = 1;
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
      BatchStroke x{};
      x.first_point = sk.first_point;
      x.npoints = sk.npoints;
      x.F = b->F;
      x.S = b->sizeMap;
      x.wr = (b->F - 1) / 2;
      x.support2 = b->support2;
      x.footprint = device_footprint<M>(b, b->width);
      x.fp_len = b->F * b->F;
      x.radius = b->radius;
      x.spacing = sk.spacing;
      for (int i = 0; i < 3; i++) {
        x.K[i] = sk.K[i];
        x.Sc[i] = sk.S[i];
      }
      const auto dk = std::make_pair(b->F, b->support2);
      auto di = disc_cache.find(dk);
      if (di == disc_cache.end()) di = disc_cache.emplace(dk, disc_count(b->F, b->support2)).first;
      disc_of.push_back(di->second);
      smax = std::max(smax, b->sizeMap);
      // stamp count (paintStroke's loop bounds) and the load estimates
      const int64_t n = stroke_stamp_count(points + 2 * sk.first_point, sk.npoints, sk.spacing);
      PG_REQUIRE(n < INT_MAX, "at most 2^31 - 1 stamps per stroke");
      total_stamps += n;
      loadN[c] += static_cast<double>(n);
      loadP[c] += static_cast<double>(n) * di->second;
      work[c] = loadN[c] * kStampFixed + kStampPerPixel * loadP[c];
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
    ensure_status(b, st);
    const size_t pk_bytes = static_cast<size_t>(b->sizeMap) * b->sizeMap * 8 * msz;
    ensure(b, &b->d_pickup, &b->d_pickup_bytes, pk_bytes);
    const int ring_reset = per[c].empty() ? kRingKeep : prepare_snapshot(cv, b, st);
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
    x.crec = cv->wet.base;
    x.srec = b->useSnapshot ? b->snapshot.base : cv->wet.base;
    x.ring = b->d_ring();
    x.stamp_count = b->d_status + 2;
    x.ring_reset = ring_reset;
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
  auto kern1k = batch_kernel<TK, TV, 1024>;
  auto kern512 = batch_kernel<TK, TV, 512>;
  // distinct stroke shapes (footprint side, map side, support-disc pixels): shared-memory
  // plans are made per shape, and per canvas the shapes it paints
  std::map<std::tuple<int, int, int>, int32_t> shape_id;
  std::vector<std::tuple<int, int, int>> shapes;
  std::vector<int32_t> shape_of(bs.size());
  std::vector<std::vector<int32_t>> canvas_shapes(nc);
  for (int32_t c = 0; c < nc; c++)
    for (size_t k = 0; k < per[c].size(); k++) {
      const size_t i = static_cast<size_t>(first[c]) + k;
      const auto key = std::make_tuple(bs[i].F, bs[i].S, disc_of[i]);
      auto it = shape_id.find(key);
      if (it == shape_id.end()) {
        it = shape_id.emplace(key, static_cast<int32_t>(shapes.size())).first;
        shapes.push_back(key);
      }
      shape_of[i] = it->second;
      auto& cs = canvas_shapes[c];
      if (std::find(cs.begin(), cs.end(), it->second) == cs.end()) cs.push_back(it->second);
    }
  // a shape's plan for a launch of nt-thread CTAs in clusters of cl (nullptr: the shape does
  // not fit 512-thread CTAs); clusters keep the pickup map in global memory
  std::map<std::tuple<int32_t, int, bool>, std::unique_ptr<SmemPlan>> plans;
  const int want_nt = env_threads("PAINTY_BATCH_THREADS") ? env_threads("PAINTY_BATCH_THREADS")
                                                          : opt.threads;
  auto shape_plan = [&](int32_t sid, int nt, int cl) -> const SmemPlan* {
    const auto key = std::make_tuple(sid, nt, cl == 1);
    auto it = plans.find(key);
    if (it != plans.end()) return it->second.get();
    std::unique_ptr<SmemPlan> pl;
    const int F = std::get<0>(shapes[sid]), S = std::get<1>(shapes[sid]);
    const int nd = std::get<2>(shapes[sid]);
    if (nt == 1024) {
      pl = std::make_unique<SmemPlan>(plan_smem_limit<M>(F, S, nd, limit1k, true, cl == 1, true));
    } else if (waves_fit(F, 512) && (want_nt == 512 || F <= kMax512Side) && limit512 > 0) {
      try {
        pl = std::make_unique<SmemPlan>(plan_smem_limit<M>(F, S, nd, limit512, true, cl == 1, true));
      } catch (const Error&) {
      }
    }
    return plans.emplace(key, std::move(pl)).first->second.get();
  };
  // a candidate launch: one persistent kernel over the canvases order[begin, end)
  struct Launch {
    int begin = 0, end = 0, nt = 1024, cl = 1, slots = 0;
    size_t dyn = 0;
    int fmax_cm = 0;  // largest footprint whose cell maps live in global memory
    double span = 1e300;
  };
  auto evaluate = [&](int begin, int end, int nt, int cl, int max_slots) {
    Launch L;
    L.begin = begin;
    L.end = end;
    L.nt = nt;
    L.cl = cl;
    std::vector<char> seen(shapes.size(), 0);
    for (int k = begin; k < end; k++)
      for (int32_t sid : canvas_shapes[order[k]]) {
        if (seen[sid]) continue;
        seen[sid] = 1;
        const SmemPlan* pl = shape_plan(sid, nt, cl);
        if (!pl) return Launch{};
        L.dyn = std::max(L.dyn, pl->layout.total);
        if (pl->cm_global) L.fmax_cm = std::max(L.fmax_cm, std::get<0>(shapes[sid]));
      }
    // in whole KB (fewer distinct occupancy queries), within the budget the plans respect
    const size_t limit = nt == 512 ? limit512 : limit1k;
    L.dyn = std::min((std::max<size_t>(L.dyn, 16) + 1023) / 1024 * 1024,
                     std::max<size_t>(L.dyn, limit));
    int fits = 0;
    if (nt == 512) {
      info512.allow_smem(kern512, L.dyn);
      fits = info512.fits(kern512, cl, L.dyn);
    } else {
      info1k.allow_smem(kern1k, L.dyn);
      fits = info1k.fits(kern1k, cl, L.dyn);
    }
    L.slots = std::min({fits, max_slots, end - begin});
    if (L.slots < 1) return Launch{};
    const std::vector<int32_t> sub(order.begin() + begin, order.begin() + end);
    L.span = batch_makespan(loadN, loadP, sub, L.slots, cl, nt);
    return L;
  };
  // thread count and cluster size: autotuned by the cost model unless PAINTY_BATCH_THREADS /
  // PAINTY_BATCH_CLUSTER (or the caller's options) set them
  const int forced = env_cluster("PAINTY_BATCH_CLUSTER");
  auto best_launch = [&](int begin, int end, int max_slots_1k, int max_slots_512) {
    Launch best;
    for (int c2 : {1, 2, 4, 8}) {
      if (forced ? c2 != forced : c2 > opt.max_cluster) continue;
      // a requested thread count, else 512-thread CTAs for clusters and 1024 for lone CTAs;
      // the other count when the first fits no launch (boxes wider than 512 threads cover)
      const int first = want_nt ? want_nt : (c2 > 1 ? 512 : 1024);
      for (int n2 : {first, first == 512 ? 1024 : 512}) {
        const int ms = n2 == 512 ? max_slots_512 : max_slots_1k;
        const Launch L = evaluate(begin, end, n2, c2, ms == INT_MAX ? ms : ms / c2);
        if (L.slots < 1) continue;
        if (L.span < best.span) best = L;
        break;
      }
    }
    return best;
  };
  const Launch single = best_launch(0, nc, INT_MAX, INT_MAX);
  PG_REQUIRE(single.slots >= 1, "no stamp cluster fits on the device");
  // the heaviest canvases on large clusters (a launch of their own, next to the rest): a
  // canvas's stamps run in order, so the heaviest canvas bounds the batch unless more CTAs
  // share its stamps
  Launch heavy, rest;
  // PAINTY_BATCH_SPLIT="<cluster>:<canvases>" forces the split (tests)
  int force_ch = 0, force_h = 0;
  if (const char* v = std::getenv("PAINTY_BATCH_SPLIT")) {
    if (std::sscanf(v, "%d:%d", &force_ch, &force_h) != 2 ||
        !(force_ch == 2 || force_ch == 4 || force_ch == 8) || force_h < 1 || force_h >= nc)
      force_ch = force_h = 0;
  }
  if (opt.done_host) force_ch = 0;  // one launch signals completion: no split
  if (force_ch) {
    heavy = evaluate(0, force_h, 512, force_ch, force_h);
    if (heavy.slots < force_h) heavy = evaluate(0, force_h, 1024, force_ch, force_h);
    int dev = 0, sms = 0;
    PG_CUDA(cudaGetDevice(&dev));
    PG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const int left = std::max(1, sms - force_h * force_ch);
    rest = best_launch(force_h, nc, left, left);
    PG_REQUIRE(heavy.slots == force_h && rest.slots >= 1, "PAINTY_BATCH_SPLIT does not fit");
  } else if (!forced && !want_nt && !opt.done_host && nc >= 2 && opt.max_cluster >= 4) {
    int dev = 0, sms = 0;
    PG_CUDA(cudaGetDevice(&dev));
    PG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    double best = single.span * 0.97;  // a split must clearly pay for its second launch
    for (int ch : {8, 4}) {
      if (ch > opt.max_cluster) continue;
      for (int h = 1; h < nc && 2 * h * ch <= sms; h++) {
        Launch A = evaluate(0, h, 512, ch, h);  // clusters: 512-thread CTAs where boxes allow
        if (A.slots < h) A = evaluate(0, h, 1024, ch, h);
        if (A.slots < h || A.span >= best) break;
        const int left = sms - h * ch;  // SMs the heavy launch leaves (one 1024-thread CTA each)
        const Launch B = best_launch(h, nc, left, left);
        if (B.slots < 1) continue;
        const double span = std::max(A.span, B.span);
        if (span < best) {
          best = span;
          heavy = A;
          rest = B;
        }
      }
    }
  }
  const bool split = heavy.slots >= 1;
  const Launch& main_l = split ? rest : single;
  g_last_batch_shape[0] = main_l.cl;
  g_last_batch_shape[1] = main_l.slots;
  g_last_batch_shape[2] = main_l.nt;
  g_last_batch_shape[3] = split ? heavy.cl : 0;
  g_last_batch_shape[4] = split ? heavy.slots : 0;
  // the strokes' plans for the launch that paints their canvas
  auto apply = [&](const Launch& L) {
    for (int k = L.begin; k < L.end; k++) {
      const int32_t c = order[k];
      for (size_t j = 0; j < per[c].size(); j++) {
        const size_t i = static_cast<size_t>(first[c]) + j;
        const SmemPlan* pl = shape_plan(shape_of[i], L.nt, L.cl);
        bs[i].ndisc = pl->ndisc;
        bs[i].plan = (pl->pick ? 1 : 0) | (pl->big ? 2 : 0) | (pl->cm_global ? 4 : 0);
      }
    }
  };
  if (split) {
    apply(heavy);
    apply(rest);
  } else {
    apply(single);
  }
  // the descriptors in one device buffer (one allocation, one copy) and the scratch of each
  // launch in another, all stream-ordered and freed after the launches; pieces 256-byte aligned
  std::vector<unsigned char> hdesc;
  auto piece = [&](const void* h, size_t bytes) -> size_t {
    const size_t off = align_up(hdesc.size(), 256);
    hdesc.resize(off + std::max<size_t>(bytes, 16));
    if (bytes) std::memcpy(hdesc.data() + off, h, bytes);
    return off;
  };
  const size_t o_canvas = piece(bc.data(), bc.size() * sizeof(bc[0]));
  const size_t o_strokes = piece(bs.data(), bs.size() * sizeof(BatchStroke));
  const size_t o_points = piece(points, static_cast<size_t>(npoints) * 2 * sizeof(double));
  const size_t o_order = piece(order.data(), order.size() * sizeof(int32_t));
  void* d_desc = nullptr;
  const bool own_desc = !(opt.device_desc && hdesc.size() <= opt.device_desc_bytes);
  d_desc = own_desc ? temp_alloc(hdesc.size(), st) : opt.device_desc;
  if (opt.desc_needed) *opt.desc_needed = hdesc.size();
  const void* hsrc = hdesc.data();
  if (opt.host_staging && hdesc.size() <= opt.host_staging_bytes) {
    std::memcpy(opt.host_staging, hdesc.data(), hdesc.size());
    hsrc = opt.host_staging;
  }
  PG_CUDA(cudaMemcpyAsync(d_desc, hsrc, hdesc.size(), cudaMemcpyHostToDevice, st));
  auto at = [&](size_t off) { return static_cast<void*>(static_cast<char*>(d_desc) + off); };
  const int64_t pstride = static_cast<int64_t>(8) * smax * smax;
  const int64_t ostride = static_cast<int64_t>(smax) * smax;
  // a launch's scratch: counter, status words 1..7 (bounds-check records at status + 4, + 5),
  // claims; then the per-cluster pickup maps, owner tables and cell maps
  struct ScratchLayout {
    size_t pick, own, cm, end;
    int64_t cmstride;
  };
  auto layout_of = [&](const Launch& L) {
    ScratchLayout S{};
    S.cmstride = static_cast<int64_t>(L.cl) * 2 * L.fmax_cm * L.fmax_cm;
    S.pick = align_up(sizeof(int) * (8 + L.slots), 256);
    S.own = align_up(S.pick + L.slots * pstride * msz, 256);
    S.cm = align_up(S.own + L.slots * ostride * sizeof(int), 256);
    S.end = align_up(S.cm + std::max<int64_t>(L.slots * S.cmstride, 4) * sizeof(int), 256);
    return S;
  };
  const Launch& first_l = split ? heavy : single;
  const ScratchLayout S1 = layout_of(first_l);
  const bool own_scratch = !(opt.device_scratch && S1.end <= opt.device_scratch_bytes);
  void* d_scratch = own_scratch ? temp_alloc(S1.end, st) : opt.device_scratch;
  if (opt.scratch_needed) *opt.scratch_needed = S1.end;
  PG_CUDA(cudaMemsetAsync(d_scratch, 0, sizeof(int) * (8 + first_l.slots), st));
  unsigned* d_status = reinterpret_cast<unsigned*>(static_cast<int*>(d_scratch) + 1);
  ScratchLayout S2{};
  void* d_scratch2 = nullptr;
  if (split) {
    S2 = layout_of(rest);
    d_scratch2 = temp_alloc(S2.end, st);
    PG_CUDA(cudaMemsetAsync(d_scratch2, 0, sizeof(int) * (8 + rest.slots), st));
  }
  auto args_for = [&](const Launch& L, void* scratch, const ScratchLayout& SL) {
    auto sat = [&](size_t off) { return static_cast<void*>(static_cast<char*>(scratch) + off); };
    BatchArgs<TK, TV> a{};
    a.canvases = static_cast<const BatchCanvas<TK, TV>*>(at(o_canvas));
    a.strokes = static_cast<const BatchStroke*>(at(o_strokes));
    a.points = static_cast<const double*>(at(o_points));
    a.order = static_cast<const int32_t*>(at(o_order)) + L.begin;
    a.norder = L.end - L.begin;
    a.ncanvas = nc;
    a.counter = static_cast<int*>(scratch);
    a.status = d_status;  // one status word for every launch of the batch
    a.claims = static_cast<int*>(scratch) + 8;
    a.scratch_pickup = static_cast<M*>(sat(SL.pick));
    a.scratch_owner = static_cast<int*>(sat(SL.own));
    a.scratch_cellmap = static_cast<int*>(sat(SL.cm));
    a.cellmap_stride = SL.cmstride;
    a.pickup_stride = pstride;
    a.owner_stride = ostride;
    a.nstrokes = static_cast<int64_t>(bs.size());
    a.npoints = npoints;
    a.nslots = L.slots;
    return a;
  };
  auto launch = [&](const Launch& L, const BatchArgs<TK, TV>& a, cudaStream_t s) {
    if (L.nt == 512)
      launch_clustered(kern512, L.slots * L.cl, L.cl, std::max<size_t>(L.dyn, 16), s, a, 512);
    else
      launch_clustered(kern1k, L.slots * L.cl, L.cl, std::max<size_t>(L.dyn, 16), s, a, 1024);
    count_launch();
    PG_CUDA(cudaGetLastError());
  };
  // a lone launch stores its final status into the caller's pinned memory itself: a copy
  // queued behind the kernel would hold back other streams' work
  unsigned* mapped_status =
    opt.status_host && !split
      ? static_cast<unsigned*>(const_cast<void*>(mapped_host(opt.status_host)))
      : nullptr;
  const bool status_in_kernel = mapped_status != nullptr;
  if (split) {  // the rest on a side stream forked from and joined back into `st`
    SideStream& side = side_stream();
    PG_CUDA(cudaEventRecord(side.fork, st));
    PG_CUDA(cudaStreamWaitEvent(side.st, side.fork, 0));
    launch(heavy, args_for(heavy, d_scratch, S1), st);
    launch(rest, args_for(rest, d_scratch2, S2), side.st);
    PG_CUDA(cudaEventRecord(side.join, side.st));
    PG_CUDA(cudaStreamWaitEvent(st, side.join, 0));
  } else {
    BatchArgs<TK, TV> a = args_for(single, d_scratch, S1);
    a.status_host = mapped_status;
    if (opt.done_host) {
      a.done_host = static_cast<unsigned*>(const_cast<void*>(mapped_host(opt.done_host)));
      PG_REQUIRE(a.done_host != nullptr, "the completion word must be pinned host memory");
      a.done_value = opt.done_value;
    }
    launch(single, a, st);
  }
  unsigned status[6] = {};
  if (!status_in_kernel) {
    PG_CUDA(cudaMemcpyAsync(opt.status_host ? opt.status_host : status, d_status,
                            opt.status_host ? sizeof(unsigned) : sizeof(status),
                            cudaMemcpyDeviceToHost, st));
  }
  if (own_desc) PG_CUDA(cudaFreeAsync(d_desc, st));
  if (own_scratch) PG_CUDA(cudaFreeAsync(d_scratch, st));
  if (d_scratch2) PG_CUDA(cudaFreeAsync(d_scratch2, st));
  if (!opt.status_host) PG_CUDA(cudaStreamSynchronize(st));
  for (int32_t c = 0; c < nc; c++) {
    if (per[c].empty()) continue;
    painty_brush* b = brushes[c];
    canvases[c]->version++;
    if (b->useSnapshot) {
      b->ring_canvas = canvases[c]->id;
      b->ring_version = canvases[c]->version;
    }
    b->pickup_clear = false;  // the last stroke's pickup map is in the brush's buffer
  }
  check_stamp_status(status, "batched stamp kernel");
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
                 int64_t npoints, int64_t* stamps_out, cudaStream_t st,
                 const BatchOptions* options) {
  const BatchOptions opt = options ? *options : BatchOptions{};
  PG_REQUIRE(opt.max_cluster == 1 || opt.max_cluster == 2 || opt.max_cluster == 4 ||
               opt.max_cluster == 8,
             "max_cluster must be 1, 2, 4 or 8");
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
      run_batch_typed<float, float>(canvases, brushes, ncanvas, strokes, nstrokes, points,
                                       npoints, stamps_out, st, opt);
      break;
    case PAINTY_STORAGE_F16:
      run_batch_typed<__half, __half>(canvases, brushes, ncanvas, strokes, nstrokes, points,
                                       npoints, stamps_out, st, opt);
      break;
    case PAINTY_STORAGE_BF16:
      run_batch_typed<__nv_bfloat16, __half>(canvases, brushes, ncanvas, strokes, nstrokes, points,
                                       npoints, stamps_out, st, opt);
      break;
    case PAINTY_STORAGE_F64:
      run_batch_typed<double, double>(canvases, brushes, ncanvas, strokes, nstrokes, points,
                                       npoints, stamps_out, st, opt);
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
// 256^2) followed by one status word. Every GPU that loads this library holds it (about
// 256 KB) until the process exits. All calls share it; calls that overlap on the GPU race.
// The footprint bound (side^2 <= 64 x 1024, side odd: at most 255) caps the map side at 256.
constexpr int kNoAllocMaxMapSide = 256;
constexpr int kNoAllocOwnerCells = kNoAllocMaxMapSide * kNoAllocMaxMapSide;
static __device__ __align__(256) int g_noalloc_scratch[kNoAllocOwnerCells + 64];

namespace pg {
namespace {
constexpr int kNoAllocMaxDevices = 64;
std::mutex g_noalloc_mu;
void* g_noalloc_addr[kNoAllocMaxDevices] = {};
unsigned long long g_noalloc_ctx[kNoAllocMaxDevices] = {};

// Identity of the calling thread's current CUDA context (cuCtxGetId: unique for the life of
// the process), through the runtime's driver entry points so the library needs no libcuda
// link; 0 when unavailable or when no context is current yet. Called under g_noalloc_mu.
unsigned long long current_context_id() {
  using GetCurrent = int (*)(void**);                     // cuCtxGetCurrent(CUcontext*)
  using GetId = int (*)(void*, unsigned long long*);      // cuCtxGetId(CUcontext, id*)
  static GetCurrent get_current = nullptr;
  static GetId get_id = nullptr;
  static bool resolved = false;
  if (!resolved) {
    resolved = true;
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q{};
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) ==
          cudaSuccess && q == cudaDriverEntryPointSuccess)
      get_current = reinterpret_cast<GetCurrent>(f);
    f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) ==
          cudaSuccess && q == cudaDriverEntryPointSuccess)
      get_id = reinterpret_cast<GetId>(f);
    cudaGetLastError();
  }
  if (!get_current || !get_id) return 0;
  void* ctx = nullptr;
  if (get_current(&ctx) != 0 || ctx == nullptr) return 0;
  unsigned long long id = 0;
  return get_id(ctx, &id) == 0 ? id : 0;
}

// Device address of the scratch array on the current device. The host-side symbol is only a
// stand-in, so the address is looked up with that device current: once per device, and again
// when the device's context was re-created since (cudaDeviceReset reloads the module, and the
// array may move).
int* noalloc_scratch() {
  int dev = 0;
  PG_CUDA(cudaGetDevice(&dev));
  PG_REQUIRE(dev >= 0 && dev < kNoAllocMaxDevices, "device ordinal out of range");
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  const unsigned long long ctx = current_context_id();
  if (!g_noalloc_addr[dev] || (ctx != 0 && ctx != g_noalloc_ctx[dev])) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || p == nullptr) {
      cudaGetLastError();
      fail(PAINTY_ERR_CUDA, std::string("cudaGetSymbolAddress(no-alloc scratch): ") +
                              cudaGetErrorString(e));
    }
    g_noalloc_addr[dev] = p;
    g_noalloc_ctx[dev] = current_context_id();  // the lookup made the context current
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
    for (void* d : {b->d_footprint, b->d_pickup, b->d_owner, b->d_cellmap, b->d_stamps,
                    static_cast<void*>(b->d_status)})
      pg::brush_free(b, d);
    if (b->has_snapshot) pg::brush_free(b, b->snapshot.base);
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
      if (b->has_snapshot) pg::brush_free(b, b->snapshot.base);
      b->has_snapshot = false;
      void* base = pg::brush_alloc(b, pg::layer_bytes(c->wet.rows, c->wet.cols, c->wet.storage, true));
      pg::layer_layout(b->snapshot, c->wet.rows, c->wet.cols, c->wet.storage, base, true);
      b->has_snapshot = true;
    }
    PG_CUDA(cudaMemcpyAsync(b->snapshot.base, c->wet.base, c->wet.bytes,
                            cudaMemcpyDeviceToDevice, st));
    b->ring_canvas = c->id;  // snapshot == canvas: the next run refreshes nothing stale
    b->ring_version = c->version;
    b->ring_pending = pg::kRingClean;
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
    char* base = static_cast<char*>(b->d_pickup);  // cell records of 8 values
    if (plane == PAINTY_PLANE_V) {
      const void* p[1] = {base + 6 * msz};
      pg::download_planes(p, 1, dt, S, S, S, host, fmt, pg::as_stream(stream), 8);
    } else {
      PG_REQUIRE(plane == PAINTY_PLANE_K || plane == PAINTY_PLANE_S, "pickup planes are K, S, V");
      const int off = plane == PAINTY_PLANE_K ? 0 : 3;
      const void* p[3] = {base + (off + 0) * msz, base + (off + 1) * msz, base + (off + 2) * msz};
      pg::download_planes(p, 3, dt, S, S, S, host, fmt, pg::as_stream(stream), 8);
    }
    (void)cells;
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
// status word live in g_noalloc_scratch. The first call on a device (and the first after its
// context was re-created) looks up the scratch address; make it before any stream capture.
// Synchronous: returns after the stamps ran.
painty_status painty_stamps_f32_noalloc(const painty_stamp_buffers_f32* b, void* stream) {
  return guard([&] {
    PG_REQUIRE(b != nullptr, "buffers is null");
    PG_REQUIRE(b->n >= 0 && b->n < INT_MAX, "stamp count must lie in [0, 2^31 - 1)");
    PG_REQUIRE(b->rows > 0 && b->cols > 0 && b->pitch >= b->cols, "bad canvas geometry");
    PG_REQUIRE(static_cast<int64_t>(b->rows) * b->pitch < (int64_t(1) << 31),
               "canvas too large for stamping (a plane holds 2^31 elements or more)");
    PG_REQUIRE(b->map_side > 0 && b->map_side <= kNoAllocMaxMapSide,
               "pickup map side above the allocation-free maximum of 256 (radius about 90)");
    PG_REQUIRE(b->footprint_side > 0 && (b->footprint_side & 1) == 1,
               "footprint side must be odd and positive");
    PG_REQUIRE(b->map_side >= b->footprint_side && b->map_side <= b->footprint_side + 1,
               "map side must be the footprint side or one more");
    PG_REQUIRE(static_cast<int64_t>(b->footprint_side) * b->footprint_side <=
                 int64_t(pg::kMaxPixelsPerThread) * pg::kStampThreads,
               "footprint side above 255");
    // the brush values painty_brush_create / set_rates / dip accept
    PG_REQUIRE(std::isfinite(b->radius) && b->radius >= 0.0, "radius must be finite and >= 0");
    PG_REQUIRE(std::isfinite(b->pickup_rate) && std::isfinite(b->deposition_rate) &&
                 std::isfinite(b->capacity),
               "rates and capacity must be finite");
    for (int i = 0; i < 3; i++)
      PG_REQUIRE(std::isfinite(b->paint_K[i]) && std::isfinite(b->paint_S[i]),
                 "paint K and S must be finite");
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
    PG_CUDA(cudaMemsetAsync(status, 0, 8 * sizeof(unsigned), st));
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
    a.ring = nullptr;  // no state kept between calls: the first stamp refreshes its whole ring
    a.stamp_count = nullptr;
    a.ring_reset = pg::kRingUnknown;
    a.pickup_zero = 0;
    a.owner_global = scratch;
    a.status = status;
    a.support2 = 2 * b->footprint_side * b->footprint_side;  // no cull: every box pixel
    // planar pickup map: 7 values per staged cell
    const pg::SmemPlan plan = pg::plan_smem<float>(
        b->footprint_side, b->map_side, pg::disc_count(b->footprint_side, a.support2), false,
        true, false, 7);
    a.ndisc = plan.ndisc;
    a.pickup_smem = plan.pick ? 1 : 0;
    a.footprint_smem = 0;
    a.footprint = b->footprint;  // global: the owner table is the scratch array
    auto kern = a.pickup_smem ? pg::stamp_kernel<true, true, false, false, float, float>
                              : pg::stamp_kernel<false, true, false, false, float, float>;
    const pg::StampSmem Lk = pg::stamp_smem_layout<float>(b->footprint_side, b->map_side, a.ndisc,
                                                          false, a.pickup_smem != 0, false, 7);
    PG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 static_cast<int>(Lk.total)));
    kern<<<1, pg::kStampThreads, Lk.total, st>>>(a);
    pg::count_launch();
    PG_CUDA(cudaGetLastError());
    unsigned hs[6] = {};
    PG_CUDA(cudaMemcpyAsync(hs, status, sizeof(hs), cudaMemcpyDeviceToHost, st));
    PG_CUDA(cudaStreamSynchronize(st));
    pg::check_stamp_status(hs, "stamp kernel");
  });
}

int32_t painty_build_flags(void) {
  return (pg::kBoundsCheck ? PAINTY_BUILD_BOUNDS_CHECK : 0) |
         (pg::kPhaseTimers ? PAINTY_BUILD_PHASE_TIMERS : 0);
}

painty_status painty_take_phase_cycles(uint64_t out[16]) {
  return guard([&] {
    PG_REQUIRE(out != nullptr, "out is null");
    if (!pg::kPhaseTimers)
      pg::fail(PAINTY_ERR_UNSUPPORTED, "not the phase-timing build (PAINTY_PHASE_TIMERS=1)");
    unsigned long long v[16] = {}, zero[16] = {};
    PG_CUDA(cudaDeviceSynchronize());
    PG_CUDA(cudaMemcpyFromSymbol(v, pg::g_phase_cycles, sizeof(v)));
    PG_CUDA(cudaMemcpyToSymbol(pg::g_phase_cycles, zero, sizeof(zero)));
    for (int i = 0; i < 16; i++) out[i] = v[i];
  });
}

painty_status painty_batch_last_split(int32_t* cluster, int32_t* canvases) {
  return guard([&] {
    if (cluster) *cluster = pg::g_last_batch_shape[3];
    if (canvases) *canvases = pg::g_last_batch_shape[4];
  });
}

painty_status painty_batch_last_shape(int32_t* cluster, int32_t* clusters, int32_t* threads) {
  return guard([&] {
    if (cluster) *cluster = pg::g_last_batch_shape[0];
    if (clusters) *clusters = pg::g_last_batch_shape[1];
    if (threads) *threads = pg::g_last_batch_shape[2];
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
