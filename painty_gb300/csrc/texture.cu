// texture.cu -- the texture brush: painty's TextureBrush<vec3> with its Smudge<vec3>
// (painty/renderer/TextureBrush.hxx:20-237, painty/renderer/Smudge.hxx:16-229) on the GPU.
//
// A stroke is three launches:
//  1. thickness: every pixel of the stroke's bounding box finds its texture coordinates by
//     generalized barycentric interpolation over the stroke outline (Math.hxx:72-147), samples
//     the thickness texture bilinearly and records the thickness map and its maximum;
//  2. smudge: one CTA walks the spine in painty's u steps; each step rotates the smudge pickup
//     map to the new heading (bilinear) and exchanges paint between it and the canvas pixels
//     under it (every cell and canvas pixel once per step, so a step is parallel);
//  3. deposit: each painted pixel blends the brush paint in by volume, V = max(Vtex, Vcan).
// The spine, the outline and the per-step rotations are computed on the host with painty's
// double arithmetic (this file's device code is built without fused multiply-adds, so F64
// storage reproduces painty bit for bit). Outline geometry and texture sampling are double in
// every storage mode; the smudge and the deposit run in the storage's math type.
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <type_traits>
#include <vector>

#include "device_common.cuh"
#include "internal.h"

// TextureBrush<vec3>: host copy of the brush and its device buffers.
struct painty_texture_brush {
  std::vector<double> tex;  // thickness texture (th x tw), painty's BrushStrokeSample map
  int32_t th = 0, tw = 0;
  double radius = 0.0;          // TextureBrush.hxx:228
  double thicknessScale = 1.0;  // BrushBase.hxx _thicknessScale
  double paintK[3] = {0.1, 0.1, 0.1}, paintS[3] = {0.1, 0.1, 0.1};  // TextureBrush.hxx:28-30
  bool useSmudge = true;        // TextureBrush.hxx:236
  // Smudge (Smudge.hxx:22-36, 147-158): maps side x side, maxSize made odd
  int32_t side = 0, maxSize = 1;
  double rotation = 0.0;
  bool maps_zero = true;  // the device maps must be cleared before their next use
  int bound = -1;         // -1 unbound, 0 FP32 math, 1 FP64 math
  void* d_tex = nullptr;
  void* d_maps = nullptr;  // two maps of 7 planes of side^2 cells; the first is the state
  size_t d_maps_bytes = 0;
  void make_smudge(int32_t size) {
    side = size;
    maxSize = (size % 2) == 0 ? size + 1 : size;
    rotation = 0.0;
    maps_zero = true;
  }
};

namespace pg {
namespace {

constexpr int kSmudgeThreads = 1024;
constexpr int kTexThreads = 256;

struct D2 {
  double x, y;
};

// ---------------------------------------------------------------------- host geometry
// Spline.hxx:27-73 and SplineEval (:183-231) in painty's operation order
double cr_pos_h(double p_1, double p0, double p1, double p2, double t) {
  constexpr double tau = 0.5;
  const double t2 = t * t, t3 = t2 * t;
  const double b1 = -tau * t + 2.0 * tau * t2 - tau * t3;
  const double b2 = 1.0 + (tau - 3.0) * t2 + (2.0 - tau) * t3;
  const double b3 = tau * t + (3.0 - 2.0 * tau) * t2 + (tau - 2.0) * t3;
  const double b4 = -tau * t2 + tau * t3;
  return p_1 * b1 + p0 * b2 + p1 * b3 + p2 * b4;
}
double cr_der_h(double p_1, double p0, double p1, double p2, double t) {
  constexpr double tau = 0.5;
  const double t2 = t * t;
  const double b1 = tau * (-3.0 * t2 + 4.0 * t - 1.0);
  const double b2 = -t * (-2.0 * tau + 3.0 * (tau - 2.0) * t + 6.0);
  const double b3 = (t - 1.0) * (3.0 * (tau - 2.0) * t - tau);
  const double b4 = tau * t * (3.0 * t - 2.0);
  return p_1 * b1 + p0 * b2 + p1 * b3 + p2 * b4;
}
D2 spline_h(const std::vector<D2>& p, double u, bool deriv) {
  const auto n = static_cast<int64_t>(p.size());
  const double x = static_cast<double>(n - 1) * u;
  const int32_t index = static_cast<int32_t>(x);
  const double t = x - std::floor(x);
  auto at = [&](int32_t i) -> const D2& {
    if (i < 0) return p.front();
    if (i >= static_cast<int32_t>(n)) return p.back();
    return p[static_cast<size_t>(i)];
  };
  const D2 &a = at(index - 1), &b = at(index), &c = at(index + 1), &d = at(index + 2);
  if (deriv) return {cr_der_h(a.x, b.x, c.x, d.x, t), cr_der_h(a.y, b.y, c.y, d.y, t)};
  return {cr_pos_h(a.x, b.x, c.x, d.x, t), cr_pos_h(a.y, b.y, c.y, d.y, t)};
}
D2 normalized_h(const D2& v) {  // Eigen normalized(): v / sqrt(squaredNorm), unchanged at 0
  const double n = v.x * v.x + v.y * v.y;
  if (n > 0.0) {
    const double r = std::sqrt(n);
    return {v.x / r, v.y / r};
  }
  return v;
}
double normalize_angle_h(double a) {  // Smudge.hxx:201-211
  constexpr double PI = 3.14159265358979323846;
  while (a <= -0.5 * PI) a += PI;
  while (a > 0.5 * PI) a -= PI;
  return a;
}

// ---------------------------------------------------------------------- device code
// r, A, D of painty's generalized barycentric coordinates for outline vertex i at (px, py):
// s_i = poly[i] - p, r = |s_i|, A = det(s_i, s_i+1) / 2, D = s_i . s_i+1 (Math.hxx:82-95).
struct BaryTerms {
  double r, A, D;
};
__device__ __forceinline__ BaryTerms bary_terms(const double2* poly, int n, int i, double px,
                                                double py) {
  const double2 pi = poly[i], pj = poly[i + 1 < n ? i + 1 : 0];
  const double sx = pi.x - px, sy = pi.y - py;
  const double tx = pj.x - px, ty = pj.y - py;
  return {sqrt(sx * sx + sy * sy), (sx * ty - tx * sy) / 2.0, sx * tx + sy * ty};
}

// generalizedBarycentricCoordinatesInterpolate (Math.hxx:72-147) of the outline `poly` at
// (px, py) with texture coordinates `uv` (n > 1 vertices, global memory). painty makes two
// passes (r, A, D and the early returns, then the weights); here one pass evaluates each
// vertex's terms once: vertex i's early returns are taken at step i, in painty's order, before
// its weight joins the sums, so the result is painty's to the bit.
__device__ D2 barycentric_uv(const double2* poly, const double2* uv, int n, double px,
                             double py) {
  constexpr double Eps = 2.220446049250313080847e-16 * 100.0;
  const BaryTerms last = bary_terms(poly, n, n - 1, px, py);
  const BaryTerms first = bary_terms(poly, n, 0, px, py);
  double fx = 0.0, fy = 0.0, W = 0.0;
  BaryTerms prv = last, cur = first;  // vertices i-1 and i
  for (int i = 0; i < n; i++) {
    const BaryTerms nxt = i + 1 == n ? first : (i + 1 == n - 1 ? last : bary_terms(poly, n, i + 1, px, py));
    // early returns (painty's first pass): on vertex i, or on its edge to vertex i+1, whose
    // |s_i+1| is nxt.r
    if (fabs(cur.r - 0.0) < Eps) return {uv[i].x, uv[i].y};
    if (fabs(cur.A - 0.0) < Eps && cur.D < 0.0) {
      const double2 fi1 = uv[i + 1 < n ? i + 1 : 0];
      const double k = 1.0 / (cur.r + nxt.r);
      return {(nxt.r * uv[i].x + cur.r * fi1.x) * k, (nxt.r * uv[i].y + cur.r * fi1.y) * k};
    }
    // the weight (painty's second pass)
    double w = 0.0;
    if (prv.A != 0.0) w = w + (prv.r - prv.D / cur.r) / prv.A;
    if (cur.A != 0.0) w = w + (nxt.r - cur.D / cur.r) / cur.A;
    fx = fx + w * uv[i].x;
    fy = fy + w * uv[i].y;
    W = W + w;
    prv = cur;
    cur = nxt;
  }
  if (!(fabs(W - 0.0) < Eps)) {
    const double k = 1.0 / W;
    return {fx * k, fy * k};
  }
  return {uv[0].x, uv[0].y};
}

__device__ __forceinline__ int reflect_d(int p, int len) {  // OpenCV BORDER_REFLECT
  if (len == 1) return 0;
  for (int guard = 0; (p < 0 || p >= len) && guard < 64; guard++) p = p < 0 ? -p - 1 : len - 1 - (p - len);
  return min(max(p, 0), len - 1);
}

// Mat.hxx:68-103: bilinear sample with BORDER_REFLECT (double)
__device__ double interp_d(const double* img, int rows, int cols, double px, double py) {
  const int x = static_cast<int>(floor(px)), y = static_cast<int>(floor(py));
  const int x0 = reflect_d(x, cols), x1 = reflect_d(x + 1, cols);
  const int y0 = reflect_d(y, rows), y1 = reflect_d(y + 1, rows);
  const double a = px - static_cast<double>(x), c = py - static_cast<double>(y);
  return (img[y0 * cols + x0] * (1.0 - a) + img[y0 * cols + x1] * a) * (1.0 - c) +
         (img[y1 * cols + x0] * (1.0 - a) + img[y1 * cols + x1] * a) * c;
}

struct TexArgs {
  const double2* poly;
  const double2* uv;
  int npoly;
  const double* tex;
  int th, tw;
  double scale;
  int x0, y0, nx, ny;     // the bounding-box loop (painty's int(boundMin) .. int(boundMax))
  int bx, by;             // int(boundMin): thickness-map origin
  int trows, tcols;       // thickness-map size
  int rows, cols;         // canvas
};

// Launch 1: thickness map (math type M), its maximum (non-negative values compare as their
// bit patterns) and the number of painted pixels; stats = {max bits, count}.
template <class M>
__global__ void __launch_bounds__(kTexThreads) tb_thickness_kernel(const TexArgs a, M* tmap,
                                                                   unsigned long long* stats) {
  using Bits = typename std::conditional<sizeof(M) == 8, unsigned long long, unsigned>::type;
  const int64_t n = static_cast<int64_t>(a.nx) * a.ny;
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  Bits vmax = 0;
  unsigned count = 0;
  // every thread runs the same trip count, so the warp reductions below see all lanes
  for (int64_t base = static_cast<int64_t>(blockIdx.x) * blockDim.x; base < n; base += stride) {
    const int64_t i = base + threadIdx.x;
    if (i >= n) continue;
    const int y = a.y0 + static_cast<int>(i / a.nx), x = a.x0 + static_cast<int>(i % a.nx);
    if (x < 0 || x >= a.cols || y < 0 || y >= a.rows) continue;
    D2 tp = barycentric_uv(a.poly, a.uv, a.npoly, static_cast<double>(x), static_cast<double>(y));
    if (tp.x < 0.0 || tp.x > 1.0 || tp.y < 0.0 || tp.y > 1.0) continue;
    tp.x *= a.tw;
    tp.y *= a.th;
    const double vtex = a.scale * interp_d(a.tex, a.th, a.tw, tp.x, tp.y);
    if (!(vtex > 0.0)) continue;
    const int s = x - a.bx, t = y - a.by;
    if (s < 0 || t < 0 || s >= a.tcols || t >= a.trows) continue;
    const M v = static_cast<M>(vtex);
    if (!(v > M(0))) continue;
    tmap[static_cast<int64_t>(t) * a.tcols + s] = v;
    Bits vb;
    if constexpr (sizeof(M) == 8) vb = static_cast<Bits>(__double_as_longlong(v));
    else vb = __float_as_uint(v);
    vmax = vb > vmax ? vb : vmax;
    count++;
  }
  for (int o = 16; o > 0; o >>= 1) {
    const Bits ov = __shfl_xor_sync(0xffffffffu, vmax, o);
    vmax = ov > vmax ? ov : vmax;
    count += __shfl_xor_sync(0xffffffffu, count, o);
  }
  if ((threadIdx.x & 31) == 0 && count > 0) {
    if constexpr (sizeof(M) == 8) atomicMax(stats, vmax);
    else atomicMax(reinterpret_cast<unsigned*>(stats), vmax);
    atomicAdd(stats + 1, static_cast<unsigned long long>(count));
  }
}

// One smudge step in the math type M: spine point, cos / sin of the heading change and the
// map's top-left canvas pixel.
template <class M>
struct SmudgeStep {
  M cx, cy;
  M c, s;
  int roi_x, roi_y;
};

template <class M>
struct SmudgeArgs {
  void* canvas;   // packed canvas records
  int rows, cols;
  int64_t pitch;
  M* maps;        // two pickup maps of 7 planes (K r,g,b, S r,g,b, V) of side^2 cells each;
                  // the first is the smudge's state between strokes
  int side;
  M ctr, radius;  // maxSize / 2 (the rotation centre) and maxSize * 0.5 (the exchange radius)
  const M* tmap;
  int trows, tcols;
  // int(cp - boundMin) of painty, in integers: boundMin = b0 + f with f in [0, 1); m = cp - b0
  // gives m - 1 for m >= 1 and f > 0, else m
  int bx0, by0, bxf, byf;
  const SmudgeStep<M>* steps;
  int64_t nsteps;
  const unsigned long long* maxbits;
  M pickupRate, depositionRate;
  uint32_t seed;  // stochastic rounding of 16-bit canvas stores (per stroke)
};

// Cells a thread exchanges per batch (its canvas loads are in flight together).
template <class M> constexpr int kSmudgeBatch = 2;

// The paint exchange of one smudge cell (values `val`: K r,g,b, S r,g,b, V) with its canvas
// pixel (record `cr` at `pix`) under thickness D (Smudge.hxx:60-142).
template <class TK, class TV, class M>
__device__ __forceinline__ void smudge_exchange(const SmudgeArgs<M>& a, M (&val)[7],
                                                PixRec<TK, TV>& cr, M D, int pix, int64_t k,
                                                M maxD, M rmaxD) {
  const M cV = ld_elem<M>(&cr.v[6]), pV = val[6];
  M cVl, pVl;
  if constexpr (sizeof(M) == 8) {  // painty divides by maxD
    cVl = cV * a.depositionRate * D / maxD;
    pVl = pV * a.pickupRate * D / maxD;
  } else {
    cVl = cV * a.depositionRate * D * rmaxD;
    pVl = pV * a.pickupRate * D * rmaxD;
  }
  const M cVr = cV - cVl;
  const M pVr = pV - pVl;
  M cK[6], pK[6];
#pragma unroll
  for (int q = 0; q < 6; q++) {
    cK[q] = ld_elem<M>(&cr.k[q]);
    pK[q] = val[q];
  }
  constexpr double MinVolume = 0.001;
  const M pVnew = pVr + cVl;
  if (pVnew > M(MinVolume)) {
    const M inv = M(1) / pVnew;
#pragma unroll
    for (int q = 0; q < 6; q++) val[q] = inv * (pVr * pK[q] + cVl * cK[q]);
    val[6] = pVnew > M(0) ? pVnew : M(0);
  }
  const M cVnew = cVr + pVl;
  if (cVnew > M(MinVolume)) {
    // 16-bit storage rounds stochastically: a step moves a pixel by a small fraction of the
    // difference, which round-to-nearest would drop (bits from stroke, step, pixel)
    uint32_t h[4] = {0u, 0u, 0u, 0u};
    if constexpr (sizeof(TK) == 2) {
      h[0] = hash32(hash32(a.seed + static_cast<uint32_t>(k)) ^
                    (static_cast<uint32_t>(pix) * 0x9e3779b1u));
#pragma unroll
      for (int q = 1; q < 4; q++) h[q] = hash32(h[q - 1] + 0x632be5abu);
    }
    const M inv = M(1) / cVnew;
#pragma unroll
    for (int q = 0; q < 6; q++)
      st_elem_sr<M>(&cr.k[q], inv * (cVr * cK[q] + pVl * pK[q]),
                    (q & 1) ? h[q >> 1] >> 16 : h[q >> 1]);
    st_elem_sr<M>(&cr.v[6], cVnew > M(0) ? cVnew : M(0), h[3]);
    store_rec<TK, TV>(a.canvas, pix, cr);
  }
}

// Geometry of one smudge cell (x, y) at a step: its canvas record, or -1 when the cell is off
// the canvas, outside the thickness map or beyond the smudge radius; D its thickness.
template <class M>
__device__ __forceinline__ int smudge_cell_pixel(const SmudgeArgs<M>& a, const SmudgeStep<M>& st,
                                                 int x, int y, M* D) {
  const int cpx = x + st.roi_x, cpy = y + st.roi_y;
  if (cpx < 0 || cpy < 0 || cpx >= a.cols || cpy >= a.rows) return -1;
  const int mx = cpx - a.bx0, my = cpy - a.by0;
  const int tpx = (a.bxf && mx >= 1) ? mx - 1 : mx;
  const int tpy = (a.byf && my >= 1) ? my - 1 : my;
  if (tpx < 0 || tpy < 0 || tpx >= a.tcols || tpy >= a.trows) return -1;
  const M dx = st.cx - static_cast<M>(cpx);
  const M dy = st.cy - static_cast<M>(cpy);
  if (sqrt(dx * dx + dy * dy) > a.radius) return -1;
  *D = __ldg(a.tmap + static_cast<int64_t>(tpy) * a.tcols + tpx);
  return static_cast<int>(static_cast<int64_t>(cpy) * a.pitch + cpx);
}

// Launch 2: Smudge::smudge (Smudge.hxx:38-145) with updateOrientation (:160-199), one CTA
// walking the steps in order. Per step the map is rotated from one buffer into the other
// (painty copies dst to src, then rotates src into dst: cells that rotate in from outside keep
// their own value), then each cell under the stroke exchanges paint with its canvas pixel.
// SM: both maps staged in shared memory (loaded at the start, written back at the end).
template <class TK, class TV, class M, bool SM>
__global__ void __launch_bounds__(kSmudgeThreads, 1) tb_smudge_kernel(const __grid_constant__ SmudgeArgs<M> a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  constexpr int J = kSmudgeBatch<M>;
  const int tid = threadIdx.x, T = blockDim.x;
  const int side = a.side, cells = side * side;
  M* cur;
  M* nxt;
  if constexpr (SM) {
    cur = reinterpret_cast<M*>(smem_raw);
    nxt = cur + 7 * cells;
    for (int i = tid; i < 7 * cells; i += T) cur[i] = a.maps[i];
    __syncthreads();
  } else {
    cur = a.maps;
    nxt = a.maps + 7 * cells;
  }
  M maxD;
  if constexpr (sizeof(M) == 8)
    maxD = __longlong_as_double(static_cast<long long>(*a.maxbits));
  else
    maxD = __uint_as_float(static_cast<unsigned>(*a.maxbits));
  // 1 / maxD: FP32 multiplies by it; FP64 divides as painty does
  const M rmaxD = M(1) / maxD;
  const M c0 = a.ctr, fside = static_cast<M>(side);
  const float rside = 1.0f / static_cast<float>(side);
  SmudgeStep<M> st = a.steps[0];
  for (int64_t k = 0; k < a.nsteps; k++) {
    // the next step's parameters load while this one runs
    const SmudgeStep<M> st_next = a.steps[k + 1 < a.nsteps ? k + 1 : k];
    const M cs = st.c, sn = st.s;
    // One pass per step: a cell's rotated value (updateOrientation: nxt = cur rotated about
    // the map centre) depends only on the previous map, and its exchange with the canvas only
    // on that value and its own canvas pixel, so each thread rotates and exchanges its cells
    // without waiting for the others; one barrier ends the step.
    for (int base = 0; base < cells; base += J * T) {
      int cxy[J], pix[J];  // cell (y << 16 | x), or -1; canvas record, or -1
      M D[J];
      PixRec<TK, TV> cr[J];
#pragma unroll
      for (int j = 0; j < J; j++) {
        const int i = base + j * T + tid;
        cxy[j] = -1;
        pix[j] = -1;
        D[j] = M(0);
        if (i >= cells) continue;
        // (x, y) of cell i: a float quotient corrected by one step is exact
        int y = static_cast<int>((static_cast<float>(i) + 0.5f) * rside);
        int x = i - y * side;
        if (x < 0) {
          y--;
          x += side;
        } else if (x >= side) {
          y++;
          x -= side;
        }
        cxy[j] = y << 16 | x;
        // the thickness and the canvas record load together, before the rotation
        pix[j] = smudge_cell_pixel(a, st, x, y, &D[j]);
        if (pix[j] >= 0) cr[j] = load_rec<false, TK, TV>(a.canvas, pix[j]);
      }
#pragma unroll
      for (int j = 0; j < J; j++) {
        if (cxy[j] < 0) continue;
        const int y = cxy[j] >> 16, x = cxy[j] & 0xffff;
        const int i = y * side + x;
        M val[7];
        const M px = static_cast<M>(x) - c0, py = static_cast<M>(y) - c0;
        const M qx = px * cs - py * sn + c0;
        const M qy = px * sn + py * cs + c0;
        if (qx < M(0) || qy < M(0) || qx >= fside || qy >= fside) {
#pragma unroll
          for (int q = 0; q < 7; q++) val[q] = cur[q * cells + i];
        } else {
          // 0 <= q < side: the BORDER_REFLECT neighbours are q's cell and the next one, which
          // reflects back onto the last cell at the border
          const int fx = static_cast<int>(floor(qx)), fy = static_cast<int>(floor(qy));
          const int x1 = min(fx + 1, side - 1), y1 = min(fy + 1, side - 1);
          const M wa = qx - static_cast<M>(fx), wc = qy - static_cast<M>(fy);
          const int o00 = fy * side + fx, o01 = fy * side + x1;
          const int o10 = y1 * side + fx, o11 = y1 * side + x1;
#pragma unroll
          for (int q = 0; q < 7; q++) {
            const M* sp = cur + q * cells;
            val[q] = (sp[o00] * (M(1) - wa) + sp[o01] * wa) * (M(1) - wc) +
                     (sp[o10] * (M(1) - wa) + sp[o11] * wa) * wc;
          }
        }
        // the exchange (Smudge.hxx:60-142) where the cell covers painted canvas
        if (pix[j] >= 0 && D[j] > M(0))
          smudge_exchange<TK, TV, M>(a, val, cr[j], D[j], pix[j], k, maxD, rmaxD);
#pragma unroll
        for (int q = 0; q < 7; q++) nxt[q * cells + i] = val[q];
      }
    }
    __syncthreads();
    M* t = cur;
    cur = nxt;
    nxt = t;
    st = st_next;
  }
  // the state map: write the current map back to the first global map
  if (SM || cur != a.maps)
    for (int i = tid; i < 7 * cells; i += T) a.maps[i] = cur[i];
}

// Distributed shared memory: the shared::cluster address of `local` (a shared address of this
// CTA) in CTA `rank` of the cluster, and loads from such addresses.
__device__ __forceinline__ unsigned dsmem_map(unsigned local, unsigned rank) {
  unsigned r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(local), "r"(rank));
  return r;
}
__device__ __forceinline__ float dsmem_ld(unsigned addr, float) {
  float v;
  asm volatile("ld.shared::cluster.f32 %0, [%1];" : "=f"(v) : "r"(addr) : "memory");
  return v;
}
__device__ __forceinline__ double dsmem_ld(unsigned addr, double) {
  double v;
  asm volatile("ld.shared::cluster.f64 %0, [%1];" : "=d"(v) : "r"(addr) : "memory");
  return v;
}

constexpr int kSmudgeClusterThreads = 256;

// Launch 2 on a thread-block cluster: the same steps with the map's rows split into bands, one
// per CTA (band b: rows [b B, b B + B), B = ceil(side / CTAs)), each band's two buffers in its
// CTA's shared memory. A cell's rotation reads its four neighbours wherever they live through
// distributed shared memory; its exchange touches only its own band and canvas pixel. One
// cluster barrier per step orders the maps and the canvas writes (canvas reads bypass L1:
// another CTA may have written the pixel in an earlier step). The FP64 rotation's work spreads
// over the cluster's SMs.
template <class TK, class TV, class M>
__global__ void __launch_bounds__(kSmudgeClusterThreads, 1)
    tb_smudge_cluster_kernel(const __grid_constant__ SmudgeArgs<M> a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  constexpr int J = kSmudgeBatch<M>;
  const int tid = threadIdx.x, T = blockDim.x;
  const int side = a.side, cells = side * side;
  const int rank = static_cast<int>(cluster_rank()), C = static_cast<int>(cluster_size());
  const int B = (side + C - 1) / C;            // band rows
  const int P = B * side;                      // band cells (plane stride in shared memory)
  const int ry0 = rank * B, ry1 = min(side, ry0 + B);
  const int nloc = ry1 > ry0 ? (ry1 - ry0) * side : 0;
  M* cur = reinterpret_cast<M*>(smem_raw);
  M* nxt = cur + 7 * P;
  for (int i = tid; i < nloc; i += T)
#pragma unroll
    for (int q = 0; q < 7; q++) cur[q * P + i] = a.maps[q * cells + ry0 * side + i];
  cluster_barrier();  // every band loaded before any remote read
  M maxD;
  if constexpr (sizeof(M) == 8)
    maxD = __longlong_as_double(static_cast<long long>(*a.maxbits));
  else
    maxD = __uint_as_float(static_cast<unsigned>(*a.maxbits));
  const M rmaxD = M(1) / maxD;
  const M c0 = a.ctr, fside = static_cast<M>(side);
  const float rside = 1.0f / static_cast<float>(side);
  constexpr unsigned ES = sizeof(M);
  SmudgeStep<M> st = a.steps[0];
  for (int64_t k = 0; k < a.nsteps; k++) {
    const SmudgeStep<M> st_next = a.steps[k + 1 < a.nsteps ? k + 1 : k];
    const M cs = st.c, sn = st.s;
    const unsigned cur_s = static_cast<unsigned>(__cvta_generic_to_shared(cur));
    for (int base = 0; base < nloc; base += J * T) {
      int cxy[J], pix[J];
      M D[J];
      PixRec<TK, TV> cr[J];
#pragma unroll
      for (int j = 0; j < J; j++) {
        const int li = base + j * T + tid;
        cxy[j] = -1;
        pix[j] = -1;
        D[j] = M(0);
        if (li >= nloc) continue;
        int yl = static_cast<int>((static_cast<float>(li) + 0.5f) * rside);
        int x = li - yl * side;
        if (x < 0) {
          yl--;
          x += side;
        } else if (x >= side) {
          yl++;
          x -= side;
        }
        const int y = ry0 + yl;
        cxy[j] = y << 16 | x;
        pix[j] = smudge_cell_pixel(a, st, x, y, &D[j]);
        if (pix[j] >= 0) cr[j] = load_rec<true, TK, TV>(a.canvas, pix[j]);
      }
#pragma unroll
      for (int j = 0; j < J; j++) {
        if (cxy[j] < 0) continue;
        const int y = cxy[j] >> 16, x = cxy[j] & 0xffff;
        const int li = (y - ry0) * side + x;
        M val[7];
        const M px = static_cast<M>(x) - c0, py = static_cast<M>(y) - c0;
        const M qx = px * cs - py * sn + c0;
        const M qy = px * sn + py * cs + c0;
        if (qx < M(0) || qy < M(0) || qx >= fside || qy >= fside) {
#pragma unroll
          for (int q = 0; q < 7; q++) val[q] = cur[q * P + li];
        } else {
          const int fx = static_cast<int>(floor(qx)), fy = static_cast<int>(floor(qy));
          const int x1 = min(fx + 1, side - 1), y1 = min(fy + 1, side - 1);
          const M wa = qx - static_cast<M>(fx), wc = qy - static_cast<M>(fy);
          // the two neighbour rows, in their bands' CTAs
          const int o0 = fy / B, o1 = y1 / B;
          const unsigned r0 = dsmem_map(cur_s + ES * static_cast<unsigned>((fy - o0 * B) * side), o0);
          const unsigned r1 = dsmem_map(cur_s + ES * static_cast<unsigned>((y1 - o1 * B) * side), o1);
          const unsigned ax0 = ES * static_cast<unsigned>(fx), ax1 = ES * static_cast<unsigned>(x1);
#pragma unroll
          for (int q = 0; q < 7; q++) {
            const unsigned pq = ES * static_cast<unsigned>(q * P);
            const M s00 = dsmem_ld(r0 + pq + ax0, M(0)), s01 = dsmem_ld(r0 + pq + ax1, M(0));
            const M s10 = dsmem_ld(r1 + pq + ax0, M(0)), s11 = dsmem_ld(r1 + pq + ax1, M(0));
            val[q] = (s00 * (M(1) - wa) + s01 * wa) * (M(1) - wc) +
                     (s10 * (M(1) - wa) + s11 * wa) * wc;
          }
        }
        if (pix[j] >= 0 && D[j] > M(0))
          smudge_exchange<TK, TV, M>(a, val, cr[j], D[j], pix[j], k, maxD, rmaxD);
#pragma unroll
        for (int q = 0; q < 7; q++) nxt[q * P + li] = val[q];
      }
    }
    cluster_barrier();  // the step's maps and canvas writes before the next step's reads
    M* t = cur;
    cur = nxt;
    nxt = t;
    st = st_next;
  }
  for (int i = tid; i < nloc; i += T)
#pragma unroll
    for (int q = 0; q < 7; q++) a.maps[q * cells + ry0 * side + i] = cur[q * P + i];
}

template <class M>
struct DepositArgs {
  void* canvas;
  int rows, cols;
  int64_t pitch;
  const M* tmap;
  int trows, tcols;
  int x0, y0, nx, ny, bx, by;
  M K[3], S[3];
};

// Launch 3: the deposit over the painted pixels (TextureBrush.hxx:179-204)
template <class TK, class TV, class M>
__global__ void __launch_bounds__(kTexThreads) tb_deposit_kernel(const DepositArgs<M> a) {
  const int64_t n = static_cast<int64_t>(a.nx) * a.ny;
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int y = a.y0 + static_cast<int>(i / a.nx), x = a.x0 + static_cast<int>(i % a.nx);
    if (x < 0 || x >= a.cols || y < 0 || y >= a.rows) continue;
    const int s = x - a.bx, t = y - a.by;
    if (s < 0 || t < 0 || s >= a.tcols || t >= a.trows) continue;
    const M vtex = a.tmap[static_cast<int64_t>(t) * a.tcols + s];
    if (!(vtex > M(0))) continue;  // not a painted pixel
    const int c = static_cast<int>(static_cast<int64_t>(y) * a.pitch + x);
    PixRec<TK, TV> r = load_rec<false, TK, TV>(a.canvas, c);
    const M vcan = ld_elem<M>(&r.v[6]);
    const M vsum = vcan + vtex;
    if (!(vsum > M(0))) continue;
    const M sc = M(1) / vsum;
#pragma unroll
    for (int q = 0; q < 3; q++) {
      const M kk = ld_elem<M>(&r.k[q]), ss = ld_elem<M>(&r.k[3 + q]);
      st_elem<M>(&r.k[q], (vcan * kk + vtex * a.K[q]) * sc);
      st_elem<M>(&r.k[3 + q], (vcan * ss + vtex * a.S[q]) * sc);
    }
    st_elem<M>(&r.v[6], vtex > vcan ? vtex : vcan);
    store_rec<TK, TV>(a.canvas, c, r);
  }
}

size_t align256(size_t n) { return (n + 255) / 256 * 256; }

int max_dyn_smem() {
  int dev = 0, v = 0;
  PG_CUDA(cudaGetDevice(&dev));
  PG_CUDA(cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  return v;
}

int grid_of(int64_t n, int block) {
  return static_cast<int>(std::max<int64_t>(1, std::min<int64_t>((n + block - 1) / block, 152 * 16)));
}

size_t smudge_cluster_smem(int side, int cl, size_t es) {
  const size_t B = static_cast<size_t>((side + cl - 1) / cl);
  return 2 * 7 * B * static_cast<size_t>(side) * es;
}

// CTAs of the smudge cluster for a map of `side`: PAINTY_SMUDGE_CLUSTER (1, 2, 4, 8, 16) when
// set, else 16 (FP64: its rotation is bound by the FP64 rate) or 8 (FP32) when the device can
// co-schedule such a cluster with the band buffers in shared memory; 1 means one CTA.
template <class TK, class TV, class M>
int smudge_cluster(int side) {
  int want = sizeof(M) == 8 ? 16 : 8;
  if (const char* v = std::getenv("PAINTY_SMUDGE_CLUSTER")) {
    const int n = std::atoi(v);
    if (n == 1 || n == 2 || n == 4 || n == 8 || n == 16) want = n;
  }
  while (want > 1 && want > side) want /= 2;  // at least one map row per CTA
  auto kern = tb_smudge_cluster_kernel<TK, TV, M>;
  for (; want > 1; want /= 2) {
    const size_t smem = smudge_cluster_smem(side, want, sizeof(M));
    if (smem > static_cast<size_t>(max_dyn_smem())) continue;
    if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             static_cast<int>(smem)) != cudaSuccess ||
        (want > 8 &&
         cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) !=
           cudaSuccess)) {
      cudaGetLastError();
      continue;
    }
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3(static_cast<unsigned>(want));
    cfg.blockDim = dim3(kSmudgeClusterThreads);
    cfg.dynamicSmemBytes = smem;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = static_cast<unsigned>(want);
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    int n = 0;
    if (cudaOccupancyMaxActiveClusters(&n, kern, &cfg) == cudaSuccess && n >= 1) return want;
    cudaGetLastError();
  }
  return 1;
}

template <class TK, class TV, class M>
void launch_smudge_cluster(const SmudgeArgs<M>& sa, int cl, cudaStream_t st) {
  auto kern = tb_smudge_cluster_kernel<TK, TV, M>;
  const size_t smem = smudge_cluster_smem(sa.side, cl, sizeof(M));
  cudaLaunchConfig_t cfg{};
  cfg.gridDim = dim3(static_cast<unsigned>(cl));
  cfg.blockDim = dim3(kSmudgeClusterThreads);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = static_cast<unsigned>(cl);
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  PG_CUDA(cudaLaunchKernelEx(&cfg, kern, sa));
}

// TextureBrush::paintStroke (TextureBrush.hxx:52-205); returns the pixels painted.
template <class TK, class TV>
int64_t paint_texture_stroke(painty_canvas* c, painty_texture_brush* b, const double* path,
                             int32_t n, cudaStream_t st) {
  using M = typename MathOf<TK>::type;
  if (n < 2) return 0;
  const int rows = c->wet.rows, cols = c->wet.cols;
  std::vector<D2> arg(static_cast<size_t>(n));
  for (int32_t i = 0; i < n; i++) arg[i] = {path[2 * i], path[2 * i + 1]};
  std::vector<D2> v;
  {
    const D2 d = normalized_h({arg[1].x - arg[0].x, arg[1].y - arg[0].y});
    v.push_back({arg[0].x - d.x * b->radius, arg[0].y - d.y * b->radius});
  }
  v.insert(v.end(), arg.begin(), arg.end());
  {
    const D2 d = normalized_h({arg[n - 1].x - arg[n - 2].x, arg[n - 1].y - arg[n - 2].y});
    v.push_back({arg[n - 1].x + d.x * b->radius, arg[n - 1].y + d.y * b->radius});
  }
  D2 bmin = v.front(), bmax = v.front();
  for (const D2& p : v) {
    bmin.x = std::min(bmin.x, p.x);
    bmin.y = std::min(bmin.y, p.y);
    bmax.x = std::max(bmax.x, p.x);
    bmax.y = std::max(bmax.y, p.y);
  }
  bmin.x = std::max(bmin.x - b->radius, 0.0);
  bmax.x = std::min(bmax.x + b->radius, static_cast<double>(cols - 1));
  bmin.y = std::max(bmin.y - b->radius, 0.0);
  bmax.y = std::min(bmax.y + b->radius, static_cast<double>(rows - 1));
  double length = 0.0;
  for (size_t i = 1; i < v.size(); ++i) {
    const double dx = v[i].x - v[i - 1].x, dy = v[i].y - v[i - 1].y;
    length += std::sqrt(dx * dx + dy * dy);
  }
  // the smudge steps u by 1 / length: about length + 1 steps
  PG_REQUIRE(!b->useSmudge || length < static_cast<double>(1 << 26),
             "stroke too long for the smudge");
  PG_REQUIRE(!b->useSmudge || b->side <= 4096, "smudge map wider than 4096 (radius above 2048)");
  // outline: the right side reversed, then the left side; uv (u, 1) then (u, 0)
  std::vector<double2> up, down, upUv, downUv;
  for (size_t i = 0; i < v.size(); ++i) {
    const double u = static_cast<double>(i) / static_cast<double>(v.size() - 1);
    const D2 p = spline_h(v, u, false);
    const D2 t = normalized_h(spline_h(v, u, true));
    const D2 d = {-t.y, t.x};
    up.push_back(make_double2(p.x - b->radius * d.x, p.y - b->radius * d.y));
    down.push_back(make_double2(p.x + b->radius * d.x, p.y + b->radius * d.y));
    upUv.push_back(make_double2(u, 0.0));
    downUv.push_back(make_double2(u, 1.0));
  }
  up.insert(up.begin(), down.rbegin(), down.rend());
  upUv.insert(upUv.begin(), downUv.rbegin(), downUv.rend());
  const int trows = static_cast<int32_t>(bmax.y - bmin.y + 1);
  const int tcols = static_cast<int32_t>(bmax.x - bmin.x + 1);
  if (trows <= 0 || tcols <= 0) return 0;  // the bounds miss the canvas (painty fails here)
  const int x0 = static_cast<int32_t>(bmin.x), x1 = static_cast<int32_t>(bmax.x);
  const int y0 = static_cast<int32_t>(bmin.y), y1 = static_cast<int32_t>(bmax.y);
  const int nx = x1 - x0 + 1, ny = y1 - y0 + 1;
  if (nx <= 0 || ny <= 0) return 0;

  // device buffers of the stroke (stream-ordered)
  const int np = static_cast<int>(up.size());
  const size_t tmap_bytes = static_cast<size_t>(trows) * tcols * sizeof(M);
  char* d = nullptr;
  const size_t off_poly = 0, off_uv = align256(np * sizeof(double2)),
               off_max = off_uv + align256(np * sizeof(double2)),
               off_tmap = off_max + 256, total = off_tmap + align256(tmap_bytes);
  d = static_cast<decltype(d)>(temp_alloc(total, st));
  PG_CUDA(cudaMemcpyAsync(d + off_poly, up.data(), np * sizeof(double2), cudaMemcpyHostToDevice, st));
  PG_CUDA(cudaMemcpyAsync(d + off_uv, upUv.data(), np * sizeof(double2), cudaMemcpyHostToDevice, st));
  PG_CUDA(cudaMemsetAsync(d + off_max, 0, 256 + align256(tmap_bytes), st));
  auto* maxbits = reinterpret_cast<unsigned long long*>(d + off_max);
  M* tmap = reinterpret_cast<M*>(d + off_tmap);

  TexArgs ta{};
  ta.poly = reinterpret_cast<const double2*>(d + off_poly);
  ta.uv = reinterpret_cast<const double2*>(d + off_uv);
  ta.npoly = np;
  ta.tex = static_cast<const double*>(b->d_tex);
  ta.th = b->th;
  ta.tw = b->tw;
  ta.scale = b->thicknessScale;
  ta.x0 = x0;
  ta.y0 = y0;
  ta.nx = nx;
  ta.ny = ny;
  ta.bx = x0;
  ta.by = y0;
  ta.trows = trows;
  ta.tcols = tcols;
  ta.rows = rows;
  ta.cols = cols;
  const int64_t npx = static_cast<int64_t>(nx) * ny;
  tb_thickness_kernel<M><<<grid_of(npx, kTexThreads), kTexThreads, 0, st>>>(ta, tmap, maxbits);
  count_launch();
  PG_CUDA(cudaGetLastError());

  // the thickness maximum and the painted-pixel count
  unsigned long long stats[2] = {0, 0};
  PG_CUDA(cudaMemcpyAsync(stats, maxbits, sizeof(stats), cudaMemcpyDeviceToHost, st));
  PG_CUDA(cudaStreamSynchronize(st));
  const int64_t painted = static_cast<int64_t>(stats[1]);
  if (painted == 0) {
    PG_CUDA(cudaFreeAsync(d, st));
    return 0;
  }
  // the smudge runs only where the map has paint (Smudge.hxx:41-47)
  if (b->useSmudge) {
    double maxD;
    if constexpr (sizeof(M) == 8) {
      std::memcpy(&maxD, &stats[0], 8);
    } else {
      float x;
      const unsigned lo = static_cast<unsigned>(stats[0]);
      std::memcpy(&x, &lo, 4);
      maxD = x;
    }
    if (maxD > 0.0) {
      std::vector<SmudgeStep<M>> steps;
      const double msz = static_cast<double>(b->side);
      for (double u = 0.0; u <= 1.0; u += 1. / length) {
        const D2 ctr = spline_h(v, u, false);
        const D2 t = normalized_h(spline_h(v, u, true));
        const double theta = std::atan2(t.y, t.x);
        const double dtheta = normalize_angle_h(theta - b->rotation);
        b->rotation = theta;
        SmudgeStep<M> s{};
        s.cx = static_cast<M>(ctr.x);
        s.cy = static_cast<M>(ctr.y);
        s.c = static_cast<M>(std::cos(dtheta));
        s.s = static_cast<M>(std::sin(dtheta));
        s.roi_x = static_cast<int32_t>(ctr.x - msz / 2.0);
        s.roi_y = static_cast<int32_t>(ctr.y - msz / 2.0);
        steps.push_back(s);
      }
      const size_t cells = static_cast<size_t>(b->side) * b->side;
      const size_t mbytes = 2 * cells * 7 * sizeof(M);
      if (b->d_maps_bytes < mbytes || !b->d_maps) {
        device_free(b->d_maps);
        b->d_maps = device_alloc(std::max<size_t>(mbytes, 256));
        b->d_maps_bytes = std::max<size_t>(mbytes, 256);
        b->maps_zero = true;
      }
      if (b->maps_zero) {
        PG_CUDA(cudaMemsetAsync(b->d_maps, 0, b->d_maps_bytes, st));
        b->maps_zero = false;
      }
      SmudgeStep<M>* dsteps = nullptr;
      dsteps = static_cast<SmudgeStep<M>*>(
        temp_alloc(std::max<size_t>(steps.size(), 1) * sizeof(SmudgeStep<M>), st));
      if (!steps.empty())
        PG_CUDA(cudaMemcpyAsync(dsteps, steps.data(), steps.size() * sizeof(SmudgeStep<M>),
                                cudaMemcpyHostToDevice, st));
      SmudgeArgs<M> sa{};
      sa.canvas = c->wet.base;
      sa.rows = rows;
      sa.cols = cols;
      sa.pitch = c->wet.pitch;
      sa.maps = static_cast<M*>(b->d_maps);
      sa.side = b->side;
      sa.ctr = static_cast<M>(b->maxSize / 2.0);
      sa.radius = static_cast<M>(b->maxSize * 0.5);
      sa.tmap = tmap;
      sa.trows = trows;
      sa.tcols = tcols;
      sa.bx0 = static_cast<int>(std::floor(bmin.x));
      sa.by0 = static_cast<int>(std::floor(bmin.y));
      sa.bxf = bmin.x > std::floor(bmin.x) ? 1 : 0;
      sa.byf = bmin.y > std::floor(bmin.y) ? 1 : 0;
      sa.steps = dsteps;
      sa.nsteps = static_cast<int64_t>(steps.size());
      sa.maxbits = maxbits;
      sa.pickupRate = static_cast<M>(0.1);      // Smudge.hxx:156
      sa.depositionRate = static_cast<M>(0.1);  // Smudge.hxx:158
      // from the canvas's write count: the same painting session gives the same bits
      sa.seed = static_cast<uint32_t>(c->version * 0x9e3779b97f4a7c15ull >> 32);
      if (!steps.empty() && cells > 0) {
        // a cluster of CTAs shares the map by bands when the device has one free; otherwise
        // one CTA holds both maps in shared memory when they fit (side <= 64 in FP32, <= 45
        // in FP64), else in global memory
        const size_t smem = 2 * cells * 7 * sizeof(M);
        const int cl = smudge_cluster<TK, TV, M>(b->side);
        if (cl > 1) {
          launch_smudge_cluster<TK, TV, M>(sa, cl, st);
        } else if (smem <= static_cast<size_t>(max_dyn_smem())) {
          auto kern = tb_smudge_kernel<TK, TV, M, true>;
          PG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       static_cast<int>(smem)));
          kern<<<1, kSmudgeThreads, smem, st>>>(sa);
        } else {
          tb_smudge_kernel<TK, TV, M, false><<<1, kSmudgeThreads, 0, st>>>(sa);
        }
        count_launch();
        PG_CUDA(cudaGetLastError());
      }
      PG_CUDA(cudaFreeAsync(dsteps, st));
    }
  }

  DepositArgs<M> da{};
  da.canvas = c->wet.base;
  da.rows = rows;
  da.cols = cols;
  da.pitch = c->wet.pitch;
  da.tmap = tmap;
  da.trows = trows;
  da.tcols = tcols;
  da.x0 = x0;
  da.y0 = y0;
  da.nx = nx;
  da.ny = ny;
  da.bx = x0;
  da.by = y0;
  for (int q = 0; q < 3; q++) {
    da.K[q] = static_cast<M>(b->paintK[q]);
    da.S[q] = static_cast<M>(b->paintS[q]);
  }
  tb_deposit_kernel<TK, TV, M><<<grid_of(npx, kTexThreads), kTexThreads, 0, st>>>(da);
  count_launch();
  PG_CUDA(cudaGetLastError());
  PG_CUDA(cudaFreeAsync(d, st));
  c->version++;
  return painted;
}

}  // namespace
}  // namespace pg

using pg::guard;

extern "C" {

painty_status painty_texture_brush_create(const double* texture, int32_t rows, int32_t cols,
                                          painty_texture_brush** out) {
  return guard([&] {
    PG_REQUIRE(out != nullptr, "out is null");
    PG_REQUIRE(texture != nullptr && rows > 0 && cols > 0, "texture is empty");
    auto* b = new painty_texture_brush();
    b->tex.assign(texture, texture + static_cast<size_t>(rows) * cols);
    b->th = rows;
    b->tw = cols;
    b->make_smudge(static_cast<int32_t>(2.0 * b->radius));  // TextureBrush.hxx:25-31
    *out = b;
  });
}

painty_status painty_texture_brush_destroy(painty_texture_brush* b) {
  return guard([&] {
    if (!b) return;
    pg::device_free(b->d_tex);
    pg::device_free(b->d_maps);
    delete b;
  });
}

painty_status painty_texture_brush_set_radius(painty_texture_brush* b, double radius) {
  return guard([&] {
    PG_REQUIRE(b != nullptr, "brush is null");
    PG_REQUIRE(std::isfinite(radius) && radius >= 0.0 && radius <= 1e6,
               "radius must be in [0, 1e6]");
    if (!(std::fabs(b->radius - radius) < 0.5)) {  // TextureBrush.hxx:33-41
      b->radius = radius;
      if (b->useSmudge) b->make_smudge(static_cast<int32_t>(2.0 * radius));
    }
  });
}

painty_status painty_texture_brush_dip(painty_texture_brush* b, const double K[3],
                                       const double S[3]) {
  return guard([&] {
    PG_REQUIRE(b && K && S, "null argument");
    for (int i = 0; i < 3; i++) {
      b->paintK[i] = K[i];
      b->paintS[i] = S[i];
    }
  });
}

painty_status painty_texture_brush_set_smudge(painty_texture_brush* b, int32_t enable) {
  return guard([&] {
    PG_REQUIRE(b != nullptr, "brush is null");
    b->useSmudge = enable != 0;
  });
}

painty_status painty_texture_brush_set_thickness_scale(painty_texture_brush* b, double scale) {
  return guard([&] {
    PG_REQUIRE(b != nullptr, "brush is null");
    PG_REQUIRE(std::isfinite(scale), "scale must be finite");
    b->thicknessScale = scale;
  });
}

painty_status painty_texture_brush_paint_stroke(painty_canvas* c, painty_texture_brush* b,
                                                const double* path_xy, int32_t n,
                                                int64_t* painted_out, void* stream) {
  return guard([&] {
    PG_REQUIRE(c && b, "null handle");
    PG_REQUIRE(n >= 0 && (n == 0 || path_xy), "path is null");
    // every pixel of the stroke's bounds walks the 2 (n + 2)-vertex outline
    PG_REQUIRE(n <= 4096, "path longer than 4096 points");
    for (int64_t i = 0; i < 2 * static_cast<int64_t>(n); i++)
      PG_REQUIRE(std::isfinite(path_xy[i]) && std::fabs(path_xy[i]) < 1e9,
                 "path coordinates must be finite and within 1e9");
    PG_REQUIRE(static_cast<int64_t>(c->wet.rows) * c->wet.pitch < (int64_t(1) << 31),
               "canvas too large for the texture brush");
    const bool f64 = c->wet.storage == PAINTY_STORAGE_F64;
    const int mode = f64 ? 1 : 0;
    if (b->bound < 0) b->bound = mode;
    PG_REQUIRE(b->bound == mode,
               "a texture brush paints either F64 canvases or F32/F16/BF16 canvases, not both");
    const cudaStream_t st = pg::as_stream(stream);
    if (!b->d_tex) {
      b->d_tex = pg::device_alloc(b->tex.size() * sizeof(double));
      PG_CUDA(cudaMemcpyAsync(b->d_tex, b->tex.data(), b->tex.size() * sizeof(double),
                              cudaMemcpyHostToDevice, st));
    }
    int64_t painted = 0;
    switch (c->wet.storage) {
      case PAINTY_STORAGE_F32:
        painted = pg::paint_texture_stroke<float, float>(c, b, path_xy, n, st);
        break;
      case PAINTY_STORAGE_F16:
        painted = pg::paint_texture_stroke<__half, __half>(c, b, path_xy, n, st);
        break;
      case PAINTY_STORAGE_BF16:
        painted = pg::paint_texture_stroke<__nv_bfloat16, __half>(c, b, path_xy, n, st);
        break;
      case PAINTY_STORAGE_F64:
        painted = pg::paint_texture_stroke<double, double>(c, b, path_xy, n, st);
        break;
    }
    if (painted_out) *painted_out = painted;
  });
}

painty_status painty_texture_brush_smudge_map(const painty_texture_brush* b,
                                                   painty_plane plane, double* host,
                                                   int32_t* side, void* stream) {
  return guard([&] {
    PG_REQUIRE(b != nullptr, "brush is null");
    if (side) *side = b->side;
    if (!host) return;
    const size_t cells = static_cast<size_t>(b->side) * b->side;
    const int nch = plane == PAINTY_PLANE_V ? 1 : 3;
    PG_REQUIRE(plane == PAINTY_PLANE_K || plane == PAINTY_PLANE_S || plane == PAINTY_PLANE_V,
               "smudge planes are K, S, V");
    if (!b->d_maps || b->maps_zero || b->bound < 0) {
      std::memset(host, 0, cells * nch * sizeof(double));
      return;
    }
    const size_t msz = b->bound == 1 ? 8 : 4;
    const int off = plane == PAINTY_PLANE_K ? 0 : plane == PAINTY_PLANE_S ? 3 : 6;
    const char* base = static_cast<const char*>(b->d_maps);
    const size_t pb = cells * msz;  // bytes per plane
    const void* p[3] = {base + off * pb, base + (off + 1) * pb, base + (off + 2) * pb};
    pg::download_planes(p, nch, b->bound == 1 ? pg::DT_F64 : pg::DT_F32, b->side, b->side,
                        b->side, host, PAINTY_HOST_F64_INTERLEAVED, pg::as_stream(stream));
  });
}

}  // extern "C"
