// canvas_gpu.cu -- painty's GL canvas path as CUDA kernels.
//
// painty's second renderer keeps the canvas in rgba32f GL textures (V in K.a, a lighting
// volume in S.a) and paints with compute and raster shaders:
//  - PaintLayerGpu::composeOnto / CanvasGpu::getComposed (PaintLayerGpu.cxx:27-41,
//    CanvasGpu.cxx:91-95) run ComposeLayerOnSubstrate.compute.glsl:13-71;
//  - CanvasGpu::dryStep (CanvasGpu.cxx:112-128) runs DryingStep.compute.glsl:30-77;
//  - TextureBrushGpu::paintStroke (TextureBrushGpu.cxx:74-167) rasterises the stroke's
//    triangle strip with a texture from TextureBrushDictionary (generateWarpedTexture,
//    :169-246; BrushTextureWarp.{vert,frag}.glsl), imprints it with
//    PaintTextureFootprintOnCanvas.compute.glsl:17-53 and clears it with
//    ClearTextureFootprint.compute.glsl.
// Here the canvas is the library's packed canvas (the record's pad element holds the lighting
// volume) and the arithmetic is float, as in the shaders. Where GL leaves a choice to the
// implementation (raster rules, texture filtering, dispatch rounding) these kernels make the
// choices the oracle restates: vertices snap to 1/256 pixel; coverage is exact at pixel
// centres with a top-left rule, the last triangle of the strip covering a centre wins;
// barycentrics divide in float; the brush texture is sampled bilinearly with clamp-to-edge and
// unquantised weights; a w x h dispatch covers the 16 x 16 tiles containing it. The device
// code is built without fused multiply-adds, so results equal the oracle's float arithmetic.
#include <algorithm>
#include <climits>
#include <cmath>
#include <cstring>
#include <limits>
#include <map>
#include <random>
#include <vector>

#include "device_common.cuh"
#include "internal.h"

// TextureBrushDictionary (TextureBrushDictionary.hxx:17-39) with a seeded pick.
struct painty_texture_dictionary {
  struct Entry {
    uint32_t radius_class = 0, length_class = 0;
    int32_t rows = 0, cols = 0;
    std::vector<float> gl;  // GL rows, bottom-up: gl[k * cols + i] = image row rows-1-k
    float* d_tex = nullptr;
  };
  std::mt19937 gen;
  std::vector<Entry> entries;
};

// TextureBrushGpu (TextureBrushGpu.hxx:21-64); the smudge pass is not provided.
struct painty_gpu_texture_brush {
  painty_texture_dictionary* dict = nullptr;
  double radius = 0.0;
  double paint[2][3] = {{0, 0, 0}, {0, 0, 0}};
  double thicknessScale = 1.0;  // BrushBase.hxx:45
  float* d_warped = nullptr;    // canvas-sized R32F warped brush texture
  int* d_owner = nullptr;       // per pixel: the last strip triangle covering it, or -1
  int32_t wrows = 0, wcols = 0;
  int32_t last_texture = -1;
};

namespace pg {
namespace {

constexpr float kGlEps = 10e-6f;  // the shaders' Eps

// coth (ComposeLayerOnSubstrate.compute.glsl:13-22): 1 above 20, cosh(x) / sinh(x) for x != 0,
// else infinity. cosh / sinh = 1 + 2 / (e^2x - 1), with expm1 accurate near 0.
__device__ __forceinline__ float glsl_coth(float x) {
  if (x > 20.0f) return 1.0f;
  if (fabsf(x) > 0.0f) return 1.0f + 2.0f / expm1f(2.0f * x);
  return __int_as_float(0x7f800000);
}

// computeReflectance (ComposeLayerOnSubstrate.compute.glsl:28-47): coth(bSh) stands where the
// CPU path has b * coth(bSh), and any channel with |bSh| < 1e-5 returns r0.
__device__ __forceinline__ void glsl_reflectance(const float K[3], const float S[3],
                                                 const float r0[3], float d, float out[3]) {
  float a[3], bSh[3];
  bool small = false;
#pragma unroll
  for (int c = 0; c < 3; c++) {
    const float K_S = K[c] / S[c];
    a[c] = 1.0f + K_S;
    const float asq = a[c] * a[c];
    const float b = sqrtf(fmaxf(asq - 1.0f, 0.0f));
    bSh[c] = b * S[c] * d;
    small = small || fabsf(bSh[c]) < kGlEps;
  }
#pragma unroll
  for (int c = 0; c < 3; c++) {
    if (small) {
      out[c] = r0[c];
    } else {
      const float bc = glsl_coth(bSh[c]);
      out[c] = (1.0f - r0[c] * (a[c] - bc)) / (a[c] - r0[c] + bc);
    }
  }
}

// Compose (DRY false: out = composeOnto of the wet layer over R0) or dry step (DRY true: R0
// takes the portion of V that leaves; V keeps the rest).
template <class TK, class TV, bool DRY>
__global__ void __launch_bounds__(256) glsl_canvas_kernel(void* canvas, float* r0_0, float* r0_1,
                                                          float* r0_2, float* out0, float* out1,
                                                          float* out2, int rows, int cols,
                                                          int64_t pitch, float portion) {
  const int64_t n = static_cast<int64_t>(rows) * cols;
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int64_t y = i / cols, x = i - y * cols;
    const int64_t p = y * pitch + x;
    PixRec<TK, TV> r = load_rec<false, TK, TV>(canvas, static_cast<int>(p));
    float K[3], S[3];
#pragma unroll
    for (int c = 0; c < 3; c++) {
      K[c] = ld_elem<float>(&r.k[c]);
      S[c] = ld_elem<float>(&r.k[3 + c]);
    }
    const float d = ld_elem<float>(&r.v[6]);
    const float r0[3] = {r0_0[p], r0_1[p], r0_2[p]};
    float o[3] = {r0[0], r0[1], r0[2]};
    if constexpr (DRY) {
      const float vRemaining = fmaxf(0.0f, d - portion);
      const float vLeaving = d - vRemaining;
      if (fabsf(vLeaving) > kGlEps) glsl_reflectance(K, S, r0, vLeaving, o);
      r0_0[p] = o[0];
      r0_1[p] = o[1];
      r0_2[p] = o[2];
      st_elem<float>(&r.v[6], vRemaining);
      store_rec<TK, TV>(canvas, static_cast<int>(p), r);
    } else {
      if (fabsf(d) > kGlEps) glsl_reflectance(K, S, r0, d, o);
      out0[p] = o[0];
      out1[p] = o[1];
      out2[p] = o[2];
    }
  }
}

int grid_for_px(int64_t n) {
  return static_cast<int>(std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, 152 * 8)));
}

template <bool DRY>
void launch_glsl(const painty_canvas* c, painty_image* out, float portion, cudaStream_t st) {
  const painty_layer& w = c->wet;
  float* r0[3] = {static_cast<float*>(c->r0.R[0]), static_cast<float*>(c->r0.R[1]),
                  static_cast<float*>(c->r0.R[2])};
  float* o[3] = {r0[0], r0[1], r0[2]};
  if (out) {
    for (int i = 0; i < 3; i++) o[i] = static_cast<float*>(out->R[i]);
  }
  const int g = grid_for_px(static_cast<int64_t>(w.rows) * w.cols);
  switch (w.storage) {
    case PAINTY_STORAGE_F32:
      glsl_canvas_kernel<float, float, DRY><<<g, 256, 0, st>>>(
        w.base, r0[0], r0[1], r0[2], o[0], o[1], o[2], w.rows, w.cols, w.pitch, portion);
      break;
    case PAINTY_STORAGE_F16:
      glsl_canvas_kernel<__half, __half, DRY><<<g, 256, 0, st>>>(
        w.base, r0[0], r0[1], r0[2], o[0], o[1], o[2], w.rows, w.cols, w.pitch, portion);
      break;
    case PAINTY_STORAGE_BF16:
      glsl_canvas_kernel<__nv_bfloat16, __half, DRY><<<g, 256, 0, st>>>(
        w.base, r0[0], r0[1], r0[2], o[0], o[1], o[2], w.rows, w.cols, w.pitch, portion);
      break;
    default: fail(PAINTY_ERR_UNSUPPORTED, "the GL canvas path is float: F32, F16 or BF16 canvases");
  }
  count_launch();
  PG_CUDA(cudaGetLastError());
}

// ------------------------------------------------------------------ texture brush (GL path)
struct D2 {
  double x, y;
};
double cr_pos(double p_1, double p0, double p1, double p2, double t) {  // Spline.hxx:27-47
  constexpr double tau = 0.5;
  const double t2 = t * t, t3 = t2 * t;
  const double b1 = -tau * t + 2.0 * tau * t2 - tau * t3;
  const double b2 = 1.0 + (tau - 3.0) * t2 + (2.0 - tau) * t3;
  const double b3 = tau * t + (3.0 - 2.0 * tau) * t2 + (tau - 2.0) * t3;
  const double b4 = -tau * t2 + tau * t3;
  return p_1 * b1 + p0 * b2 + p1 * b3 + p2 * b4;
}
double cr_der(double p_1, double p0, double p1, double p2, double t) {  // Spline.hxx:49-73
  constexpr double tau = 0.5;
  const double t2 = t * t;
  const double b1 = tau * (-3.0 * t2 + 4.0 * t - 1.0);
  const double b2 = -t * (-2.0 * tau + 3.0 * (tau - 2.0) * t + 6.0);
  const double b3 = (t - 1.0) * (3.0 * (tau - 2.0) * t - tau);
  const double b4 = tau * t * (3.0 * t - 2.0);
  return p_1 * b1 + p0 * b2 + p1 * b3 + p2 * b4;
}
D2 spline_at(const std::vector<D2>& p, double u, bool deriv) {  // SplineEval (Spline.hxx:183-231)
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
  if (deriv) return {cr_der(a.x, b.x, c.x, d.x, t), cr_der(a.y, b.y, c.y, d.y, t)};
  return {cr_pos(a.x, b.x, c.x, d.x, t), cr_pos(a.y, b.y, c.y, d.y, t)};
}
D2 normalized(const D2& v) {  // Eigen normalized()
  const double n = v.x * v.x + v.y * v.y;
  if (n > 0.0) {
    const double r = std::sqrt(n);
    return {v.x / r, v.y / r};
  }
  return v;
}

// cv::normalize(.., 0, 1, NORM_MINMAX) of a double image
void normalize_minmax(std::vector<double>& v) {
  if (v.empty()) return;
  double lo = v[0], hi = v[0];
  for (double x : v) {
    lo = std::fmin(lo, x);
    hi = std::fmax(hi, x);
  }
  const double range = hi - lo;
  const double scale = range > std::numeric_limits<double>::epsilon() ? 1.0 / range : 0.0;
  const double shift = 0.0 - lo * scale;
  for (double& x : v) x = x * scale + shift;
}

// TextureBrushDictionary::lookup (TextureBrushDictionary.cxx:25-69) over the classes its
// constructor builds (:128-179): size classes by radius token and length classes by length
// token, ascending, with their mean texture rows and cols. The length scan stops at the chosen
// size's length classes (painty bounds it by the number of size classes, :46). The pick is a
// seeded std::mt19937 draw mapped by multiply-shift (painty seeds from std::random_device).
int32_t dict_lookup(painty_texture_dictionary* d, const double* path, int32_t n,
                    double brushSize) {
  PG_REQUIRE(!d->entries.empty(), "the texture dictionary is empty");
  double length = 0.0;
  for (int32_t i = 0; i + 1 < n; i++) {
    const double dx = path[2 * i] - path[2 * (i + 1)], dy = path[2 * i + 1] - path[2 * (i + 1) + 1];
    length += std::sqrt(dx * dx + dy * dy);
  }
  std::map<uint32_t, std::map<uint32_t, std::vector<int32_t>>> m;
  for (size_t i = 0; i < d->entries.size(); i++)
    m[d->entries[i].radius_class][d->entries[i].length_class].push_back(static_cast<int32_t>(i));
  std::vector<std::vector<std::vector<int32_t>>> cls;
  for (const auto& e : m) {
    cls.emplace_back();
    for (const auto& a : e.second) cls.back().push_back(a.second);
  }
  std::vector<double> avgSizes(cls.size(), 0.0);
  std::vector<std::vector<double>> avgLen(cls.size());
  for (size_t i = 0; i < cls.size(); i++) {
    uint32_t ns = 0;
    avgLen[i].assign(cls[i].size(), 0.0);
    for (size_t j = 0; j < cls[i].size(); j++) {
      uint32_t nl = 0;
      for (int32_t e : cls[i][j]) {
        avgSizes[i] += static_cast<double>(d->entries[static_cast<size_t>(e)].rows);
        avgLen[i][j] += static_cast<double>(d->entries[static_cast<size_t>(e)].cols);
        ns++;
        nl++;
      }
      avgLen[i][j] *= (1.0 / static_cast<double>(nl));
    }
    avgSizes[i] *= (1.0 / static_cast<double>(ns));
  }
  uint32_t i0 = 0, i1 = 1;
  double mr = avgSizes[0];
  for (uint32_t i = 0; i < avgSizes.size(); i++) {
    const double dd = std::fabs(avgSizes[i] - brushSize);
    if (dd < mr) {
      mr = dd;
      i0 = i;
    }
  }
  double ml = avgLen[i0][0];
  for (uint32_t i = 0; i < avgSizes.size() && i < avgLen[i0].size(); i++) {
    const double dd = std::fabs(avgLen[i0][i] - length);
    if (dd < ml) {
      ml = dd;
      i1 = i;
    }
  }
  PG_REQUIRE(i1 < cls[i0].size() && !cls[i0][i1].empty(), "no candidate found");
  const auto& cand = cls[i0][i1];
  const uint64_t r = static_cast<uint64_t>(d->gen()) * static_cast<uint64_t>(cand.size());
  return cand[static_cast<size_t>(r >> 32)];
}

struct StripArgs {
  const long long* X;  // window coordinates of the strip vertices, 1/256 pixel
  const long long* Y;
  const float* tu;
  const float* tv;
  int nv;
  int rows, cols;
  int* owner;
  float* warped;
  const float* tex;  // GL rows of the brush texture
  int th, tw;
  int wx0, wy0, wnx, wny;  // the strip's pixel box in window coordinates
};

__device__ __forceinline__ long long floordiv256(long long a) {
  return a >= 0 ? a / 256 : -((-a + 255) / 256);
}
__device__ __forceinline__ long long edge_fn(long long ax, long long ay, long long bx,
                                             long long by, long long px, long long py) {
  return (bx - ax) * (py - ay) - (by - ay) * (px - ax);
}
// GL top-left rule for a counter-clockwise triangle in window coordinates (y up): a horizontal
// edge running in -x is a top edge, an edge running in -y a left edge.
__device__ __forceinline__ bool top_left(long long ax, long long ay, long long bx, long long by) {
  return (ay == by && bx < ax) || by < ay;
}

struct Tri {
  int ia, ib, ic;
  long long area;
};
__device__ __forceinline__ Tri strip_tri(const StripArgs& a, int k) {
  Tri t{k, k + 1, k + 2, 0};
  t.area = edge_fn(a.X[t.ia], a.Y[t.ia], a.X[t.ib], a.Y[t.ib], a.X[t.ic], a.Y[t.ic]);
  if (t.area < 0) {
    const int s = t.ib;
    t.ib = t.ic;
    t.ic = s;
    t.area = -t.area;
  }
  return t;
}
__device__ __forceinline__ bool covers(const StripArgs& a, const Tri& t, long long px,
                                       long long py, long long w[3]) {
  const long long xa = a.X[t.ia], ya = a.Y[t.ia], xb = a.X[t.ib], yb = a.Y[t.ib];
  const long long xc = a.X[t.ic], yc = a.Y[t.ic];
  w[0] = edge_fn(xb, yb, xc, yc, px, py);
  w[1] = edge_fn(xc, yc, xa, ya, px, py);
  w[2] = edge_fn(xa, ya, xb, yb, px, py);
  return (w[0] > 0 || (w[0] == 0 && top_left(xb, yb, xc, yc))) &&
         (w[1] > 0 || (w[1] == 0 && top_left(xc, yc, xa, ya))) &&
         (w[2] > 0 || (w[2] == 0 && top_left(xa, ya, xb, yb)));
}

// Raster pass 1: each strip triangle marks the centres it covers with its index (the last
// triangle wins, as GL draws the strip in order without blending). A triangle's pixel box is
// cut into 16 x 16 tiles shared out over the CTAs of its grid row; a tile whose four corner
// regions all lie outside one edge is skipped whole (the strip's triangles are long and thin,
// so most of a box is empty), otherwise each thread tests one pixel centre.
constexpr int kCoverSplit = 16;  // CTAs per triangle
__global__ void __launch_bounds__(256) strip_cover_kernel(const StripArgs a) {
  const int k = blockIdx.x;
  const Tri t = strip_tri(a, k);
  if (t.area == 0) return;
  const long long xa = a.X[t.ia], ya = a.Y[t.ia], xb = a.X[t.ib], yb = a.Y[t.ib];
  const long long xc = a.X[t.ic], yc = a.Y[t.ic];
  const long long xmin = min(xa, min(xb, xc)), xmax = max(xa, max(xb, xc));
  const long long ymin = min(ya, min(yb, yc)), ymax = max(ya, max(yb, yc));
  // pixel centres 256 x + 128 inside [xmin, xmax]
  const long long x0 = max(0LL, floordiv256(xmin - 128 + 255));
  const long long x1 = min(static_cast<long long>(a.cols - 1), floordiv256(xmax - 128));
  const long long y0 = max(0LL, floordiv256(ymin - 128 + 255));
  const long long y1 = min(static_cast<long long>(a.rows - 1), floordiv256(ymax - 128));
  if (x0 > x1 || y0 > y1) return;
  const long long tx = (x1 - x0) / 16 + 1, ty = (y1 - y0) / 16 + 1;
  const int lx = threadIdx.x & 15, ly = threadIdx.x >> 4;
  for (long long tile = blockIdx.y; tile < tx * ty; tile += gridDim.y) {
    const long long bx = x0 + (tile % tx) * 16, by = y0 + (tile / tx) * 16;
    // the tile's centre box [bx, bx + 15] x [by, by + 15] in 1/256 units
    const long long cx0 = 256 * bx + 128, cx1 = cx0 + 256 * 15;
    const long long cy0 = 256 * by + 128, cy1 = cy0 + 256 * 15;
    bool outside = false;
    const long long ex[3][4] = {{xb, yb, xc, yc}, {xc, yc, xa, ya}, {xa, ya, xb, yb}};
#pragma unroll
    for (int e = 0; e < 3; e++) {
      // an edge function is affine: its maximum over the box is at a corner
      const long long dx = ex[e][2] - ex[e][0], dy = ex[e][3] - ex[e][1];
      const long long px = dy > 0 ? cx0 : cx1;  // maximises -dy * px
      const long long py = dx > 0 ? cy1 : cy0;  // maximises dx * py
      if (edge_fn(ex[e][0], ex[e][1], ex[e][2], ex[e][3], px, py) < 0) outside = true;
    }
    if (outside) continue;  // uniform over the CTA
    const long long x = bx + lx, wy = by + ly;
    if (x > x1 || wy > y1) continue;
    long long w[3];
    if (!covers(a, t, 256 * x + 128, 256 * wy + 128, w)) continue;
    const long long y = a.rows - 1 - wy;  // canvas row of window row wy
    atomicMax(a.owner + y * a.cols + x, k);
  }
}

// Raster pass 2: the covering triangle's interpolated texture coordinate samples the brush
// texture (BrushTextureWarp.frag.glsl:9-12) into the warped texture; the owner map resets.
__global__ void __launch_bounds__(256) strip_sample_kernel(const StripArgs a) {
  const long long n = static_cast<long long>(a.wnx) * a.wny;
  for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<long long>(gridDim.x) * blockDim.x) {
    const long long wy = a.wy0 + i / a.wnx, x = a.wx0 + i % a.wnx;
    const long long y = a.rows - 1 - wy;
    int* own = a.owner + y * a.cols + x;
    const int k = *own;
    if (k < 0) continue;
    *own = -1;
    const Tri t = strip_tri(a, k);
    long long w[3];
    covers(a, t, 256 * x + 128, 256 * wy + 128, w);
    const float fa = static_cast<float>(t.area);
    const float l0 = static_cast<float>(w[0]) / fa, l1 = static_cast<float>(w[1]) / fa,
                l2 = static_cast<float>(w[2]) / fa;
    const float u = l0 * a.tu[t.ia] + l1 * a.tu[t.ib] + l2 * a.tu[t.ic];
    const float v = l0 * a.tv[t.ia] + l1 * a.tv[t.ib] + l2 * a.tv[t.ic];
    // bilinear, clamp to edge, texel centres at (i + 0.5) / size
    const float s = u * static_cast<float>(a.tw) - 0.5f;
    const float r = v * static_cast<float>(a.th) - 0.5f;
    const float fs = floorf(s), fr = floorf(r);
    const float wa = s - fs, wc = r - fr;
    const long long is = static_cast<long long>(fs), ir = static_cast<long long>(fr);
    const int i0 = static_cast<int>(min(max(is, 0LL), static_cast<long long>(a.tw - 1)));
    const int i1 = static_cast<int>(min(max(is + 1, 0LL), static_cast<long long>(a.tw - 1)));
    const int k0 = static_cast<int>(min(max(ir, 0LL), static_cast<long long>(a.th - 1)));
    const int k1 = static_cast<int>(min(max(ir + 1, 0LL), static_cast<long long>(a.th - 1)));
    const float* g = a.tex;
    a.warped[y * a.cols + x] =
      (g[k0 * a.tw + i0] * (1.0f - wa) + g[k0 * a.tw + i1] * wa) * (1.0f - wc) +
      (g[k1 * a.tw + i0] * (1.0f - wa) + g[k1 * a.tw + i1] * wa) * wc;
  }
}

struct ImprintArgs {
  void* canvas;
  int64_t pitch;
  float* warped;
  int rows, cols;
  int x0, y0, nx, ny;  // the dispatch's tiles, clipped to the canvas
  float K[3], S[3];
  float scale;
};

// PaintTextureFootprintOnCanvas.compute.glsl:17-53, then ClearTextureFootprint for the pixel.
template <class TK, class TV>
__global__ void __launch_bounds__(256) strip_imprint_kernel(const ImprintArgs a) {
  const int64_t n = static_cast<int64_t>(a.nx) * a.ny;
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int y = a.y0 + static_cast<int>(i / a.nx), x = a.x0 + static_cast<int>(i % a.nx);
    float* wp = a.warped + static_cast<int64_t>(y) * a.cols + x;
    const float vTex = a.scale * *wp;
    *wp = 0.0f;
    const int p = static_cast<int>(static_cast<int64_t>(y) * a.pitch + x);
    PixRec<TK, TV> r = load_rec<false, TK, TV>(a.canvas, p);
    const float vCan = ld_elem<float>(&r.v[6]);
    const float vSum = vCan + vTex;
    if (vSum < kGlEps) continue;
#pragma unroll
    for (int c = 0; c < 3; c++) {
      const float K = ld_elem<float>(&r.k[c]), S = ld_elem<float>(&r.k[3 + c]);
      st_elem<float>(&r.k[c], (vCan * K + vTex * a.K[c]) / vSum);
      st_elem<float>(&r.k[3 + c], (vCan * S + vTex * a.S[c]) / vSum);
    }
    st_elem<float>(&r.v[6], vSum);
    st_elem<float>(&r.v[7], vTex > 0.0f ? vTex : vCan);
    store_rec<TK, TV>(a.canvas, p, r);
  }
}

// TextureBrushGpu::paintStroke (TextureBrushGpu.cxx:74-167), smudge off.
void gl_paint_stroke(painty_canvas* c, painty_gpu_texture_brush* b, const double* path,
                     int32_t n, cudaStream_t st) {
  if (n < 2) return;  // painty's guard is commented out; fewer points have no strip
  const int rows = c->wet.rows, cols = c->wet.cols;
  std::vector<D2> v(static_cast<size_t>(n));
  for (int32_t i = 0; i < n; i++) v[static_cast<size_t>(i)] = {path[2 * i], path[2 * i + 1]};
  D2 bmin = v.front(), bmax = v.front();
  for (const D2& p : v) {
    bmin.x = std::fmin(bmin.x, p.x);
    bmin.y = std::fmin(bmin.y, p.y);
    bmax.x = std::fmax(bmax.x, p.x);
    bmax.y = std::fmax(bmax.y, p.y);
  }
  bmin.x = std::fmax(bmin.x - b->radius, 0.0);
  bmax.x = std::fmin(bmax.x + b->radius, static_cast<double>(cols - 1));
  bmin.y = std::fmax(bmin.y - b->radius, 0.0);
  bmax.y = std::fmin(bmax.y + b->radius, static_cast<double>(rows - 1));

  // generateWarpedTexture (:169-246): the strip (right, left per spline sample), snapped
  const int nv = 2 * n;
  std::vector<long long> X(static_cast<size_t>(nv)), Y(static_cast<size_t>(nv));
  std::vector<float> tu(static_cast<size_t>(nv)), tv(static_cast<size_t>(nv));
  auto snap = [](float f) { return static_cast<long long>(std::nearbyint(static_cast<double>(f) * 256.0)); };
  long long xmin = LLONG_MAX, xmax = LLONG_MIN, ymin = LLONG_MAX, ymax = LLONG_MIN;
  for (int32_t i = 0; i < n; i++) {
    const double u = static_cast<double>(i) / static_cast<double>(n - 1);
    const D2 cc = spline_at(v, u, false);
    const D2 t = normalized(spline_at(v, u, true));
    const D2 d = {-t.y, t.x};
    const D2 l = {cc.x - b->radius * d.x, cc.y - b->radius * d.y};
    const D2 r = {cc.x + b->radius * d.x, cc.y + b->radius * d.y};
    const float vx[2] = {static_cast<float>(r.x), static_cast<float>(l.x)};
    const float vy[2] = {static_cast<float>(r.y), static_cast<float>(l.y)};
    // window coordinates in 1/256 pixel stay below 2^31 and their edge products below 2^63
    PG_REQUIRE(std::fabs(vx[0]) < 4e6f && std::fabs(vx[1]) < 4e6f && std::fabs(vy[0]) < 4e6f &&
                 std::fabs(vy[1]) < 4e6f,
               "stroke outline beyond 4e6 pixels");
    for (int s = 0; s < 2; s++) {
      const size_t j = static_cast<size_t>(2 * i + s);
      X[j] = snap(vx[s]);
      Y[j] = snap(static_cast<float>(rows) - vy[s]);
      tu[j] = static_cast<float>(u);
      tv[j] = s == 0 ? 0.0f : 1.0f;
      xmin = std::min(xmin, X[j]);
      xmax = std::max(xmax, X[j]);
      ymin = std::min(ymin, Y[j]);
      ymax = std::max(ymax, Y[j]);
    }
  }
  const int32_t tex = dict_lookup(b->dict, path, n, 2.0 * b->radius);
  b->last_texture = tex;
  auto& e = b->dict->entries[static_cast<size_t>(tex)];
  if (!e.d_tex) {
    e.d_tex = static_cast<float*>(device_alloc(e.gl.size() * sizeof(float)));
    PG_CUDA(cudaMemcpyAsync(e.d_tex, e.gl.data(), e.gl.size() * sizeof(float),
                            cudaMemcpyHostToDevice, st));
  }
  if (b->wrows != rows || b->wcols != cols) {
    device_free(b->d_warped);
    device_free(b->d_owner);
    b->d_warped = nullptr;
    b->d_owner = nullptr;
    const size_t px = static_cast<size_t>(rows) * cols;
    b->d_warped = static_cast<float*>(device_alloc(px * sizeof(float)));
    b->d_owner = static_cast<int*>(device_alloc(px * sizeof(int)));
    PG_CUDA(cudaMemsetAsync(b->d_warped, 0, px * sizeof(float), st));
    PG_CUDA(cudaMemsetAsync(b->d_owner, 0xff, px * sizeof(int), st));
    b->wrows = rows;
    b->wcols = cols;
  }
  // vertex arrays in one stream-ordered allocation
  const size_t bx = static_cast<size_t>(nv) * sizeof(long long), bf = static_cast<size_t>(nv) * sizeof(float);
  std::vector<char> host(2 * bx + 2 * bf);
  std::memcpy(host.data(), X.data(), bx);
  std::memcpy(host.data() + bx, Y.data(), bx);
  std::memcpy(host.data() + 2 * bx, tu.data(), bf);
  std::memcpy(host.data() + 2 * bx + bf, tv.data(), bf);
  char* dv = nullptr;
  dv = static_cast<decltype(dv)>(temp_alloc(host.size(), st));
  PG_CUDA(cudaMemcpyAsync(dv, host.data(), host.size(), cudaMemcpyHostToDevice, st));
  StripArgs sa{};
  sa.X = reinterpret_cast<const long long*>(dv);
  sa.Y = reinterpret_cast<const long long*>(dv + bx);
  sa.tu = reinterpret_cast<const float*>(dv + 2 * bx);
  sa.tv = reinterpret_cast<const float*>(dv + 2 * bx + bf);
  sa.nv = nv;
  sa.rows = rows;
  sa.cols = cols;
  sa.owner = b->d_owner;
  sa.warped = b->d_warped;
  sa.tex = e.d_tex;
  sa.th = e.rows;
  sa.tw = e.cols;
  // window pixels whose centres can lie in the strip
  auto fdiv = [](long long a) { return a >= 0 ? a / 256 : -((-a + 255) / 256); };
  const long long px0 = std::max(0LL, fdiv(xmin - 128) - 1), px1 = std::min<long long>(cols - 1, fdiv(xmax - 128) + 1);
  const long long wy0 = std::max(0LL, fdiv(ymin - 128) - 1), wy1 = std::min<long long>(rows - 1, fdiv(ymax - 128) + 1);
  if (px0 <= px1 && wy0 <= wy1) {
    sa.wx0 = static_cast<int>(px0);
    sa.wy0 = static_cast<int>(wy0);
    sa.wnx = static_cast<int>(px1 - px0 + 1);
    sa.wny = static_cast<int>(wy1 - wy0 + 1);
    strip_cover_kernel<<<dim3(nv - 2, kCoverSplit), 256, 0, st>>>(sa);
    count_launch();
    PG_CUDA(cudaGetLastError());
    strip_sample_kernel<<<grid_for_px(static_cast<int64_t>(sa.wnx) * sa.wny), 256, 0, st>>>(sa);
    count_launch();
    PG_CUDA(cudaGetLastError());
  }
  PG_CUDA(cudaFreeAsync(dv, st));

  // imprint and clear over the area of interest, rounded up to the shaders' 16 x 16 tiles
  const int32_t aoiW = static_cast<int32_t>(bmax.x - bmin.x) + 1;
  const int32_t aoiH = static_cast<int32_t>(bmax.y - bmin.y) + 1;
  if (aoiW <= 0 || aoiH <= 0) return;
  const int32_t ax0 = static_cast<int32_t>(bmin.x), ay0 = static_cast<int32_t>(bmin.y);
  const int64_t ax1 = std::min<int64_t>(cols, ax0 + static_cast<int64_t>(aoiW + 15) / 16 * 16);
  const int64_t ay1 = std::min<int64_t>(rows, ay0 + static_cast<int64_t>(aoiH + 15) / 16 * 16);
  const int32_t cx0 = std::max(ax0, 0), cy0 = std::max(ay0, 0);
  if (ax1 <= cx0 || ay1 <= cy0) return;
  ImprintArgs ia{};
  ia.canvas = c->wet.base;
  ia.pitch = c->wet.pitch;
  ia.warped = b->d_warped;
  ia.rows = rows;
  ia.cols = cols;
  ia.x0 = cx0;
  ia.y0 = cy0;
  ia.nx = static_cast<int>(ax1 - cx0);
  ia.ny = static_cast<int>(ay1 - cy0);
  for (int i = 0; i < 3; i++) {
    ia.K[i] = static_cast<float>(b->paint[0][i]);
    ia.S[i] = static_cast<float>(b->paint[1][i]);
  }
  ia.scale = static_cast<float>(b->thicknessScale);
  const int g = grid_for_px(static_cast<int64_t>(ia.nx) * ia.ny);
  switch (c->wet.storage) {
    case PAINTY_STORAGE_F32: strip_imprint_kernel<float, float><<<g, 256, 0, st>>>(ia); break;
    case PAINTY_STORAGE_F16: strip_imprint_kernel<__half, __half><<<g, 256, 0, st>>>(ia); break;
    case PAINTY_STORAGE_BF16:
      strip_imprint_kernel<__nv_bfloat16, __half><<<g, 256, 0, st>>>(ia);
      break;
    default: fail(PAINTY_ERR_UNSUPPORTED, "the GL canvas path is float: F32, F16 or BF16 canvases");
  }
  count_launch();
  PG_CUDA(cudaGetLastError());
  c->version++;
}

}  // namespace
}  // namespace pg

using pg::guard;

extern "C" {

painty_status painty_canvas_compose_glsl(const painty_canvas* c, painty_image* out,
                                         void* stream) {
  return guard([&] {
    PG_REQUIRE(c && out, "null handle");
    PG_REQUIRE(out->rows == c->wet.rows && out->cols == c->wet.cols, "image size differs");
    PG_REQUIRE(out->storage == PAINTY_STORAGE_F32 && c->r0.storage == PAINTY_STORAGE_F32,
               "the GL canvas path composes into F32 images");
    pg::launch_glsl<false>(c, out, 0.0f, pg::as_stream(stream));
  });
}

painty_status painty_canvas_dry_step(painty_canvas* c, float portion, void* stream) {
  return guard([&] {
    PG_REQUIRE(c != nullptr, "canvas is null");
    PG_REQUIRE(c->r0.storage == PAINTY_STORAGE_F32,
               "the GL canvas path is float: F32, F16 or BF16 canvases");
    c->version++;
    pg::launch_glsl<true>(c, nullptr, portion, pg::as_stream(stream));
  });
}

painty_status painty_texture_dictionary_create(uint32_t seed, painty_texture_dictionary** out) {
  return guard([&] {
    PG_REQUIRE(out != nullptr, "out is null");
    auto* d = new painty_texture_dictionary();
    d->gen.seed(seed);
    *out = d;
  });
}

painty_status painty_texture_dictionary_destroy(painty_texture_dictionary* d) {
  return guard([&] {
    if (!d) return;
    for (auto& e : d->entries) pg::device_free(e.d_tex);
    delete d;
  });
}

painty_status painty_texture_dictionary_add(painty_texture_dictionary* d, uint32_t radius_class,
                                            uint32_t length_class, const double* height,
                                            int32_t rows, int32_t cols, int32_t* index_out) {
  return guard([&] {
    PG_REQUIRE(d != nullptr, "dictionary is null");
    PG_REQUIRE(height != nullptr && rows > 0 && cols > 0, "texture is empty");
    std::vector<double> v(height, height + static_cast<size_t>(rows) * cols);
    for (double x : v) PG_REQUIRE(std::isfinite(x), "texture values must be finite");
    // loadHeightMap normalises, the GPU copy is normalised again, flipped and made float
    // (TextureBrushDictionary.cxx:112-124)
    pg::normalize_minmax(v);
    pg::normalize_minmax(v);
    painty_texture_dictionary::Entry e;
    e.radius_class = radius_class;
    e.length_class = length_class;
    e.rows = rows;
    e.cols = cols;
    e.gl.resize(v.size());
    for (int32_t k = 0; k < rows; k++)
      for (int32_t i = 0; i < cols; i++)
        e.gl[static_cast<size_t>(k) * cols + i] =
          static_cast<float>(v[static_cast<size_t>(rows - 1 - k) * cols + i]);
    d->entries.push_back(std::move(e));
    if (index_out) *index_out = static_cast<int32_t>(d->entries.size() - 1);
  });
}

painty_status painty_texture_dictionary_lookup(painty_texture_dictionary* d,
                                               const double* path_xy, int32_t n,
                                               double brush_size, int32_t* index_out) {
  return guard([&] {
    PG_REQUIRE(d && index_out, "null argument");
    PG_REQUIRE(n >= 1 && path_xy, "path is empty");
    *index_out = pg::dict_lookup(d, path_xy, n, brush_size);
  });
}

painty_status painty_gpu_texture_brush_create(painty_texture_dictionary* dict,
                                              painty_gpu_texture_brush** out) {
  return guard([&] {
    PG_REQUIRE(dict && out, "null argument");
    auto* b = new painty_gpu_texture_brush();
    b->dict = dict;
    b->radius = 5.0;  // TextureBrushGpu.cxx:45 (setRadius(5.0) from radius 0)
    *out = b;
  });
}

painty_status painty_gpu_texture_brush_destroy(painty_gpu_texture_brush* b) {
  return guard([&] {
    if (!b) return;
    pg::device_free(b->d_warped);
    pg::device_free(b->d_owner);
    delete b;
  });
}

painty_status painty_gpu_texture_brush_set_radius(painty_gpu_texture_brush* b, double radius) {
  return guard([&] {
    PG_REQUIRE(b != nullptr, "brush is null");
    PG_REQUIRE(std::isfinite(radius) && radius >= 0.0 && radius <= 1e6,
               "radius must be in [0, 1e6]");
    if (!(std::fabs(b->radius - radius) < 0.5)) b->radius = radius;  // TextureBrushGpu.cxx:48-61
  });
}

painty_status painty_gpu_texture_brush_dip(painty_gpu_texture_brush* b, const double K[3],
                                           const double S[3]) {
  return guard([&] {
    PG_REQUIRE(b && K && S, "null argument");
    for (int i = 0; i < 3; i++) {
      b->paint[0][i] = K[i];
      b->paint[1][i] = S[i];
    }
  });
}

painty_status painty_gpu_texture_brush_set_thickness_scale(painty_gpu_texture_brush* b,
                                                           double scale) {
  return guard([&] {
    PG_REQUIRE(b != nullptr, "brush is null");
    PG_REQUIRE(std::isfinite(scale), "scale must be finite");
    b->thicknessScale = scale;
  });
}

painty_status painty_gpu_texture_brush_set_smudge(painty_gpu_texture_brush* b, int32_t enable) {
  return guard([&] {
    PG_REQUIRE(b != nullptr, "brush is null");
    if (enable)
      pg::fail(PAINTY_ERR_UNSUPPORTED,
               "the GL smudge pass is not provided: its window pixels race for truncated "
               "smudge-map cells (Smudge.compute.glsl:57-92); use painty_texture_brush");
  });
}

painty_status painty_gpu_texture_brush_last_texture(const painty_gpu_texture_brush* b,
                                                    int32_t* index_out) {
  return guard([&] {
    PG_REQUIRE(b && index_out, "null argument");
    *index_out = b->last_texture;
  });
}

painty_status painty_gpu_texture_brush_paint_stroke(painty_canvas* c,
                                                    painty_gpu_texture_brush* b,
                                                    const double* path_xy, int32_t n,
                                                    void* stream) {
  return guard([&] {
    PG_REQUIRE(c && b, "null handle");
    PG_REQUIRE(n >= 0 && (n == 0 || path_xy), "path is null");
    PG_REQUIRE(n <= (1 << 20), "path too long");
    for (int64_t i = 0; i < 2 * static_cast<int64_t>(n); i++)
      PG_REQUIRE(std::isfinite(path_xy[i]) && std::fabs(path_xy[i]) < 1e7,
                 "path coordinates must be finite and within 1e7");
    PG_REQUIRE(c->wet.storage != PAINTY_STORAGE_F64,
               "the GL canvas path is float: F32, F16 or BF16 canvases");
    PG_REQUIRE(static_cast<int64_t>(c->wet.rows) * c->wet.pitch < (int64_t(1) << 31),
               "canvas too large");
    pg::gl_paint_stroke(c, b, path_xy, n, pg::as_stream(stream));
  });
}

}  // extern "C"
