// gl_path.cpp -- the oracle's CPU restatement of painty's GL canvas path, in float.
//
// TEST INFRASTRUCTURE ONLY (see painty_oracle.h). The GL path runs as compute and raster
// shaders; their arithmetic is restated here from the shader sources:
//   painty/renderer/shaders/ComposeLayerOnSubstrate.compute.glsl:13-71  (PaintLayerGpu::composeOnto)
//   painty/renderer/shaders/DryingStep.compute.glsl:13-77               (CanvasGpu::dryStep)
//   painty/renderer/src/TextureBrushGpu.cxx:48-246                      (setRadius, paintStroke,
//        generateWarpedTexture) with BrushTextureWarp.{vert,frag}.glsl,
//        PaintTextureFootprintOnCanvas.compute.glsl:17-53 and ClearTextureFootprint.compute.glsl
//   painty/renderer/src/TextureBrushDictionary.cxx:21-181               (lookup, texture classes)
// A GL canvas is K4 / S4 / R4: rows*cols pixels of 4 floats (painty's rgba32f textures, V in
// K.a, the lighting volume in S.a), row-major with a top-left origin (the GpuMat upload flips
// rows into GL's bottom-up textures; the shaders address those flipped rows, so in image
// coordinates every pass below reads and writes the pixel it names).
// Where GL leaves a choice to the implementation, this file and the CUDA kernels make the
// same one: vertices snap to 1/256 pixel, coverage is tested exactly at pixel centres with a
// top-left rule, barycentrics are divided in float, the brush texture is sampled bilinearly
// with clamp-to-edge and unquantised weights, and a compute dispatch of w x h covers the
// 16 x 16 tiles that contain it (the shaders check only the image bounds).
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <map>
#include <random>
#include <vector>

#include "painty_oracle.h"

namespace {

// ------------------------------------------------------------------ compute shaders
float glsl_coth(float x) {  // ComposeLayerOnSubstrate.compute.glsl:13-22
  if (x > 20.0f) return 1.0f;
  if (std::fabs(x) > 0.0f) return std::cosh(x) / std::sinh(x);
  return std::numeric_limits<float>::infinity();
}

// computeReflectance (ComposeLayerOnSubstrate.compute.glsl:28-47). Unlike the CPU path the
// shader uses coth(bSh) where painty's KubelkaMunk.hxx has b * coth(bSh), and returns r0 when
// any channel's |bSh| < 1e-5.
void glsl_reflectance(const float K[3], const float S[3], const float r0[3], float d,
                      float out[3]) {
  constexpr float Eps = 10e-6f;
  float a[3], b[3], bSh[3];
  bool small = false;
  for (int c = 0; c < 3; c++) {
    const float K_S = K[c] / S[c];
    a[c] = 1.0f + K_S;
    const float asq = a[c] * a[c];
    b[c] = std::sqrt(std::fmax(asq - 1.0f, 0.0f));
    bSh[c] = b[c] * S[c] * d;
    small = small || std::fabs(bSh[c]) < Eps;
  }
  if (small) {
    for (int c = 0; c < 3; c++) out[c] = r0[c];
    return;
  }
  for (int c = 0; c < 3; c++) {
    const float bc = glsl_coth(bSh[c]);
    out[c] = (1.0f - r0[c] * (a[c] - bc)) / (a[c] - r0[c] + bc);
  }
}

// ------------------------------------------------------------------ texture dictionary
struct TexEntry {
  uint32_t radius_class = 0, length_class = 0;
  int32_t rows = 0, cols = 0;
  std::vector<float> gl;  // GL texture rows (bottom-up): gl[k * cols + i] = image row rows-1-k
};

// cv::normalize(src, dst, 0, 1, NORM_MINMAX) on doubles: dst = src * scale + shift
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

}  // namespace

struct orc_tdict {
  std::mt19937 gen;
  std::vector<TexEntry> entries;  // insertion order
};

namespace {

// The classes of TextureBrushDictionary (TextureBrushDictionary.cxx:128-179): size classes by
// radius token, length classes by length token (both ascending), with mean rows / mean cols.
struct Classes {
  std::vector<std::vector<std::vector<int32_t>>> byClass;  // [size][length] -> entry indices
  std::vector<double> avgSizes;
  std::vector<std::vector<double>> avgLengths;
};

Classes make_classes(const orc_tdict* d) {
  std::map<uint32_t, std::map<uint32_t, std::vector<int32_t>>> m;
  for (size_t i = 0; i < d->entries.size(); i++)
    m[d->entries[i].radius_class][d->entries[i].length_class].push_back(static_cast<int32_t>(i));
  Classes c;
  for (const auto& e : m) {
    c.byClass.emplace_back();
    for (const auto& a : e.second) c.byClass.back().push_back(a.second);
  }
  c.avgSizes.assign(c.byClass.size(), 0.0);
  c.avgLengths.resize(c.byClass.size());
  for (size_t i = 0; i < c.byClass.size(); i++) {
    uint32_t n = 0;
    c.avgLengths[i].assign(c.byClass[i].size(), 0.0);
    for (size_t j = 0; j < c.byClass[i].size(); j++) {
      uint32_t nl = 0;
      for (int32_t e : c.byClass[i][j]) {
        c.avgSizes[i] += static_cast<double>(d->entries[static_cast<size_t>(e)].rows);
        c.avgLengths[i][j] += static_cast<double>(d->entries[static_cast<size_t>(e)].cols);
        n++;
        nl++;
      }
      c.avgLengths[i][j] *= (1.0 / static_cast<double>(nl));
    }
    c.avgSizes[i] *= (1.0 / static_cast<double>(n));
  }
  return c;
}

// ------------------------------------------------------------------ raster helpers
struct V2d {
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
V2d spline(const std::vector<V2d>& p, double u, bool deriv) {  // SplineEval, Spline.hxx:183-231
  const auto n = static_cast<int64_t>(p.size());
  const double x = static_cast<double>(n - 1) * u;
  const int32_t index = static_cast<int32_t>(x);
  const double t = x - std::floor(x);
  auto at = [&](int32_t i) -> const V2d& {
    if (i < 0) return p.front();
    if (i >= static_cast<int32_t>(n)) return p.back();
    return p[static_cast<size_t>(i)];
  };
  const V2d &a = at(index - 1), &b = at(index), &c = at(index + 1), &d = at(index + 2);
  if (deriv) return {cr_der(a.x, b.x, c.x, d.x, t), cr_der(a.y, b.y, c.y, d.y, t)};
  return {cr_pos(a.x, b.x, c.x, d.x, t), cr_pos(a.y, b.y, c.y, d.y, t)};
}
V2d normalized(const V2d& v) {
  const double n = v.x * v.x + v.y * v.y;
  if (n > 0.0) {
    const double r = std::sqrt(n);
    return {v.x / r, v.y / r};
  }
  return v;
}

int64_t snap(float v) { return static_cast<int64_t>(std::nearbyint(static_cast<double>(v) * 256.0)); }

// bilinear sample of a GL texture (bottom-up rows), clamp to edge
float sample_tex(const TexEntry& e, float u, float t) {
  const float s = u * static_cast<float>(e.cols) - 0.5f;
  const float r = t * static_cast<float>(e.rows) - 0.5f;
  const float fs = std::floor(s), fr = std::floor(r);
  const float a = s - fs, c = r - fr;
  auto cl = [](int64_t v, int32_t n) { return static_cast<int32_t>(v < 0 ? 0 : (v >= n ? n - 1 : v)); };
  const int32_t i0 = cl(static_cast<int64_t>(fs), e.cols), i1 = cl(static_cast<int64_t>(fs) + 1, e.cols);
  const int32_t k0 = cl(static_cast<int64_t>(fr), e.rows), k1 = cl(static_cast<int64_t>(fr) + 1, e.rows);
  const float* g = e.gl.data();
  return (g[k0 * e.cols + i0] * (1.0f - a) + g[k0 * e.cols + i1] * a) * (1.0f - c) +
         (g[k1 * e.cols + i0] * (1.0f - a) + g[k1 * e.cols + i1] * a) * c;
}

}  // namespace

struct orc_gtbrush {
  double radius = 0.0;
  double paint[2][3] = {{0, 0, 0}, {0, 0, 0}};
  double thicknessScale = 1.0;
  std::vector<float> warped;  // the canvas-sized warped brush texture (R32F)
  int32_t wrows = 0, wcols = 0;
  int32_t last_texture = -1;
};

extern "C" {

void orc_glsl_compose(int64_t npix, const float* K4, const float* S4, const float* R4,
                      float* out4) {
  for (int64_t p = 0; p < npix; p++) {
    const float* k = K4 + 4 * p;
    const float* s = S4 + 4 * p;
    const float* r0 = R4 + 4 * p;
    const float d = k[3];
    float r[3] = {r0[0], r0[1], r0[2]};
    if (std::fabs(d) > 10e-6f) glsl_reflectance(k, s, r0, d, r);
    out4[4 * p + 0] = r[0];
    out4[4 * p + 1] = r[1];
    out4[4 * p + 2] = r[2];
    out4[4 * p + 3] = 1.0f;
  }
}

void orc_glsl_dry_step(int64_t npix, float* K4, const float* S4, float* R4, float portion) {
  for (int64_t p = 0; p < npix; p++) {
    float* k = K4 + 4 * p;
    const float* s = S4 + 4 * p;
    float* r0 = R4 + 4 * p;
    const float d = k[3];
    const float vRemaining = std::fmax(0.0f, d - portion);  // DryingStep.compute.glsl:137-138
    const float vLeaving = d - vRemaining;
    float r[3] = {r0[0], r0[1], r0[2]};
    if (std::fabs(vLeaving) > 10e-6f) glsl_reflectance(k, s, r0, vLeaving, r);
    r0[0] = r[0];
    r0[1] = r[1];
    r0[2] = r[2];
    r0[3] = 1.0f;
    k[3] = vRemaining;
  }
}

orc_tdict* orc_tdict_create(uint32_t seed) {
  auto* d = new orc_tdict();
  d->gen.seed(seed);
  return d;
}
void orc_tdict_destroy(orc_tdict* d) { delete d; }

// Entry `index`'s GL texture (rows x cols floats, GL row order): copies it into `out` when
// not NULL; returns 0, or -1 for an index out of range.
int32_t orc_tdict_texture(const orc_tdict* d, int32_t index, int32_t* rows, int32_t* cols,
                          float* out) {
  if (index < 0 || static_cast<size_t>(index) >= d->entries.size()) return -1;
  const TexEntry& e = d->entries[static_cast<size_t>(index)];
  *rows = e.rows;
  *cols = e.cols;
  if (out) std::memcpy(out, e.gl.data(), e.gl.size() * sizeof(float));
  return 0;
}

// createBrushTexturesFromFolder (TextureBrushDictionary.cxx:112-126): loadHeightMap normalises
// min-max, the GPU copy is normalised again, flipped to GL rows and converted to float
int32_t orc_tdict_add(orc_tdict* d, uint32_t radius_class, uint32_t length_class,
                      const double* height, int32_t rows, int32_t cols) {
  std::vector<double> v(height, height + static_cast<size_t>(rows) * cols);
  normalize_minmax(v);
  normalize_minmax(v);
  TexEntry e;
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
  return static_cast<int32_t>(d->entries.size() - 1);
}

// lookup (TextureBrushDictionary.cxx:25-69). The reference scans length classes with the
// count of size classes (:46); here the scan stops at the chosen size's length classes. Its
// random pick (std::random_device) is a seeded std::mt19937 draw mapped by multiply-shift.
int32_t orc_tdict_lookup(orc_tdict* d, const double* path, int32_t n, double brushSize) {
  if (d->entries.empty() || n < 1) return -1;
  double length = 0.0;
  for (int32_t i = 0; i + 1 < n; i++) {
    const double dx = path[2 * i] - path[2 * (i + 1)], dy = path[2 * i + 1] - path[2 * (i + 1) + 1];
    length += std::sqrt(dx * dx + dy * dy);
  }
  const Classes c = make_classes(d);
  uint32_t i0 = 0, i1 = 1;
  double mr = c.avgSizes[0];
  for (uint32_t i = 0; i < c.avgSizes.size(); i++) {
    const double dd = std::fabs(c.avgSizes[i] - brushSize);
    if (dd < mr) {
      mr = dd;
      i0 = i;
    }
  }
  double ml = c.avgLengths[i0][0];
  for (uint32_t i = 0; i < c.avgSizes.size() && i < c.avgLengths[i0].size(); i++) {
    const double dd = std::fabs(c.avgLengths[i0][i] - length);
    if (dd < ml) {
      ml = dd;
      i1 = i;
    }
  }
  if (i1 >= c.byClass[i0].size() || c.byClass[i0][i1].empty()) return -1;  // "no candidate found"
  const auto& cand = c.byClass[i0][i1];
  const uint64_t r = static_cast<uint64_t>(d->gen()) * static_cast<uint64_t>(cand.size());
  return cand[static_cast<size_t>(r >> 32)];
}

orc_gtbrush* orc_gtbrush_create(void) {
  auto* b = new orc_gtbrush();
  orc_gtbrush_set_radius(b, 5.0);  // TextureBrushGpu.cxx:45
  return b;
}
void orc_gtbrush_destroy(orc_gtbrush* b) { delete b; }
void orc_gtbrush_set_radius(orc_gtbrush* b, double radius) {  // TextureBrushGpu.cxx:48-61
  if (!(std::fabs(b->radius - radius) < 0.5)) b->radius = radius;
}
void orc_gtbrush_dip(orc_gtbrush* b, const double K[3], const double S[3]) {
  for (int i = 0; i < 3; i++) {
    b->paint[0][i] = K[i];
    b->paint[1][i] = S[i];
  }
}
void orc_gtbrush_set_thickness_scale(orc_gtbrush* b, double s) { b->thicknessScale = s; }
int32_t orc_gtbrush_last_texture(const orc_gtbrush* b) { return b->last_texture; }
const float* orc_gtbrush_warped(const orc_gtbrush* b) { return b->warped.data(); }

// TextureBrushGpu::paintStroke(path, CanvasGpu&) (TextureBrushGpu.cxx:74-167), smudge off.
// Returns 0, or -1 when the dictionary has no candidate.
int32_t orc_gtbrush_paint_stroke(orc_gtbrush* b, orc_tdict* dict, int32_t rows, int32_t cols,
                                 float* K4, float* S4, const double* path, int32_t n) {
  if (n < 2) return 0;  // the reference's guard is commented out; fewer points are undefined
  std::vector<V2d> v(static_cast<size_t>(n));
  for (int32_t i = 0; i < n; i++) v[static_cast<size_t>(i)] = {path[2 * i], path[2 * i + 1]};
  V2d bmin = v.front(), bmax = v.front();
  for (const V2d& p : v) {
    bmin.x = std::fmin(bmin.x, p.x);
    bmin.y = std::fmin(bmin.y, p.y);
    bmax.x = std::fmax(bmax.x, p.x);
    bmax.y = std::fmax(bmax.y, p.y);
  }
  bmin.x = std::fmax(bmin.x - b->radius, 0.0);
  bmax.x = std::fmin(bmax.x + b->radius, static_cast<double>(cols - 1));
  bmin.y = std::fmax(bmin.y - b->radius, 0.0);
  bmax.y = std::fmin(bmax.y + b->radius, static_cast<double>(rows - 1));

  // generateWarpedTexture (:169-246)
  if (b->wrows != rows || b->wcols != cols) {
    b->warped.assign(static_cast<size_t>(rows) * cols, 0.0f);
    b->wrows = rows;
    b->wcols = cols;
  }
  std::vector<float> xy(static_cast<size_t>(4) * n), uv(static_cast<size_t>(4) * n);
  orc_gl_strip_vertices(path, n, b->radius, xy.data(), uv.data());
  std::vector<float> vx, vy, tu, tv;
  for (int32_t i = 0; i < 2 * n; i++) {
    vx.push_back(xy[static_cast<size_t>(2 * i)]);
    vy.push_back(xy[static_cast<size_t>(2 * i + 1)]);
    tu.push_back(uv[static_cast<size_t>(2 * i)]);
    tv.push_back(uv[static_cast<size_t>(2 * i + 1)]);
  }
  const int32_t tex = orc_tdict_lookup(dict, path, n, 2.0 * b->radius);
  if (tex < 0) return -1;
  b->last_texture = tex;
  const TexEntry& e = dict->entries[static_cast<size_t>(tex)];
  // window coordinates (ortho(0, cols, rows, 0) then the viewport: x, rows - y), snapped
  const int32_t nv = 2 * n;
  std::vector<int64_t> X(static_cast<size_t>(nv)), Y(static_cast<size_t>(nv));
  int64_t xmin = INT64_MAX, xmax = INT64_MIN, ymin = INT64_MAX, ymax = INT64_MIN;
  for (int32_t i = 0; i < nv; i++) {
    X[static_cast<size_t>(i)] = snap(vx[static_cast<size_t>(i)]);
    Y[static_cast<size_t>(i)] = snap(static_cast<float>(rows) - vy[static_cast<size_t>(i)]);
    xmin = std::min(xmin, X[static_cast<size_t>(i)]);
    xmax = std::max(xmax, X[static_cast<size_t>(i)]);
    ymin = std::min(ymin, Y[static_cast<size_t>(i)]);
    ymax = std::max(ymax, Y[static_cast<size_t>(i)]);
  }
  // canvas pixels whose centres can lie in the strip
  const int64_t px0 = std::max<int64_t>(0, (xmin - 128) / 256 - 1);
  const int64_t px1 = std::min<int64_t>(cols - 1, (xmax - 128) / 256 + 1);
  const int64_t wy0 = std::max<int64_t>(0, (ymin - 128) / 256 - 1);
  const int64_t wy1 = std::min<int64_t>(rows - 1, (ymax - 128) / 256 + 1);
  for (int64_t wy = wy0; wy <= wy1; wy++) {
    const int64_t y = rows - 1 - wy;  // canvas row of window row wy
    for (int64_t x = px0; x <= px1; x++) {
      const int64_t Px = 256 * x + 128, Py = 256 * wy + 128;
      for (int32_t k = nv - 3; k >= 0; k--) {  // the last triangle covering the centre wins
        int32_t ia = k, ib = k + 1, ic = k + 2;
        auto E = [&](int32_t a, int32_t bb, int64_t qx, int64_t qy) {
          return (X[static_cast<size_t>(bb)] - X[static_cast<size_t>(a)]) * (qy - Y[static_cast<size_t>(a)]) -
                 (Y[static_cast<size_t>(bb)] - Y[static_cast<size_t>(a)]) * (qx - X[static_cast<size_t>(a)]);
        };
        int64_t area = E(ia, ib, X[static_cast<size_t>(ic)], Y[static_cast<size_t>(ic)]);
        if (area == 0) continue;
        if (area < 0) {
          std::swap(ib, ic);
          area = -area;
        }
        auto topleft = [&](int32_t a, int32_t bb) {
          const int64_t ay = Y[static_cast<size_t>(a)], by = Y[static_cast<size_t>(bb)];
          return (ay == by && X[static_cast<size_t>(bb)] < X[static_cast<size_t>(a)]) || by < ay;
        };
        const int64_t w0 = E(ib, ic, Px, Py), w1 = E(ic, ia, Px, Py), w2 = E(ia, ib, Px, Py);
        const bool in0 = w0 > 0 || (w0 == 0 && topleft(ib, ic));
        const bool in1 = w1 > 0 || (w1 == 0 && topleft(ic, ia));
        const bool in2 = w2 > 0 || (w2 == 0 && topleft(ia, ib));
        if (!(in0 && in1 && in2)) continue;
        const float fa = static_cast<float>(area);
        const float l0 = static_cast<float>(w0) / fa, l1 = static_cast<float>(w1) / fa,
                    l2 = static_cast<float>(w2) / fa;
        const float u = l0 * tu[static_cast<size_t>(ia)] + l1 * tu[static_cast<size_t>(ib)] +
                        l2 * tu[static_cast<size_t>(ic)];
        const float t = l0 * tv[static_cast<size_t>(ia)] + l1 * tv[static_cast<size_t>(ib)] +
                        l2 * tv[static_cast<size_t>(ic)];
        b->warped[static_cast<size_t>(y) * cols + static_cast<size_t>(x)] = sample_tex(e, u, t);
        break;
      }
    }
  }

  // imprint and clear over the AOI's tiles
  const int32_t aoiW = static_cast<int32_t>(bmax.x - bmin.x) + 1;
  const int32_t aoiH = static_cast<int32_t>(bmax.y - bmin.y) + 1;
  if (aoiW <= 0 || aoiH <= 0) return 0;
  const int32_t x0 = static_cast<int32_t>(bmin.x), y0 = static_cast<int32_t>(bmin.y);
  const float Kb[3] = {static_cast<float>(b->paint[0][0]), static_cast<float>(b->paint[0][1]),
                       static_cast<float>(b->paint[0][2])};
  const float Sb[3] = {static_cast<float>(b->paint[1][0]), static_cast<float>(b->paint[1][1]),
                       static_cast<float>(b->paint[1][2])};
  orc_glsl_imprint(rows, cols, b->warped.data(), K4, S4, x0, y0, aoiW, aoiH, Kb, Sb,
                   static_cast<float>(b->thicknessScale));
  orc_glsl_clear(rows, cols, b->warped.data(), x0, y0, aoiW, aoiH);
  return 0;
}

// The triangle strip of generateWarpedTexture (TextureBrushGpu.cxx:183-207): for each of the
// n control points, u = i / (n - 1), the spine's Catmull-Rom point c and unit tangent t
// (SplineEval), and the vertices c + radius * (-t.y, t.x) then c - radius * (-t.y, t.x) as
// floats, with texture coordinates (u, 0) and (u, 1). xy and uv receive 2n pairs each.
void orc_gl_strip_vertices(const double* path, int32_t n, double radius, float* xy, float* uv) {
  std::vector<V2d> v(static_cast<size_t>(n));
  for (int32_t i = 0; i < n; i++) v[static_cast<size_t>(i)] = {path[2 * i], path[2 * i + 1]};
  for (int32_t i = 0; i < n; i++) {
    const double u = static_cast<double>(i) / static_cast<double>(n - 1);
    const V2d c = spline(v, u, false);
    const V2d t = normalized(spline(v, u, true));
    const V2d d = {-t.y, t.x};
    const V2d l = {c.x - radius * d.x, c.y - radius * d.y};
    const V2d r = {c.x + radius * d.x, c.y + radius * d.y};
    float* p = xy + 4 * i;
    float* q = uv + 4 * i;
    p[0] = static_cast<float>(r.x);
    p[1] = static_cast<float>(r.y);
    p[2] = static_cast<float>(l.x);
    p[3] = static_cast<float>(l.y);
    q[0] = static_cast<float>(u);
    q[1] = 0.0f;
    q[2] = static_cast<float>(u);
    q[3] = 1.0f;
  }
}

// PaintTextureFootprintOnCanvas.compute.glsl:17-53 over the area of interest (aoi_w x aoi_h
// pixels from (x0, y0), image coordinates), dispatched as whole 16 x 16 tiles: the pixels of
// those tiles that lie on the canvas mix the warped texture's paint volume into K4 / S4.
void orc_glsl_imprint(int32_t rows, int32_t cols, const float* warped, float* K4, float* S4,
                      int32_t x0, int32_t y0, int32_t aoi_w, int32_t aoi_h, const float Kb[3],
                      const float Sb[3], float scale) {
  if (aoi_w <= 0 || aoi_h <= 0) return;
  const int32_t x1 = x0 + (aoi_w + 15) / 16 * 16, y1 = y0 + (aoi_h + 15) / 16 * 16;
  for (int32_t y = std::max(y0, 0); y < std::min(y1, rows); y++)
    for (int32_t x = std::max(x0, 0); x < std::min(x1, cols); x++) {
      const size_t p = static_cast<size_t>(y) * cols + x;
      float* k = K4 + 4 * p;
      float* s = S4 + 4 * p;
      const float vCan = k[3];
      const float vTex = scale * warped[p];
      const float vSum = vCan + vTex;
      if (vSum < 10e-6f) continue;
      for (int c = 0; c < 3; c++) {
        k[c] = (vCan * k[c] + vTex * Kb[c]) / vSum;
        s[c] = (vCan * s[c] + vTex * Sb[c]) / vSum;
      }
      k[3] = vSum;
      s[3] = vTex > 0.0f ? vTex : vCan;
    }
}

// ClearTextureFootprint.compute.glsl over the same tiles.
void orc_glsl_clear(int32_t rows, int32_t cols, float* warped, int32_t x0, int32_t y0,
                    int32_t aoi_w, int32_t aoi_h) {
  if (aoi_w <= 0 || aoi_h <= 0) return;
  const int32_t x1 = x0 + (aoi_w + 15) / 16 * 16, y1 = y0 + (aoi_h + 15) / 16 * 16;
  for (int32_t y = std::max(y0, 0); y < std::min(y1, rows); y++)
    for (int32_t x = std::max(x0, 0); x < std::min(x1, cols); x++)
      warped[static_cast<size_t>(y) * cols + x] = 0.0f;
}

}  // extern "C"
