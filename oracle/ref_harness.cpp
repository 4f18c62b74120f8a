// ref_harness.cpp -- TEST INFRASTRUCTURE ONLY.
//
// Compiles lindemeier/painty's own header-only hot-path code, unmodified, from the reference
// checkout (include root passed by oracle/Makefile), against the repository's minimal Eigen
// and OpenCV stand-ins in oracle/ref_shim/, and exposes it through a C API (prefix ref_) that
// mirrors the oracle's (prefix orc_). Tests use it to pin the restated oracle bit for bit.
// It exists only where the reference checkout exists; nothing on the product path uses it.
//
// What is the reference's code here: KubelkaMunk.hxx, Math.hxx (coth), Spline.hxx,
// Color.hxx (CIEDE2000), image/Mat.hxx (Interpolate, PaddedMat), renderer/PaintLayer.hxx,
// Canvas.hxx, FootprintBrush.hxx, Renderer.hxx, mixer/src/PaintMixer.cxx (its Ceres fitting
// routines compiled against oracle/ref_shim/ceres, not run) and mixer/src/Serialization.cxx
// (palette JSON through oracle/ref_shim/nlohmann, the palette swatch image). What is the harness's: the footprint
// "image" source (painty::io::imRead below returns the registered full-size footprint),
// and the stroke loop of FootprintBrush::paintStroke, re-driven here over the reference's
// own CatmullRom/imprint because that loop reads path[SIZE_MAX] at i = 0
// (FootprintBrush.hxx:252).
#include <cmath>
#include <cstdint>
#include <cstring>
#include <sstream>
#include <string>
#include <vector>

#include "painty/core/Color.hxx"
#include "painty/core/KubelkaMunk.hxx"
#include "painty/core/Math.hxx"
#include "painty/core/Spline.hxx"
#include "painty/image/ColorExtraction.hxx"
#include "painty/image/Mat.hxx"
#include "painty/mixer/PaintMixer.hxx"
#include "painty/mixer/Serialization.hxx"
#include "painty/renderer/Canvas.hxx"
#include "painty/renderer/FootprintBrush.hxx"
#include "painty/renderer/PaintLayer.hxx"
#include "painty/renderer/Renderer.hxx"
#include "painty/renderer/TextureBrush.hxx"

using painty::vec2;
using painty::vec3;

namespace {
painty::Mat<double> g_footprint_full;
painty::Mat<double> g_texture;  // the thickness texture the next TextureBrush loads
}

namespace cv {
void shim_resize_bilinear(const Mat_<double>& src, Mat_<double>& dst, int rows, int cols) {
  Mat_<double> out(rows, cols);
  const double sy = static_cast<double>(src.rows) / static_cast<double>(rows);
  const double sx = static_cast<double>(src.cols) / static_cast<double>(cols);
  for (int i = 0; i < rows; i++)
    for (int j = 0; j < cols; j++) {
      const vec2 pos = {(static_cast<double>(j) + 0.5) * sx - 0.5,
                        (static_cast<double>(i) + 0.5) * sy - 0.5};
      out(i, j) = painty::Interpolate(src, pos);
    }
  dst = out;
}
}  // namespace cv

namespace painty {
namespace io {
void imRead(const std::string&, Mat<double>& gray, bool) { gray = g_footprint_full.clone(); }
}  // namespace io

// PaintMixer.cxx (linked for mixSinglePaint) also references the palette extraction of
// painty/image/src/ColorExtraction.cxx, which needs OpenCV's clustering; the oracle build never
// calls it.
void ExtractColorPaletteAharoni(const Mat<vec3>&, std::vector<vec3>&, uint32_t) {
  throw std::logic_error("ExtractColorPaletteAharoni is not part of the oracle build");
}

// The harness's stand-ins for the two out-of-line classes TextureBrush.hxx needs
// (painty/renderer/src/BrushStrokeSample.cxx, painty/image/src/TextureWarp.cxx load stroke
// samples from disk): the sample's thickness map is the registered texture.
TextureWarp::TextureWarp() {}
BrushStrokeSample::BrushStrokeSample(const std::string&) { _thickness_map = g_texture.clone(); }
const Mat<double>& BrushStrokeSample::getThicknessMap() const { return _thickness_map; }
}  // namespace painty

struct ref_canvas {
  painty::Canvas<vec3> c;
  ref_canvas(int r, int cc) : c(r, cc) {}
};
struct ref_tbrush {
  painty::TextureBrush<vec3> b;
  ref_tbrush() : b("sample") {}
};
struct ref_brush {
  painty::FootprintBrush<vec3> b;
  explicit ref_brush(double r) : b(r) {}
};

static vec3 v3(const double* p) { return vec3(p[0], p[1], p[2]); }

extern "C" {

double ref_coth(double x) { return painty::coth(x); }

void ref_compute_reflectance(const double K[3], const double S[3], const double R0[3],
                             double d, double out[3]) {
  const vec3 r = painty::ComputeReflectance<double, 3>(v3(K), v3(S), v3(R0), d);
  for (int i = 0; i < 3; i++) out[i] = r[i];
}

double ref_catmull_rom_1d(double p_1, double p0, double p1, double p2, double t) {
  return painty::CatmullRom(p_1, p0, p1, p2, t);
}

void ref_spline_catmull_rom(const double* pts, int32_t n, double u, double out[2]) {
  std::vector<vec2> v;
  for (int i = 0; i < n; i++) v.emplace_back(pts[2 * i], pts[2 * i + 1]);
  painty::SplineEval<std::vector<vec2>::const_iterator> s(v.cbegin(), v.cend());
  const vec2 r = s.catmullRom(u);
  out[0] = r[0];
  out[1] = r[1];
}

// The triangle strip of TextureBrushGpu::generateWarpedTexture (TextureBrushGpu.cxx:183-207)
// over painty's SplineEval. That loop sits in a .cxx built around prgl's GL objects, so the
// harness repeats its few lines of vertex arithmetic; the spline is painty's.
void ref_gl_strip_vertices(const double* pts, int32_t n, double radius, float* xy, float* uv) {
  std::vector<vec2> v;
  for (int i = 0; i < n; i++) v.emplace_back(pts[2 * i], pts[2 * i + 1]);
  painty::SplineEval<std::vector<vec2>::const_iterator> spine(v.cbegin(), v.cend());
  for (int32_t i = 0; i < n; i++) {
    const auto u = static_cast<double>(i) / static_cast<double>(v.size() - 1);
    const auto c = spine.catmullRom(u);
    auto t = spine.catmullRomDerivativeFirst(u).normalized();
    const vec2 d = {-t[1], t[0]};
    const vec2 l = c - radius * d;
    const vec2 r = c + radius * d;
    xy[4 * i + 0] = static_cast<float>(r[0U]);
    xy[4 * i + 1] = static_cast<float>(r[1U]);
    xy[4 * i + 2] = static_cast<float>(l[0U]);
    xy[4 * i + 3] = static_cast<float>(l[1U]);
    uv[4 * i + 0] = static_cast<float>(u);
    uv[4 * i + 1] = static_cast<float>(0.0);
    uv[4 * i + 2] = static_cast<float>(u);
    uv[4 * i + 3] = static_cast<float>(1.0);
  }
}

// PaintMixer::mixSinglePaint (painty/mixer/src/PaintMixer.cxx:327-355) over a palette of n
// paints (K, S: n x 3); 0, or -1 when painty throws.
int32_t ref_mix_single_paint(const double* weights, int32_t n, const double* K, const double* S,
                             double out_K[3], double out_S[3]) {
  painty::Palette palette(static_cast<size_t>(n));
  for (int32_t i = 0; i < n; i++)
    for (int c = 0; c < 3; c++) {
      palette[static_cast<size_t>(i)].K[c] = K[3 * i + c];
      palette[static_cast<size_t>(i)].S[c] = S[3 * i + c];
    }
  try {
    const painty::PaintMixer mixer(palette);
    const painty::PaintCoeff p =
      mixer.mixSinglePaint(std::vector<double>(weights, weights + n));
    for (int c = 0; c < 3; c++) {
      out_K[c] = p.K[c];
      out_S[c] = p.S[c];
    }
  } catch (...) {
    return -1;
  }
  return 0;
}

// LoadPalette (painty/mixer/src/Serialization.cxx:38-44) of a JSON text: the number of paints,
// their K and S (n x 3) copied out up to `cap` paints; -1 when painty throws.
int32_t ref_load_palette(const char* text, double* K, double* S, int32_t cap) {
  painty::Palette palette;
  try {
    std::istringstream in(text);
    painty::LoadPalette(in, palette);
  } catch (...) {
    return -1;
  }
  for (size_t i = 0; i < palette.size() && static_cast<int32_t>(i) < cap; i++)
    for (int c = 0; c < 3; c++) {
      K[3 * i + c] = palette[i].K[c];
      S[3 * i + c] = palette[i].S[c];
    }
  return static_cast<int32_t>(palette.size());
}

// VisualizePalette (Serialization.cxx:64-137) of n paints at `thickness`: 200 x 100n x 3
// doubles (sRGB) into `out`.
void ref_visualize_palette(const double* K, const double* S, int32_t n, double thickness,
                           double* out) {
  painty::Palette palette(static_cast<size_t>(n));
  for (int32_t i = 0; i < n; i++)
    for (int c = 0; c < 3; c++) {
      palette[static_cast<size_t>(i)].K[c] = K[3 * i + c];
      palette[static_cast<size_t>(i)].S[c] = S[3 * i + c];
    }
  const painty::Mat<vec3> img = painty::VisualizePalette(palette, thickness);
  for (int32_t y = 0; y < img.rows; y++)
    for (int32_t x = 0; x < img.cols; x++)
      for (int c = 0; c < 3; c++)
        out[(static_cast<size_t>(y) * img.cols + x) * 3 + c] = img(y, x)[c];
}

double ref_interpolate(const double* img, int32_t rows, int32_t cols, double x, double y) {
  painty::Mat<double> m(rows, cols);
  for (int i = 0; i < rows * cols; i++) m(i) = img[i];
  return painty::Interpolate(m, vec2(x, y));
}

void ref_rgb2lab(const double rgb[3], double lab[3]) {
  painty::ColorConverter<double> conv;
  vec3 out;
  conv.rgb2lab(v3(rgb), out);
  for (int i = 0; i < 3; i++) lab[i] = out[i];
}

double ref_ciede2000(const double a[3], const double b[3]) {
  return painty::ColorConverter<double>::ColorDifferenceCIEDE2000(v3(a), v3(b));
}

ref_canvas* ref_canvas_create(int32_t rows, int32_t cols) { return new ref_canvas(rows, cols); }
void ref_canvas_destroy(ref_canvas* c) { delete c; }

// which: 0 K (npix*3), 1 S, 2 V (npix), 3 R0 (npix*3), 4 h (npix)
void ref_canvas_get(ref_canvas* c, int32_t which, double* out) {
  auto& L = c->c.getPaintLayer();
  const int n = L.getRows() * L.getCols();
  for (int i = 0; i < n; i++) {
    switch (which) {
      case 0: for (int ch = 0; ch < 3; ch++) out[i * 3 + ch] = L.getK_buffer()(i)[ch]; break;
      case 1: for (int ch = 0; ch < 3; ch++) out[i * 3 + ch] = L.getS_buffer()(i)[ch]; break;
      case 2: out[i] = L.getV_buffer()(i); break;
      case 3: for (int ch = 0; ch < 3; ch++) out[i * 3 + ch] = c->c.getR0()(i)[ch]; break;
      case 4: out[i] = c->c.get_h()(i); break;
      default: break;
    }
  }
}

void ref_canvas_set(ref_canvas* c, int32_t which, const double* in) {
  auto& L = c->c.getPaintLayer();
  const int n = L.getRows() * L.getCols();
  for (int i = 0; i < n; i++) {
    switch (which) {
      case 0: L.getK_buffer()(i) = v3(in + 3 * i); break;
      case 1: L.getS_buffer()(i) = v3(in + 3 * i); break;
      case 2: L.getV_buffer()(i) = in[i]; break;
      case 3: c->c.getR0()(i) = v3(in + 3 * i); break;
      case 4: c->c.get_h()(i) = in[i]; break;
      default: break;
    }
  }
}

void ref_canvas_dry(ref_canvas* c) { c->c.dryCanvas(); }

void ref_canvas_compose(ref_canvas* c, double* out) {
  painty::Renderer<vec3> r;
  const auto R = r.compose(c->c);
  for (size_t i = 0; i < R.total(); i++)
    for (int ch = 0; ch < 3; ch++) out[i * 3 + ch] = R(static_cast<int>(i))[ch];
}

void ref_canvas_render(ref_canvas* c, double* out) {
  painty::Renderer<vec3> r;
  const auto R = r.render(c->c);
  for (size_t i = 0; i < R.total(); i++)
    for (int ch = 0; ch < 3; ch++) out[i * 3 + ch] = R(static_cast<int>(i))[ch];
}

ref_brush* ref_brush_create(double radius, const double* fp, int32_t fh, int32_t fw) {
  g_footprint_full = painty::Mat<double>(fh, fw);
  for (int i = 0; i < fh * fw; i++) g_footprint_full(i) = fp[i];
  return new ref_brush(radius);
}
void ref_brush_destroy(ref_brush* b) { delete b; }
void ref_brush_set_radius(ref_brush* b, double r) { b->b.setRadius(r); }
void ref_brush_set_rates(ref_brush* b, double pickup, double deposit) {
  b->b.setPickupRate(pickup);
  b->b.setDepositionRate(deposit);
}
void ref_brush_set_snapshot(ref_brush* b, int32_t use) { b->b.setUseSnapshotBuffer(use != 0); }
void ref_brush_dip(ref_brush* b, const double K[3], const double S[3]) {
  b->b.dip({v3(K), v3(S)});
}
void ref_brush_update_snapshot(ref_brush* b, ref_canvas* c) { b->b.updateSnapshot(c->c); }
void ref_brush_imprint(ref_brush* b, ref_canvas* c, double cx, double cy, double theta) {
  b->b.imprint(vec2(cx, cy), theta, c->c);
}
void ref_brush_stamps(ref_brush* b, ref_canvas* c, const double* s, int64_t n) {
  for (int64_t i = 0; i < n; i++) b->b.imprint(vec2(s[3 * i], s[3 * i + 1]), s[3 * i + 2], c->c);
}

// FootprintBrush.hxx:251-267 with painty's CatmullRom / CatmullRomDerivativeFirst and
// imprint, path[0] for the predecessor of the first segment.
int64_t ref_brush_paint_stroke(ref_brush* b, ref_canvas* c, const double* path, int32_t n) {
  if (n < 2) return 0;
  std::vector<vec2> p;
  for (int i = 0; i < n; i++) p.emplace_back(path[2 * i], path[2 * i + 1]);
  int64_t count = 0;
  for (size_t i = 0; i + 1 < p.size(); i++) {
    const auto p_pre = p[i == 0 ? 0 : i - 1];
    const auto p_0 = p[i];
    const auto p_1 = p[i + 1];
    const auto p_next = p[std::min(i + 2, p.size() - 1)];
    const auto dist = (p_1 - p_0).norm();
    for (int32_t pd = 1; pd <= static_cast<int32_t>(dist); pd++) {
      const auto t = static_cast<double>(pd) / dist;
      const auto dir = painty::CatmullRomDerivativeFirst(p_pre, p_0, p_1, p_next, t);
      b->b.imprint(painty::CatmullRom(p_pre, p_0, p_1, p_next, t), std::atan2(dir[1], dir[0]),
                   c->c);
      count++;
    }
  }
  return count;
}

// F (footprint side) and S (pickup-map side)
void ref_brush_info(ref_brush* b, int32_t* F, int32_t* S) {
  *F = b->b.getFootprint().rows;
  *S = b->b.getPickupMap().getRows();
}
void ref_brush_footprint(ref_brush* b, double* out) {
  const auto& f = b->b.getFootprint();
  for (size_t i = 0; i < f.total(); i++) out[i] = f(static_cast<int>(i));
}
// which: 0 K (S*S*3), 1 S, 2 V
void ref_brush_pickup(ref_brush* b, int32_t which, double* out) {
  const auto& L = b->b.getPickupMap();
  const int n = L.getRows() * L.getCols();
  for (int i = 0; i < n; i++) {
    switch (which) {
      case 0: for (int ch = 0; ch < 3; ch++) out[i * 3 + ch] = L.getK_buffer()(i)[ch]; break;
      case 1: for (int ch = 0; ch < 3; ch++) out[i * 3 + ch] = L.getS_buffer()(i)[ch]; break;
      case 2: out[i] = L.getV_buffer()(i); break;
      default: break;
    }
  }
}

// TextureBrush<vec3> (TextureBrush.hxx) with the registered thickness texture
ref_tbrush* ref_tbrush_create(const double* tex, int32_t th, int32_t tw) {
  g_texture = painty::Mat<double>(th, tw);
  for (int32_t i = 0; i < th; i++)
    for (int32_t j = 0; j < tw; j++) g_texture(i, j) = tex[static_cast<size_t>(i) * tw + j];
  return new ref_tbrush();
}
void ref_tbrush_destroy(ref_tbrush* b) { delete b; }
void ref_tbrush_set_radius(ref_tbrush* b, double r) { b->b.setRadius(r); }
void ref_tbrush_dip(ref_tbrush* b, const double K[3], const double S[3]) {
  b->b.dip({v3(K), v3(S)});
}
void ref_tbrush_set_smudge(ref_tbrush* b, int32_t on) { b->b.enableSmudge(on != 0); }
void ref_tbrush_set_thickness_scale(ref_tbrush* b, double s) { b->b.setThicknessScale(s); }
void ref_tbrush_paint_stroke(ref_tbrush* b, ref_canvas* c, const double* path, int32_t n) {
  std::vector<vec2> v;
  for (int32_t i = 0; i < n; i++) v.emplace_back(path[2 * i], path[2 * i + 1]);
  b->b.paintStroke(v, c->c);
}

}  // extern "C"
