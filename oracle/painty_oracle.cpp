// painty_oracle.cpp -- CPU oracle (test infrastructure only; see painty_oracle.h).
//
// Double precision, the reference's loop order and branches, no FMA contraction
// (built with -ffp-contract=off so x86-64 and aarch64 give the same bits).
#include "painty_oracle.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>
#include <thread>
#include <vector>

namespace {

constexpr double kMinVolume = 0.001;  // FootprintBrush.hxx:26

// ---------------------------------------------------------------- core math
// Math.hxx:157-169
double coth_ref(double x) {
  if (x > 20.0) return 1.0;
  if (std::fabs(x) > 0.0) {
    const double res = std::cosh(x) / std::sinh(x);
    return std::isnan(res) ? 1.0 : res;
  }
  return std::numeric_limits<double>::infinity();
}

// KubelkaMunk.hxx:25-83, one channel at a time (the reference's loops are per channel and
// independent, so evaluating channel by channel gives the same bits).
void reflectance_ref(const double* K, const double* S_in, const double* R0, double d,
                     double* out) {
  const double eps = std::numeric_limits<double>::epsilon() * 10000.0;
  if (std::fabs(d) < eps) {
    for (int i = 0; i < 3; i++) out[i] = R0[i];
    return;
  }
  for (int i = 0; i < 3; i++) {
    const double S = (std::fabs(S_in[i]) > eps) ? S_in[i] : 0.00000000001;
    const double K_S = K[i] / S;
    const double a = 1.0 + K_S;
    const double asq = a * a;
    const double v = asq - 1.0;
    const double b = (v < 0.0) ? 0.0 : std::sqrt(v);
    const double bSh = b * S * d;
    const double bcoth = b * coth_ref(bSh);
    out[i] = (1.0 - R0[i] * (a - bcoth)) / (a - R0[i] + bcoth);
  }
}

// FP64 oracle. x*coth(x), sinh(x)/x and cosh(x) by their Taylor series below |x| = 1e-3
// (next terms below 1e-20 relative); closed forms through exp(-|x|) above, which stay finite
// for any x. Finite for K = 0, where the reference's b*coth(bSh) is 0*inf = NaN.
//   R = (1 - R0 (a - b coth x)) / (a - R0 + b coth x),  b coth x = (x coth x) / (S d)
//   T = b / (a sinh x + b cosh x)
void km_fp64(const double* K, const double* S_in, const double* R0, double d, double* R,
             double* T) {
  const double eps = std::numeric_limits<double>::epsilon() * 10000.0;
  for (int i = 0; i < 3; i++) {
    if (std::fabs(d) < eps) {
      R[i] = R0[i];
      T[i] = 1.0;
      continue;
    }
    const double S = (std::fabs(S_in[i]) > eps) ? S_in[i] : 0.00000000001;
    const double q = K[i] / S;
    const double a = 1.0 + q;
    const double bb = q * (2.0 + q);  // a^2 - 1 without cancellation
    const double b = bb > 0.0 ? std::sqrt(bb) : 0.0;
    const double x = b * S * d;
    const double ax = std::fabs(x);
    double bc, t;
    if (ax < 1e-3) {
      const double x2 = x * x;
      const double g = 1.0 + x2 / 3.0 - x2 * x2 / 45.0 + 2.0 * x2 * x2 * x2 / 945.0;
      const double shc = 1.0 + x2 / 6.0 + x2 * x2 / 120.0;
      const double ch = 1.0 + x2 / 2.0 + x2 * x2 / 24.0;
      bc = g / (S * d);
      t = 1.0 / (a * S * d * shc + ch);
    } else {
      const double e2 = std::exp(-2.0 * ax);
      const double g = ax * (1.0 + e2) / (1.0 - e2);
      bc = g / (S * d);
      const double e1 = std::exp(-ax);
      const double den = a * (1.0 - e1 * e1) + b * (1.0 + e1 * e1);
      t = den > 0.0 ? 2.0 * b * e1 / den : 0.0;
    }
    R[i] = (1.0 - R0[i] * (a - bc)) / (a - R0[i] + bc);
    T[i] = t;
  }
}

// Spline.hxx:27-47
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

// Spline.hxx:49-73
double catmull_rom_deriv(double p_1, double p0, double p1, double p2, double t) {
  constexpr double tau = 0.5;
  const double t2 = t * t;
  const double b1 = tau * (-3.0 * t2 + 4.0 * t - 1.0);
  const double b2 = -t * (-2.0 * tau + 3.0 * (tau - 2.0) * t + 6.0);
  const double b3 = (t - 1.0) * (3.0 * (tau - 2.0) * t - tau);
  const double b4 = tau * t * (3.0 * t - 2.0);
  return p_1 * b1 + p0 * b2 + p1 * b3 + p2 * b4;
}

// OpenCV BORDER_REFLECT as documented: "fedcba|abcdefgh|hgfedcb".
int border_reflect(int p, int len) {
  if (len == 1) return 0;
  while (p < 0 || p >= len) {
    if (p < 0)
      p = -p - 1;
    else
      p = len - 1 - (p - len);
  }
  return p;
}

// Mat.hxx:68-103 (single-channel branch)
double interpolate(const double* in, int rows, int cols, double px, double py) {
  const int x = static_cast<int>(std::floor(px));
  const int y = static_cast<int>(std::floor(py));
  const int x0 = border_reflect(x, cols);
  const int x1 = border_reflect(x + 1, cols);
  const int y0 = border_reflect(y, rows);
  const int y1 = border_reflect(y + 1, rows);
  const double a = px - static_cast<double>(x);
  const double c = py - static_cast<double>(y);
  return (in[y0 * cols + x0] * (1.0 - a) + in[y0 * cols + x1] * a) * (1.0 - c) +
         (in[y1 * cols + x0] * (1.0 - a) + in[y1 * cols + x1] * a) * c;
}

void resample(const double* src, int rows, int cols, int out_rows, int out_cols,
              double* out) {
  const double sy = static_cast<double>(rows) / static_cast<double>(out_rows);
  const double sx = static_cast<double>(cols) / static_cast<double>(out_cols);
  for (int i = 0; i < out_rows; i++) {
    for (int j = 0; j < out_cols; j++) {
      const double y = (static_cast<double>(i) + 0.5) * sy - 0.5;
      const double x = (static_cast<double>(j) + 0.5) * sx - 0.5;
      out[i * out_cols + j] = interpolate(src, rows, cols, x, y);
    }
  }
}

// ---------------------------------------------------------------- layers
// PaintLayer.hxx:21-145: K, S (vec3 per cell) and V per cell.
struct Layer {
  int rows = 0, cols = 0;
  std::vector<double> K, S, V;
  void resize(int r, int c) {
    rows = r;
    cols = c;
    K.assign(static_cast<size_t>(r) * c * 3, 0.0);
    S.assign(static_cast<size_t>(r) * c * 3, 0.0);
    V.assign(static_cast<size_t>(r) * c, 0.0);
  }
  void clear() {  // PaintLayer.hxx:67-73
    std::fill(K.begin(), K.end(), 0.0);
    std::fill(S.begin(), S.end(), 0.0);
    std::fill(V.begin(), V.end(), 0.0);
  }
  void copy_to(Layer& o) const {  // PaintLayer.hxx:102-110
    if (o.rows != rows || o.cols != cols) o.resize(rows, cols);
    o.K = K;
    o.S = S;
    o.V = V;
  }
  size_t idx(int row, int col) const { return static_cast<size_t>(row) * cols + col; }
};

}  // namespace

// ---------------------------------------------------------------- objects
struct orc_canvas {
  Layer wet;
  std::vector<double> R0, h;
};

struct orc_brush {
  double radius = 0.0;      // FootprintBrush.hxx:437
  int sizeMap = 0;          // :443
  int F = 0;                // _footprint.rows == _footprint.cols
  std::vector<double> footprint;
  std::vector<double> full;  // full-size footprint (stands in for the footprint PNG)
  int fh = 0, fw = 0;
  Layer pickup;
  Layer snapshot;
  bool useSnapshot = true;        // :477
  double capacity = 1.0;          // :483
  double pickupRate = 0.9;        // :489
  double depositionRate = 0.05;   // :495
  double paintK[3] = {0, 0, 0};   // :501 (uninitialised in the reference until dip())
  double paintS[3] = {0, 0, 0};
};

namespace {

// FootprintBrush.hxx:46-63
void set_radius(orc_brush* b, double radius) {
  constexpr double Eps = 0.5;
  if (!(std::fabs(b->radius - radius) < Eps)) {
    b->radius = radius;
    const int width = static_cast<int>(2.0 * std::ceil(radius) + 1.0);
    b->sizeMap = static_cast<int>(std::ceil(std::sqrt(2.0) * width));
    const int pad = (b->sizeMap - width) / 2;
    std::vector<double> scaled(static_cast<size_t>(width) * width);
    resample(b->full.data(), b->fh, b->fw, width, width, scaled.data());
    b->F = width + 2 * pad;  // PaddedMat, Mat.hxx:115-129
    b->footprint.assign(static_cast<size_t>(b->F) * b->F, 0.0);
    for (int i = 0; i < width; i++)
      for (int j = 0; j < width; j++)
        b->footprint[static_cast<size_t>(i + pad) * b->F + (j + pad)] =
          scaled[static_cast<size_t>(i) * width + j];
    b->pickup.resize(b->sizeMap, b->sizeMap);
    b->pickup.clear();
  }
}

// Footprint height at a pickup-map cell. The pickup map is sizeMap wide; the footprint is
// F = width + 2*((sizeMap - width)/2) wide, one less than sizeMap when sizeMap - width is
// odd. For such cells the reference reads past the footprint row or buffer
// (FootprintBrush.hxx:352, 396); the padding value 0 is the evident intent and is used here.
double footprint_at(const orc_brush* b, int my, int mx) {
  if (my >= b->F || mx >= b->F) return 0.0;
  return b->footprint[static_cast<size_t>(my) * b->F + mx];
}

// FootprintBrush.hxx:331-340, channel-wise
inline void blend3(double v_a, const double* a, double v_b, const double* b, double* res) {
  const double vTotal = v_a + v_b;
  if (vTotal > kMinVolume) {
    for (int i = 0; i < 3; i++) res[i] = (v_a * a[i] + v_b * b[i]) / vTotal;
  } else {
    for (int i = 0; i < 3; i++) res[i] = a[i];
  }
}

// FootprintBrush.hxx:278-319
void update_snapshot_ring(orc_brush* b, const orc_canvas* c, double cx, double cy) {
  const Layer& layer = c->wet;
  if (layer.cols != b->snapshot.cols || layer.rows != b->snapshot.rows) {
    layer.copy_to(b->snapshot);
  }
  const int hr = (b->F - 1) / 2;
  const int wr = (b->F - 1) / 2;
  const int tlx = static_cast<int>(cx - wr), tly = static_cast<int>(cy - hr);
  const int brx = static_cast<int>(cx + wr), bry = static_cast<int>(cy + hr);
  const int tlax = std::max(static_cast<int>(cx - wr - b->radius), 0);
  const int tlay = std::max(static_cast<int>(cy - hr - b->radius), 0);
  const int brax = std::min(static_cast<int>(cx + wr + b->radius), layer.cols - 1);
  const int bray = std::min(static_cast<int>(cy + hr + b->radius), layer.rows - 1);
  for (int row = tlay; row <= bray; row++) {
    for (int col = tlax; col <= brax; col++) {
      if (row > tly && row < bry && col > tlx && col < brx) continue;
      const size_t i = layer.idx(row, col);
      for (int ch = 0; ch < 3; ch++) {
        b->snapshot.K[i * 3 + ch] = layer.K[i * 3 + ch];
        b->snapshot.S[i * 3 + ch] = layer.S[i * 3 + ch];
      }
      b->snapshot.V[i] = layer.V[i];
    }
  }
}

// FootprintBrush.hxx:349-384
void pickup_paint(orc_brush* b, int xc, int yc, int mx, int my, Layer& src) {
  const double fp = footprint_at(b, my, mx);
  if (fp > 0.0) {
    const size_t m = b->pickup.idx(my, mx);
    const size_t p = src.idx(yc, xc);
    const double v_pickupIs = b->pickup.V[m];
    const double v_canvasIs = src.V[p];
    const double v_canvasLeave = b->pickupRate * v_canvasIs * fp;
    if (v_canvasLeave > kMinVolume) {
      src.V[p] = v_canvasIs - v_canvasLeave;
      double k[3], s[3];
      blend3(v_pickupIs, &b->pickup.K[m * 3], v_canvasLeave, &src.K[p * 3], k);
      blend3(v_pickupIs, &b->pickup.S[m * 3], v_canvasLeave, &src.S[p * 3], s);
      for (int ch = 0; ch < 3; ch++) {
        b->pickup.K[m * 3 + ch] = k[ch];
        b->pickup.S[m * 3 + ch] = s[ch];
      }
      b->pickup.V[m] = v_pickupIs + v_canvasLeave;
    }
  }
}

// FootprintBrush.hxx:393-431
void deposit_paint(orc_brush* b, int xc, int yc, int mx, int my, Layer& dst) {
  const double fp = footprint_at(b, my, mx);
  if (fp > 0.0) {
    const size_t m = b->pickup.idx(my, mx);
    const size_t p = dst.idx(yc, xc);
    const double v_pickupIs = b->pickup.V[m];
    const double v_pickupFree = std::max(0.0, b->capacity - v_pickupIs);
    double ksrc[3], ssrc[3];
    blend3(v_pickupIs, &b->pickup.K[m * 3], v_pickupFree, b->paintK, ksrc);
    blend3(v_pickupIs, &b->pickup.S[m * 3], v_pickupFree, b->paintS, ssrc);
    const double v_pickupLeave = b->depositionRate * v_pickupIs * fp;
    b->pickup.V[m] = v_pickupIs - v_pickupLeave;
    const double v_canvasIs = dst.V[p];
    const double v_Blend = b->capacity * fp;
    double k[3], s[3];
    blend3(v_Blend, ksrc, v_canvasIs, &dst.K[p * 3], k);
    blend3(v_Blend, ssrc, v_canvasIs, &dst.S[p * 3], s);
    for (int ch = 0; ch < 3; ch++) {
      dst.K[p * 3 + ch] = k[ch];
      dst.S[p * 3 + ch] = s[ch];
    }
    dst.V[p] = v_Blend + v_canvasIs;
  }
}

// FootprintBrush.hxx:73-143. Canvas::checkDry (Canvas.hxx:123-155) only writes the time
// map unless a full drying time has elapsed between two stamps; it is left out.
void imprint(orc_brush* b, orc_canvas* c, double cx, double cy, double theta) {
  const int h = b->F, w = b->F;
  const int hr = (h - 1) / 2;
  const int wr = (w - 1) / 2;
  if (b->useSnapshot) update_snapshot_ring(b, c, cx, cy);
  Layer& src = b->useSnapshot ? b->snapshot : c->wet;
  const double cosTheta = std::cos(-theta);
  const double sinTheta = std::sin(-theta);
  for (int row = -hr; row <= hr; row++) {
    for (int col = -wr; col <= wr; col++) {
      const int xc = static_cast<int>(col + cx);
      const int yc = static_cast<int>(row + cy);
      const double rotatedCol = col * cosTheta - row * sinTheta;
      const double rotatedRow = col * sinTheta + row * cosTheta;
      const int mx = static_cast<int>(std::round(rotatedCol + wr));
      const int my = static_cast<int>(std::round(rotatedRow + hr));
      if (yc < 0 || xc < 0 || xc >= c->wet.cols || yc >= c->wet.rows) continue;
      if (my < 0 || mx < 0 || mx >= b->sizeMap || my >= b->sizeMap) continue;
      pickup_paint(b, xc, yc, mx, my, src);
      deposit_paint(b, xc, yc, mx, my, c->wet);
    }
  }
}

// FootprintBrush.hxx:206-268 with chord spacing as a parameter (1.0 reproduces the
// reference). At i = 0 the reference's std::max(i - 1UL, 0UL) wraps around (:252); the
// evident intent, path[0], is used.
template <class Fn>
int64_t for_each_stroke_stamp(const double* path, int n, double spacing, Fn&& fn) {
  int64_t count = 0;
  if (n < 2) return 0;
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
      const double cxs = catmull_rom(pp[0], p0[0], p1[0], pn[0], t);
      const double cys = catmull_rom(pp[1], p0[1], p1[1], pn[1], t);
      fn(cxs, cys, std::atan2(diry, dirx));
      count++;
    }
  }
  return count;
}

// Color.hxx:186-198 (RGB2XYZ_MATRIX, sRGB D65) and :77-81 with the D65 white (:49-51)
void rgb2lab(const double* rgb, double* lab) {
  const double X = 0.4124564 * rgb[0] + 0.3575761 * rgb[1] + 0.1804375 * rgb[2];
  const double Y = 0.2126729 * rgb[0] + 0.7151522 * rgb[1] + 0.0721750 * rgb[2];
  const double Z = 0.0193339 * rgb[0] + 0.1191920 * rgb[1] + 0.9503041 * rgb[2];
  auto f = [](double t) {
    return (t > std::pow(6. / 29., 3.)) ? std::pow(t, 1. / 3.)
                                        : (1. / 3.) * std::pow(29. / 6., 2.) * t + (4. / 29.);
  };
  const double wx = 0.95047, wy = 1.0, wz = 1.08883;
  lab[0] = 116. * f(Y / wy) - 16.;
  lab[1] = 500. * (f(X / wx) - f(Y / wy));
  lab[2] = 200. * (f(Y / wy) - f(Z / wz));
}

// CIEDE2000 (Sharma, Wu, Dalal 2005), with painty's conventions for hue wrap and zero
// chroma (Color.hxx:658-763).
double ciede2000(const double* l1, const double* l2) {
  const double pi = 3.14159265358979323846;
  const double eps = std::numeric_limits<double>::epsilon() * 1000.0;
  const double C1 = std::sqrt(l1[1] * l1[1] + l1[2] * l1[2]);
  const double C2 = std::sqrt(l2[1] * l2[1] + l2[2] * l2[2]);
  const double Cm = (C1 + C2) / 2.;
  const double Cm7 = std::pow(Cm, 7.);
  const double G = 0.5 * (1. - std::sqrt(Cm7 / (Cm7 + std::pow(25., 7.))));
  const double a1 = (1. + G) * l1[1];
  const double a2 = (1. + G) * l2[1];
  const double Cp1 = std::sqrt(a1 * a1 + l1[2] * l1[2]);
  const double Cp2 = std::sqrt(a2 * a2 + l2[2] * l2[2]);
  const double Cprod = Cp1 * Cp2;
  double h1 = std::atan2(l1[2], a1);
  if (h1 < 0) h1 += 2. * pi;
  double h2 = std::atan2(l2[2], a2);
  if (h2 < 0) h2 += 2. * pi;
  if (std::fabs(std::fabs(a2) + std::fabs(l2[2])) < eps) h2 = 0.;
  const double dL = l2[0] - l1[0];
  const double dC = Cp2 - Cp1;
  double dh = h2 - h1;
  if (dh > pi) dh -= 2. * pi;
  if (dh < -pi) dh += 2. * pi;
  if (std::fabs(Cprod) < eps) dh = 0.;
  const double dH = 2. * std::sqrt(Cprod) * std::sin(dh / 2.);
  const double Lp = (l1[0] + l2[0]) / 2.;
  const double Cp = (Cp1 + Cp2) / 2.;
  double hp = (h1 + h2) / 2.;
  if (std::fabs(h1 - h2) > pi) hp -= pi;
  if (hp < 0) hp += 2. * pi;
  if (std::fabs(Cprod) < eps) hp = h1 + h2;
  const double L50 = (Lp - 50.) * (Lp - 50.);
  const double Sl = 1. + 0.015 * L50 / std::sqrt(20.0 + L50);
  const double Sc = 1. + 0.045 * Cp;
  const double Tt = 1. - 0.17 * std::cos(hp - pi / 6.) + 0.24 * std::cos(2. * hp) +
                    0.32 * std::cos(3. * hp + pi / 30.) -
                    0.20 * std::cos(4. * hp - 63. * pi / 180.);
  const double Sh = 1. + 0.015 * Cp * Tt;
  const double dtheta =
    (30. * pi / 180.) * std::exp(-std::pow(((180. / pi * hp - 275.) / 25.), 2.));
  const double Cp7 = std::pow(Cp, 7.);
  const double Rc = 2. * std::sqrt(Cp7 / (Cp7 + std::pow(25., 7.)));
  const double RT = -std::sin(2.0 * dtheta) * Rc;
  return std::sqrt(std::pow(dL / Sl, 2.) + std::pow(dC / Sc, 2.) + std::pow(dH / Sh, 2.) +
                   RT * (dC / Sc) * (dH / Sh));
}

template <class Fn>
void parallel_for(int64_t n, int nthreads, Fn&& fn) {
  if (nthreads <= 1 || n < 4096) {
    fn(int64_t(0), n, 0);
    return;
  }
  std::vector<std::thread> th;
  const int64_t chunk = (n + nthreads - 1) / nthreads;
  for (int t = 0; t < nthreads; t++) {
    const int64_t lo = t * chunk, hi = std::min(n, lo + chunk);
    if (lo >= hi) break;
    th.emplace_back([&fn, lo, hi, t] { fn(lo, hi, t); });
  }
  for (auto& x : th) x.join();
}

}  // namespace

extern "C" {

double orc_coth(double x) { return coth_ref(x); }

void orc_compute_reflectance(const double K[3], const double S[3], const double R0[3],
                             double d, double out[3]) {
  reflectance_ref(K, S, R0, d, out);
}

void orc_km_fp64(const double K[3], const double S[3], const double R0[3], double d,
                 double R[3], double T[3]) {
  km_fp64(K, S, R0, d, R, T);
}

void orc_catmull_rom(const double p_1[2], const double p0[2], const double p1[2],
                     const double p2[2], double t, double out[2]) {
  for (int i = 0; i < 2; i++) out[i] = catmull_rom(p_1[i], p0[i], p1[i], p2[i], t);
}

void orc_catmull_rom_deriv(const double p_1[2], const double p0[2], const double p1[2],
                           const double p2[2], double t, double out[2]) {
  for (int i = 0; i < 2; i++) out[i] = catmull_rom_deriv(p_1[i], p0[i], p1[i], p2[i], t);
}

double orc_catmull_rom_1d(double p_1, double p0, double p1, double p2, double t) {
  return catmull_rom(p_1, p0, p1, p2, t);
}

// Spline.hxx:183-190, 202-219
void orc_spline_catmull_rom(const double* pts, int32_t n, double u, double out[2]) {
  const double x = static_cast<double>(n - 1U) * u;
  const int index = static_cast<int>(x);
  const double t = x - std::floor(x);
  auto clamp_idx = [n](int i) { return i < 0 ? 0 : (i >= n ? n - 1 : i); };
  const double* a = pts + 2 * clamp_idx(index - 1);
  const double* b = pts + 2 * clamp_idx(index);
  const double* c = pts + 2 * clamp_idx(index + 1);
  const double* d = pts + 2 * clamp_idx(index + 2);
  for (int i = 0; i < 2; i++) out[i] = catmull_rom(a[i], b[i], c[i], d[i], t);
}

double orc_interpolate(const double* img, int32_t rows, int32_t cols, double x, double y) {
  return interpolate(img, rows, cols, x, y);
}

void orc_resample(const double* src, int32_t rows, int32_t cols, int32_t out_rows,
                  int32_t out_cols, double* out) {
  resample(src, rows, cols, out_rows, out_cols, out);
}

void orc_compose_layers(int64_t npix, int32_t L, const double* K, const double* S,
                        const double* V, const double* R0, double* out, int32_t mode,
                        int32_t nthreads) {
  parallel_for(npix, nthreads, [&](int64_t lo, int64_t hi, int) {
    for (int64_t p = lo; p < hi; p++) {
      double r[3] = {R0[p * 3], R0[p * 3 + 1], R0[p * 3 + 2]};
      for (int l = 0; l < L; l++) {
        const size_t o = static_cast<size_t>(l) * npix;
        double nr[3], tt[3];
        if (mode == 0)
          reflectance_ref(&K[(o + p) * 3], &S[(o + p) * 3], r, V[o + p], nr);
        else
          km_fp64(&K[(o + p) * 3], &S[(o + p) * 3], r, V[o + p], nr, tt);
        r[0] = nr[0];
        r[1] = nr[1];
        r[2] = nr[2];
      }
      out[p * 3] = r[0];
      out[p * 3 + 1] = r[1];
      out[p * 3 + 2] = r[2];
    }
  });
}

extern "C++" {
namespace {
// Renderer::compose over float32 planar stacks in double (PaintLayer.hxx:81-96 per layer),
// written through `put(p, r)`.
template <class Put>
void compose_f32_soa(int64_t npix, int32_t L, const float* K, const float* S, const float* V,
                     const float* R0, int32_t nthreads, Put put) {
  parallel_for(npix, nthreads, [&](int64_t lo, int64_t hi, int) {
    for (int64_t p = lo; p < hi; p++) {
      double r[3] = {R0[p], R0[npix + p], R0[2 * npix + p]};
      for (int l = 0; l < L; l++) {
        double k[3], s[3], nr[3];
        for (int ch = 0; ch < 3; ch++) {
          k[ch] = K[(static_cast<int64_t>(l) * 3 + ch) * npix + p];
          s[ch] = S[(static_cast<int64_t>(l) * 3 + ch) * npix + p];
        }
        reflectance_ref(k, s, r, V[static_cast<int64_t>(l) * npix + p], nr);
        r[0] = nr[0];
        r[1] = nr[1];
        r[2] = nr[2];
      }
      put(p, r);
    }
  });
}
}  // namespace
}  // extern "C++"

// The same composite with the double result kept, interleaved (npix, 3): the reference values
// that reduced-precision results are measured against.
void orc_compose_layers_f32_soa_f64(int64_t npix, int32_t L, const float* K, const float* S,
                                    const float* V, const float* R0, double* out,
                                    int32_t nthreads) {
  compose_f32_soa(npix, L, K, S, V, R0, nthreads, [&](int64_t p, const double* r) {
    for (int ch = 0; ch < 3; ch++) out[3 * p + ch] = r[ch];
  });
}

void orc_compose_layers_f32_soa(int64_t npix, int32_t L, const float* K, const float* S,
                                const float* V, const float* R0, float* out,
                                int32_t nthreads) {
  // Planes: K[(l*3 + ch)*npix + p], V[l*npix + p], R0[ch*npix + p], out likewise.
  parallel_for(npix, nthreads, [&](int64_t lo, int64_t hi, int) {
    for (int64_t p = lo; p < hi; p++) {
      double r[3] = {R0[p], R0[npix + p], R0[2 * npix + p]};
      for (int l = 0; l < L; l++) {
        double k[3], s[3], nr[3];
        for (int ch = 0; ch < 3; ch++) {
          k[ch] = K[(static_cast<int64_t>(l) * 3 + ch) * npix + p];
          s[ch] = S[(static_cast<int64_t>(l) * 3 + ch) * npix + p];
        }
        reflectance_ref(k, s, r, V[static_cast<int64_t>(l) * npix + p], nr);
        r[0] = nr[0];
        r[1] = nr[1];
        r[2] = nr[2];
      }
      for (int ch = 0; ch < 3; ch++) out[ch * npix + p] = static_cast<float>(r[ch]);
    }
  });
}

// Canvas.hxx:26-58: wet layer zero, R0 = background (1.0), h = 0
orc_canvas* orc_canvas_create(int32_t rows, int32_t cols) {
  auto* c = new orc_canvas();
  c->wet.resize(rows, cols);
  c->R0.assign(static_cast<size_t>(rows) * cols * 3, 1.0);
  c->h.assign(static_cast<size_t>(rows) * cols, 0.0);
  return c;
}

void orc_canvas_destroy(orc_canvas* c) { delete c; }

double* orc_canvas_plane(orc_canvas* c, int32_t which) {
  switch (which) {
    case 0: return c->wet.K.data();
    case 1: return c->wet.S.data();
    case 2: return c->wet.V.data();
    case 3: return c->R0.data();
    case 4: return c->h.data();
    default: return nullptr;
  }
}

// Canvas.hxx:105-121
void orc_canvas_dry(orc_canvas* c) {
  const size_t n = c->wet.V.size();
  for (size_t i = 0; i < n; i++) {
    const double v = c->wet.V[i];
    c->h[i] += v;
    double r[3];
    reflectance_ref(&c->wet.K[i * 3], &c->wet.S[i * 3], &c->R0[i * 3], v, r);
    for (int ch = 0; ch < 3; ch++) {
      c->R0[i * 3 + ch] = r[ch];
      c->wet.K[i * 3 + ch] = 0.0;
      c->wet.S[i * 3 + ch] = 0.0;
    }
    c->wet.V[i] = 0.0;
  }
}

// Renderer.hxx:26-53
void orc_canvas_compose(const orc_canvas* c, double* out_rgb) {
  const size_t n = c->wet.V.size();
  for (size_t i = 0; i < n; i++)
    reflectance_ref(&c->wet.K[i * 3], &c->wet.S[i * 3], &c->R0[i * 3], c->wet.V[i],
                    &out_rgb[i * 3]);
}

// Renderer::render (Renderer.hxx:60-156): the composed canvas lit by a point light with a
// Beckmann / Cook-Torrance specular term; normals from the wet layer's volume (central
// differences through Interpolate). Vector arithmetic per coefficient as Eigen's: squared norm
// and dot products summed left to right, normalized() divides by sqrt(squaredNorm).
void orc_canvas_render(const orc_canvas* c, double* out_rgb) {
  const int H = c->wet.rows, W = c->wet.cols;
  std::vector<double> comp(static_cast<size_t>(H) * W * 3);
  orc_canvas_compose(c, comp.data());
  constexpr double Pi = 3.141592653589793238462643383279502884197169399375105820974;
  struct V3 {
    double x, y, z;
  };
  auto sub = [](V3 a, V3 b) { return V3{a.x - b.x, a.y - b.y, a.z - b.z}; };
  auto dot = [](V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; };
  auto nrm = [&](V3 a) {
    const double n = dot(a, a);
    if (n > 0.0) {
      const double r = std::sqrt(n);
      return V3{a.x / r, a.y / r, a.z / r};
    }
    return a;
  };
  const double m = 0.5, s = 0.2;
  const V3 lightPos = {-200, -1500, -2000.};
  const V3 eyePos = {W / 2.0, H / 2.0, -100.};
  const std::vector<double>& hm = c->wet.V;
  for (int i = 0; i < H; ++i)
    for (int j = 0; j < W; ++j) {
      const double s11 = hm[static_cast<size_t>(i) * W + j];
      const double s01 = interpolate(hm.data(), H, W, static_cast<double>(j) - 1.0, i);
      const double s21 = interpolate(hm.data(), H, W, static_cast<double>(j) + 1.0, i);
      const double s10 = interpolate(hm.data(), H, W, j, static_cast<double>(i) - 1.0);
      const double s12 = interpolate(hm.data(), H, W, j, static_cast<double>(i) + 1.0);
      const V3 va = nrm({2.0, 0.0, s21 - s01});
      const V3 vb = nrm({0.0, 2.0, s12 - s10});
      V3 n = nrm({va.y * vb.z - va.z * vb.y, va.z * vb.x - va.x * vb.z, va.x * vb.y - va.y * vb.x});
      n.z *= -1.;
      const V3 pixPos = {static_cast<double>(j), static_cast<double>(i), s11};
      const V3 lightDirection = nrm(sub(lightPos, pixPos));
      const V3 l = nrm(lightDirection);
      const V3 v = nrm(sub(eyePos, pixPos));
      const V3 h = nrm({v.x + l.x, v.y + l.y, v.z + l.z});
      const double* Kd = &comp[(static_cast<size_t>(i) * W + j) * 3];
      const double NdotH = std::max(0.0, dot(n, h));
      const double VdotH = std::max(0.0, dot(v, h));
      const double NdotV = std::max(0.0, dot(n, v));
      const double NdotL = std::max(0.0, dot(n, l));
      double spec[3] = {0.0, 0.0, 0.0};
      if (NdotL > 0.0 && NdotV > 0.0) {
        const double A = 1.0 / (std::pow(m, 2.0) + std::pow(NdotH, 4.0) * Pi);
        const double B = std::exp(-std::pow(std::tan(std::acos(NdotH)), 2.0) / std::pow(m, 2.0));
        const double G1 = 2.0 * NdotH * NdotV / VdotH;
        const double G2 = 2.0 * NdotH * NdotL / VdotH;
        const double G = std::min(1.0, std::min(G1, G2));
        const double f5 = std::pow(1.0 - VdotH, 5.0);
        const double bg = A * B * G;
        for (int k = 0; k < 3; k++) {
          const double RF = 1.0 + (1.0 - 1.0) * f5;  // Ks = 1
          spec[k] = bg * RF / (NdotL * NdotV);
        }
      }
      const double beta = 15.0 * (1.0 / (4.0 * Pi * std::pow(std::sqrt(dot(lightDirection, lightDirection)), 2.0)));
      for (int k = 0; k < 3; k++) {
        const double ambient = Kd[k] * 0.2;
        const double r = (beta * NdotL) * ((1.0 - s) * Kd[k] + s * spec[k]) + ambient * Kd[k];
        out_rgb[(static_cast<size_t>(i) * W + j) * 3 + k] = std::min(std::max(r, 0.0), 1.0);
      }
    }
}

orc_brush* orc_brush_create(double radius, const double* footprint_full, int32_t fh,
                            int32_t fw) {
  auto* b = new orc_brush();
  b->full.assign(footprint_full, footprint_full + static_cast<size_t>(fh) * fw);
  b->fh = fh;
  b->fw = fw;
  set_radius(b, radius);  // FootprintBrush.hxx:29-37
  return b;
}

void orc_brush_destroy(orc_brush* b) { delete b; }
void orc_brush_set_radius(orc_brush* b, double radius) { set_radius(b, radius); }

void orc_brush_set_rates(orc_brush* b, double pickup_rate, double deposition_rate) {
  b->pickupRate = pickup_rate;          // :182-184
  b->depositionRate = deposition_rate;  // :186-188
}

void orc_brush_set_snapshot(orc_brush* b, int32_t use) { b->useSnapshot = use != 0; }

// FootprintBrush.hxx:150-166
void orc_brush_dip(orc_brush* b, const double K[3], const double S[3]) {
  b->pickup.clear();
  for (int i = 0; i < 3; i++) {
    b->paintK[i] = K[i];
    b->paintS[i] = S[i];
  }
}

// FootprintBrush.hxx:168-172
void orc_brush_update_snapshot(orc_brush* b, const orc_canvas* c) {
  c->wet.copy_to(b->snapshot);
}

void orc_brush_imprint(orc_brush* b, orc_canvas* c, double cx, double cy, double theta) {
  imprint(b, c, cx, cy, theta);
}

void orc_brush_stamps(orc_brush* b, orc_canvas* c, const double* s, int64_t n) {
  for (int64_t i = 0; i < n; i++) imprint(b, c, s[3 * i], s[3 * i + 1], s[3 * i + 2]);
}

int64_t orc_brush_paint_stroke(orc_brush* b, orc_canvas* c, const double* path, int32_t n,
                               double spacing) {
  return for_each_stroke_stamp(path, n, spacing,
                               [&](double x, double y, double th) { imprint(b, c, x, y, th); });
}

int64_t orc_stroke_stamps(const double* path, int32_t n, double spacing, double* out,
                          int64_t cap) {
  int64_t k = 0;
  return for_each_stroke_stamp(path, n, spacing, [&](double x, double y, double th) {
    if (k < cap) {
      out[3 * k] = x;
      out[3 * k + 1] = y;
      out[3 * k + 2] = th;
    }
    k++;
  });
}

double orc_brush_info(const orc_brush* b, int32_t* F, int32_t* S) {
  if (F) *F = b->F;
  if (S) *S = b->sizeMap;
  return b->radius;
}

const double* orc_brush_footprint(const orc_brush* b) { return b->footprint.data(); }

const double* orc_brush_pickup(const orc_brush* b, int32_t which) {
  switch (which) {
    case 0: return b->pickup.K.data();
    case 1: return b->pickup.S.data();
    case 2: return b->pickup.V.data();
    default: return nullptr;
  }
}

const double* orc_brush_snapshot(const orc_brush* b, int32_t which, int32_t* rows,
                                 int32_t* cols) {
  if (rows) *rows = b->snapshot.rows;
  if (cols) *cols = b->snapshot.cols;
  switch (which) {
    case 0: return b->snapshot.K.data();
    case 1: return b->snapshot.S.data();
    case 2: return b->snapshot.V.data();
    default: return nullptr;
  }
}

// PaintMixer.cxx:327-355 (Eps = 10e-6, :278)
void orc_mix_single_paint(const double* w, int32_t n, const double* palK, const double* palS,
                          double K[3], double S[3]) {
  double norm = 1.0, wSum = 0.0;
  for (int i = 0; i < n; i++) wSum += w[i];
  if (!(std::fabs(wSum - 1.0) < 10e-6)) norm = 1. / wSum;
  for (int i = 0; i < 3; i++) {
    K[i] = 0.0;
    S[i] = 0.0;
  }
  for (int l = 0; l < n; l++) {
    for (int i = 0; i < 3; i++) {
      K[i] += norm * w[l] * palK[l * 3 + i];
      S[i] += norm * w[l] * palS[l * 3 + i];
    }
  }
}

// PaintMixer.cxx:536-548
void orc_mixed(const double K1[3], const double S1[3], double v1, const double K2[3],
               const double S2[3], double v2, double K[3], double S[3]) {
  const double totalV = v1 + v2;
  const double inv = 1.0 / totalV;
  for (int i = 0; i < 3; i++) {
    K[i] = ((v1 * K1[i]) + (v2 * K2[i])) * inv;
    S[i] = ((v1 * S1[i]) + (v2 * S2[i])) * inv;
  }
}

void orc_rgb2lab(const double rgb[3], double lab[3]) { rgb2lab(rgb, lab); }
double orc_ciede2000(const double lab1[3], const double lab2[3]) { return ciede2000(lab1, lab2); }

double orc_delta_e_images(int64_t npix, const double* a, const double* b, double* mean_out,
                          int32_t nthreads) {
  const int nt = std::max(1, static_cast<int>(nthreads));
  std::vector<double> mx(nt, 0.0), sum(nt, 0.0);
  parallel_for(npix, nt, [&](int64_t lo, int64_t hi, int t) {
    for (int64_t p = lo; p < hi; p++) {
      double la[3], lb[3];
      rgb2lab(a + 3 * p, la);
      rgb2lab(b + 3 * p, lb);
      const double d = ciede2000(la, lb);
      mx[t] = std::max(mx[t], d);
      sum[t] += d;
    }
  });
  double m = 0.0, s = 0.0;
  for (int t = 0; t < nt; t++) {
    m = std::max(m, mx[t]);
    s += sum[t];
  }
  if (mean_out) *mean_out = npix > 0 ? s / static_cast<double>(npix) : 0.0;
  return m;
}

}  // extern "C"

// ---------------------------------------------------------------- texture brush
// TextureBrush<vec3> (painty/renderer/TextureBrush.hxx:20-237) with its Smudge<vec3>
// (painty/renderer/Smudge.hxx:16-229). The thickness texture stands in for
// BrushStrokeSample::getThicknessMap(), which painty loads from a sample directory.
namespace {

struct V2 {
  double x, y;
};

// SplineEval::catmullRom / catmullRomDerivativeFirst over all points (Spline.hxx:183-231):
// x = (n-1) u, index = int(x), t = x - floor(x), control points clamped to the ends.
V2 spline_eval(const std::vector<V2>& p, double u, bool deriv) {
  const auto n = static_cast<int64_t>(p.size());
  const double x = static_cast<double>(n - 1) * u;
  const int32_t index = static_cast<int32_t>(x);
  const double t = x - std::floor(x);
  auto at = [&](int32_t i) -> const V2& {
    if (i < 0) return p.front();
    if (i >= static_cast<int32_t>(n)) return p.back();
    return p[static_cast<size_t>(i)];
  };
  const V2 &a = at(index - 1), &b = at(index), &c = at(index + 1), &d = at(index + 2);
  if (deriv)
    return {catmull_rom_deriv(a.x, b.x, c.x, d.x, t), catmull_rom_deriv(a.y, b.y, c.y, d.y, t)};
  return {catmull_rom(a.x, b.x, c.x, d.x, t), catmull_rom(a.y, b.y, c.y, d.y, t)};
}

double norm2(const V2& v) { return std::sqrt(v.x * v.x + v.y * v.y); }
V2 normalized2(const V2& v) {  // Eigen normalized(): v / sqrt(squaredNorm) when positive
  const double n = v.x * v.x + v.y * v.y;
  if (n > 0.0) {
    const double r = std::sqrt(n);
    return {v.x / r, v.y / r};
  }
  return v;
}

// generalizedBarycentricCoordinatesInterpolate (painty/core/Math.hxx:72-147) for vec2 values
V2 barycentric_interpolate(const std::vector<V2>& polygon, const V2& pos,
                           const std::vector<V2>& values) {
  const size_t n = polygon.size();
  constexpr double Eps = std::numeric_limits<double>::epsilon() * 100.0;
  if (n == 1U) return values.front();
  std::vector<V2> sv(n);
  for (size_t i = 0; i < n; ++i) sv[i] = {polygon[i].x - pos.x, polygon[i].y - pos.y};
  std::vector<double> r(n), A(n), D(n);
  for (size_t i = 0; i < n; ++i) {
    const V2 si1 = (i == n - 1) ? sv[0] : sv[i + 1];
    const V2 si = sv[i];
    r[i] = norm2(si);
    if (std::fabs(r[i] - 0.0) < Eps) return values[i];
    const double det = si.x * si1.y - si1.x * si.y;
    A[i] = det / 2.0;
    D[i] = si.x * si1.x + si.y * si1.y;
    if (std::fabs(A[i] - 0.0) < Eps && D[i] < 0.0) {
      const double ri1 = norm2(si1);
      const V2 fi1 = (i == n - 1) ? values.front() : values[i + 1];
      const double k = 1.0 / (r[i] + ri1);
      return {(ri1 * values[i].x + r[i] * fi1.x) * k, (ri1 * values[i].y + r[i] * fi1.y) * k};
    }
  }
  V2 f = {0.0, 0.0};
  double W = 0.0;
  for (size_t i = 0; i < n; ++i) {
    double w = 0.0;
    const double A_1 = (i == 0) ? A.back() : A[i - 1];
    if (A_1 != 0.0) {
      const double r_1 = (i == 0) ? r.back() : r[i - 1];
      const double D_1 = (i == 0) ? D.back() : D[i - 1];
      w = w + (r_1 - D_1 / r[i]) / A_1;
    }
    if (A[i] != 0.0) {
      const double ri1 = (i == n - 1) ? r[0] : r[i + 1];
      w = w + (ri1 - D[i] / r[i]) / A[i];
    }
    f = {f.x + w * values[i].x, f.y + w * values[i].y};
    W = W + w;
  }
  if (!(std::fabs(W - 0.0) < Eps)) {
    const double k = 1.0 / W;
    return {f.x * k, f.y * k};
  }
  return values.front();
}

// Mat.hxx:68-103, three channels of an interleaved layer plane
void interpolate3(const std::vector<double>& in, int rows, int cols, double px, double py,
                  double out[3]) {
  const int x = static_cast<int>(std::floor(px));
  const int y = static_cast<int>(std::floor(py));
  const int x0 = border_reflect(x, cols), x1 = border_reflect(x + 1, cols);
  const int y0 = border_reflect(y, rows), y1 = border_reflect(y + 1, rows);
  const double a = px - static_cast<double>(x);
  const double c = py - static_cast<double>(y);
  for (int k = 0; k < 3; k++) {
    auto v = [&](int yy, int xx) { return in[(static_cast<size_t>(yy) * cols + xx) * 3 + k]; };
    out[k] = (v(y0, x0) * (1.0 - a) + v(y0, x1) * a) * (1.0 - c) +
             (v(y1, x0) * (1.0 - a) + v(y1, x1) * a) * c;
  }
}

}  // namespace

struct orc_tbrush {
  std::vector<double> tex;  // thickness texture (th x tw)
  int th = 0, tw = 0;
  double radius = 0.0;           // TextureBrush.hxx:228
  double thicknessScale = 1.0;   // BrushBase.hxx _thicknessScale
  double paint[2][3] = {{0.1, 0.1, 0.1}, {0.1, 0.1, 0.1}};  // TextureBrush.hxx:28-30
  bool useSmudge = true;         // TextureBrush.hxx:236
  // Smudge (Smudge.hxx:147-158)
  int maxSize = 0;
  Layer pickSrc, pickDst;
  double rotation = 0.0;
  double smPickupRate = 0.1, smDepositionRate = 0.1;
  void make_smudge(int32_t size) {  // Smudge.hxx:22-36
    maxSize = size;
    pickSrc.resize(size, size);
    pickDst.resize(size, size);
    if ((maxSize % 2) == 0) maxSize++;
    pickSrc.clear();
    pickDst.clear();
    rotation = 0.0;
  }
};

namespace {

double normalize_angle(double angle) {  // Smudge.hxx:201-211
  constexpr double HALF_PI = 0.5 * 3.14159265358979323846;
  constexpr double PI = 3.14159265358979323846;
  double a = angle;
  while (a <= -HALF_PI) a += PI;
  while (a > HALF_PI) a -= PI;
  return a;
}

// Smudge::updateOrientation (Smudge.hxx:160-199)
void smudge_orient(orc_tbrush* b, const V2& heading) {
  const double theta = std::atan2(heading.y, heading.x);
  const double dtheta = normalize_angle(theta - b->rotation);
  b->rotation = theta;
  b->pickDst.copy_to(b->pickSrc);
  const double cx = b->maxSize / 2.0, cy = b->maxSize / 2.0;
  const double sn = std::sin(dtheta), cs = std::cos(dtheta);
  Layer& d = b->pickDst;
  const Layer& sr = b->pickSrc;
  for (int x = 0; x < d.cols; x++)
    for (int y = 0; y < d.rows; y++) {
      const double px = x - cx, py = y - cy;
      const double qx = px * cs - py * sn + cx;
      const double qy = px * sn + py * cs + cy;
      const size_t o = d.idx(y, x);
      if (qx < 0 || qy < 0 || qx >= d.cols || qy >= d.rows) {
        for (int k = 0; k < 3; k++) {
          d.K[o * 3 + k] = sr.K[o * 3 + k];
          d.S[o * 3 + k] = sr.S[o * 3 + k];
        }
        d.V[o] = sr.V[o];
      } else {
        d.V[o] = interpolate(sr.V.data(), sr.rows, sr.cols, qx, qy);
        interpolate3(sr.K, sr.rows, sr.cols, qx, qy, &d.K[o * 3]);
        interpolate3(sr.S, sr.rows, sr.cols, qx, qy, &d.S[o * 3]);
      }
    }
}

// Smudge::smudge (Smudge.hxx:38-145)
void smudge_run(orc_tbrush* b, orc_canvas* c, const V2& boundMin, const std::vector<V2>& verts,
                double length, const std::vector<double>& tmap, int trows, int tcols) {
  double maxD = 0.0;
  for (double m : tmap) maxD = std::max(m, maxD);
  if (maxD <= 0.) return;
  Layer& pm = b->pickDst;
  Layer& cw = c->wet;
  for (double u = 0.0; u <= 1.0; u += 1. / length) {
    const V2 center = spline_eval(verts, u, false);
    const V2 t = normalized2(spline_eval(verts, u, true));
    smudge_orient(b, t);
    const double radius = b->maxSize * 0.5;
    const int32_t roi_x = static_cast<int32_t>(center.x - pm.cols / 2.0);
    const int32_t roi_y = static_cast<int32_t>(center.y - pm.rows / 2.0);
    for (int x = 0; x < pm.cols; x++)
      for (int y = 0; y < pm.rows; y++) {
        const int cpx = x + roi_x, cpy = y + roi_y;
        const int tpx = static_cast<int32_t>(cpx - boundMin.x);
        const int tpy = static_cast<int32_t>(cpy - boundMin.y);
        if (cpx < 0 || cpy < 0 || cpx >= cw.cols || cpy >= cw.rows) continue;
        if (tpx < 0 || tpy < 0 || tpx >= tcols || tpy >= trows) continue;
        const double dx = center.x - static_cast<double>(cpx);
        const double dy = center.y - static_cast<double>(cpy);
        if (std::sqrt(dx * dx + dy * dy) > radius) continue;
        const double D = tmap[static_cast<size_t>(tpy) * tcols + tpx];
        if (D <= 0.0) continue;
        const size_t co = cw.idx(cpy, cpx), po = pm.idx(y, x);
        const double cV = cw.V[co], pV = pm.V[po];
        const double cVl = cV * b->smDepositionRate * D / maxD;
        const double cVr = cV - cVl;
        const double pVl = pV * b->smPickupRate * D / maxD;
        const double pVr = pV - pVl;
        double canvasK[3], canvasS[3], pickK[3], pickS[3];
        for (int k = 0; k < 3; k++) {
          canvasK[k] = cw.K[co * 3 + k];
          canvasS[k] = cw.S[co * 3 + k];
          pickK[k] = pm.K[po * 3 + k];
          pickS[k] = pm.S[po * 3 + k];
        }
        constexpr double MinVolume = 0.001;
        const double pVnew = pVr + cVl;
        if (pVnew > MinVolume) {
          const double pVnew_ = 1.0 / pVnew;
          for (int k = 0; k < 3; k++) {
            pm.K[po * 3 + k] = pVnew_ * (pVr * pickK[k] + cVl * canvasK[k]);
            pm.S[po * 3 + k] = pVnew_ * (pVr * pickS[k] + cVl * canvasS[k]);
          }
          pm.V[po] = std::max(pVnew, 0.0);
        }
        const double cVnew = cVr + pVl;
        if (cVnew > MinVolume) {
          const double cVnew_ = 1. / cVnew;
          for (int k = 0; k < 3; k++) {
            cw.K[co * 3 + k] = cVnew_ * (cVr * canvasK[k] + pVl * pickK[k]);
            cw.S[co * 3 + k] = cVnew_ * (cVr * canvasS[k] + pVl * pickS[k]);
          }
          cw.V[co] = std::max(cVnew, 0.0);
        }
      }
  }
}

}  // namespace

extern "C" {

orc_tbrush* orc_tbrush_create(const double* tex, int32_t th, int32_t tw) {
  auto* b = new orc_tbrush();
  b->tex.assign(tex, tex + static_cast<size_t>(th) * tw);
  b->th = th;
  b->tw = tw;
  b->make_smudge(static_cast<int32_t>(2.0 * b->radius));  // TextureBrush.hxx:25-31
  return b;
}
void orc_tbrush_destroy(orc_tbrush* b) { delete b; }
void orc_tbrush_set_radius(orc_tbrush* b, double radius) {  // TextureBrush.hxx:33-41
  if (!(std::fabs(b->radius - radius) < 0.5)) {
    b->radius = radius;
    if (b->useSmudge) b->make_smudge(static_cast<int32_t>(2.0 * radius));
  }
}
void orc_tbrush_dip(orc_tbrush* b, const double K[3], const double S[3]) {  // :48-50
  for (int k = 0; k < 3; k++) {
    b->paint[0][k] = K[k];
    b->paint[1][k] = S[k];
  }
}
void orc_tbrush_set_smudge(orc_tbrush* b, int32_t on) { b->useSmudge = on != 0; }  // :207-209
void orc_tbrush_set_thickness_scale(orc_tbrush* b, double s) { b->thicknessScale = s; }
// the smudge pickup map (which: 0 K, 1 S, 2 V) and its side
const double* orc_tbrush_smudge_map(const orc_tbrush* b, int32_t which, int32_t* side) {
  if (side) *side = b->pickDst.rows;
  return which == 0 ? b->pickDst.K.data() : which == 1 ? b->pickDst.S.data() : b->pickDst.V.data();
}

// TextureBrush::paintStroke (TextureBrush.hxx:52-205); returns the pixels painted
int64_t orc_tbrush_paint_stroke(orc_tbrush* b, orc_canvas* c, const double* path, int32_t n) {
  if (n < 2) return 0;
  std::vector<V2> arg(static_cast<size_t>(n));
  for (int32_t i = 0; i < n; i++) arg[i] = {path[2 * i], path[2 * i + 1]};
  std::vector<V2> v;
  {
    const V2 d = normalized2({arg[1].x - arg[0].x, arg[1].y - arg[0].y});
    v.push_back({arg[0].x - d.x * b->radius, arg[0].y - d.y * b->radius});
  }
  v.insert(v.end(), arg.begin(), arg.end());
  {
    const V2 d = normalized2({arg[n - 1].x - arg[n - 2].x, arg[n - 1].y - arg[n - 2].y});
    v.push_back({arg[n - 1].x + d.x * b->radius, arg[n - 1].y + d.y * b->radius});
  }
  Layer& cw = c->wet;
  V2 bmin = v.front(), bmax = v.front();
  for (const V2& p : v) {
    bmin.x = std::min(bmin.x, p.x);
    bmin.y = std::min(bmin.y, p.y);
    bmax.x = std::max(bmax.x, p.x);
    bmax.y = std::max(bmax.y, p.y);
  }
  bmin.x = std::max(bmin.x - b->radius, 0.0);
  bmax.x = std::min(bmax.x + b->radius, static_cast<double>(cw.cols - 1));
  bmin.y = std::max(bmin.y - b->radius, 0.0);
  bmax.y = std::min(bmax.y + b->radius, static_cast<double>(cw.rows - 1));
  double length = 0.0;
  for (size_t i = 1; i < v.size(); ++i) length += norm2({v[i].x - v[i - 1].x, v[i].y - v[i - 1].y});
  // the outline: right side reversed, then left side; uv (u, 1) then (u, 0)
  std::vector<V2> up, down, upUv, downUv;
  for (size_t i = 0; i < v.size(); ++i) {
    const double u = static_cast<double>(i) / static_cast<double>(v.size() - 1);
    const V2 cpt = spline_eval(v, u, false);
    const V2 t = normalized2(spline_eval(v, u, true));
    const V2 d = {-t.y, t.x};
    up.push_back({cpt.x - b->radius * d.x, cpt.y - b->radius * d.y});
    down.push_back({cpt.x + b->radius * d.x, cpt.y + b->radius * d.y});
    upUv.push_back({u, 0.0});
    downUv.push_back({u, 1.0});
  }
  up.insert(up.begin(), down.rbegin(), down.rend());
  upUv.insert(upUv.begin(), downUv.rbegin(), downUv.rend());
  const int trows = static_cast<int32_t>(bmax.y - bmin.y + 1);
  const int tcols = static_cast<int32_t>(bmax.x - bmin.x + 1);
  std::vector<double> tmap(static_cast<size_t>(std::max(trows, 0)) * std::max(tcols, 0), 0.0);
  std::vector<std::pair<int, int>> pixels;
  for (int x = static_cast<int32_t>(bmin.x); x <= static_cast<int32_t>(bmax.x); x++)
    for (int y = static_cast<int32_t>(bmin.y); y <= static_cast<int32_t>(bmax.y); y++) {
      if (x < 0 || x >= cw.cols || y < 0 || y >= cw.rows) continue;
      V2 tp = barycentric_interpolate(up, {static_cast<double>(x), static_cast<double>(y)}, upUv);
      if (tp.x < 0.0 || tp.x > 1.0 || tp.y < 0.0 || tp.y > 1.0) continue;
      tp.x *= b->tw;
      tp.y *= b->th;
      const double Vtex = b->thicknessScale * interpolate(b->tex.data(), b->th, b->tw, tp.x, tp.y);
      if (Vtex > 0.0) {
        const int sx = x - static_cast<int32_t>(bmin.x), sy = y - static_cast<int32_t>(bmin.y);
        if (sx >= 0 && sy >= 0 && sx < tcols && sy < trows) {
          tmap[static_cast<size_t>(sy) * tcols + sx] = Vtex;
          pixels.emplace_back(x, y);
        }
      }
    }
  if (b->useSmudge) smudge_run(b, c, bmin, v, length, tmap, trows, tcols);
  for (const auto& px : pixels) {
    const int x = px.first, y = px.second;
    if (x < 0 || y < 0 || x >= cw.cols || y >= cw.rows) continue;
    const int ty = std::min(trows - 1, std::max(y - static_cast<int32_t>(bmin.y), 0));
    const int tx = std::min(tcols - 1, std::max(x - static_cast<int32_t>(bmin.x), 0));
    const double Vtex = tmap[static_cast<size_t>(ty) * tcols + tx];
    const size_t o = cw.idx(y, x);
    const double Vcan = cw.V[o];
    const double Vsum = Vcan + Vtex;
    if (Vsum > 0.0) {
      const double sc = 1.0 / Vsum;
      for (int k = 0; k < 3; k++) {
        cw.K[o * 3 + k] = (Vcan * cw.K[o * 3 + k] + Vtex * b->paint[0][k]) * sc;
        cw.S[o * 3 + k] = (Vcan * cw.S[o * 3 + k] + Vtex * b->paint[1][k]) * sc;
      }
      cw.V[o] = std::max(Vtex, Vcan);
    }
  }
  return static_cast<int64_t>(pixels.size());
}

}  // extern "C"
