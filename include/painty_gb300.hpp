/*
 * painty_gb300.hpp -- C++17 facade over the C ABI (painty_gb300.h), mirroring painty's class
 * names and signatures for the paint path so that code written against painty's
 * Canvas / PaintLayer / FootprintBrush / Renderer compiles against this one with the
 * container types changed:
 *
 *   painty (painty/renderer/...)                   this facade
 *   Canvas<vec3>(rows, cols)          Canvas.hxx:26  painty_gb300::Canvas(rows, cols, storage)
 *   Canvas::clear / setBackground     :72-87         Canvas::clear / setBackground
 *   Canvas::getPaintLayer             :89            Canvas::getPaintLayer (a view)
 *   Canvas::getR0 / get_h             :91-103        Canvas::getR0 / get_h (host copies)
 *   Canvas::dryCanvas                 :105-121       Canvas::dryCanvas
 *   PaintLayer::getK/S/V_buffer       PaintLayer.hxx  PaintLayer::getK/S/V_buffer (host copies)
 *   PaintLayer::composeOnto / copyTo  :81-115        PaintLayer::composeOnto / copyTo
 *   FootprintBrush(radius)            FootprintBrush.hxx:29-37  FootprintBrush(radius, footprint)
 *   setRadius / dip / paintStroke     :46-63, 150-268  the same
 *   imprint(center, theta, canvas)    :73-143        the same
 *   set/get Pickup / Deposition rate, UseSnapshotBuffer, getPickupMap, getFootprint,
 *   updateSnapshot                    :168-204, 477-495  the same
 *   Renderer::compose(canvas | layer, R0)  Renderer.hxx:26-53  Renderer::compose
 *   Renderer::render(canvas)          Renderer.hxx:60-156  Renderer::render
 *   TextureBrush<vec3>(sampleDir)     TextureBrush.hxx:25-237  TextureBrush(texture, rows, cols)
 *   CanvasGpu::getComposed / dryStep  CanvasGpu.cxx:91-128  Canvas::getComposedGlsl / dryStep
 *   TextureBrushDictionary / TextureBrushGpu  TextureBrushGpu.cxx:17-250  the same
 *   LoadPalette / SavePalette         mixer/src/Serialization.cxx:38-53  the same
 *   SbrRenderThread                   SbrRenderThread.hxx:19-116  the same (no window)
 *
 * Host images are row-major, pixel-interleaved doubles (cv::Mat_<vec3>'s layout): rows*cols*3
 * values for three channels, rows*cols for one. Errors are painty's exception types:
 * std::invalid_argument for bad arguments (PAINTY_ERR_INVALID_ARGUMENT), std::bad_alloc for
 * device memory exhaustion, std::runtime_error otherwise.
 */
#ifndef PAINTY_GB300_HPP
#define PAINTY_GB300_HPP

#include <array>
#include <cctype>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <functional>
#include <future>
#include <memory>
#include <mutex>
#include <thread>
#include <cstring>
#include <cstdint>
#include <cstdlib>
#include <istream>
#include <iterator>
#include <new>
#include <ostream>
#include <sstream>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "painty_gb300.h"

namespace painty_gb300 {

using vec3 = std::array<double, 3>;
struct vec2 {
  double x = 0.0, y = 0.0;
};

enum class Storage : int {
  F32 = PAINTY_STORAGE_F32,
  F16 = PAINTY_STORAGE_F16,
  BF16 = PAINTY_STORAGE_BF16,
  F64 = PAINTY_STORAGE_F64
};

// Status -> painty's exception types.
inline void check(painty_status s) {
  if (s == PAINTY_OK) return;
  const std::string msg = std::string(painty_status_string(s)) + ": " + painty_last_error();
  if (s == PAINTY_ERR_INVALID_ARGUMENT) throw std::invalid_argument(msg);
  if (s == PAINTY_ERR_OUT_OF_MEMORY) throw std::bad_alloc();
  throw std::runtime_error(msg);
}

namespace detail {
// Move-only owner of a C handle.
template <class H, painty_status (*Destroy)(H*)>
class Handle {
 public:
  Handle() = default;
  explicit Handle(H* h) : h_(h) {}
  Handle(const Handle&) = delete;
  Handle& operator=(const Handle&) = delete;
  Handle(Handle&& o) noexcept : h_(std::exchange(o.h_, nullptr)) {}
  Handle& operator=(Handle&& o) noexcept {
    if (this != &o) {
      reset();
      h_ = std::exchange(o.h_, nullptr);
    }
    return *this;
  }
  ~Handle() { reset(); }
  H* get() const { return h_; }

 private:
  void reset() {
    if (h_) Destroy(h_);
    h_ = nullptr;
  }
  H* h_ = nullptr;
};
}  // namespace detail

// A reflectance image on the device (painty's Mat<vec3> result of a composite).
class Image {
 public:
  Image(int32_t rows, int32_t cols, Storage storage = Storage::F32) : rows_(rows), cols_(cols) {
    painty_image* h = nullptr;
    check(painty_image_create(rows, cols, static_cast<painty_storage>(storage), &h));
    own_ = Owner(h);
    h_ = h;
  }
  int32_t rows() const { return rows_; }
  int32_t cols() const { return cols_; }
  void fill(const vec3& c) { check(painty_image_fill(h_, c[0], c[1], c[2], nullptr)); }
  void upload(const std::vector<double>& rgb) {
    require(rgb.size() == size_t(rows_) * cols_ * 3, "image buffer size");
    check(painty_image_upload(h_, rgb.data(), PAINTY_HOST_F64_INTERLEAVED, nullptr));
  }
  std::vector<double> download() const {
    std::vector<double> out(size_t(rows_) * cols_ * 3);
    check(painty_image_download(h_, out.data(), PAINTY_HOST_F64_INTERLEAVED, nullptr));
    return out;
  }
  painty_image* handle() const { return h_; }

 private:
  friend class Canvas;
  Image(painty_image* borrowed, int32_t rows, int32_t cols)
      : rows_(rows), cols_(cols), h_(borrowed) {}
  static void require(bool ok, const char* what) {
    if (!ok) throw std::invalid_argument(what);
  }
  using Owner = detail::Handle<painty_image, painty_image_destroy>;
  int32_t rows_, cols_;
  Owner own_;
  painty_image* h_ = nullptr;
};

// painty::PaintLayer<vec3>: K, S (3 channels) and V (volume) planes on the device.
class PaintLayer {
 public:
  PaintLayer(int32_t rows, int32_t cols, Storage storage = Storage::F32) {
    painty_layer* h = nullptr;
    check(painty_layer_create(rows, cols, static_cast<painty_storage>(storage), &h));
    own_ = Owner(h);
    h_ = h;
  }
  int32_t getRows() const { return info().first; }
  int32_t getCols() const { return info().second; }
  void clear() { check(painty_layer_clear(h_, nullptr)); }
  // PaintLayer::set: K, S interleaved rows*cols*3, V rows*cols
  void set(const std::vector<double>& K, const std::vector<double>& S,
           const std::vector<double>& V) {
    check(painty_layer_upload(h_, PAINTY_PLANE_K, K.data(), PAINTY_HOST_F64_INTERLEAVED, nullptr));
    check(painty_layer_upload(h_, PAINTY_PLANE_S, S.data(), PAINTY_HOST_F64_INTERLEAVED, nullptr));
    check(painty_layer_upload(h_, PAINTY_PLANE_V, V.data(), PAINTY_HOST_F64_INTERLEAVED, nullptr));
  }
  // PaintLayer::set(i, j, k, s, v) (PaintLayer.hxx:122-127)
  void set(int32_t i, int32_t j, const vec3& k, const vec3& s, double v) {
    const int32_t rc[2] = {i, j};
    check(painty_layer_set_cells(h_, 1, rc, k.data(), s.data(), &v, nullptr));
  }
  std::vector<double> getK_buffer() const { return plane(PAINTY_PLANE_K, 3); }
  std::vector<double> getS_buffer() const { return plane(PAINTY_PLANE_S, 3); }
  std::vector<double> getV_buffer() const { return plane(PAINTY_PLANE_V, 1); }
  void copyTo(PaintLayer& other) const { check(painty_layer_copy(h_, other.h_, nullptr)); }
  // PaintLayer::composeOnto (PaintLayer.hxx:81-96): R0 <- KM(K, S, R0, V)
  void composeOnto(Image& R0) const {
    const painty_layer* L[1] = {h_};
    check(painty_compose_layers(L, 1, R0.handle(), R0.handle(), nullptr));
  }
  painty_layer* handle() const { return h_; }

 private:
  friend class Canvas;
  explicit PaintLayer(painty_layer* borrowed) : h_(borrowed) {}
  std::pair<int32_t, int32_t> info() const {
    int32_t r = 0, c = 0;
    painty_storage s{};
    check(painty_layer_info(h_, &r, &c, &s));
    return {r, c};
  }
  std::vector<double> plane(painty_plane p, int nch) const {
    const auto [r, c] = info();
    std::vector<double> out(size_t(r) * c * nch);
    check(painty_layer_download(h_, p, out.data(), PAINTY_HOST_F64_INTERLEAVED, nullptr));
    return out;
  }
  using Owner = detail::Handle<painty_layer, painty_layer_destroy>;
  Owner own_;
  painty_layer* h_ = nullptr;
};

// painty::Canvas<vec3> (Canvas.hxx:20-198): the wet layer, the substrate R0 and height map h.
class Canvas {
 public:
  Canvas(int32_t rows, int32_t cols, Storage storage = Storage::F32) : rows_(rows), cols_(cols) {
    painty_canvas* h = nullptr;
    check(painty_canvas_create(rows, cols, static_cast<painty_storage>(storage), &h));
    own_ = Owner(h);
  }
  int32_t rows() const { return rows_; }
  int32_t cols() const { return cols_; }
  void clear() { check(painty_canvas_clear(own_.get(), nullptr)); }
  // Canvas::setBackground (Canvas.hxx:80-87): clear, then R0 = background
  void setBackground(const std::vector<double>& rgb) {
    require(rgb.size() == size_t(rows_) * cols_ * 3, "background size");
    clear();
    check(painty_canvas_upload(own_.get(), PAINTY_PLANE_R0, rgb.data(),
                               PAINTY_HOST_F64_INTERLEAVED, nullptr));
  }
  std::vector<double> getR0() const { return plane(PAINTY_PLANE_R0, 3); }
  std::vector<double> get_h() const { return plane(PAINTY_PLANE_H, 1); }
  // A view of the canvas's wet layer (valid while the canvas lives)
  PaintLayer getPaintLayer() {
    painty_layer* l = nullptr;
    check(painty_canvas_layer(own_.get(), &l));
    return PaintLayer(l);
  }
  Image r0Image() {
    painty_image* i = nullptr;
    check(painty_canvas_r0(own_.get(), &i));
    return Image(i, rows_, cols_);
  }
  void dryCanvas() { check(painty_canvas_dry(own_.get(), nullptr)); }
  // the GL canvas path (CanvasGpu.cxx:91-128): its composite and its partial drying step
  Image getComposedGlsl() const {
    Image out(rows_, cols_, Storage::F32);
    check(painty_canvas_compose_glsl(own_.get(), out.handle(), nullptr));
    return out;
  }
  void dryStep(float step = 0.01F) { check(painty_canvas_dry_step(own_.get(), step, nullptr)); }
  painty_canvas* handle() const { return own_.get(); }

 private:
  static void require(bool ok, const char* what) {
    if (!ok) throw std::invalid_argument(what);
  }
  std::vector<double> plane(painty_plane p, int nch) const {
    std::vector<double> out(size_t(rows_) * cols_ * nch);
    check(painty_canvas_download(own_.get(), p, out.data(), PAINTY_HOST_F64_INTERLEAVED, nullptr));
    return out;
  }
  using Owner = detail::Handle<painty_canvas, painty_canvas_destroy>;
  int32_t rows_, cols_;
  Owner own_;
};

// painty::FootprintBrush<vec3> (FootprintBrush.hxx:22-502). `footprint` is the full-size
// footprint image (fh x fw values in [0, 1]) that stands in for painty's footprint PNG.
class FootprintBrush {
 public:
  FootprintBrush(double radius, const std::vector<double>& footprint, int32_t fh, int32_t fw) {
    painty_brush* h = nullptr;
    check(painty_brush_create(radius, footprint.data(), fh, fw, &h));
    own_ = Owner(h);
  }
  void setRadius(double radius) { check(painty_brush_set_radius(own_.get(), radius)); }
  double getRadius() const {
    double r = 0.0;
    check(painty_brush_info(own_.get(), &r, nullptr, nullptr));
    return r;
  }
  // BrushBase::dip (FootprintBrush.hxx:150-158): paint = {K, S}; cleans the pickup map
  void dip(const std::array<vec3, 2>& paint) {
    check(painty_brush_dip(own_.get(), paint[0].data(), paint[1].data(), nullptr));
  }
  void setPickupRate(double r) { check(painty_brush_set_rates(own_.get(), r, getDepositionRate())); }
  void setDepositionRate(double r) { check(painty_brush_set_rates(own_.get(), getPickupRate(), r)); }
  double getPickupRate() const { return rates().first; }
  double getDepositionRate() const { return rates().second; }
  void setUseSnapshotBuffer(bool use) { check(painty_brush_set_snapshot(own_.get(), use ? 1 : 0)); }
  // FootprintBrush::imprint (FootprintBrush.hxx:73-143)
  void imprint(const vec2& center, double theta, Canvas& canvas) {
    check(painty_imprint(canvas.handle(), own_.get(), center.x, center.y, theta, nullptr));
  }
  // stamps (cx, cy, theta) in order, as repeated imprint calls
  void stamps(const std::vector<std::array<double, 3>>& s, Canvas& canvas) {
    check(painty_stamps(canvas.handle(), own_.get(), s.empty() ? nullptr : s[0].data(),
                        static_cast<int64_t>(s.size()), nullptr));
  }
  // FootprintBrush::paintStroke (FootprintBrush.hxx:206-268); returns the stamps applied.
  // spacing 1.0 is painty's; other values space stamps along each segment's chord.
  int64_t paintStroke(const std::vector<vec2>& path, Canvas& canvas, double spacing = 1.0) {
    std::vector<double> xy;
    xy.reserve(path.size() * 2);
    for (const auto& p : path) {
      xy.push_back(p.x);
      xy.push_back(p.y);
    }
    int64_t n = 0;
    check(painty_stroke(canvas.handle(), own_.get(), xy.data(),
                        static_cast<int32_t>(path.size()), spacing, &n, nullptr));
    return n;
  }
  // FootprintBrush::updateSnapshot(canvas) (FootprintBrush.hxx:168-172)
  void updateSnapshot(const Canvas& canvas) {
    check(painty_brush_update_snapshot(own_.get(), canvas.handle(), nullptr));
  }
  // getPickupMap: plane K or S (S*S*3 interleaved) or V (S*S)
  std::vector<double> getPickupMap(painty_plane plane) const {
    int32_t F = 0, S = 0;
    check(painty_brush_info(own_.get(), nullptr, &F, &S));
    std::vector<double> out(size_t(S) * S * (plane == PAINTY_PLANE_V ? 1 : 3));
    check(painty_brush_download_pickup(own_.get(), plane, out.data(),
                                       PAINTY_HOST_F64_INTERLEAVED, nullptr));
    return out;
  }
  std::vector<double> getFootprint() const {
    int32_t F = 0;
    check(painty_brush_info(own_.get(), nullptr, &F, nullptr));
    std::vector<double> out(size_t(F) * F);
    check(painty_brush_footprint(own_.get(), out.data()));
    return out;
  }
  painty_brush* handle() const { return own_.get(); }

 private:
  std::pair<double, double> rates() const {
    double p = 0.0, d = 0.0;
    check(painty_brush_get_rates(own_.get(), &p, &d));
    return {p, d};
  }
  using Owner = detail::Handle<painty_brush, painty_brush_destroy>;
  Owner own_;
};

// painty::Renderer<vec3>::compose (Renderer.hxx:26-53)
class Renderer {
 public:
  Image compose(const Canvas& canvas, Storage storage = Storage::F32) const {
    Image out(canvas.rows(), canvas.cols(), storage);
    check(painty_canvas_compose(canvas.handle(), out.handle(), nullptr));
    return out;
  }
  // compose(layer, R0): the layer composed onto a copy of R0
  Image compose(const PaintLayer& layer, const Image& R0) const {
    Image out(R0.rows(), R0.cols());
    const painty_layer* L[1] = {layer.handle()};
    check(painty_compose_layers(L, 1, R0.handle(), out.handle(), nullptr));
    return out;
  }
  // Renderer::render (Renderer.hxx:60-156): the composite lit by painty's point light;
  // storage F64 for F64 canvases, F32 otherwise
  Image render(const Canvas& canvas, Storage storage = Storage::F32) const {
    Image out(canvas.rows(), canvas.cols(), storage);
    check(painty_canvas_render(canvas.handle(), out.handle(), nullptr));
    return out;
  }
};

namespace detail {
inline std::vector<double> flatten(const std::vector<vec2>& path) {
  std::vector<double> xy;
  xy.reserve(path.size() * 2);
  for (const auto& p : path) {
    xy.push_back(p.x);
    xy.push_back(p.y);
  }
  return xy;
}
}  // namespace detail

// painty::TextureBrush<vec3> (TextureBrush.hxx:20-237) with its Smudge. `texture` is the
// brush-stroke sample's thickness map (rows x cols), which painty reads from a sample folder.
class TextureBrush {
 public:
  TextureBrush(const std::vector<double>& texture, int32_t rows, int32_t cols) {
    if (texture.size() != size_t(rows) * size_t(cols)) throw std::invalid_argument("texture size");
    painty_texture_brush* h = nullptr;
    check(painty_texture_brush_create(texture.data(), rows, cols, &h));
    own_ = Owner(h);
  }
  void setRadius(double radius) { check(painty_texture_brush_set_radius(own_.get(), radius)); }
  void dip(const std::array<vec3, 2>& paint) {
    check(painty_texture_brush_dip(own_.get(), paint[0].data(), paint[1].data()));
  }
  void enableSmudge(bool enable) { check(painty_texture_brush_set_smudge(own_.get(), enable ? 1 : 0)); }
  void setThicknessScale(double s) { check(painty_texture_brush_set_thickness_scale(own_.get(), s)); }
  // TextureBrush::paintStroke (TextureBrush.hxx:52-205); returns the pixels painted
  int64_t paintStroke(const std::vector<vec2>& path, Canvas& canvas) {
    const auto xy = detail::flatten(path);
    int64_t n = 0;
    check(painty_texture_brush_paint_stroke(canvas.handle(), own_.get(), xy.data(),
                                            static_cast<int32_t>(path.size()), &n, nullptr));
    return n;
  }

 private:
  using Owner = detail::Handle<painty_texture_brush, painty_texture_brush_destroy>;
  Owner own_;
};

// painty::TextureBrushDictionary (TextureBrushDictionary.hxx:17-39): brush textures in
// (radius, length) classes; the random pick is seeded.
class TextureBrushDictionary {
 public:
  explicit TextureBrushDictionary(uint32_t seed = 0) {
    painty_texture_dictionary* h = nullptr;
    check(painty_texture_dictionary_create(seed, &h));
    own_ = Owner(h);
  }
  int32_t add(uint32_t radiusClass, uint32_t lengthClass, const std::vector<double>& height,
              int32_t rows, int32_t cols) {
    if (height.size() != size_t(rows) * size_t(cols)) throw std::invalid_argument("texture size");
    int32_t i = -1;
    check(painty_texture_dictionary_add(own_.get(), radiusClass, lengthClass, height.data(),
                                        rows, cols, &i));
    return i;
  }
  // lookup(path, brushSize) (TextureBrushDictionary.cxx:25-69): the chosen texture's index
  int32_t lookup(const std::vector<vec2>& path, double brushSize) {
    const auto xy = detail::flatten(path);
    int32_t i = -1;
    check(painty_texture_dictionary_lookup(own_.get(), xy.data(),
                                           static_cast<int32_t>(path.size()), brushSize, &i));
    return i;
  }
  painty_texture_dictionary* handle() const { return own_.get(); }

 private:
  using Owner = detail::Handle<painty_texture_dictionary, painty_texture_dictionary_destroy>;
  Owner own_;
};

// painty::TextureBrushGpu (TextureBrushGpu.hxx:21-64) on the GL canvas path; the dictionary
// must outlive the brush.
class TextureBrushGpu {
 public:
  explicit TextureBrushGpu(TextureBrushDictionary& dict) {
    painty_gpu_texture_brush* h = nullptr;
    check(painty_gpu_texture_brush_create(dict.handle(), &h));
    own_ = Owner(h);
  }
  void setRadius(double radius) { check(painty_gpu_texture_brush_set_radius(own_.get(), radius)); }
  void dip(const std::array<vec3, 2>& paint) {
    check(painty_gpu_texture_brush_dip(own_.get(), paint[0].data(), paint[1].data()));
  }
  void setThicknessScale(double s) {
    check(painty_gpu_texture_brush_set_thickness_scale(own_.get(), s));
  }
  void enableSmudge(bool enable) { check(painty_gpu_texture_brush_set_smudge(own_.get(), enable ? 1 : 0)); }
  // paintStroke(path, CanvasGpu&) (TextureBrushGpu.cxx:74-167)
  void paintStroke(const std::vector<vec2>& path, Canvas& canvas) {
    const auto xy = detail::flatten(path);
    check(painty_gpu_texture_brush_paint_stroke(canvas.handle(), own_.get(), xy.data(),
                                                static_cast<int32_t>(path.size()), nullptr));
  }

 private:
  using Owner = detail::Handle<painty_gpu_texture_brush, painty_gpu_texture_brush_destroy>;
  Owner own_;
};

// painty::SbrRenderThread (renderer/SbrRenderThread.hxx:19-116, src/SbrRenderThread.cxx):
// one worker thread owns a canvas and a TextureBrushGpu (the GL canvas path) and runs the
// requests in submission order; calls return futures. Like painty's, the worker dries the
// canvas by CanvasGpu::dryStep() every `dryInterval` (250 ms in painty; zero turns it off,
// which makes results independent of timing). painty's window refresh has no counterpart.
// The dictionary must outlive the object.
class SbrRenderThread {
 public:
  SbrRenderThread(int32_t rows, int32_t cols, TextureBrushDictionary& dict,
                  const std::vector<double>& background = {},
                  std::chrono::milliseconds dryInterval = std::chrono::milliseconds(250))
      : rows_(rows), cols_(cols), dryInterval_(dryInterval) {
    // painty creates the brush and canvas on its GL thread; here the worker does too
    auto ready = post([this, &dict, background] {
      brush_ = std::make_unique<TextureBrushGpu>(dict);
      canvas_ = std::make_unique<Canvas>(rows_, cols_, Storage::F32);
      if (!background.empty()) canvas_->setBackground(background);
    });
    worker_ = std::thread([this] { loop(); });
    try {
      ready.get();
    } catch (...) {
      shutdown();
      throw;
    }
  }
  SbrRenderThread(const SbrRenderThread&) = delete;
  SbrRenderThread& operator=(const SbrRenderThread&) = delete;
  ~SbrRenderThread() { shutdown(); }
  std::pair<int32_t, int32_t> getSize() const { return {rows_, cols_}; }
  double getBrushThicknessScale() const { return thicknessScale_; }
  // render(path, radius, ks) (SbrRenderThread.cxx:70-78): dip, setRadius, paintStroke
  std::future<void> render(const std::vector<vec2>& path, double radius,
                           const std::array<vec3, 2>& ks) {
    return post([this, path, radius, ks] {
      brush_->dip(ks);
      brush_->setRadius(radius);
      brush_->paintStroke(path, *canvas_);
    });
  }
  // getLinearRgbImage (:80-85): CanvasGpu::getCompositionLinearRgb, rows*cols*3 doubles
  std::future<std::vector<double>> getLinearRgbImage() {
    return post([this] { return canvas_->getComposedGlsl().download(); });
  }
  void setBrushThicknessScale(double scale) {
    thicknessScale_ = scale;
    post([this, scale] { brush_->setThicknessScale(scale); });
  }
  // enableSmudge (:94-98): the GL smudge pass is not provided (see TextureBrushGpu)
  void enableSmudge(bool enable) {
    if (enable)
      throw std::runtime_error("unsupported: the GL smudge pass is not provided");
  }
  // dryCanvas (:100-104): dryStep(1.0)
  std::future<void> dryCanvas() {
    return post([this] { canvas_->dryStep(1.0F); });
  }

 private:
  template <class F>
  auto post(F&& f) -> std::future<decltype(f())> {
    using R = decltype(f());
    auto task = std::make_shared<std::packaged_task<R()>>(std::forward<F>(f));
    std::future<R> fut = task->get_future();
    {
      std::lock_guard<std::mutex> g(m_);
      q_.emplace_back([task] { (*task)(); });
    }
    cv_.notify_one();
    return fut;
  }
  // drains the queue (the last job releases the brush and canvas on the worker), then joins
  void shutdown() {
    if (!worker_.joinable()) return;
    post([this] {
      brush_.reset();
      canvas_.reset();
    });
    {
      std::lock_guard<std::mutex> g(m_);
      stop_ = true;
    }
    cv_.notify_one();
    worker_.join();
  }
  void loop() {
    using clock = std::chrono::steady_clock;
    const bool timer = dryInterval_.count() > 0;
    auto nextDry = clock::now() + dryInterval_;
    for (;;) {
      std::function<void()> job;
      bool dry = false;
      {
        std::unique_lock<std::mutex> lk(m_);
        for (;;) {
          if (timer && clock::now() >= nextDry) {
            dry = true;
            break;
          }
          if (!q_.empty()) {
            job = std::move(q_.front());
            q_.pop_front();
            break;
          }
          if (stop_) return;
          if (timer)
            cv_.wait_until(lk, nextDry);
          else
            cv_.wait(lk);
        }
      }
      if (dry) {  // the drying timer (SbrRenderThread.cxx:37-41): dryStep() every interval
        nextDry = clock::now() + dryInterval_;
        if (canvas_) {
          try {
            canvas_->dryStep();
          } catch (...) {
          }
        }
        continue;
      }
      job();
    }
  }
  int32_t rows_, cols_;
  std::chrono::milliseconds dryInterval_;
  double thicknessScale_ = 1.0;
  std::unique_ptr<TextureBrushGpu> brush_;
  std::unique_ptr<Canvas> canvas_;
  std::mutex m_;
  std::condition_variable cv_;
  std::deque<std::function<void()>> q_;
  bool stop_ = false;
  std::thread worker_;
};

// painty::PaintCoeff (mixer/PaintCoeff.hxx) and its palette JSON files.
struct PaintCoeff {
  vec3 K{}, S{};
};
using Palette = std::vector<PaintCoeff>;

namespace detail {
// The palette JSON grammar: an array of objects whose "K" and "S" members are arrays of three
// numbers (other members are skipped). Throws std::invalid_argument on malformed input.
class PaletteParser {
 public:
  explicit PaletteParser(std::string text) : t_(std::move(text)) {}
  Palette parse() {
    Palette out;
    expect('[');
    if (peek() == ']') {
      ++i_;
      return out;
    }
    for (;;) {
      out.push_back(entry());
      const char c = next();
      if (c == ']') break;
      if (c != ',') fail("',' or ']'");
    }
    return out;
  }

 private:
  PaintCoeff entry() {
    PaintCoeff p;
    bool hasK = false, hasS = false;
    expect('{');
    if (peek() == '}') fail("K and S");
    for (;;) {
      const std::string key = str();
      expect(':');
      if (key == "K" || key == "S") {
        vec3 v{};
        expect('[');
        for (int c = 0; c < 3; c++) {
          if (c) expect(',');
          v[static_cast<size_t>(c)] = num();
        }
        if (peek() == ',') fail("three coefficients");
        expect(']');
        (key == "K" ? p.K : p.S) = v;
        (key == "K" ? hasK : hasS) = true;
      } else {
        skip();
      }
      const char c = next();
      if (c == '}') break;
      if (c != ',') fail("',' or '}'");
    }
    if (!hasK || !hasS) fail("K and S");
    return p;
  }
  void skip() {  // any JSON value
    const char c = peek();
    if (c == '"') {
      str();
    } else if (c == '[' || c == '{') {
      const char close = c == '[' ? ']' : '}';
      ++i_;
      if (peek() == close) {
        ++i_;
        return;
      }
      for (;;) {
        if (c == '{') {
          str();
          expect(':');
        }
        skip();
        const char d = next();
        if (d == close) break;
        if (d != ',') fail("separator");
      }
    } else {
      size_t j = i_;
      while (j < t_.size() && !std::strchr(",]} \t\r\n", t_[j])) ++j;
      if (j == i_) fail("value");
      i_ = j;
    }
  }
  double num() {
    ws();
    const char* b = t_.c_str() + i_;
    char* e = nullptr;
    const double v = std::strtod(b, &e);
    if (e == b) fail("number");
    i_ += static_cast<size_t>(e - b);
    return v;
  }
  std::string str() {
    expect('"');
    std::string s;
    while (i_ < t_.size() && t_[i_] != '"') {
      if (t_[i_] == '\\' && i_ + 1 < t_.size()) ++i_;
      s.push_back(t_[i_++]);
    }
    if (i_ >= t_.size()) fail("closing quote");
    ++i_;
    return s;
  }
  void ws() {
    while (i_ < t_.size() && std::isspace(static_cast<unsigned char>(t_[i_]))) ++i_;
  }
  char peek() {
    ws();
    return i_ < t_.size() ? t_[i_] : '\0';
  }
  char next() {
    const char c = peek();
    if (i_ < t_.size()) ++i_;
    return c;
  }
  void expect(char c) {
    if (next() != c) fail(std::string("'") + c + "'");
  }
  [[noreturn]] void fail(const std::string& what) {
    throw std::invalid_argument("palette JSON: expected " + what + " at offset " +
                                std::to_string(i_));
  }
  std::string t_;
  size_t i_ = 0;
};
}  // namespace detail

// LoadPalette (mixer/src/Serialization.cxx:38-44): appends the stream's paints
inline void LoadPalette(std::istream& stream, Palette& palette) {
  const std::string text((std::istreambuf_iterator<char>(stream)), std::istreambuf_iterator<char>());
  const Palette p = detail::PaletteParser(text).parse();
  palette.insert(palette.end(), p.begin(), p.end());
}

// SavePalette (mixer/src/Serialization.cxx:46-53): compact JSON with sorted keys, numbers in
// the shortest form that reads back to the same double
inline void SavePalette(std::ostream& stream, const Palette& palette) {
  auto number = [](double v) {
    for (int prec = 1; prec <= 17; prec++) {
      std::ostringstream o;
      o.precision(prec);
      o << v;
      if (std::strtod(o.str().c_str(), nullptr) == v) {
        std::string s = o.str();
        if (s.find_first_of(".eEn") == std::string::npos) s += ".0";
        return s;
      }
    }
    return std::to_string(v);
  };
  stream << '[';
  for (size_t i = 0; i < palette.size(); i++) {
    if (i) stream << ',';
    stream << "{\"K\":[" << number(palette[i].K[0]) << ',' << number(palette[i].K[1]) << ','
           << number(palette[i].K[2]) << "],\"S\":[" << number(palette[i].S[0]) << ','
           << number(palette[i].S[1]) << ',' << number(palette[i].S[2]) << "]}";
  }
  stream << ']';
}

// PaintMixer::mixSinglePaint (mixer/src/PaintMixer.cxx:327-355) over a palette of n paints
inline std::array<vec3, 2> mixSinglePaint(const std::vector<double>& weights,
                                          const std::vector<vec3>& K, const std::vector<vec3>& S) {
  if (weights.size() != K.size() || K.size() != S.size())
    throw std::invalid_argument("weights and palette sizes differ");
  std::array<vec3, 2> out{};
  check(painty_mix_paint(weights.data(), static_cast<int32_t>(weights.size()), K.data()->data(),
                         S.data()->data(), out[0].data(), out[1].data()));
  return out;
}

}  // namespace painty_gb300

#endif  // PAINTY_GB300_HPP
