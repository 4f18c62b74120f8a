// Exercises include/painty_gb300.hpp the way painty's own code uses its classes.
//   facade_demo errors            argument errors surface as std::invalid_argument (no GPU)
//   facade_demo paint IN OUT      paints the stroke described in IN, writes the canvas to OUT
//   facade_demo palette IN OUT    LoadPalette(IN) then SavePalette(OUT) (no GPU)
//   facade_demo texture IN OUT    TextureBrush stroke + Renderer::render (F64), canvas to OUT
//                                 IN: rows, cols, th, tw, tex[th*tw], npts, path[2*npts],
//                                 radius, K[3], S[3]; OUT: painted, K, S, V, lit[rows*cols*3]
//   facade_demo sbr               strokes through SbrRenderThread equal the same strokes
//                                 painted directly with TextureBrushGpu (GPU)
// IN (doubles): rows, cols, fh, fw, footprint[fh*fw], npts, path[2*npts], radius, spacing,
//               pickup, deposition, K[3], S[3], R0[rows*cols*3]
// OUT (doubles): stamps, K[rows*cols*3], S[rows*cols*3], V[rows*cols], composite[rows*cols*3]
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iostream>
#include <sstream>
#include <stdexcept>
#include <vector>

#include "painty_gb300.hpp"

namespace pg = painty_gb300;

static int errors() {
  int ok = 0;
  try {
    pg::Canvas bad(0, 5);
  } catch (const std::invalid_argument&) {
    ok++;
  }
  try {
    std::vector<double> fp(4, 1.0);
    pg::FootprintBrush b(-1.0, fp, 2, 2);
  } catch (const std::invalid_argument&) {
    ok++;
  }
  for (const char* bad : {"[{\"K\":[1,2,3]}]", "[{\"K\":[1,2],\"S\":[1,2,3]}]", "{", "[1]"}) {
    try {
      std::istringstream in(bad);
      pg::Palette p;
      pg::LoadPalette(in, p);
    } catch (const std::invalid_argument&) {
      ok++;
    }
  }
  std::printf("%s\n", ok == 6 ? "errors ok" : "errors FAILED");
  return ok == 6 ? 0 : 1;
}

static int palette(const char* in, const char* out) {
  std::ifstream f(in);
  pg::Palette p;
  pg::LoadPalette(f, p);
  std::ofstream o(out);
  pg::SavePalette(o, p);
  std::printf("palette of %zu paints\n", p.size());
  return 0;
}

static int paint(const char* in, const char* out) {
  std::ifstream f(in, std::ios::binary | std::ios::ate);
  const std::streamsize bytes = f.tellg();
  f.seekg(0);
  std::vector<double> v(static_cast<size_t>(bytes) / sizeof(double));
  f.read(reinterpret_cast<char*>(v.data()), static_cast<std::streamsize>(v.size() * sizeof(double)));
  size_t i = 0;
  auto take = [&](size_t n) {
    std::vector<double> r(v.begin() + i, v.begin() + i + n);
    i += n;
    return r;
  };
  const int rows = static_cast<int>(v[i++]), cols = static_cast<int>(v[i++]);
  const int fh = static_cast<int>(v[i++]), fw = static_cast<int>(v[i++]);
  const auto footprint = take(size_t(fh) * fw);
  const int npts = static_cast<int>(v[i++]);
  const auto xy = take(size_t(npts) * 2);
  const double radius = v[i++], spacing = v[i++], pickup = v[i++], deposition = v[i++];
  const auto K = take(3), S = take(3);
  const auto R0 = take(size_t(rows) * cols * 3);

  pg::Canvas canvas(rows, cols, pg::Storage::F64);
  canvas.setBackground(R0);
  pg::FootprintBrush brush(radius, footprint, fh, fw);
  brush.setPickupRate(pickup);
  brush.setDepositionRate(deposition);
  brush.dip({pg::vec3{K[0], K[1], K[2]}, pg::vec3{S[0], S[1], S[2]}});
  std::vector<pg::vec2> path;
  for (int p = 0; p < npts; p++) path.push_back({xy[2 * p], xy[2 * p + 1]});
  const int64_t n = brush.paintStroke(path, canvas, spacing);
  auto layer = canvas.getPaintLayer();
  const auto k = layer.getK_buffer(), s = layer.getS_buffer(), vol = layer.getV_buffer();
  const auto rgb = pg::Renderer().compose(canvas, pg::Storage::F64).download();
  std::ofstream o(out, std::ios::binary);
  const double nd = static_cast<double>(n);
  o.write(reinterpret_cast<const char*>(&nd), sizeof(double));
  for (const auto* vec : {&k, &s, &vol, &rgb})
    o.write(reinterpret_cast<const char*>(vec->data()),
            static_cast<std::streamsize>(vec->size() * sizeof(double)));
  std::printf("painted %lld stamps\n", static_cast<long long>(n));
  return 0;
}

// deterministic values in [0, 1) (a 64-bit LCG; the demo needs no particular generator)
static double unit(uint64_t& s) {
  s = s * 6364136223846793005ULL + 1442695040888963407ULL;
  return static_cast<double>(s >> 11) * (1.0 / 9007199254740992.0);
}

static void fill_dictionary(pg::TextureBrushDictionary& d) {
  uint64_t s = 99;
  for (int rc = 0; rc < 2; rc++)
    for (int lc = 0; lc < 2; lc++)
      for (int k = 0; k < 2; k++) {
        const int rows = rc ? 34 : 10, cols = lc ? 220 : 60;
        std::vector<double> h(size_t(rows) * cols);
        for (auto& x : h) x = unit(s);
        d.add(rc ? 16 : 4, lc ? 200 : 50, h, rows, cols);
      }
}

static int sbr() {
  const int rows = 96, cols = 128;
  std::vector<double> bg(size_t(rows) * cols * 3, 0.9);
  struct Stroke {
    std::vector<pg::vec2> path;
    double radius;
    std::array<pg::vec3, 2> ks;
  };
  std::vector<Stroke> strokes;
  uint64_t s = 7;
  for (int i = 0; i < 12; i++) {
    Stroke st;
    const int n = 2 + static_cast<int>(unit(s) * 5);
    for (int p = 0; p < n; p++) st.path.push_back({unit(s) * cols, unit(s) * rows});
    st.radius = 2.0 + 18.0 * unit(s);
    st.ks = {pg::vec3{unit(s) * 5, unit(s) * 5, unit(s) * 5},
             pg::vec3{0.05 + unit(s) * 3, 0.05 + unit(s) * 3, 0.05 + unit(s) * 3}};
    strokes.push_back(st);
  }
  std::vector<double> a, b;
  {
    pg::TextureBrushDictionary dict(5);
    fill_dictionary(dict);
    pg::SbrRenderThread sbr(rows, cols, dict, bg, std::chrono::milliseconds(0));
    std::vector<std::future<void>> done;
    for (const auto& st : strokes) done.push_back(sbr.render(st.path, st.radius, st.ks));
    a = sbr.getLinearRgbImage().get();
    for (auto& f : done) f.get();
    sbr.dryCanvas().get();
    const auto dried = sbr.getLinearRgbImage().get();
    if (dried.size() != a.size()) return 1;
  }
  {
    pg::TextureBrushDictionary dict(5);
    fill_dictionary(dict);
    pg::TextureBrushGpu brush(dict);
    pg::Canvas canvas(rows, cols, pg::Storage::F32);
    canvas.setBackground(bg);
    for (const auto& st : strokes) {
      brush.dip(st.ks);
      brush.setRadius(st.radius);
      brush.paintStroke(st.path, canvas);
    }
    b = canvas.getComposedGlsl().download();
  }
  const bool same = a.size() == b.size() && std::memcmp(a.data(), b.data(), a.size() * 8) == 0;
  bool painted = false;
  for (size_t i = 0; i < a.size(); i++) painted = painted || a[i] != 0.9f;
  std::printf("%s\n", same && painted ? "sbr ok" : "sbr FAILED");
  return same && painted ? 0 : 1;
}

static int texture(const char* in, const char* out) {
  std::ifstream f(in, std::ios::binary | std::ios::ate);
  const std::streamsize bytes = f.tellg();
  f.seekg(0);
  std::vector<double> v(static_cast<size_t>(bytes) / sizeof(double));
  f.read(reinterpret_cast<char*>(v.data()), static_cast<std::streamsize>(v.size() * sizeof(double)));
  size_t i = 0;
  auto take = [&](size_t n) {
    std::vector<double> r(v.begin() + i, v.begin() + i + n);
    i += n;
    return r;
  };
  const int rows = static_cast<int>(v[i++]), cols = static_cast<int>(v[i++]);
  const int th = static_cast<int>(v[i++]), tw = static_cast<int>(v[i++]);
  const auto tex = take(size_t(th) * tw);
  const int npts = static_cast<int>(v[i++]);
  const auto xy = take(size_t(npts) * 2);
  const double radius = v[i++];
  const auto K = take(3), S = take(3);
  pg::Canvas canvas(rows, cols, pg::Storage::F64);
  canvas.setBackground(std::vector<double>(size_t(rows) * cols * 3, 0.9));
  pg::TextureBrush brush(tex, th, tw);
  brush.setRadius(radius);
  brush.dip({pg::vec3{K[0], K[1], K[2]}, pg::vec3{S[0], S[1], S[2]}});
  std::vector<pg::vec2> path;
  for (int p = 0; p < npts; p++) path.push_back({xy[2 * p], xy[2 * p + 1]});
  const int64_t painted = brush.paintStroke(path, canvas);
  auto layer = canvas.getPaintLayer();
  const auto k = layer.getK_buffer(), s = layer.getS_buffer(), vol = layer.getV_buffer();
  const auto lit = pg::Renderer().render(canvas, pg::Storage::F64).download();
  std::ofstream o(out, std::ios::binary);
  const double nd = static_cast<double>(painted);
  o.write(reinterpret_cast<const char*>(&nd), sizeof(double));
  for (const auto* vec : {&k, &s, &vol, &lit})
    o.write(reinterpret_cast<const char*>(vec->data()),
            static_cast<std::streamsize>(vec->size() * sizeof(double)));
  std::printf("painted %lld pixels\n", static_cast<long long>(painted));
  return 0;
}

int main(int argc, char** argv) {
  if (argc >= 4 && std::strcmp(argv[1], "texture") == 0) return texture(argv[2], argv[3]);
  if (argc >= 2 && std::strcmp(argv[1], "sbr") == 0) return sbr();
  if (argc >= 2 && std::strcmp(argv[1], "errors") == 0) return errors();
  if (argc >= 4 && std::strcmp(argv[1], "paint") == 0) return paint(argv[2], argv[3]);
  if (argc >= 4 && std::strcmp(argv[1], "palette") == 0) return palette(argv[2], argv[3]);
  std::fprintf(stderr, "usage: facade_demo errors | paint IN OUT\n");
  return 2;
}
