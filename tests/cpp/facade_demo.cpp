// Exercises include/painty_gb300.hpp the way painty's own code uses its classes.
//   facade_demo errors            argument errors surface as std::invalid_argument (no GPU)
//   facade_demo paint IN OUT      paints the stroke described in IN, writes the canvas to OUT
//   facade_demo palette IN OUT    LoadPalette(IN) then SavePalette(OUT) (no GPU)
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

int main(int argc, char** argv) {
  if (argc >= 2 && std::strcmp(argv[1], "errors") == 0) return errors();
  if (argc >= 4 && std::strcmp(argv[1], "paint") == 0) return paint(argv[2], argv[3]);
  if (argc >= 4 && std::strcmp(argv[1], "palette") == 0) return palette(argv[2], argv[3]);
  std::fprintf(stderr, "usage: facade_demo errors | paint IN OUT\n");
  return 2;
}
