// tdict_ref.cpp -- TEST INFRASTRUCTURE ONLY.
//
// Links lindemeier/painty's own painty/renderer/src/TextureBrushDictionary.cxx, compiled
// unmodified from the reference checkout against the stand-ins in oracle/ref_shim/ (OpenCV's
// normalize / flip / convertTo, prgl's Texture2d), and exposes it through a C API (prefix
// tref_) so tests can pin the oracle's restatement (orc_tdict_*) to it.
//
// The dictionary's constructor scans "data/textures" relative to the working directory and
// reads each file through painty::io::imRead. The harness supplies both: tests create empty
// files named <radius>_<length>_<k>.tex in such a folder, register each file's height map
// under its path here, and tref_create scans the folder from its parent. Everything else --
// the file-name parsing, the size and length classes and their averages, both min-max
// normalisations, the flip into GL rows, the float conversion and the lookup's class choice --
// is painty's code. Its random pick among a class's candidates (std::random_device) is not
// reproducible; tests compare classes, not picks.
#include <unistd.h>

#include <cstdint>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "painty/renderer/TextureBrushDictionary.hxx"

namespace {
std::map<std::string, painty::Mat<double>> g_files;
std::string g_last_read;
}  // namespace

namespace painty {
namespace io {
void imRead(const std::string& filename, Mat<double>& gray, bool) {
  g_last_read = filename;
  gray = g_files.at(filename).clone();
}
}  // namespace io
}  // namespace painty

namespace prgl {
std::shared_ptr<Texture2d> Texture2d::Create(int width, int height, TextureFormatInternal,
                                             TextureFormat, DataType) {
  auto t = std::make_shared<Texture2d>();
  t->width = width;
  t->height = height;
  t->source = g_last_read;
  return t;
}
void Texture2d::upload(const void* data) {
  texels.resize(static_cast<size_t>(width) * height);
  std::memcpy(texels.data(), data, texels.size() * sizeof(float));
}
}  // namespace prgl

extern "C" {

// Registers the height map (rows x cols doubles, row-major) that imRead returns for `path`.
void tref_register(const char* path, const double* height, int32_t rows, int32_t cols) {
  painty::Mat<double> m(rows, cols);
  for (int32_t r = 0; r < rows; r++)
    for (int32_t c = 0; c < cols; c++) m(r, c) = height[static_cast<size_t>(r) * cols + c];
  g_files[path] = m;
}

void tref_clear_registry(void) { g_files.clear(); }

// A dictionary built by painty's constructor from `root`/data/textures (NULL on failure).
void* tref_create(const char* root) {
  char cwd[4096];
  if (!getcwd(cwd, sizeof(cwd)) || chdir(root) != 0) return nullptr;
  painty::TextureBrushDictionary* d = nullptr;
  try {
    d = new painty::TextureBrushDictionary();
  } catch (...) {
    d = nullptr;
  }
  if (chdir(cwd) != 0) {
    delete d;
    return nullptr;
  }
  return d;
}

void tref_destroy(void* d) { delete static_cast<painty::TextureBrushDictionary*>(d); }

// lookup(path, brushSize): copies the picked texture's source path into `source` (cap bytes)
// and, when `texels` is not NULL, its uploaded R32F texels (rows x cols floats, GL row order).
// Returns 0, or -1 when painty throws.
int32_t tref_lookup(void* d, const double* path_xy, int32_t n, double brush_size, char* source,
                    int32_t cap, int32_t* rows, int32_t* cols, float* texels) {
  std::vector<painty::vec2> path(static_cast<size_t>(n));
  for (int32_t i = 0; i < n; i++) path[static_cast<size_t>(i)] = {path_xy[2 * i], path_xy[2 * i + 1]};
  try {
    const auto e = static_cast<painty::TextureBrushDictionary*>(d)->lookup(path, brush_size);
    std::strncpy(source, e.texGpu->source.c_str(), static_cast<size_t>(cap) - 1);
    source[cap - 1] = '\0';
    *rows = e.texGpu->height;
    *cols = e.texGpu->width;
    if (texels) std::memcpy(texels, e.texGpu->texels.data(), e.texGpu->texels.size() * sizeof(float));
  } catch (...) {
    return -1;
  }
  return 0;
}

}  // extern "C"
