// Minimal stand-in for prgl's Texture2d (the GL texture wrapper painty's
// TextureBrushDictionary stores its brush textures in), written for this repository so that
// painty/renderer/src/TextureBrushDictionary.cxx compiles unmodified in the oracle build. A
// texture keeps its uploaded texels in host memory; Create and upload are defined by the
// harness that links it (oracle/tdict_ref.cpp).
#pragma once
#include <memory>
#include <string>
#include <vector>

namespace prgl {
enum class TextureFormatInternal { R32F };
enum class TextureFormat { Red };
enum class DataType { Float };

class Texture2d {
 public:
  static std::shared_ptr<Texture2d> Create(int width, int height, TextureFormatInternal internal,
                                           TextureFormat format, DataType type);
  void upload(const void* data);

  int width = 0, height = 0;
  std::vector<float> texels;  // height rows of width R32F texels, as uploaded
  std::string source;         // the file the harness read just before the texture was made
};
}  // namespace prgl
