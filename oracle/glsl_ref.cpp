// glsl_ref.cpp -- painty's own GL compute shaders, compiled as C++: the reference side of the
// GL-path parity tests.
//
// TEST INFRASTRUCTURE ONLY. `make glsl` (oracle/Makefile) copies the shader sources from the
// reference checkout into oracle/_ref/glsl/ without their #version line and compiles this
// file against them; nothing of the shaders is kept in the repository. Each shader is
// included inside a namespace of its own, with the GLSL stand-ins of glsl_shim.inc:
//   painty/renderer/shaders/ComposeLayerOnSubstrate.compute.glsl      (PaintLayerGpu::composeOnto)
//   painty/renderer/shaders/DryingStep.compute.glsl                   (CanvasGpu::dryStep)
//   painty/renderer/shaders/PaintTextureFootprintOnCanvas.compute.glsl (TextureBrushGpu imprint)
//   painty/renderer/shaders/ClearTextureFootprint.compute.glsl        (TextureBrushGpu clear)
// Images are rows x cols arrays, top row first, of 4 floats (rgba32f: K4 / S4 / R4, V in K.a,
// the lighting volume in S.a) or 1 float (r32f: the warped brush texture).
#include <cmath>
#include <cstdint>

#define layout(...)
#define uniform
#define highp
#define readonly
#define writeonly
#define in

namespace glsl_compose {
#include "glsl_shim.inc"
#define main run
#include "ComposeLayerOnSubstrate.compute.glsl"
#undef main
}  // namespace glsl_compose

namespace glsl_dry {
#include "glsl_shim.inc"
#define main run
#include "DryingStep.compute.glsl"
#undef main
}  // namespace glsl_dry

namespace glsl_imprint {
#include "glsl_shim.inc"
#define main run
#include "PaintTextureFootprintOnCanvas.compute.glsl"
#undef main
}  // namespace glsl_imprint

namespace glsl_clear {
#include "glsl_shim.inc"
#define main run
#include "ClearTextureFootprint.compute.glsl"
#undef main
}  // namespace glsl_clear

namespace {

int groups(int n) { return n > 0 ? (n + 15) / 16 : 0; }

}  // namespace

extern "C" {

// CanvasGpu::getComposed: ComposeLayerOnSubstrate over the whole canvas; R4 is composed in
// place (the caller passes a copy of R0).
void glref_compose(int32_t rows, int32_t cols, const float* K4, const float* S4, float* R4) {
  using namespace glsl_compose;
  tex_R0 = {R4, cols, rows, 4};
  tex_K = {const_cast<float*>(K4), cols, rows, 4};
  tex_S = {const_cast<float*>(S4), cols, rows, 4};
  offset = ivec2(0, 0);
  dispatch(groups(cols), groups(rows), run);
}

// CanvasGpu::dryStep: DryingStep with `dry_portion`, in place on K4 and R4.
void glref_dry_step(int32_t rows, int32_t cols, float* K4, float* S4, float* R4,
                    float dry_portion) {
  using namespace glsl_dry;
  tex_R0 = {R4, cols, rows, 4};
  tex_K = {K4, cols, rows, 4};
  tex_S = {S4, cols, rows, 4};
  offset = ivec2(0, 0);
  dryPortion = dry_portion;
  dispatch(groups(cols), groups(rows), run);
}

// TextureBrushGpu's imprint: PaintTextureFootprintOnCanvas over the area of interest
// (aoi_w x aoi_h pixels from (x0, y0), in image coordinates), in place on K4 and S4.
void glref_imprint(int32_t rows, int32_t cols, const float* warped, float* K4, float* S4,
                   int32_t x0, int32_t y0, int32_t aoi_w, int32_t aoi_h, const float Kb[3],
                   const float Sb[3], float thickness_scale) {
  using namespace glsl_imprint;
  warpedBrushTexture = {const_cast<float*>(warped), cols, rows, 1};
  tex_K = {K4, cols, rows, 4};
  tex_S = {S4, cols, rows, 4};
  offset = ivec2(x0, y0);
  K_brush = vec3(Kb[0], Kb[1], Kb[2]);
  S_brush = vec3(Sb[0], Sb[1], Sb[2]);
  thicknessScale = thickness_scale;
  dispatch(groups(aoi_w), groups(aoi_h), run);
}

// TextureBrushGpu's clear: ClearTextureFootprint over the same area, in place on `warped`.
void glref_clear(int32_t rows, int32_t cols, float* warped, int32_t x0, int32_t y0,
                 int32_t aoi_w, int32_t aoi_h) {
  using namespace glsl_clear;
  warpedBrushTexture = {warped, cols, rows, 1};
  offset = ivec2(x0, y0);
  dispatch(groups(aoi_w), groups(aoi_h), run);
}

}  // extern "C"
