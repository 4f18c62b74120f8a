/*
 * painty_oracle.h -- CPU oracle for the Kubelka-Munk paint path of lindemeier/painty.
 *
 * TEST INFRASTRUCTURE ONLY. This library checks the GPU results: only tests/, the smoke check
 * in __graft_entry__.py and bench.py's CPU-baseline leg may load it. The product library
 * (painty_gb300) never links or calls it.
 *
 * It restates, in double precision and with the reference's own loop order and branches:
 *   painty/core/KubelkaMunk.hxx:25-83      ComputeReflectance
 *   painty/core/Math.hxx:157-169           coth
 *   painty/core/Spline.hxx:27-73, 127-220  CatmullRom, derivative, SplineEval
 *   painty/image/Mat.hxx:68-129            Interpolate (BORDER_REFLECT), PaddedMat
 *   painty/renderer/PaintLayer.hxx:21-127  PaintLayer (clear, composeOnto, copyTo)
 *   painty/renderer/Canvas.hxx:26-121      Canvas (ctor, setBackground, dryCanvas)
 *   painty/renderer/FootprintBrush.hxx:46-431  setRadius, imprint, dip/clean, paintStroke,
 *                                          updateSnapshot, blend, pickupPaint, depositPaint
 *   painty/renderer/Renderer.hxx:26-156    Renderer::compose, Renderer::render (lit)
 *   painty/renderer/TextureBrush.hxx:20-237, Smudge.hxx:16-229  the texture brush
 *   painty/mixer/src/PaintMixer.cxx:327-355, 536-548  mixSinglePaint, mixed
 *   painty/core/Color.hxx:186-198, 248-252, 658-763   rgb2xyz, xyz2lab, CIEDE2000
 * and, in float (gl_path.cpp), the GL canvas path's shaders (CanvasGpu, TextureBrushGpu),
 * plus an FP64 Kubelka-Munk oracle (reflectance R and transmittance T) that uses the series
 * form of x*coth(x) near x -> 0 and is finite where the reference returns NaN (K = 0).
 *
 * Layouts: images are row-major, top-left origin. Three-channel planes are interleaved
 * (pixel-major, r,g,b), the way painty's cv::Mat_<vec3> stores them.
 */
#ifndef PAINTY_ORACLE_H
#define PAINTY_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- core math ---- */
double orc_coth(double x);
void orc_compute_reflectance(const double K[3], const double S[3], const double R0[3],
                             double d, double out[3]);
void orc_km_fp64(const double K[3], const double S[3], const double R0[3], double d,
                 double R[3], double T[3]);
void orc_catmull_rom(const double p_1[2], const double p0[2], const double p1[2],
                     const double p2[2], double t, double out[2]);
void orc_catmull_rom_deriv(const double p_1[2], const double p0[2], const double p1[2],
                           const double p2[2], double t, double out[2]);
double orc_catmull_rom_1d(double p_1, double p0, double p1, double p2, double t);
void orc_spline_catmull_rom(const double* pts_xy, int32_t n, double u, double out[2]);
double orc_interpolate(const double* img, int32_t rows, int32_t cols, double x, double y);
/* Footprint setup used by FootprintBrush::setRadius: resample the full-size footprint to
 * width x width (bilinear, pixel-centre aligned, BORDER_REFLECT) and zero-pad by `pad`. */
void orc_resample(const double* src, int32_t rows, int32_t cols, int32_t out_rows,
                  int32_t out_cols, double* out);

/* ---- multi-layer composite (PaintLayer::composeOnto applied layer by layer) ----
 * K,S: L planes of npix*3; V: L planes of npix; R0: npix*3; out: npix*3.
 * mode 0: the reference's ComputeReflectance; mode 1: the FP64 series oracle. */
void orc_compose_layers(int64_t npix, int32_t L, const double* K, const double* S,
                        const double* V, const double* R0, double* out, int32_t mode,
                        int32_t nthreads);
/* Same with float inputs (timed CPU baseline over the GPU's own fp32 planes, SoA). */
void orc_compose_layers_f32_soa_f64(int64_t npix, int32_t L, const float* K, const float* S,
                                    const float* V, const float* R0, double* out,
                                    int32_t nthreads);
void orc_compose_layers_f32_soa(int64_t npix, int32_t L, const float* K, const float* S,
                                const float* V, const float* R0, float* out,
                                int32_t nthreads);

/* ---- canvas / brush objects ---- */
typedef struct orc_canvas orc_canvas;
typedef struct orc_brush orc_brush;

orc_canvas* orc_canvas_create(int32_t rows, int32_t cols);
void orc_canvas_destroy(orc_canvas* c);
/* which: 0 K (npix*3), 1 S (npix*3), 2 V (npix), 3 R0 (npix*3), 4 h (npix) */
double* orc_canvas_plane(orc_canvas* c, int32_t which);
void orc_canvas_dry(orc_canvas* c);
void orc_canvas_compose(const orc_canvas* c, double* out_rgb);

orc_brush* orc_brush_create(double radius, const double* footprint_full, int32_t fh,
                            int32_t fw);
void orc_brush_destroy(orc_brush* b);
void orc_brush_set_radius(orc_brush* b, double radius);
void orc_brush_set_rates(orc_brush* b, double pickup_rate, double deposition_rate);
void orc_brush_set_snapshot(orc_brush* b, int32_t use);
void orc_brush_dip(orc_brush* b, const double K[3], const double S[3]);
void orc_brush_update_snapshot(orc_brush* b, const orc_canvas* c);
void orc_brush_imprint(orc_brush* b, orc_canvas* c, double cx, double cy, double theta);
/* cx_cy_theta: n triples, applied in order */
void orc_brush_stamps(orc_brush* b, orc_canvas* c, const double* cx_cy_theta, int64_t n);
/* FootprintBrush::paintStroke with chord spacing `spacing` (1.0 = the reference). */
int64_t orc_brush_paint_stroke(orc_brush* b, orc_canvas* c, const double* path_xy, int32_t n,
                               double spacing);
/* Stamp list the stroke expands to (cx, cy, theta per stamp); returns the count. Writes at
 * most `cap` triples. */
int64_t orc_stroke_stamps(const double* path_xy, int32_t n, double spacing, double* out,
                          int64_t cap);
/* F: footprint side, S: pickup-map side; returns the brush's current radius */
double orc_brush_info(const orc_brush* b, int32_t* F, int32_t* S);
const double* orc_brush_footprint(const orc_brush* b);
/* which: 0 K (S*S*3), 1 S (S*S*3), 2 V (S*S) */
const double* orc_brush_pickup(const orc_brush* b, int32_t which);
/* snapshot planes, same layout as the canvas wet layer; rows/cols 0 before first use */
const double* orc_brush_snapshot(const orc_brush* b, int32_t which, int32_t* rows,
                                 int32_t* cols);

/* ---- mixing ---- */
void orc_mix_single_paint(const double* weights, int32_t n, const double* palK,
                          const double* palS, double K[3], double S[3]);
void orc_mixed(const double K1[3], const double S1[3], double v1, const double K2[3],
               const double S2[3], double v2, double K[3], double S[3]);

/* ---- colour difference (measurement) ---- */
void orc_rgb2lab(const double rgb[3], double lab[3]);
double orc_ciede2000(const double lab1[3], const double lab2[3]);
/* per-pixel CIEDE2000 between two linear-RGB images (npix*3); returns max, writes mean */
double orc_delta_e_images(int64_t npix, const double* rgb_a, const double* rgb_b,
                          double* mean_out, int32_t nthreads);

/* Renderer::render (Renderer.hxx:60-156): lit rendering of the canvas, out npix*3 */
void orc_canvas_render(const orc_canvas* c, double* out_rgb);

/* TextureBrush<vec3> (TextureBrush.hxx) with its Smudge; the texture is the thickness map. */
typedef struct orc_tbrush orc_tbrush;
orc_tbrush* orc_tbrush_create(const double* tex, int32_t th, int32_t tw);
void orc_tbrush_destroy(orc_tbrush* b);
void orc_tbrush_set_radius(orc_tbrush* b, double radius);
void orc_tbrush_dip(orc_tbrush* b, const double K[3], const double S[3]);
void orc_tbrush_set_smudge(orc_tbrush* b, int32_t on);
void orc_tbrush_set_thickness_scale(orc_tbrush* b, double s);
const double* orc_tbrush_smudge_map(const orc_tbrush* b, int32_t which, int32_t* side);
int64_t orc_tbrush_paint_stroke(orc_tbrush* b, orc_canvas* c, const double* path_xy, int32_t n);

/* ---- the GL canvas path (gl_path.cpp), float: K4/S4/R4 = npix pixels of 4 floats ---- */
/* PaintLayerGpu::composeOnto of one layer onto a copy of R0 (CanvasGpu::getComposed) */
void orc_glsl_compose(int64_t npix, const float* K4, const float* S4, const float* R4,
                      float* out4);
/* CanvasGpu::dryStep(portion) */
void orc_glsl_dry_step(int64_t npix, float* K4, const float* S4, float* R4, float portion);
/* TextureBrushGpu's triangle strip for an n-point path: 2n vertices (xy) and texture
 * coordinates (uv), float pairs */
void orc_gl_strip_vertices(const double* path_xy, int32_t n, double radius, float* xy,
                           float* uv);
/* TextureBrushGpu's imprint and clear passes over an area of interest of aoi_w x aoi_h pixels
 * from (x0, y0), dispatched as whole 16 x 16 tiles; warped: rows*cols floats (R32F) */
void orc_glsl_imprint(int32_t rows, int32_t cols, const float* warped, float* K4, float* S4,
                      int32_t x0, int32_t y0, int32_t aoi_w, int32_t aoi_h, const float Kb[3],
                      const float Sb[3], float scale);
void orc_glsl_clear(int32_t rows, int32_t cols, float* warped, int32_t x0, int32_t y0,
                    int32_t aoi_w, int32_t aoi_h);
/* TextureBrushDictionary with a seeded pick */
typedef struct orc_tdict orc_tdict;
orc_tdict* orc_tdict_create(uint32_t seed);
void orc_tdict_destroy(orc_tdict* d);
int32_t orc_tdict_add(orc_tdict* d, uint32_t radius_class, uint32_t length_class,
                      const double* height, int32_t rows, int32_t cols);
int32_t orc_tdict_lookup(orc_tdict* d, const double* path_xy, int32_t n, double brush_size);
int32_t orc_tdict_texture(const orc_tdict* d, int32_t index, int32_t* rows, int32_t* cols,
                          float* out);
/* TextureBrushGpu (smudge off) */
typedef struct orc_gtbrush orc_gtbrush;
orc_gtbrush* orc_gtbrush_create(void);
void orc_gtbrush_destroy(orc_gtbrush* b);
void orc_gtbrush_set_radius(orc_gtbrush* b, double radius);
void orc_gtbrush_dip(orc_gtbrush* b, const double K[3], const double S[3]);
void orc_gtbrush_set_thickness_scale(orc_gtbrush* b, double s);
int32_t orc_gtbrush_last_texture(const orc_gtbrush* b);
const float* orc_gtbrush_warped(const orc_gtbrush* b);
int32_t orc_gtbrush_paint_stroke(orc_gtbrush* b, orc_tdict* dict, int32_t rows, int32_t cols,
                                 float* K4, float* S4, const double* path_xy, int32_t n);

#ifdef __cplusplus
}
#endif
#endif
