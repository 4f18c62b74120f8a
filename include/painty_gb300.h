/*
 * painty_gb300.h -- C ABI of the GB300-native Kubelka-Munk paint path.
 *
 * A drop-in for lindemeier/painty's paint-rendering hot path: the imprint brush's stamp
 * deposition onto the wet/dry canvas layers, the volume-weighted K,S mixing of pickup and
 * deposit, and the per-pixel Kubelka-Munk layer composite onto the substrate reflectance.
 * The C++ facade in painty_gb300.hpp mirrors painty's Canvas / FootprintBrush / Renderer
 * classes on top of these entry points.
 *
 * Conventions
 *  - Every call returns painty_status; nothing throws across this boundary.
 *    painty_last_error() gives a message for the calling thread's last failure.
 *  - Handles own device memory; the caller owns host buffers. Host images are row-major with
 *    a top-left origin (painty's cv::Mat_ layout, no y-flip).
 *  - `stream` is a cudaStream_t (NULL = the legacy default stream). Calls that take host
 *    buffers are synchronous with respect to those buffers: they return once the host
 *    memory may be reused (upload) or holds the result (download).
 *  - A handle may be used from one thread at a time.
 *  - Storage formats: F32 (default), F16 / BF16 (K and S in that type, volume in FP16; all
 *    arithmetic in FP32), F64 (double storage and arithmetic: the parity mode whose stamping
 *    reproduces painty's double-precision CPU results bit for bit).
 */
#ifndef PAINTY_GB300_H
#define PAINTY_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PAINTY_GB300_ABI_VERSION 2

typedef enum painty_status {
  PAINTY_OK = 0,
  PAINTY_ERR_INVALID_ARGUMENT = 1, /* painty throws std::invalid_argument */
  PAINTY_ERR_OUT_OF_MEMORY = 2,
  PAINTY_ERR_CUDA = 3,
  PAINTY_ERR_UNSUPPORTED = 4,
  PAINTY_ERR_BUDGET = 5,    /* serving: request larger than the memory budget */
  PAINTY_ERR_TIMEOUT = 6,   /* a bounded device wait ran out */
  PAINTY_ERR_CANCELLED = 7, /* serving: request cancelled before it ran */
  PAINTY_ERR_STATE = 8      /* handle in the wrong state for the call */
} painty_status;

typedef enum painty_storage {
  PAINTY_STORAGE_F32 = 0,
  PAINTY_STORAGE_F16 = 1,
  PAINTY_STORAGE_BF16 = 2,
  PAINTY_STORAGE_F64 = 3
} painty_storage;

/* Host buffer formats. INTERLEAVED = pixel-major channels (cv::Mat_<vec3>);
 * PLANAR = one full rows*cols plane per channel. One-channel planes read the same either way. */
typedef enum painty_host_format {
  PAINTY_HOST_F64_INTERLEAVED = 0,
  PAINTY_HOST_F32_INTERLEAVED = 1,
  PAINTY_HOST_F64_PLANAR = 2,
  PAINTY_HOST_F32_PLANAR = 3
} painty_host_format;

/* Planes of a paint layer / canvas. */
typedef enum painty_plane {
  PAINTY_PLANE_K = 0,  /* absorption, 3 channels */
  PAINTY_PLANE_S = 1,  /* scattering, 3 channels */
  PAINTY_PLANE_V = 2,  /* paint volume (layer thickness), 1 channel */
  PAINTY_PLANE_R0 = 3, /* canvas only: substrate reflectance, 3 channels */
  PAINTY_PLANE_H = 4,  /* canvas only: height map, 1 channel */
  PAINTY_PLANE_VL = 5  /* canvas only: the GL path's lighting volume (S.a of painty's
                          PaintLayerGpu, PaintTextureFootprintOnCanvas.compute.glsl:51-52) */
} painty_plane;

typedef struct painty_layer painty_layer;   /* PaintLayer<vec3>  (K, S, V) */
typedef struct painty_image painty_image;   /* Mat<vec3> reflectance image on the device */
typedef struct painty_canvas painty_canvas; /* Canvas<vec3>: wet layer + R0 + h */
typedef struct painty_brush painty_brush;   /* FootprintBrush<vec3> */

/* ------------------------------------------------------------------ library */
int32_t painty_abi_version(void);
/* Build properties of the loaded library: PAINTY_BUILD_BOUNDS_CHECK is set in the
 * bounds-checked build (libpainty_gb300_checked.so), whose stamp kernels test every computed
 * index against its buffer and return PAINTY_ERR_CUDA naming the access instead of faulting.
 * No counterpart in painty. */
#define PAINTY_BUILD_BOUNDS_CHECK 1
/* PAINTY_BUILD_PHASE_TIMERS is set in the phase-timing build (libpainty_gb300_phases.so), whose
 * stamp loop adds each warp's clock cycles per phase into device counters read with
 * painty_take_phase_cycles. */
#define PAINTY_BUILD_PHASE_TIMERS 2
int32_t painty_build_flags(void);
/* Phase-timing build only: reads and clears the stamp loop's counters (synchronises the
 * device). out[0..7]: warp cycles summed over warps and stamps in painting, the snapshot ring
 * refresh, classification, parameter derivation, per-stamp setup, the CTA barrier, the
 * cluster barrier, and edge-duplicate (wave) painting with its refresh; out[8]: stamps summed
 * over CTAs; out[9]: warp-stamps (stamps times warps per CTA, summed over CTAs); out[10..15]:
 * 0. PAINTY_ERR_UNSUPPORTED in other builds. No counterpart in painty. */
painty_status painty_take_phase_cycles(uint64_t out[16]);
const char* painty_status_string(painty_status s);
const char* painty_last_error(void);
/* Number of this library's kernel launches so far in this process (all devices). */
int64_t painty_kernel_launch_count(void);
/* Reads and clears the current device's pipeline-fault word: nonzero when a kernel's
 * shared-memory copy pipeline stalled beyond its one-second wait limit since the last call
 * (that kernel wrote NaN where it stopped instead of hanging). Synchronises the device.
 * No counterpart in painty. */
painty_status painty_take_device_faults(uint32_t* faults);

/* ------------------------------------------------------------------ layers
 * replaces PaintLayer<vec>::PaintLayer(rows, cols) + clear()  (painty/renderer/PaintLayer.hxx:27-30, 68-74) */
painty_status painty_layer_create(int32_t rows, int32_t cols, painty_storage storage,
                                  painty_layer** out);
painty_status painty_layer_destroy(painty_layer* layer);
/* replaces PaintLayer::clear (PaintLayer.hxx:68-74) */
painty_status painty_layer_clear(painty_layer* layer, void* stream);
/* replaces writes through getK_buffer/getS_buffer/getV_buffer (PaintLayer.hxx:32-54) */
painty_status painty_layer_upload(painty_layer* layer, painty_plane plane, const void* host,
                                  painty_host_format fmt, void* stream);
painty_status painty_layer_download(const painty_layer* layer, painty_plane plane, void* host,
                                    painty_host_format fmt, void* stream);
/* replaces PaintLayer::set(i, j, k, s, v) (PaintLayer.hxx:122-127) for n cells in order:
 * rows_cols = n (row, col) pairs, K and S = n triples, V = n values (host). Later cells win
 * where cells repeat. At most 2^24 cells per call. */
painty_status painty_layer_set_cells(painty_layer* layer, int64_t n, const int32_t* rows_cols,
                                     const double* K, const double* S, const double* V,
                                     void* stream);
/* replaces PaintLayer::copyTo (PaintLayer.hxx:103-111); same size and storage */
painty_status painty_layer_copy(const painty_layer* src, painty_layer* dst, void* stream);
painty_status painty_layer_info(const painty_layer* layer, int32_t* rows, int32_t* cols,
                                painty_storage* storage);

/* ------------------------------------------------------------------ images (R0, R1)
 * F32 or F64 storage. */
painty_status painty_image_create(int32_t rows, int32_t cols, painty_storage storage,
                                  painty_image** out);
painty_status painty_image_destroy(painty_image* img);
painty_status painty_image_fill(painty_image* img, double r, double g, double b, void* stream);
painty_status painty_image_upload(painty_image* img, const void* host, painty_host_format fmt,
                                  void* stream);
painty_status painty_image_download(const painty_image* img, void* host,
                                    painty_host_format fmt, void* stream);

/* ------------------------------------------------------------------ composite
 * replaces PaintLayer::composeOnto applied to layers[0..L-1] in order
 * (painty/renderer/PaintLayer.hxx:81-96, per pixel painty/core/KubelkaMunk.hxx:25-83),
 * fused into one pass: out = KM(layer L-1, ... KM(layer 0, r0)). `out` may be `r0`
 * (in place, as composeOnto). Layers share size; out/r0 storage F32, or F64 with F64 layers. */
painty_status painty_compose_layers(const painty_layer* const* layers, int32_t L,
                                    const painty_image* r0, painty_image* out, void* stream);
/* The same one layer per launch (the plain drop-in composeOnto, R0 read and written per layer). */
painty_status painty_compose_layers_unfused(const painty_layer* const* layers, int32_t L,
                                            const painty_image* r0, painty_image* out,
                                            void* stream);
/* Renderer::compose of layer stacks held in host memory into a host image
 * (painty/renderer/Renderer.hxx:26-53, returning a host Mat; per layer PaintLayer.hxx:81-96).
 * Host layout, FP32 planar, rows x cols per plane, contiguous: K and S [L][3][rows][cols],
 * V [L][rows][cols], R0 and out [3][rows][cols]. When every buffer is pinned (mapped into the
 * device's address space; rows * cols a multiple of 4, planes 16-byte aligned) the fused
 * composite reads and writes them in place over the host link; otherwise the transfers run
 * in row bands on three internal streams, the upload of one band, the composite of another and
 * the download of a third overlapping. Returns once `out` holds the result. */
painty_status painty_compose_layers_host(const float* K, const float* S, const float* V,
                                         int32_t L, const float* R0, float* out, int32_t rows,
                                         int32_t cols, void* stream);

/* ------------------------------------------------------------------ canvas
 * replaces Canvas<vec>::Canvas(rows, cols) (painty/renderer/Canvas.hxx:26-35): wet layer
 * cleared, R0 = background 1.0, h = 0. */
painty_status painty_canvas_create(int32_t rows, int32_t cols, painty_storage storage,
                                   painty_canvas** out);
painty_status painty_canvas_destroy(painty_canvas* canvas);
/* replaces Canvas::clear (Canvas.hxx:37-58) */
painty_status painty_canvas_clear(painty_canvas* canvas, void* stream);
/* plane K/S/V: the wet layer; R0: substrate (replaces Canvas::setBackground, :80-87); H */
painty_status painty_canvas_upload(painty_canvas* canvas, painty_plane plane, const void* host,
                                   painty_host_format fmt, void* stream);
painty_status painty_canvas_download(const painty_canvas* canvas, painty_plane plane,
                                     void* host, painty_host_format fmt, void* stream);
/* Borrowed handles (valid while the canvas lives): Canvas::getPaintLayer, Canvas::getR0 */
painty_status painty_canvas_layer(painty_canvas* canvas, painty_layer** out);
painty_status painty_canvas_r0(painty_canvas* canvas, painty_image** out);
painty_status painty_canvas_info(const painty_canvas* canvas, int32_t* rows, int32_t* cols,
                                 painty_storage* storage);
/* replaces Renderer<vec>::compose(canvas) (painty/renderer/Renderer.hxx:26-53) */
painty_status painty_canvas_compose(const painty_canvas* canvas, painty_image* out, void* stream);
/* replaces Renderer::render(canvas) (painty/renderer/Renderer.hxx:60-156): the composite lit
 * by painty's point light (Cook-Torrance with its Beckmann and geometric terms; normals from
 * the wet layer's volume), clamped to [0, 1]. out: F64 for F64 canvases, F32 otherwise. */
painty_status painty_canvas_render(const painty_canvas* canvas, painty_image* out, void* stream);
/* replaces Canvas::dryCanvas (Canvas.hxx:105-121): h += V, R0 = KM(K,S,R0,V), wet = 0 */
painty_status painty_canvas_dry(painty_canvas* canvas, void* stream);

/* ------------------------------------------------------------------ imprint brush
 * replaces FootprintBrush<vec>::FootprintBrush(radius) (painty/renderer/FootprintBrush.hxx:29-37).
 * `footprint` (fh x fw, row-major, values in [0,1]) stands in for data/footprint/footprint.png:
 * setRadius resamples it to the brush width (bilinear, pixel-centre aligned, BORDER_REFLECT)
 * and pads it to cover all rotations (FootprintBrush.hxx:46-63). */
painty_status painty_brush_create(double radius, const double* footprint, int32_t fh,
                                  int32_t fw, painty_brush** out);
painty_status painty_brush_destroy(painty_brush* brush);
/* replaces FootprintBrush::setRadius (:46-63); no change unless |radius - current| >= 0.5 */
painty_status painty_brush_set_radius(painty_brush* brush, double radius);
/* replaces setPickupRate / setDepositionRate (:182-188) */
painty_status painty_brush_set_rates(painty_brush* brush, double pickup_rate,
                                     double deposition_rate);
painty_status painty_brush_get_rates(const painty_brush* brush, double* pickup_rate,
                                     double* deposition_rate);
/* replaces setUseSnapshotBuffer (:202-204) */
painty_status painty_brush_set_snapshot(painty_brush* brush, int32_t use);
/* replaces dip (:150-154): clears the pickup map, sets the paint {K, S} */
painty_status painty_brush_dip(painty_brush* brush, const double K[3], const double S[3],
                               void* stream);
/* replaces updateSnapshot(canvas) (:168-172) */
painty_status painty_brush_update_snapshot(painty_brush* brush, const painty_canvas* canvas,
                                           void* stream);
/* F = footprint side, S = pickup-map side (getFootprint / getPickupMap sizes) */
painty_status painty_brush_info(const painty_brush* brush, double* radius, int32_t* F,
                                int32_t* S);
/* getFootprint (:178-180): F*F doubles */
painty_status painty_brush_footprint(const painty_brush* brush, double* host);
/* getPickupMap (:174-176): plane K/S (S*S*3 interleaved) or V (S*S) */
painty_status painty_brush_download_pickup(const painty_brush* brush, painty_plane plane,
                                           void* host, painty_host_format fmt, void* stream);

/* replaces FootprintBrush::imprint(center, theta, canvas) (:73-143) */
painty_status painty_imprint(painty_canvas* canvas, painty_brush* brush, double cx, double cy,
                             double theta, void* stream);
/* n imprints in order; cx_cy_theta = n triples (host) */
painty_status painty_stamps(painty_canvas* canvas, painty_brush* brush,
                            const double* cx_cy_theta, int64_t n, void* stream);
/* replaces FootprintBrush::paintStroke(path, canvas) (:206-268): Catmull-Rom through the
 * path, a stamp every `spacing` of chord length per segment (1.0 = the reference), angle
 * from the spline derivative. path_xy = n (x, y) pairs (host). Returns the stamp count. */
painty_status painty_stroke(painty_canvas* canvas, painty_brush* brush, const double* path_xy,
                            int32_t n, double spacing, int64_t* stamps_out, void* stream);

/* ------------------------------------------------------------------ batched painting
 * Many canvases, each with its own brush, painted in one persistent launch. For every canvas,
 * its strokes (in array order) are applied as painty's
 *     brush.setRadius(radius); brush.dip({K, S}); brush.paintStroke(path, canvas)
 * (FootprintBrush.hxx:46-63, 150-154, 206-268) with stamps every `spacing` of chord length
 * (1.0 = painty). Canvases are independent and run concurrently, heaviest first; a canvas's
 * strokes run in order. Results equal the sequential calls, except that the stamp angles'
 * atan2/cos/sin come from the device's double functions (within 1-2 ulp of libm's).
 * All canvases share one storage format; a brush belongs to one canvas of the batch. */
typedef struct painty_stroke_desc {
  int32_t canvas;      /* index into canvases[] */
  int32_t npoints;     /* control points, at most 512 */
  int64_t first_point; /* first (x, y) pair in points[] */
  double radius;       /* setRadius before the stroke */
  double spacing;      /* stamp spacing along each segment's chord */
  double K[3], S[3];   /* dip before the stroke */
} painty_stroke_desc;
painty_status painty_paint_batch(painty_canvas* const* canvases, painty_brush* const* brushes,
                                 int32_t ncanvas, const painty_stroke_desc* strokes, int64_t nstrokes,
                                 const double* points, int64_t npoints, int64_t* stamps_out,
                                 void* stream);

/* The launch shape the last painty_paint_batch on this thread chose: CTAs per canvas (a
 * thread-block cluster sharing each stamp), the number of clusters launched, and threads per
 * CTA (one CTA per SM: 1024 threads, or 512 with twice the registers per thread, used by
 * clusters for boxes up to side 127). Picked by a makespan model of the batch unless the
 * environment variables PAINTY_BATCH_CLUSTER / PAINTY_BATCH_THREADS set them. Any pointer may
 * be NULL. No counterpart in painty. */
painty_status painty_batch_last_shape(int32_t* cluster, int32_t* clusters, int32_t* threads);
/* Whether the last painty_paint_batch on this thread gave its heaviest canvases a launch of
 * their own, next to the rest, on clusters of `cluster` CTAs (0: no such launch), and how
 * many canvases that launch painted. The shape above is then that of the rest. A canvas's
 * stamps run in order, so the heaviest canvas bounds a batch unless more CTAs share its
 * stamps. No counterpart in painty. */
painty_status painty_batch_last_split(int32_t* cluster, int32_t* canvases);

/* ------------------------------------------------------------------ texture brush
 * TextureBrush<vec3> (painty/renderer/TextureBrush.hxx:20-237) with its Smudge<vec3>
 * (painty/renderer/Smudge.hxx:16-229). The texture is the brush-stroke sample's thickness
 * map (BrushStrokeSample::getThicknessMap), rows x cols doubles, row-major; painty's
 * constructor loads it from the sample directory, which this interface leaves to the
 * caller. A brush binds to F64 canvases or to F32/F16/BF16 canvases at its first stroke. */
typedef struct painty_texture_brush painty_texture_brush;
/* replaces TextureBrush(sampleDir) (:25-31): paint {0.1, 0.1, 0.1} x2, smudge on, radius 0 */
painty_status painty_texture_brush_create(const double* texture, int32_t rows, int32_t cols,
                                          painty_texture_brush** out);
painty_status painty_texture_brush_destroy(painty_texture_brush* brush);
/* replaces setRadius (:33-41): no change unless |radius - current| >= 0.5; a change makes a
 * new smudge of side int(2 radius) (clear pickup map, rotation 0) */
painty_status painty_texture_brush_set_radius(painty_texture_brush* brush, double radius);
/* replaces dip (:48-50) */
painty_status painty_texture_brush_dip(painty_texture_brush* brush, const double K[3],
                                       const double S[3]);
/* replaces enableSmudge (:207-209) */
painty_status painty_texture_brush_set_smudge(painty_texture_brush* brush, int32_t enable);
/* replaces BrushBase::setThicknessScale (painty/renderer/BrushBase.hxx:31-33) */
painty_status painty_texture_brush_set_thickness_scale(painty_texture_brush* brush,
                                                       double scale);
/* replaces paintStroke(verts, canvas) (:52-205): path_xy = n (x, y) pairs (host, n >= 2 to
 * paint; at most 4096 points). painted_out (may be null) receives the pixels the stroke
 * deposited on. A stroke whose bounds lie off the canvas paints nothing (painty fails on it).
 * With the smudge on, the smudge map is at most 4096 wide (radius below 2048). Synchronises
 * the stream. */
painty_status painty_texture_brush_paint_stroke(painty_canvas* canvas,
                                                painty_texture_brush* brush,
                                                const double* path_xy, int32_t n,
                                                int64_t* painted_out, void* stream);
/* the smudge pickup map (Smudge.hxx _pickupMapDst): plane K/S (side*side*3 interleaved) or
 * V (side*side) doubles; side_out receives the side; host may be null to query it */
painty_status painty_texture_brush_smudge_map(const painty_texture_brush* brush,
                                              painty_plane plane, double* host,
                                              int32_t* side_out, void* stream);

/* ------------------------------------------------------------------ the GL canvas path
 * painty's second renderer (CanvasGpu, PaintLayerGpu, TextureBrushGpu) keeps the canvas in
 * rgba32f textures and paints with compute and raster shaders. These entry points run that
 * path's arithmetic on the library's canvas (F32, F16 or BF16; float arithmetic): V is the
 * textures' K.a and PAINTY_PLANE_VL their S.a. The shaders' thresholds differ from the CPU
 * path's (|d| > 1e-5; any channel with |b S d| < 1e-5 keeps R0; no S floor), and their
 * reflectance uses coth(bSd) where the CPU path has b coth(bSd). */
/* replaces CanvasGpu::getComposed (CanvasGpu.cxx:91-95): out = the wet layer composed onto a
 * copy of R0 by ComposeLayerOnSubstrate.compute.glsl:49-71; out is an F32 image */
painty_status painty_canvas_compose_glsl(const painty_canvas* canvas, painty_image* out,
                                         void* stream);
/* replaces CanvasGpu::dryStep(step) (CanvasGpu.cxx:112-128, DryingStep.compute.glsl:122-147):
 * min(V, portion) of the paint dries into R0, V keeps the rest */
painty_status painty_canvas_dry_step(painty_canvas* canvas, float portion, void* stream);

/* TextureBrushDictionary (painty/renderer/TextureBrushDictionary.hxx:17-39): brush textures
 * in classes (radius token, length token), as painty reads them from data/textures/
 * <radius>_<length>_*.png. lookup picks the class nearest the brush size (mean texture rows)
 * and path length (mean cols), then a texture of the class at random: here from a
 * std::mt19937 seeded at creation (painty seeds from std::random_device). */
typedef struct painty_texture_dictionary painty_texture_dictionary;
painty_status painty_texture_dictionary_create(uint32_t seed, painty_texture_dictionary** out);
painty_status painty_texture_dictionary_destroy(painty_texture_dictionary* dict);
/* one texture: a height map rows x cols (normalised min-max to [0, 1], as loadHeightMap,
 * TextureBrushDictionary.cxx:112-120); index_out (may be null) receives its index */
painty_status painty_texture_dictionary_add(painty_texture_dictionary* dict,
                                            uint32_t radius_class, uint32_t length_class,
                                            const double* height, int32_t rows, int32_t cols,
                                            int32_t* index_out);
/* replaces lookup(path, brushSize) (TextureBrushDictionary.cxx:25-69) */
painty_status painty_texture_dictionary_lookup(painty_texture_dictionary* dict,
                                               const double* path_xy, int32_t n,
                                               double brush_size, int32_t* index_out);

/* TextureBrushGpu (painty/renderer/TextureBrushGpu.hxx:21-64) over a dictionary that must
 * outlive it. Radius 5 after creation (TextureBrushGpu.cxx:45); paint {0, 0}. */
typedef struct painty_gpu_texture_brush painty_gpu_texture_brush;
painty_status painty_gpu_texture_brush_create(painty_texture_dictionary* dict,
                                              painty_gpu_texture_brush** out);
painty_status painty_gpu_texture_brush_destroy(painty_gpu_texture_brush* brush);
/* replaces setRadius (TextureBrushGpu.cxx:48-61) */
painty_status painty_gpu_texture_brush_set_radius(painty_gpu_texture_brush* brush, double radius);
/* replaces dip (:63-65) */
painty_status painty_gpu_texture_brush_dip(painty_gpu_texture_brush* brush, const double K[3],
                                           const double S[3]);
painty_status painty_gpu_texture_brush_set_thickness_scale(painty_gpu_texture_brush* brush,
                                                           double scale);
/* replaces enableSmudge (:248-250); enabling returns PAINTY_ERR_UNSUPPORTED (the GL smudge
 * pass has racing writes, so it has no result to reproduce; painty's default is off) */
painty_status painty_gpu_texture_brush_set_smudge(painty_gpu_texture_brush* brush,
                                                  int32_t enable);
/* the dictionary index of the texture the last stroke used (-1 before the first) */
painty_status painty_gpu_texture_brush_last_texture(const painty_gpu_texture_brush* brush,
                                                    int32_t* index_out);
/* replaces paintStroke(path, CanvasGpu&) (:74-167): the strip through the path's Catmull-Rom
 * spline is rasterised with a dictionary texture into a canvas-sized warped texture, which is
 * imprinted (V = Vcan + Vtex; K, S volume-weighted; lighting volume Vtex, or Vcan where
 * Vtex = 0) over the stroke's bounds and cleared. n < 2 paints nothing. Asynchronous. */
painty_status painty_gpu_texture_brush_paint_stroke(painty_canvas* canvas,
                                                    painty_gpu_texture_brush* brush,
                                                    const double* path_xy, int32_t n,
                                                    void* stream);

/* ------------------------------------------------------------------ serving
 * A continuous-batching render server (no counterpart in painty, whose SbrRenderThread runs
 * one stroke at a time on a GL thread: painty/renderer/SbrRenderThread.hxx:50-74). Requests
 * paint strokes on a new canvas or continue a canvas an earlier request created; a worker
 * thread paints a slice of every admitted request per step in one batched launch, so
 * requests that arrive while others run join at the next step. Canvases stay resident
 * between requests within a device-memory budget (idle canvases are moved to host memory,
 * least recently used first, and restored when continued). A canvas's requests run in
 * submission order; each completes with its canvas's KM composite in the caller's buffer.
 * Every canvas gets its own brush (the server's footprint and rates, snapshot on). */
typedef struct painty_server painty_server;
typedef struct painty_server_options {
  uint64_t budget_bytes;   /* device memory for resident canvases (state, snapshot, maps) */
  painty_storage storage;  /* canvas storage format */
  int32_t max_active;      /* requests painted at once: one stream each (<= 0: 256; at most 1024) */
  int64_t step_stamps;     /* stamps per launch of a request (whole strokes; <= 0: 16384) */
  double pickup_rate, deposition_rate;
  const double* footprint; /* brush footprint image (copied) */
  int32_t footprint_rows, footprint_cols;
} painty_server_options;
typedef struct painty_request {
  uint64_t canvas_id;      /* 0: a new canvas of rows x cols; else continue that canvas */
  int32_t rows, cols;
  const float* r0;         /* new canvas substrate, rows*cols*3 interleaved (NULL: 1.0); pinned
                              host memory is read in place when the canvas is created (keep it
                              valid until the request finishes), other memory is copied */
  const painty_stroke_desc* strokes; /* `canvas` ignored; copied at submit */
  int64_t nstrokes;
  const double* points;    /* copied at submit */
  int64_t npoints;
  float* out_rgb;          /* composite result, rows*cols*3 interleaved (NULL: none); must
                              stay valid until the request finishes */
} painty_request;
typedef struct painty_server_counters {
  int64_t submitted, completed, failed, cancelled;
  int64_t steps, stamps, evictions, restores;  /* steps: stamp-kernel launches */
  uint64_t resident_bytes, peak_resident_bytes;
  int64_t active, pending, canvases;
  int64_t worker_busy_us;  /* time the worker thread spent issuing device work, of which: */
  int64_t worker_create_us, worker_launch_us, worker_finish_us; /* new canvases, stamp
                              launches, composite + download launches */
  uint64_t heap_bytes;     /* the device reservation canvases are carved from */
  int64_t heap_fallbacks;  /* allocations it could not hold (stream-ordered instead) */
} painty_server_counters;
painty_status painty_server_create(const painty_server_options* options, painty_server** out);
/* Non-blocking. Returns the request id and its canvas id (new canvases get one here). */
painty_status painty_server_submit(painty_server* server, const painty_request* request,
                                   uint64_t* request_id, uint64_t* canvas_id);
/* Blocks until the request finished (timeout_s < 0: no limit); returns its status:
 * PAINTY_OK, PAINTY_ERR_BUDGET (canvas larger than the budget), PAINTY_ERR_CANCELLED, or
 * PAINTY_ERR_TIMEOUT when it has not finished in time. */
painty_status painty_server_wait(painty_server* server, uint64_t request_id, double timeout_s,
                                 double* latency_s, int64_t* stamps);
/* Blocks until a request has finished that no earlier poll returned (timeout_s < 0: no
 * limit) and returns its id in completion order; PAINTY_ERR_TIMEOUT when none finished in
 * time. Every request appears once, whether or not it was also waited for. Its result and
 * status then come from painty_server_wait with a zero timeout. */
painty_status painty_server_poll(painty_server* server, double timeout_s, uint64_t* request_id);
/* Cancels a request: before it runs it is dropped; while it runs it stops after its current
 * chunk of strokes (its canvas keeps the strokes painted so far). */
painty_status painty_server_cancel(painty_server* server, uint64_t request_id);
/* Drops a canvas: once the requests already queued on it have finished, its device memory,
 * brush and any host copy are freed; later submits to it fail. No counterpart in painty (its
 * canvases are freed by their owner); a serving host calls it after a canvas's last request. */
painty_status painty_server_release(painty_server* server, uint64_t canvas_id);
painty_status painty_server_stats(painty_server* server, painty_server_counters* out);
/* Stops the worker after its current step; unfinished requests end as cancelled. */
painty_status painty_server_destroy(painty_server* server);

/* ------------------------------------------------------------------ mixing (host)
 * replaces PaintMixer::mixSinglePaint (painty/mixer/src/PaintMixer.cxx:327-355) */
painty_status painty_mix_paint(const double* weights, int32_t n, const double* palette_K,
                               const double* palette_S, double K[3], double S[3]);

/* ------------------------------------------------------------------ allocation-free stamping
 * No counterpart in the reference (painty's brush owns its buffers; this entry exists for
 * callers that cannot allocate device memory).
 *
 * Some callers cannot call cudaMalloc: a plugin whose host application owns every byte of
 * device memory and hands out fixed buffers, or a real-time paint loop that must not pay the
 * device-wide synchronisation an allocation can cause. painty_stamps allocates on first use
 * (snapshot, pickup map, scratch); this entry point allocates nothing. The caller passes every
 * input and output as its own device memory, and the only scratch -- an owner table of
 * map_side^2 ints and a status word -- is a fixed array inside the library (about 256 KB,
 * held on every GPU that loads the library until the process exits).
 *
 * Semantics are painty_stamps' on an F32 canvas: stamps applied in order, each one
 * FootprintBrush::imprint. Limits: map_side <= PAINTY_NOALLOC_MAX_MAP_SIDE (256; with the
 * footprint side at most 255 this is radius 90); larger sizes return
 * PAINTY_ERR_INVALID_ARGUMENT, as do a negative or non-finite radius and non-finite rates,
 * capacity or paint. The stamp records are device data and are not checked: they must be
 * finite, with |cx|, |cy| < 1e9 (painty_stamps' bound).
 *
 * The first call on a device -- and the first after that device's context was re-created,
 * e.g. by cudaDeviceReset -- looks up the scratch array's device address; make that call
 * before any stream capture. Calls share the scratch: calls that overlap on the GPU (other
 * streams, other threads) race, so serialise them. The call waits for its stream: it
 * returns after the stamps ran (it reads the kernel's status word back to the host).
 *
 * Buffers (device memory, FP32):
 *   canvas_*:   the wet layer, rows x pitch elements per plane (pitch >= cols)
 *   snapshot_*: the pickup source (FootprintBrush's snapshot buffer), same geometry; all NULL
 *               to pick up from the canvas. The caller initialises it (a copy of the canvas,
 *               as painty does on first use) and keeps it between calls.
 *   pickup_*:   the pickup map, map_side x map_side per plane; zero it to dip the brush
 *   footprint:  footprint_side x footprint_side heights (painty_brush_footprint, as float)
 *   stamps:     n records of 4 doubles: cx, cy, cos(-theta), sin(-theta)
 * Brush values: radius (the brush's current radius), rates, capacity (painty uses 1.0) and the
 * dipped paint. */
#define PAINTY_NOALLOC_MAX_MAP_SIDE 256
typedef struct painty_stamp_buffers_f32 {
  float* canvas_K[3];
  float* canvas_S[3];
  float* canvas_V;
  float* snapshot_K[3];
  float* snapshot_S[3];
  float* snapshot_V;
  float* pickup_K[3];
  float* pickup_S[3];
  float* pickup_V;
  const float* footprint;
  const double* stamps;
  int64_t n;
  int32_t rows, cols;
  int64_t pitch;
  int32_t footprint_side, map_side;
  double radius, pickup_rate, deposition_rate, capacity;
  double paint_K[3], paint_S[3];
} painty_stamp_buffers_f32;
painty_status painty_stamps_f32_noalloc(const painty_stamp_buffers_f32* buffers, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* PAINTY_GB300_H */
