/*
 * fractal_gb300.h - C ABI of the GB300 deep-zoom field renderer.
 *
 * Part 1 is the drop-in boundary: the hot subset of the reference's
 * renderer.h ABI version 10, byte-compatible (same struct layouts, same
 * prototypes, same 0/1 and NULL error convention with a thread-local
 * fractal_last_error()).  Each declaration cites the renderer.h prototype it
 * replaces.  A caller that loads the reference's mandelbrot.so through ctypes
 * (visualizer.py:1512-2387) can load libfractal_gb300.so instead.
 *
 * Part 2 adds entry points the reference has no counterpart for: renders into
 * caller-owned device memory on a caller-chosen CUDA stream, used by
 * benchmarks and by callers that keep fields resident in HBM.
 *
 * Every render in this library runs on the GPU.  There is no CPU fallback:
 * without a usable CUDA device the calls fail with a message.
 */
#ifndef FRACTAL_GB300_H
#define FRACTAL_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FRACTAL_ABI_VERSION 10
#define FRACTAL_RENDER_OPTIONS_VERSION 2
#define FRACTAL_KFP_OPTIONS_VERSION 3
#define FRACTAL_KFP_PLANES_VERSION 1
#define FRACTAL_RENDER_PLANES_VERSION 1
#define FRACTAL_KFP_MAX_MULTI_COLORS 256

#define FRACTAL_FORMULA_MANDELBROT 0
#define FRACTAL_FORMULA_JULIA 1
#define FRACTAL_FORMULA_BURNING_SHIP 2
#define FRACTAL_FORMULA_TRICORN 3

#define FRACTAL_COORDINATE_MODE_PROJECT 0
#define FRACTAL_COORDINATE_MODE_KALLES 1

#define FRACTAL_RENDER_HINT_SKIP_PHASE (1u << 0)
#define FRACTAL_RENDER_HINT_SKIP_ANALYTIC_DE (1u << 1)

/* Backend id of this library.  The reference uses 0 scalar, 1 AVX2,
 * 2 OpenCL and capability bits 1/2/4/8; its loader tests 1 << backend
 * (visualizer.py:1286), so the CUDA backend takes id 4 and bit 16.
 * Backend 0 (the struct default) also selects the CUDA path here. */
#define FRACTAL_BACKEND_CUDA 4
#define FRACTAL_CAPABILITY_CUDA (1 << FRACTAL_BACKEND_CUDA)

/* renderer.h:43-67 */
typedef struct FractalRenderOptions {
    uint32_t struct_size;
    uint32_t version;
    int32_t strict;
    int32_t allow_recovery;
    int32_t time_budget_ms;
    int32_t disable_bla;
    int32_t disable_cycle;
    int32_t strict_cycle;
    int32_t series_min_terms;
    int32_t series_max_terms;
    int32_t max_bla_length;
    int32_t max_linear_bla_length;
    int32_t backend;
    int32_t escape_radius_mode;
    int32_t coordinate_mode;
    int32_t reserved[1];
    double output_bias;
} FractalRenderOptions;

/* renderer.h:75-119 */
typedef struct FractalKfpOptions {
    uint32_t struct_size;
    uint32_t version;
    double iter_div;
    double color_offset;
    double ratio;
    int32_t color_method;
    int32_t smooth_method;
    int32_t smooth;
    int32_t flat;
    int32_t inverse_transition;
    double phase_color_strength;
    int32_t multi_color;
    int32_t blend_multi_color;
    uint32_t multi_color_count;
    double multi_color_period[FRACTAL_KFP_MAX_MULTI_COLORS];
    int32_t multi_color_start[FRACTAL_KFP_MAX_MULTI_COLORS];
    int32_t multi_color_type[FRACTAL_KFP_MAX_MULTI_COLORS];
    double power;
    int32_t slopes;
    double slope_power;
    double slope_ratio;
    double slope_angle;
    int32_t differences;
    int32_t interior_color[3];
    double field_bias;
    int32_t bailout_radius_preset;
    double bailout_radius_custom;
    int32_t bailout_norm_preset;
    double bailout_norm_custom;
    int32_t texture_enabled;
    double texture_merge;
    double texture_power;
    double texture_ratio;
    int32_t texture_resize;
    int32_t use_opengl;
    int32_t use_srgb;
    int32_t show_glitches;
} FractalKfpOptions;

/* renderer.h:135-153: per-pixel Kalles metadata read by the KFP plane
 * path (row-major, width*height entries; any array may be NULL). */
typedef struct FractalKfpPlanes {
    uint32_t struct_size;
    uint32_t version;
    const int64_t *orbit_iteration;
    const double *bailout;
    const int64_t *iteration;
    const double *transition;
    const double *phase;
    const double *de_x;
    const double *de_y;
    const double *test1;
    const double *test2;
    const uint8_t *texture_rgb;
    int32_t texture_width;
    int32_t texture_height;
    int32_t texture_stride;
} FractalKfpPlanes;

/* renderer.h:155-170 */
typedef struct FractalRenderPlanes {
    uint32_t struct_size;
    uint32_t version;
    int64_t *orbit_iteration;
    double *phase;
    double *de_x;
    double *de_y;
    double *test1;
    double *test2;
} FractalRenderPlanes;

/* ---------------------------------------------------------------------
 * Part 1: renderer.h v10 hot subset
 * ------------------------------------------------------------------- */

int fractal_abi_version(void);                                    /* renderer.h:172 */
int fractal_render_options_version(void);                         /* renderer.h:173 */
void fractal_render_options_default(FractalRenderOptions *options); /* renderer.h:174 */
/* renderer.h:175-177; returns FRACTAL_CAPABILITY_CUDA when a device is usable. */
int fractal_backend_capabilities(void);
const char *fractal_last_error(void);                             /* renderer.h:178 */

void fractal_set_stats_enabled(int enabled);                      /* renderer.h:180 */
int fractal_get_last_stats(uint64_t *values, int capacity);       /* renderer.h:181 */
int fractal_get_last_stats_ex(uint64_t *values, int capacity);    /* renderer.h:182 */

/* renderer.h:184-191 */
void *fractal_create_reference(const char *x_center, const char *y_center,
                               const char *viewport_zoom, int max_iter,
                               int precision_bits, int series_order);
/* renderer.h:193-200 */
void *fractal_create_reference_reusable(const char *x_center, const char *y_center,
                                        const char *viewport_zoom, int max_iter,
                                        int precision_bits, int series_order);
/* renderer.h:203-211 */
void *fractal_create_reference_reusable_options(const char *x_center, const char *y_center,
                                                const char *viewport_zoom, int max_iter,
                                                int precision_bits, int series_order,
                                                const FractalRenderOptions *options);
/* renderer.h:215-225 */
void *fractal_create_reference_ex(const char *x_center, const char *y_center,
                                  const char *viewport_zoom, int max_iter, int precision_bits,
                                  int series_order, int formula, const char *julia_real,
                                  const char *julia_imag);
/* renderer.h:226-237 */
void *fractal_create_reference_ex_options(const char *x_center, const char *y_center,
                                          const char *viewport_zoom, int max_iter,
                                          int precision_bits, int series_order, int formula,
                                          const char *julia_real, const char *julia_imag,
                                          const FractalRenderOptions *options);
void *fractal_clone_reference(void *source_handle, const char *viewport_zoom); /* renderer.h:239 */
void fractal_destroy_reference(void *handle);                                 /* renderer.h:240 */
int fractal_get_reference_stats(void *handle, uint64_t *values, int capacity); /* renderer.h:241 */

/* renderer.h:243-254 */
int fractal_render_mandelbrot_reference_ex(float *output, int width, int height,
                                           const char *zoom_text, void *handle, int max_iter,
                                           int threads, int series_order, int series_block,
                                           const FractalRenderOptions *options);
/* renderer.h:257-268 */
int fractal_render_reference_ex(float *output, int width, int height, const char *zoom_text,
                                void *handle, int max_iter, int threads, int series_order,
                                int series_block, const FractalRenderOptions *options);
/* renderer.h:273-285 */
int fractal_render_reference_ex_planes(float *output, int width, int height,
                                       const char *zoom_text, void *handle, int max_iter,
                                       int threads, int series_order, int series_block,
                                       const FractalRenderOptions *options,
                                       FractalRenderPlanes *planes);
/* renderer.h:323-335 */
int render_mandelbrot_ex(float *output, int width, int height, const char *zoom_text,
                         const char *x_center, const char *y_center, int max_iter,
                         int precision_bits, int use_perturbation, int threads,
                         const FractalRenderOptions *options);
/* renderer.h:338-353 */
int render_fractal_ex(float *output, int width, int height, const char *zoom_text,
                      const char *x_center, const char *y_center, int max_iter,
                      int precision_bits, int use_perturbation, int threads, int formula,
                      double julia_real, double julia_imag, const FractalRenderOptions *options);
/* renderer.h:357-373 */
int render_fractal_ex_planes(float *output, int width, int height, const char *zoom_text,
                             const char *x_center, const char *y_center, int max_iter,
                             int precision_bits, int use_perturbation, int threads, int formula,
                             double julia_real, double julia_imag,
                             const FractalRenderOptions *options, FractalRenderPlanes *planes);
/* renderer.h:376-386 */
int render_mandelbrot_reference(float *output, int width, int height, const char *zoom_text,
                                void *handle, int max_iter, int threads, int series_order,
                                int series_block);
/* renderer.h:387-398 */
int render_mandelbrot(float *output, int width, int height, const char *zoom_text,
                      const char *x_center, const char *y_center, int max_iter,
                      int precision_bits, int use_perturbation, int threads);

/* renderer.h:287-300: render an arbitrary list of offsets from the
 * reference centre, point i at (real[i] + i imag[i]) * 2^exponents[i]; one
 * float per point.  The largest offset replaces the view radius in the BLA and
 * series decisions.  Strict Mandelbrot lists of at most 8192 points repair
 * their glitch points exactly (MPFR iteration from scratch, on the host). */
int fractal_render_points(float *output, int point_count, const char *zoom_text,
                          const double *real_mantissa, const double *imag_mantissa,
                          const int32_t *exponents, void *handle, int max_iter, int threads,
                          int series_order, int series_block, const FractalRenderOptions *options);
/* renderer.h:302-320: the same with the six render planes (point_count
 * entries each). */
int fractal_render_points_ex_planes(float *output, int point_count, const char *zoom_text,
                                    const double *real_mantissa, const double *imag_mantissa,
                                    const int32_t *exponents, void *handle, int max_iter,
                                    int threads, int series_order, int series_block,
                                    const FractalRenderOptions *options,
                                    FractalRenderPlanes *planes);

/* renderer.h:400-411: aurora palette. */
int fractal_colourise(const float *field, uint8_t *output, int width, int height, int max_iter,
                      double phase, double vocal, double instrumental, double pitch,
                      int threads);

/* renderer.h:450-463: Kalles .kfp transfer on the scalar field (1024-entry
 * cyclic LUT supplied by the caller, distance/slope shading, dither). */
int fractal_colourise_kfp(const float *field, uint8_t *output, int width, int height, int max_iter,
                          double phase, double vocal, double instrumental, double pitch,
                          const FractalKfpOptions *options, const uint8_t *lut, int lut_size,
                          int threads);
/* renderer.h:483-497: the KFP transfer fed by Kalles metadata planes:
 * orbit iteration + test1/test2/bailout smoothing (or stored iteration and
 * transition), the phase colour, analytic DE for Differences 7, hidden
 * glitch pixels.  Texture merging is not supported: a texture with
 * texture_enabled fails with a message. */
int fractal_colourise_kfp_planes(const float *field, uint8_t *output, int width, int height,
                                 int max_iter, double phase, double vocal, double instrumental,
                                 double pitch, const FractalKfpOptions *options,
                                 const FractalKfpPlanes *planes, const uint8_t *lut, int lut_size,
                                 int threads);
/* renderer.h:503-516: compatibility name of the same transfer. */
int fractal_colourise_kfp_precise(const float *field, uint8_t *output, int width, int height,
                                  int max_iter, double phase, double vocal, double instrumental,
                                  double pitch, const FractalKfpOptions *options,
                                  const uint8_t *lut, int lut_size, int threads);
/* renderer.h:426-440: aurora palette projected through three RGB accents
 * (9 bytes), with an interior colour.  NULL accents fail with "ordinary palette accents are required". */
int fractal_colourise_accents(const float *field, uint8_t *output, int width, int height, int max_iter,
                              double phase, double vocal, double instrumental, double pitch,
                              const uint8_t *accents, int interior_red, int interior_green,
                              int interior_blue, int threads);

/* Atlas compositor: one output frame from a parent keyframe field and the
 * next, deeper child field.  The parent is cropped by `parent_zoom` about its
 * centre and resampled bilinearly; the child fills the centred rectangle of
 * `child_fraction` of the frame, feathered by a smoothstep at its edges.
 * Bilinear samples keep interior: an interior weight >= 1/2 gives interior,
 * otherwise the exterior corners are renormalised.  Host buffers; the frame
 * is composed on the GPU and copied back. */

/* renderer.h:797-813: scalar frame (no biases, child zoom 1, 48-px seam). */
int fractal_atlas_field(const float *parent, int parent_width, int parent_height, int parent_max_iter,
                        const float *child, int child_width, int child_height, int child_max_iter,
                        float *output, int output_width, int output_height, double parent_zoom,
                        double child_fraction, int palette_max_iter, int threads);
/* renderer.h:815-836: scalar frame with field biases (value + bias is the
 * true smooth count), child crop zoom and seam width. */
int fractal_atlas_field_ex(const float *parent, int parent_width, int parent_height, int parent_max_iter,
                           const float *child, int child_width, int child_height, int child_max_iter,
                           float *output, int output_width, int output_height, double parent_zoom,
                           double child_fraction, double child_zoom, double parent_field_bias,
                           double child_field_bias, double output_field_bias, int palette_max_iter,
                           int feather, int threads);
/* renderer.h:997-1017: the frame coloured with the aurora palette (seam
 * min(48, visible/8), blended in RGB). */
int fractal_atlas_colourise(const float *parent, int parent_width, int parent_height, int parent_max_iter,
                            const float *child, int child_width, int child_height, int child_max_iter,
                            uint8_t *output, int output_width, int output_height, double parent_zoom,
                            double child_fraction, int palette_max_iter, double phase, double vocal,
                            double instrumental, double pitch, int threads);
/* renderer.h:1018-1042: the same with an explicit interior colour. */
int fractal_atlas_colourise_interior(const float *parent, int parent_width, int parent_height,
                                     int parent_max_iter, const float *child, int child_width,
                                     int child_height, int child_max_iter, uint8_t *output,
                                     int output_width, int output_height, double parent_zoom,
                                     double child_fraction, int palette_max_iter, double phase,
                                     double vocal, double instrumental, double pitch, int interior_red,
                                     int interior_green, int interior_blue, int threads);
/* renderer.h:1043-1067: accent palette and interior colour. */
int fractal_atlas_colourise_accents(const float *parent, int parent_width, int parent_height,
                                    int parent_max_iter, const float *child, int child_width,
                                    int child_height, int child_max_iter, uint8_t *output,
                                    int output_width, int output_height, double parent_zoom,
                                    double child_fraction, int palette_max_iter, double phase,
                                    double vocal, double instrumental, double pitch,
                                    const uint8_t *accents, int interior_red, int interior_green,
                                    int interior_blue, int threads);

/* fractal_atlas_colourise_kfp (renderer.h:554-576) and its _precise twin
 * (renderer.h:577-603): parent and child coloured as separate KFP tiles at
 * output scale (the parent is output-sized; the child covers the rectangle
 * at child_left/child_top), each with its own stencil edges and ColorMethod 4
 * bounds, blended across a smoothstep band of `feather` pixels. */
int fractal_atlas_colourise_kfp(const float *parent, int parent_width, int parent_height, const float *child,
                                int child_width, int child_height, uint8_t *output, int output_width,
                                int output_height, int max_iter, int child_left, int child_top, int feather,
                                double phase, double vocal, double instrumental, double pitch,
                                const FractalKfpOptions *options, const uint8_t *lut, int lut_size, int threads);
int fractal_atlas_colourise_kfp_precise(const float *parent, int parent_width, int parent_height, const float *child,
                                        int child_width, int child_height, uint8_t *output, int output_width,
                                        int output_height, int max_iter, int child_left, int child_top, int feather,
                                        double phase, double vocal, double instrumental, double pitch,
                                        const FractalKfpOptions *options, const uint8_t *lut, int lut_size,
                                        int threads);

/* fractal_atlas_colourise_kfp_planes (renderer.h:604-631) and its _precise
 * twin (renderer.h:632-662): the scalar surface and every render plane present
 * in either tile reprojected to the output (integer planes by nearest sample,
 * double planes bilinearly, glitch transitions kept, interior samples reset),
 * the child blended in over its centred rectangle, then the plane-aware KFP
 * pass (texture merging included) over the composed frame. */
int fractal_atlas_colourise_kfp_planes(const float *parent, int parent_width, int parent_height, int parent_max_iter,
                                       const FractalKfpPlanes *parent_planes, const float *child, int child_width,
                                       int child_height, int child_max_iter, const FractalKfpPlanes *child_planes,
                                       uint8_t *output, int output_width, int output_height, double parent_zoom,
                                       double child_fraction, double child_zoom, int max_iter, int centered_input,
                                       double phase, double vocal, double instrumental, double pitch,
                                       const FractalKfpOptions *options, const uint8_t *lut, int lut_size,
                                       int threads);
int fractal_atlas_colourise_kfp_planes_precise(const float *parent, int parent_width, int parent_height,
                                               int parent_max_iter, const FractalKfpPlanes *parent_planes,
                                               const float *child, int child_width, int child_height,
                                               int child_max_iter, const FractalKfpPlanes *child_planes,
                                               uint8_t *output, int output_width, int output_height,
                                               double parent_zoom, double child_fraction, double child_zoom,
                                               int max_iter, int centered_input, double phase, double vocal,
                                               double instrumental, double pitch, const FractalKfpOptions *options,
                                               const uint8_t *lut, int lut_size, int threads);

/* renderer.h:660-687: raw KFP atlas frame.  The parent (crop by
 * parent_zoom) and the child (visible rectangle of child_fraction, crop by
 * child_zoom) are composed into one scalar surface encoded relative to the
 * options' field_bias (a positive bias means each source is stored relative
 * to its own cap), with a smoothstep seam inside the child rectangle; one
 * KFP pass then colours the surface, so differences and slopes stay
 * continuous across the seam. */
int fractal_atlas_colourise_kfp_raw(const float *parent, int parent_width, int parent_height,
                                    int parent_max_iter, const float *child, int child_width,
                                    int child_height, int child_max_iter, uint8_t *output,
                                    int output_width, int output_height, double parent_zoom,
                                    double child_fraction, double child_zoom, int max_iter,
                                    double phase, double vocal, double instrumental, double pitch,
                                    const FractalKfpOptions *options, const uint8_t *lut,
                                    int lut_size, int threads);
/* renderer.h:688-711: compatibility name of the same call. */
int fractal_atlas_colourise_kfp_raw_precise(const float *parent, int parent_width, int parent_height,
                                            int parent_max_iter, const float *child, int child_width,
                                            int child_height, int child_max_iter, uint8_t *output,
                                            int output_width, int output_height, double parent_zoom,
                                            double child_fraction, double child_zoom, int max_iter,
                                            double phase, double vocal, double instrumental,
                                            double pitch, const FractalKfpOptions *options,
                                            const uint8_t *lut, int lut_size, int threads);

/* Crops of one source by a zoom factor (at least 1) about its centre,
 * resampled bilinearly to the output size. */
/* renderer.h:786-795: plain bilinear crop of a scalar field. */
int fractal_crop_field(const float *source, int source_width, int source_height, float *output,
                       int output_width, int output_height, double zoom_factor, int threads);
/* renderer.h:716-725: bilinear crop of an RGB8 image. */
int fractal_crop_rgb(const uint8_t *source, int source_width, int source_height, uint8_t *output,
                     int output_width, int output_height, double zoom_factor, int threads);
/* renderer.h:726-741: coloured parent and child tiles composed per frame
 * (child crop by child_zoom in the centred rectangle of child_fraction, a
 * smoothstep seam of `feather` pixels). */
int fractal_atlas_composite_rgb(const uint8_t *parent, int parent_width, int parent_height,
                                const uint8_t *child, int child_width, int child_height,
                                uint8_t *output, int output_width, int output_height,
                                double parent_zoom, double child_fraction, double child_zoom,
                                int feather, int threads);
/* renderer.h:943-956: interior-preserving crop coloured with the aurora
 * palette. */
int fractal_crop_colourise(const float *source, int source_width, int source_height, uint8_t *output,
                           int output_width, int output_height, double zoom_factor, int max_iter,
                           double phase, double vocal, double instrumental, double pitch, int threads);
/* renderer.h:957-975: with an interior colour. */
int fractal_crop_colourise_interior(const float *source, int source_width, int source_height,
                                    uint8_t *output, int output_width, int output_height,
                                    double zoom_factor, int max_iter, double phase, double vocal,
                                    double instrumental, double pitch, int interior_red,
                                    int interior_green, int interior_blue, int threads);
/* renderer.h:976-996: with accents (NULL: the plain palette) and an
 * interior colour. */
int fractal_crop_colourise_accents(const float *source, int source_width, int source_height,
                                   uint8_t *output, int output_width, int output_height,
                                   double zoom_factor, int max_iter, double phase, double vocal,
                                   double instrumental, double pitch, const uint8_t *accents,
                                   int interior_red, int interior_green, int interior_blue,
                                   int threads);
/* renderer.h:518-535: interior-preserving crop encoded by the KFP field
 * bias, then one KFP pass. */
int fractal_crop_colourise_kfp(const float *source, int source_width, int source_height,
                               uint8_t *output, int output_width, int output_height,
                               double zoom_factor, int max_iter, double phase, double vocal,
                               double instrumental, double pitch, const FractalKfpOptions *options,
                               const uint8_t *lut, int lut_size, int threads);
/* renderer.h:536-553: compatibility name of the same call. */
int fractal_crop_colourise_kfp_precise(const float *source, int source_width, int source_height,
                                       uint8_t *output, int output_width, int output_height,
                                       double zoom_factor, int max_iter, double phase, double vocal,
                                       double instrumental, double pitch,
                                       const FractalKfpOptions *options, const uint8_t *lut,
                                       int lut_size, int threads);

/* ---------------------------------------------------------------------
 * Part 2: GB300 extensions (no counterpart in the reference)
 *
 * Device-pointer variants: every buffer argument is device memory on the
 * current CUDA device; `stream` is a cudaStream_t (NULL = the calling
 * thread's library stream).  The calls enqueue work and return without
 * synchronising; results are ready when the stream reaches them.
 * ------------------------------------------------------------------- */

/* Where reference creation builds the BLA hierarchies: 1 (default) on the
 * GPU, 0 on the host.  Both builders use the same arithmetic and give
 * identical tables; the switch exists so tests can compare them. */
void fractal_gb300_set_table_builder(int on_device);

/* Number of usable CUDA devices (0 when none). */
int fractal_gb300_device_count(void);
/* Duration in ms of the last render/colour kernel issued by this thread,
 * measured with CUDA events on its stream (after a synchronous call). */
/* Self-check: of all 2^32 float inputs, how many give a quotient by
 * `divisor` through the KFP pass's constant division (a rounded-reciprocal
 * product with one FMA correction) that differs from IEEE division. */
int fractal_gb300_check_division(float divisor, unsigned long long *mismatches);
double fractal_gb300_last_kernel_ms(void);

/* Deep or direct render of one field from a prepared reference into device
 * buffers: `field` float[width*height], `counts` uint32[width*height] (escape
 * index, max_iter for interior, 0 for an unresolved glitch; may be NULL).
 * `form` selects the arithmetic: 0 = plain FP64 form (parity with the
 * reference), 1 = FP32-mantissa floatexp form. */
int fractal_gb300_render_reference_device(float *field, uint32_t *counts, int width, int height,
                                          const char *zoom_text, void *handle, int max_iter,
                                          int series_order, int series_block,
                                          const FractalRenderOptions *options, int form,
                                          void *stream);

/* Direct (shallow) render into device buffers; same conventions as above. */
int fractal_gb300_render_direct_device(float *field, uint32_t *counts, int width, int height,
                                       const char *zoom_text, const char *x_center,
                                       const char *y_center, int max_iter, int formula,
                                       double julia_real, double julia_imag,
                                       const FractalRenderOptions *options, void *stream);

/* FMA-pipe throughput of the current device in TFLOP/s (2 flops per FMA),
 * measured with eight independent FMA chains per thread; precision_bits is
 * 64 or 32.  Returns 0 on success.  Used as the roofline denominator of the
 * iteration kernels. */
int fractal_gb300_fma_peak(int precision_bits, double *tflops);

/* KFP colour pass from a device field to device RGB8; `lut` is device
 * memory (lut_size x 3 bytes). */
int fractal_gb300_colourise_kfp_device(const float *field, uint8_t *rgb, int width, int height,
                                       int max_iter, const FractalKfpOptions *options,
                                       const uint8_t *lut, int lut_size, void *stream);

/* Aurora colour pass from a device field to device RGB8. */
int fractal_gb300_colourise_device(const float *field, uint8_t *rgb, int width, int height,
                                   int max_iter, double phase, double vocal, double instrumental,
                                   double pitch, void *stream);

/* Atlas frames (fractal_atlas_field_ex / fractal_atlas_colourise_*) from
 * device parent and child fields into device output; `interior_rgb` (three
 * ints, or NULL for black) and `accents` (9 bytes, or NULL for the plain
 * aurora palette) are host memory. */
int fractal_gb300_atlas_field_device(const float *parent, int parent_width, int parent_height,
                                     int parent_max_iter, const float *child, int child_width,
                                     int child_height, int child_max_iter, float *output,
                                     int output_width, int output_height, double parent_zoom,
                                     double child_fraction, double child_zoom,
                                     double parent_field_bias, double child_field_bias,
                                     double output_field_bias, int palette_max_iter, int feather,
                                     void *stream);
int fractal_gb300_atlas_colourise_device(const float *parent, int parent_width, int parent_height,
                                         int parent_max_iter, const float *child, int child_width,
                                         int child_height, int child_max_iter, uint8_t *output,
                                         int output_width, int output_height, double parent_zoom,
                                         double child_fraction, int palette_max_iter, double phase,
                                         double vocal, double instrumental, double pitch,
                                         const int *interior_rgb, const uint8_t *accents,
                                         void *stream);

/* Raw KFP atlas frame from device parent/child fields and a device LUT
 * into device RGB8 (fractal_atlas_colourise_kfp_raw without the colour
 * controls it ignores). */
int fractal_gb300_atlas_colourise_kfp_raw_device(const float *parent, int parent_width,
                                                 int parent_height, int parent_max_iter,
                                                 const float *child, int child_width, int child_height,
                                                 int child_max_iter, uint8_t *output, int output_width,
                                                 int output_height, double parent_zoom,
                                                 double child_fraction, double child_zoom, int max_iter,
                                                 const FractalKfpOptions *options, const uint8_t *lut,
                                                 int lut_size, void *stream);
/* The scalar surface of the raw KFP atlas frame alone, into device
 * `surface` (output_width x output_height floats), for `field_bias`. */
int fractal_gb300_atlas_kfp_surface_device(const float *parent, int parent_width, int parent_height,
                                           int parent_max_iter, const float *child, int child_width,
                                           int child_height, int child_max_iter, float *surface,
                                           int output_width, int output_height, double parent_zoom,
                                           double child_fraction, double child_zoom, int max_iter,
                                           double field_bias, void *stream);

/* Pixels of the last atlas frame of the calling thread that the fast
 * (FP32 / double-float) pass could not decide and the exact FP64 pass
 * computed; synchronises the device.  -1 before any atlas frame. */
long long fractal_gb300_atlas_last_exact_pixels(void);

/* Video-frame handoff: device RGB8 (width x height x 3) packed into the
 * layout an encoder pipe takes.  format: 0 rgb24, 1 rgb0 (R,G,B,0), 2 rgba
 * (R,G,B,255), 3 yuv420p and 4 nv12, both BT.709 limited range with the 2x2
 * mean as chroma.  packed_frame_bytes gives the output size (-1: invalid). */
long long fractal_gb300_packed_frame_bytes(int width, int height, int format);
int fractal_gb300_pack_frame_device(const uint8_t *rgb, int width, int height, int format,
                                    uint8_t *output, void *stream);

/* One keyframe of a batch: device outputs (`counts` may be NULL), its zoom,
 * the reference handle it renders from (NULL: the direct FP64 path at the
 * batch centre, which the reference pipeline takes below 1e12,
 * visualizer.py:6152), its iteration cap and flags (0 or
 * FRACTAL_GB300_KEYFRAME_SHALLOW). */
typedef struct FractalGb300Keyframe {
    float *field;
    uint32_t *counts;
    const char *zoom_text;
    void *reference;
    int max_iter;
    int flags;
} FractalGb300Keyframe;

/* Keyframe flag: a frame the reference pipeline renders on the direct path
 * (below 1e12) that also names a reference handle at the batch centre.  In
 * form 0 it takes the direct FP64 path at the batch centre (the handle is
 * not used); in form 1 it renders by FP32 perturbation against the handle's
 * orbit (shallow mode: from iteration 0, unlimited rebasing, no series or
 * BLA), which removes the FP64 direct iteration from the floatexp form. */
#define FRACTAL_GB300_KEYFRAME_SHALLOW 1

/* Capture the batch's launches into a CUDA graph and replay the graph when
 * the same batch (same buffers, zooms, handles and options) comes again. */
#define FRACTAL_GB300_BATCH_GRAPH 1u
/* Time the persistent queues' launch shapes (pixels per warp claim, blocks
 * per SM) on this batch first and keep the fastest for batches of its kind.
 * The shapes change the schedule only, never a pixel. */
#define FRACTAL_GB300_BATCH_AUTOTUNE 2u
/* Floatexp frames run as a queue of 64x64 tiles (work unit: a band of rows
 * of one tile); per-tile cost (SM cycles) and the queue's makespan and tail
 * (time from the last claim to the last finish) are recorded for
 * fractal_gb300_last_tiles.  Without _LEARNED the tiles go in ascending order
 * (fields in the order given, row-major within a field): the static order. */
#define FRACTAL_GB300_BATCH_TILES 4u
/* Tile queue in the order predicted by the attached cost network (heaviest
 * first), from a 16x16 coarse probe of every tile; implies _TILES. */
#define FRACTAL_GB300_BATCH_LEARNED 8u
/* With _TILES: compute the probe and the network features without using them
 * (training data: fractal_gb300_last_tiles returns features and costs). */
#define FRACTAL_GB300_BATCH_PROBE 16u
/* Form 1: render julia / burning-ship / tricorn fields (from 1e6) in the
 * FP32 queue too.  Without it they stay in the FP64 plain form: their deep
 * views hold long post-linear orbits that FP32 deltas do not follow (on the
 * test views 0-31 % of counts differ from FP64, whose counts a direct mpmath
 * iteration confirms), so this trades accuracy for about 10x speed. */
#define FRACTAL_GB300_BATCH_FP32_ALTERNATES 32u

/* Render many keyframes in a few launches: all direct frames in one
 * persistent lane-refill FP64 queue on a second stream, all floatexp frames
 * (form 1) in one persistent queue on `stream`, plain-form deep frames
 * (form 0, or frames the floatexp form does not cover) one launch each;
 * the second stream joins `stream` before the call's work ends.  Frames are
 * claimed in the order given: put the costliest first.  Per-frame results are
 * those of fractal_gb300_render_reference_device / _render_direct_device with
 * the same arguments, except that with form 1 the direct frames' smooth
 * values take their logarithms in FP32 (iteration counts unchanged, smooth
 * values within a few float ulps). */
int fractal_gb300_render_keyframes_device(const FractalGb300Keyframe *frames, int count, int width,
                                          int height, const char *x_center, const char *y_center,
                                          int series_order, int series_block,
                                          const FractalRenderOptions *options, int form,
                                          unsigned flags, void *stream);

/* One field of a general batch (no counterpart in the reference): device
 * outputs (`counts` and the derivative planes may be NULL; de_x / de_y both
 * or neither: the analytic distance estimate of render_plane_de,
 * renderer.cpp:7844-7990, as in FractalRenderPlanes), its zoom, the reference
 * handle it renders from (its formula, centre and, for Julia, c; NULL: the
 * direct FP64 Mandelbrot path at the batch centre), its own size and cap,
 * and flags (0 or FRACTAL_GB300_KEYFRAME_SHALLOW). */
typedef struct FractalGb300Field {
    float *field;
    uint32_t *counts;
    double *de_x;
    double *de_y;
    const char *zoom_text;
    void *reference;
    int width;
    int height;
    int max_iter;
    int flags;
} FractalGb300Field;

/* fractal_gb300_render_keyframes_device for fields of uneven size and of
 * every formula, with optional derivative planes.  Form 1 renders the
 * floatexp-covered fields (strict, no cycle detection, no time budget:
 * Mandelbrot from any zoom; the other formulas from 1e6 with
 * FRACTAL_GB300_BATCH_FP32_ALTERNATES) in one persistent FP32 queue; the
 * direct fields run in the FP64 lane-refill queue (one launch per formula
 * and plane set) and the plain-form fields one launch each, on a second
 * stream beside it.  Form 0 is the plain FP64 form, whose
 * pixels and planes equal the per-field entry points'.  At most 64 floatexp
 * fields with the tile flags; no limit otherwise. */
int fractal_gb300_render_fields_device(const FractalGb300Field *fields, int count, const char *x_center,
                                       const char *y_center, int series_order, int series_block,
                                       const FractalRenderOptions *options, int form, unsigned flags,
                                       void *stream);

/* Pin the launch shapes of the calling thread's next batches (same order as
 * fractal_gb300_queue_shapes; a 0 chunk keeps the default, a 0 blocks/SM
 * means as many as fit); values NULL or count 0 unpins.  Pinned shapes
 * override tuned ones and switch autotuning off. */
int fractal_gb300_set_queue_shapes(const int *values, int count);

/* Attach a cost network (fractal_gb300_costnet_create) to the calling
 * thread's batches for FRACTAL_GB300_BATCH_LEARNED; NULL detaches.  The
 * network is not owned. */
int fractal_gb300_set_cost_network(void *net);

/* Results of the calling thread's last tile-scheduled batch (synchronises its
 * stream): the tile count, per-tile cost in SM cycles (float[tiles]), the
 * features when the batch computed them (BF16 bits [tiles x 320]) and
 * timing_ms[0] = makespan, timing_ms[1] = tail.  cost/features/timing_ms may
 * be NULL; capacity is their tile capacity. */
int fractal_gb300_last_tiles(int *tiles, float *cost, uint16_t *features, int capacity, double *timing_ms);

/* Iterations the direct queue actually computed in the calling thread's last
 * direct launch (escaped pixels count their escape index, pixels the cycle
 * probe settled count the steps taken before it did); synchronises.  Fails
 * when that launch was a fractal_gb300_render_direct_device_noalloc call
 * (its counters are not kept) and when the thread has made no direct launch;
 * fails too, after the count is copied, when the launch's spill queue
 * reported an unpublished entry (the render is then incomplete). */
int fractal_gb300_last_direct_steps(unsigned long long *steps);

/* Test hook (no counterpart in the reference): the calling thread's next
 * direct launches wait at most `spin_limit` polls (1 .. 1 << 22; 0 = the
 * default 1 << 22) for a spilled pixel's publish mark, and with
 * withhold_publish = 1 write spilled pixels without publishing them, so a
 * test can drive the wait to its bound: the kernel then drops those pixels,
 * ends normally and fractal_gb300_last_direct_steps reports the queue error.
 * (0, 0) restores normal operation.  The failure is made on the device by
 * data only; no fault, trap or unbounded wait is involved. */
int fractal_gb300_set_direct_fault_injection(int spin_limit, int withhold_publish);

/* Launch shapes the calling thread's last batch used: direct chunk, direct
 * blocks per SM, floatexp chunk, floatexp blocks per SM (0 = as many as fit). */
int fractal_gb300_queue_shapes(int *values, int capacity);

/* No counterpart in the reference.  The direct render of
 * fractal_gb300_render_direct_device (same arguments, same pixels) for callers
 * that cannot allocate device memory: inside an allocator hook, under a
 * reserve-everything-up-front memory policy, or in a real-time loop where an
 * allocation's implicit synchronisation is not acceptable.  It calls no
 * cudaMalloc/cudaFree and creates no stream: `stream` NULL means the legacy
 * default stream (fractal_gb300_render_direct_device's NULL means the calling
 * thread's own non-blocking stream, so NULL-stream calls of the two entry
 * points are ordered differently).  It runs without the spill list (long
 * pixels finish in their own lane), so its pixels are the same but its tail
 * latency on interior-heavy views can be longer.  Its scratch is a fixed 128 KiB array inside the library,
 * so width + height must be at most 16352 (larger fields fail with an error,
 * before any launch).  All calls share that array: calls ordered on one
 * stream are independent (each call resets what it uses), calls that overlap
 * on the GPU race.  The first call on each device looks the array's address
 * up (cudaGetSymbolAddress); make it before any stream capture. */
int fractal_gb300_render_direct_device_noalloc(float *field, uint32_t *counts, int width, int height,
                                               const char *zoom_text, const char *x_center,
                                               const char *y_center, int max_iter, int formula,
                                               double julia_real, double julia_imag,
                                               const FractalRenderOptions *options, void *stream);

/* ----- Tile-cost network (no counterpart in the reference) -----------
 * A small MLP predicting the render cost of a 64x64 tile from a 16x16 coarse
 * probe of its iteration counts plus log zoom and log cap (320 BF16 features
 * per row: 256 probe values, 2 field values, zeros).  Layers 320 -> 256 ->
 * 256 -> 1 with ReLU; BF16 weights and activations, FP32 accumulation on the
 * tensor cores (tcgen05), FP32 master weights updated by Adam.  It orders
 * work only; it never changes a pixel. */
void *fractal_gb300_costnet_create(unsigned seed);
void fractal_gb300_costnet_destroy(void *net);
int fractal_gb300_costnet_parameter_count(void);
/* Read (write = 0) or replace (write = 1) the FP32 parameters: W1 [256 x 320],
 * b1 [256], W2 [256 x 256], b2 [256], w3 [256], b3 [1], row-major. */
int fractal_gb300_costnet_parameters(void *net, float *values, int count, int write);
/* One step of mean-squared-error training on `batch` rows (a multiple of
 * 128): device features (BF16 [batch x 320]) and targets (float [batch]).
 * update = 0 computes the loss and gradient only.  `loss` and `gradients`
 * (parameter order, host memory) may be NULL.  Synchronises `stream`. */
int fractal_gb300_costnet_train_step(void *net, const void *features, const float *targets, int batch,
                                     float learning_rate, int update, float *loss, float *gradients,
                                     void *stream);
/* Predictions for `rows` rows (a multiple of 128) into device `out`. */
int fractal_gb300_costnet_predict(void *net, const void *features, int rows, float *out, void *stream);
/* The network's tensor-core product on its own: C[m x n] (float) =
 * A[m x k] * B[n x k]^T with BF16 row-major A and B; m % 128 == 0,
 * n % 16 == 0, k % 64 == 0, and B allocated with b_rows >= n rows, b_rows a
 * multiple of 256 (rows beyond n are read but unused). */
int fractal_gb300_gemm_bf16(const void *a, const void *b, float *c, int m, int n, int k, int b_rows,
                            void *stream);

#ifdef __cplusplus
}
#endif

#endif
