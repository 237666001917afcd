/*
 * pxg — GB300 (sm_103a) implementation of pixie's raster hot path behind a
 * plain C ABI: extern "C" entry points, plain pointers and sizes, no C++ or
 * torch types.  It mirrors the C bindings the reference generates for this
 * path (bindings/bindings.nim: Image.fillPath/strokePath/draw/blur/shadow,
 * checkError/takeError) with images that stay resident on the GPU.
 *
 * Conventions (src/pixie/common.nim:34-57):
 *   - an image is premultiplied RGBX, 4 bytes per pixel (r, g, b, a),
 *     row-major with no row padding; dataIndex = width * y + x;
 *   - a path is pixie's command buffer: float32 records [kind, params...]
 *     with the PathCommandKind ordinals of src/pixie/paths.nim:18-22;
 *   - a colour is chroma's Color: 4 float32, straight (not premultiplied),
 *     each in [0, 1];
 *   - a transform is vmath's Mat3: 9 float32, column-major, translation in
 *     elements 6 and 7; NULL means identity;
 *   - blend modes use the BlendMode ordinals of common.nim:6-29 (0 Normal ...
 *     15 Luminosity, 16 Mask, 17 Overwrite, 18 SubtractMask, 19 ExcludeMask);
 *     winding rules: 0 NonZero, 1 EvenOdd (paths.nim:5-8); line caps:
 *     0 Butt, 1 Round, 2 Square; line joins: 0 Miter, 1 Round, 2 Bevel.
 *
 * Errors: every entry point returns 0 on success and non-zero on failure;
 * the failure's message (the reference's PixieError text where one exists)
 * is kept per thread until pxg_take_error() returns it
 * (bindings/bindings.nim:3-10).  Entry points never throw.
 *
 * Calls are issued on the library's stream (pxg_set_stream) and return after
 * the GPU work of that call completed, as the reference's procs do.
 */
#ifndef PXG_H
#define PXG_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct pxg_image pxg_image;

/* Errors — replaces checkError/takeError (bindings/bindings.nim:3-10). */
int pxg_check_error(void);
const char* pxg_take_error(void);

/* Device and stream.  pxg_init selects the CUDA device (called implicitly on
 * first use with device 0).  pxg_set_stream takes a cudaStream_t (NULL for
 * the library's own stream); no counterpart in the reference, which has no
 * device. */
int pxg_init(int device);
int pxg_set_stream(void* cuda_stream);
int pxg_synchronize(void);

/* Images — replaces newImage (src/pixie/common.nim:39-47): a transparent
 * width x height image in device memory.  Returns NULL and sets the error
 * "Image width and height must be > 0" like the reference. */
pxg_image* pxg_new_image(int64_t width, int64_t height);
/* Wraps caller-owned device memory (4 * width * height bytes, 16-byte
 * aligned) without copying; pxg_image_free then releases only the handle. */
pxg_image* pxg_image_wrap(void* device_ptr, int64_t width, int64_t height);
void pxg_image_free(pxg_image* image);
int64_t pxg_image_width(const pxg_image* image);
int64_t pxg_image_height(const pxg_image* image);
void* pxg_image_device_ptr(pxg_image* image);
int pxg_image_upload(pxg_image* image, const void* host_rgbx, int64_t nbytes);
int pxg_image_download(const pxg_image* image, void* host_rgbx, int64_t nbytes);
/* fill(Image, Color)  src/pixie/images.nim:55-57 */
int pxg_image_fill(pxg_image* image, const float color[4]);

/* fillPath(Image, Path, Paint, Mat3, WindingRule) with a solid paint
 * src/pixie/paths.nim:2093-2113 (bindings/bindings.nim:143) */
int pxg_image_fill_path(pxg_image* image, const float* commands, int64_t n_commands,
                        const float color[4], float opacity, int blend_mode,
                        const float transform[9], int winding_rule);

/* strokePath(Image, Path, Paint, Mat3, strokeWidth, LineCap, LineJoin,
 * miterLimit, dashes) with a solid paint  src/pixie/paths.nim:2144-2175
 * (bindings/bindings.nim:144) */
int pxg_image_stroke_path(pxg_image* image, const float* commands, int64_t n_commands,
                          const float color[4], float opacity, int blend_mode,
                          const float transform[9], float stroke_width, int line_cap,
                          int line_join, float miter_limit, const float* dashes,
                          int64_t n_dashes);

/* draw(Image, Image, Mat3, BlendMode) for an integer translation, the
 * blendRect branch  src/pixie/images.nim:636-678, :468-529
 * (bindings/bindings.nim:137) */
int pxg_image_draw(pxg_image* a, const pxg_image* b, int64_t translate_x, int64_t translate_y,
                   int blend_mode);

/* blur(Image, float32, Color)  src/pixie/images.nim:304-365
 * (bindings/bindings.nim:133) */
int pxg_image_blur(pxg_image* image, float radius, const float out_of_bounds[4]);

/* spread(Image, float32)  src/pixie/images.nim:700-758 (private in the
 * reference; shadow's first pass) */
int pxg_image_spread(pxg_image* image, float spread);

/* shadow(Image, Vec2, spread, blur, Color) -> new Image
 * src/pixie/images.nim:760-776 (bindings/bindings.nim:135).  Offsets must be
 * integral (the blendRect branch of draw); the result is a new image. */
pxg_image* pxg_image_shadow(const pxg_image* image, float offset_x, float offset_y, float spread,
                            float blur, const float color[4]);
/* The same shadow written into `out` (an image of the same size), with no
 * allocation: the reference allocates the result inside shadow(). */
int pxg_image_shadow_into(const pxg_image* image, pxg_image* out, float offset_x, float offset_y,
                          float spread, float blur, const float color[4]);

/* One blend mode over pixel arrays in device memory: out[i] =
 * blender(mode)(backdrop[i], source[i])  src/pixie/blends.nim:275-299 */
int pxg_blend_pixels(int blend_mode, const void* backdrop, const void* source, void* out,
                     int64_t n_pixels);

/* Batched fills: n_jobs independent fillPath calls, each onto its own image,
 * in one launch of the setup and row kernels.  Job j draws commands
 * [cmd_offsets[j], cmd_offsets[j+1]) of `commands` onto images[j] with
 * colors[4j..4j+3], opacities[j], blend_modes[j], transforms[9j..] (or
 * identity when transforms is NULL) and winding_rules[j].  On failure
 * status[j] holds 0 (drawn) or the error of that job. */
int pxg_fill_paths_batch(pxg_image* const* images, int64_t n_jobs, const float* commands,
                         const int64_t* cmd_offsets, const float* colors, const float* opacities,
                         const int32_t* blend_modes, const float* transforms,
                         const int32_t* winding_rules, int32_t* status);

/* Blur without allocating: the same result as pxg_image_blur, for callers
 * that cannot call cudaMalloc (programs whose device memory is owned by their
 * own pool allocator, or latency-critical paths where an allocation's
 * blocking and device-wide synchronisation are not acceptable).  It works in
 * place on the caller's image (`rgbx`, 4 * width * height bytes, 16-byte
 * aligned) on the caller's stream and takes its work space from a fixed
 * 8 MiB + 16 KiB array in the library's device image, so images are limited
 * to 2097152 pixels and radii to 2048 (larger ones are rejected).  Every call
 * shares that array: calls whose GPU work overlaps race.  The first call on a
 * device sets the array up (cudaGetSymbolAddress) and should come before any
 * stream capture.  It returns once the work is enqueued.  No counterpart in
 * the reference, which has no device memory. */
int pxg_image_blur_noalloc(void* rgbx, int64_t width, int64_t height, float radius,
                           const float out_of_bounds[4], void* cuda_stream);

/* Time of the last blocking call's GPU work in milliseconds (CUDA events on
 * the library's stream); for measurement only. */
float pxg_last_gpu_ms(void);

/* blocking = 1 (default): every call returns after its GPU work finished,
 * like the reference's synchronous procs.  blocking = 0: draw, fill, blur,
 * spread and shadow only enqueue their kernels on the library's stream and
 * report launch errors; pxg_synchronize() waits.  fillPath/strokePath always
 * wait (their errors come from the GPU).  No counterpart in the reference. */
int pxg_set_blocking(int blocking);

/* Number of kernels this library has launched since it was loaded. */
int64_t pxg_launch_count(void);

#ifdef __cplusplus
}
#endif

#endif /* PXG_H */
