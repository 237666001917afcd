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
/* The image's device address.  Once it has been handed out it stays fixed
 * for the image's lifetime (a blur of radius 1..8 then runs in place instead
 * of exchanging the image's buffer with the library's scratch buffer). */
void* pxg_image_device_ptr(pxg_image* image);
int pxg_image_upload(pxg_image* image, const void* host_rgbx, int64_t nbytes);
int pxg_image_download(const pxg_image* image, void* host_rgbx, int64_t nbytes);
/* applyOpacity(Image, float32)  src/pixie/images.nim:261-277: every channel
 * times round(255 * opacity), div 255 (0 clears, 255 keeps the image). */
int pxg_image_apply_opacity(pxg_image* image, float opacity);

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

/* draw(Image, Image, Mat3, BlendMode) with any transform
 * src/pixie/images.nim:636-678 (bindings/bindings.nim:137): the minifyBy2 /
 * magnifyBy2 pre-passes while the transform scales by 2 or more (or by 1/2 or
 * less), then drawSmooth (:531-634, bilinear getRgbaSmooth :367-403) unless the
 * transform is a whole-pixel translation, which takes blendRect as
 * pxg_image_draw does.  transform is vmath's Mat3: 9 floats, column-major
 * (translation in transform[6], transform[7]). */
int pxg_image_draw_transform(pxg_image* a, const pxg_image* b, const float transform[9], int blend_mode);

/* minifyBy2(Image, power) / magnifyBy2(Image, power)  src/pixie/images.nim:168-259:
 * a new image (NULL on error: "Cannot minifyBy2 with negative power",
 * "Cannot magnifyBy2 with negative power"); power 0 returns a copy. */
pxg_image* pxg_image_minify_by2(const pxg_image* image, int power);
pxg_image* pxg_image_magnify_by2(const pxg_image* image, int power);

/* drawTiled(Image, Image, Mat3, BlendMode)  src/pixie/images.nim:680-683 (drawCorrect
 * :405-445 with wrapped sampling): every destination pixel samples the source,
 * repeated, through the inverse transform. */
int pxg_image_draw_tiled(pxg_image* a, const pxg_image* b, const float transform[9], int blend_mode);

/* A paint (src/pixie/paints.nim:12-26, bindings/bindings.nim Paint):
 * kind is PaintKind (0 solid, 1 image, 2 tiled image, 3 linear gradient,
 * 4 radial gradient, 5 angular gradient); color is chroma's straight float
 * Color (solid); image / image_mat the image paint's image and vmath Mat3
 * (column-major); handles n_handles (x, y) pairs and stops n_stops
 * (r, g, b, a, position) records (gradients). */
typedef struct pxg_paint {
  int32_t kind;
  int32_t blend_mode;
  float opacity;
  float color[4];
  const pxg_image* image;
  float image_mat[9];
  int32_t n_handles;
  const float* handles;
  int32_t n_stops;
  const float* stops;
} pxg_paint;

/* fillPath / strokePath with any paint  src/pixie/paths.nim:2093-2142,
 * :2144-2210 (bindings/bindings.nim:143-144): a solid paint takes
 * pxg_image_fill_path / pxg_image_stroke_path; the others fill a mask with
 * the path, fill an image with the paint (image, tiled image or gradient),
 * apply the paint's opacity to the mask, MaskBlend the mask onto it and draw
 * it onto the image with the paint's blend mode.  Errors as the reference:
 * "Linear gradient requires 2 handles", "Radial gradient requires 3 handles",
 * "Angular gradient requires 2 handles" (sic, for 3),
 * "Gradient must have at least 1 color stop". */
int pxg_image_fill_path_paint(pxg_image* image, const float* commands, int64_t n_commands,
                              const pxg_paint* paint, const float transform[9], int winding_rule);
int pxg_image_stroke_path_paint(pxg_image* image, const float* commands, int64_t n_commands,
                                const pxg_paint* paint, const float transform[9], float stroke_width,
                                int line_cap, int line_join, float miter_limit, const float* dashes,
                                int64_t n_dashes);

/* fill(Image, Paint)  src/pixie.nim:120-131: the colour, the image paint
 * through a full-image rectangle, or the gradient written in place. */
int pxg_image_fill_paint(pxg_image* image, const pxg_paint* paint);

/* blur(Image, float32, Color)  src/pixie/images.nim:304-365
 * (bindings/bindings.nim:133) */
int pxg_image_blur(pxg_image* image, float radius, const float out_of_bounds[4]);

/* Stroke outlines: 1 (default) builds the outline of a stroke without
 * dashes on the GPU (strokeShapes, src/pixie/paths.nim:1922-2082: the host
 * flattens the path into polylines, one kernel thread per polyline point
 * writes its rectangle, join and caps); 0 builds every outline on the host.
 * Both give the same bytes: a join whose angle lies within 1e-5 of one of the
 * join's decision thresholds is rebuilt on the host with the C library's
 * atan2f, as the reference computes it.  No counterpart in the reference. */
int pxg_stroke_config(int gpu_outline);

/* Joins the GPU outline found ambiguous and rebuilt on the host, since the
 * library was loaded.  No counterpart in the reference. */
int64_t pxg_stroke_fixups(void);

/* Blur kernels: 3 (default) runs radii 1..8 on register-blocked CUDA-core
 * passes and radii 9..128 on the tensor cores with TMA-fed input rings in
 * tensor memory (images whose sides are multiples of 4; others take mode 1's
 * kernels); 1 runs radii 8..128 on the tensor cores with the warp-specialised
 * kernel that loads through registers; 2 uses the single-stage tensor-core
 * kernel (radii 8..128); 0 the tiled CUDA-core kernels (which every mode uses
 * for the radii it does not take).  All write the same bytes.  No
 * counterpart in the reference. */
int pxg_blur_config(int use_tensor_cores);

/* The kernel family the last blur ran on: 5 (the fused one-launch kernel of
 * mode 3 for radii 1..8, on images the library allocated whose device
 * address was never handed out: the result lands in the library's scratch
 * buffer and the two buffers change owners), 4 (the two small-radius passes
 * of mode 3, in place), 3 (the ring passes), 2, 1 or 0 as above (-1 before
 * any blur).  No counterpart in the reference. */
int pxg_last_blur_kernel(void);

/* Converter trace of the ring blur passes, a profiling aid: enable != 0
 * switches it on (and clears it) for the passes launched afterwards, 0 off.
 * If out is not NULL it receives up to n int64 values from the last traced
 * pass, laid out [converter group 0..1][ring chunk 0..255][event 0..2]: the
 * clock64 of CTA 0's second converter warp before its barrier waits for the
 * chunk, after them, and after its tensor-memory stores (0 where nothing was
 * recorded).  Synchronizes the device.  No counterpart in the reference. */
int pxg_ring_trace(int enable, int64_t* out, int64_t n);

/* spread(Image, float32)  src/pixie/images.nim:700-758 (private in the
 * reference; shadow's first pass) */
int pxg_image_spread(pxg_image* image, float spread);

/* shadow(Image, Vec2, spread, blur, Color) -> new Image
 * src/pixie/images.nim:760-776 (bindings/bindings.nim:135).  A whole-pixel
 * offset moves the mask as draw's blendRect branch does; a fractional one
 * resamples it with drawSmooth (OverwriteBlend) first.  The result is a new
 * image. */
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

/* Scenes: a recorded sequence of fillPath/strokePath calls painted onto one
 * image in order -- what a caller of the reference does when it draws many
 * paths onto one image (src/pixie/paths.nim:2093-2175 called in a loop, as
 * svg.nim:557-600 and contexts.nim:384-400 do).  pxg_scene_fill_path and
 * pxg_scene_stroke_path take the arguments of pxg_image_fill_path and
 * pxg_image_stroke_path, check them and build the path's geometry at once
 * (geometry errors are returned by the recording call, and that path is not
 * recorded); paths whose paint draws nothing are skipped, as fillPath skips
 * them.  pxg_image_draw_scene paints every recorded path in order with one
 * setup launch and one row launch (MaskBlend paths, whose clears reach rows
 * outside the path, are drawn alone between the runs around them).  If a
 * path fails while drawing (e.g. "Unable to discretize cubic"), the paths
 * before it are drawn, it and the later paths are not, and the error is
 * returned -- the state the reference leaves when that call raises. */
typedef struct pxg_scene pxg_scene;
pxg_scene* pxg_scene_new(void);
void pxg_scene_free(pxg_scene* scene);
int pxg_scene_clear(pxg_scene* scene);
int64_t pxg_scene_len(const pxg_scene* scene);
int pxg_scene_fill_path(pxg_scene* scene, const float* commands, int64_t n_commands,
                        const float color[4], float opacity, int blend_mode,
                        const float transform[9], int winding_rule);
int pxg_scene_stroke_path(pxg_scene* scene, const float* commands, int64_t n_commands,
                          const float color[4], float opacity, int blend_mode,
                          const float transform[9], float stroke_width, int line_cap,
                          int line_join, float miter_limit, const float* dashes, int64_t n_dashes);

/* n recordings in one call, as n calls of pxg_scene_fill_path (kinds[i] 0)
 * or pxg_scene_stroke_path (kinds[i] 1, no dashes) would make them: path i's
 * commands are cmds[offs[i] .. offs[i + 1]), its paint colors[4 i ..],
 * opacities[i], blends[i], its transform transforms[9 i ..] (NULL:
 * identity), windings[i] (fills), widths / caps / joins / miters[i]
 * (strokes).  The geometry is built on `threads` host threads (0: all) and the
 * paths are appended in submission order.  status[i] (may be NULL) is 1 where
 * path i failed -- it is skipped, as a failed call records nothing, and the
 * first failure's message is left for pxg_take_error -- else 0. */
int pxg_scene_record_batch(pxg_scene* scene, int64_t n, const int32_t* kinds, const float* cmds,
                           const int64_t* offs, const float* colors, const float* opacities,
                           const int32_t* blends, const float* transforms, const int32_t* windings,
                           const float* widths, const int32_t* caps, const int32_t* joins,
                           const float* miters, int32_t* status, int threads);
int pxg_image_draw_scene(pxg_image* image, const pxg_scene* scene);
/* Scene drawing configuration (every choice writes the same bytes):
 * slice_width is the part of a canvas row one warp of the drawing pass owns
 * (>= 32 pixels; default 256), or 0 to choose it per launch from the canvas
 * rows and the GPU's resident warps.  coverage_bytes >= 0 replaces the arena
 * in which the recording pass stores rows' coverage bytes (default: 4 GB or
 * an eighth of free memory); rows that do not fit are recorded as sample
 * spans and accumulated by the drawing pass instead; a negative value keeps
 * the current arena. */
int pxg_scene_config(int slice_width, int64_t coverage_bytes);

/* Mask batches: many paths, each filled with color(1, 1, 1, 1) onto a
 * transparent image of its own size, kept as the 8-bit alpha of that image
 * (every channel of such an image equals its alpha).  This is the first half
 * of rendering glyphs in the reference: fillPath of each glyph's path into
 * its own image (src/pixie/paths.nim:2093-2113; fonts.nim:566-596 fills
 * glyph paths).  pxg_masks_add_path builds the primitives on the host;
 * pxg_masks_render renders every mask of the batch in one setup launch and
 * one persistent row launch (a device work queue of row items), captured
 * once in a CUDA graph and replayed while the batch's shape is unchanged;
 * pxg_masks_download copies mask i (width * height bytes) to the host.
 * pxg_image_draw_masks is the second half: draw(page, mask_i,
 * translate(xy[2i], xy[2i+1]), blend_mode) for i = 0..n-1 in order
 * (images.nim:636-678, blendRect :468-529) in one launch; MaskBlend, whose
 * draw clears the whole page outside each mask, is rejected.  No
 * counterpart in the reference's bindings. */
typedef struct pxg_masks pxg_masks;
pxg_masks* pxg_masks_new(void);
void pxg_masks_free(pxg_masks* masks);
int64_t pxg_masks_len(const pxg_masks* masks);
int pxg_masks_add_path(pxg_masks* masks, const float* commands, int64_t n_commands, int64_t width,
                       int64_t height, const float transform[9], int winding_rule);

/* n glyphs in one call, as n calls of pxg_masks_add_path would add them
 * (path i: cmds[offs[i] .. offs[i + 1]), widths[i] x heights[i],
 * transforms[9 i ..] or NULL, windings[i] or NULL for NonZero); the geometry
 * is built on `threads` host threads (0: all).  All or nothing: if a path
 * fails, no glyph is added and its error is returned. */
int pxg_masks_add_paths(pxg_masks* masks, int64_t n, const float* cmds, const int64_t* offs,
                        const int64_t* widths, const int64_t* heights, const float* transforms,
                        const int32_t* windings, int threads);
int pxg_masks_render(pxg_masks* masks);
/* Renders with a given row-kernel configuration instead of the tuned one
 * (variant 0: 256-crossing scratch, 1: 32-crossing scratch; rows per work
 * item 1..64); for tests and tuning. */
int pxg_masks_render_config(pxg_masks* masks, int variant, int rows_per_item);
int pxg_masks_download(const pxg_masks* masks, int64_t index, void* out, int64_t nbytes);
const void* pxg_masks_device_ptr(const pxg_masks* masks, int64_t index);
int pxg_image_draw_masks(pxg_image* page, const pxg_masks* masks, const int64_t* xy, int blend_mode);

/* Serving: render jobs admitted against a device-memory budget and advanced
 * together by continuous batching.  A job paints a recorded scene onto a
 * fresh transparent width x height canvas (the reference's newImage + the
 * scene's fillPath/strokePath calls), then blurs it when blur_radius rounds
 * to a radius > 0 (images.nim:304-365, transparent out-of-bounds colour).
 * pxg_server_submit queues a job (the scene must stay alive and unchanged
 * until the job's result is taken) and returns its id (0 on error).
 * pxg_server_step admits queued jobs in arrival order while their canvases
 * (and blur work space) fit the budget, then advances every admitted job by
 * up to paths_per_job of its paths -- at most paths_per_step paths and 8M
 * path-rows (paths x canvas height) in all -- in one scene launch sequence
 * (setup, recording, drawing); jobs whose paths are all painted
 * are blurred and finish, freeing their memory for the next admissions.
 * pxg_server_poll returns finished job ids; pxg_server_take copies a
 * finished job's canvas to the host (out may be NULL), reports its submit,
 * admit and finish times (seconds, steady clock) and releases it; a job
 * whose path raised returns that error from pxg_server_take.
 * pxg_server_stats: steps, bytes in use, peak bytes, peak admitted jobs,
 * queued jobs, admitted jobs.  No counterpart in the reference. */
typedef struct pxg_server pxg_server;
pxg_server* pxg_server_new(int64_t budget_bytes, int64_t paths_per_job, int64_t paths_per_step);
void pxg_server_free(pxg_server* server);
int64_t pxg_server_submit(pxg_server* server, const pxg_scene* scene, int64_t width, int64_t height,
                          float blur_radius);
int pxg_server_step(pxg_server* server);
int64_t pxg_server_pending(const pxg_server* server);
int64_t pxg_server_poll(pxg_server* server, int64_t* ids, int64_t capacity);
int pxg_server_take(pxg_server* server, int64_t id, void* out_rgbx, int64_t nbytes, double times[3]);
int pxg_server_stats(const pxg_server* server, int64_t out[6]);

/* Autotuner: for each operation and shape class, the fastest of a few launch
 * configurations (row-kernel scratch size and rows per work item for mask
 * batches; the page tile of the mask composite), timed once the first time
 * the class is seen.  Every configuration writes the same bytes.  On by
 * default; pxg_autotune_report writes one line per tuned class into buf and
 * returns the report's length.  No counterpart in the reference. */
int pxg_autotune(int enable);
int64_t pxg_autotune_report(char* buf, int64_t capacity);

/* Counts of the last fill launch (fillPath, strokePath, batch or scene):
 * out[0] paths, out[1] primitives, out[2] segments after flattening, out[3]
 * band entries, out[4] pixel blends of a scene's drawing pass (0 for other
 * launches), out[5] rows whose crossings exceeded the shared-memory scratch.
 * No counterpart in the reference. */
int pxg_last_fill_stats(int64_t out[6]);

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
 * report launch errors; pxg_image_upload / pxg_image_download run on their
 * own copy streams, ordered after the calls before them and before the calls
 * after them (an upload's host buffer must stay unchanged, and a download's
 * holds the image, only after pxg_synchronize), so copies overlap other
 * images' work; pxg_synchronize() waits for everything.  fillPath/strokePath
 * always wait (their errors come from the GPU).  Enqueued calls keep the
 * order of the calls for every image: a draw, blur or shadow whose images no
 * kernel still running touches may start before the kernel before it has
 * finished, and finishes only after it.  No counterpart in the reference. */
int pxg_set_blocking(int blocking);

/* Number of kernels this library has launched since it was loaded. */
int64_t pxg_launch_count(void);

#ifdef __cplusplus
}
#endif

#endif /* PXG_H */
