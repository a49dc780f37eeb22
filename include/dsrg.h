/*
 * dsrg: C ABI of the GB300 (sm_103a) implementation of DFPSR's triangle-rendering path.
 *
 * Plain C types only: pointers, sizes and status codes.  Every entry point names the
 * reference interface it replaces (paths relative to the reference's Source/ directory).
 * Every call returns DSRG_OK (0) or a nonzero status; dsrg_context_last_error() then holds
 * a message whose prefix matches the reference's error text where the reference has one.
 *
 * Threading: a context, and everything created from it, is driven by one host thread at a
 * time, like a dsr::Renderer (api/rendererAPI.h:54-55).  All work runs on the context's
 * CUDA stream; the render calls return when their results are in the target images.
 */
#ifndef DSRG_H
#define DSRG_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes. */
#define DSRG_OK 0
#define DSRG_ERROR_INVALID_ARGUMENT 1
#define DSRG_ERROR_CUDA 2
#define DSRG_ERROR_OUT_OF_MEMORY 3
#define DSRG_ERROR_CALL_ORDER 4
#define DSRG_ERROR_UNSUPPORTED 5
#define DSRG_ERROR_DEVICE 6

/* Filter of a model (implementation/render/constants.h:33). */
#define DSRG_FILTER_SOLID 0
#define DSRG_FILTER_ALPHA 1

/* PackOrderIndex of a colour image (implementation/image/PackOrder.h:37-42). */
#define DSRG_PACK_RGBA 0
#define DSRG_PACK_BGRA 1
#define DSRG_PACK_ARGB 2
#define DSRG_PACK_ABGR 3

typedef struct dsrg_context_s *dsrg_context;
typedef struct dsrg_texture_s *dsrg_texture;
typedef struct dsrg_model_s *dsrg_model;
typedef struct dsrg_renderer_s *dsrg_renderer;

/* A camera as Camera::createPerspective / Camera::createOrthogonal build it
 * (implementation/render/Camera.h:144-156).  location = position(3), xAxis(3), yAxis(3),
 * zAxis(3) of the camera's Transform3D; slope = widthSlope (perspective) or halfWidth
 * (orthogonal); nearClip/farClip are ignored for orthogonal cameras. */
typedef struct {
	float location[12];
	int32_t perspective;
	float slope;
	float nearClip;
	float farClip;
	int32_t width;
	int32_t height;
} dsrg_camera;

/* A target image: ImageRgbaU8 (4 bytes per pixel in packOrder) or ImageF32/AlignedImageF32
 * (float per pixel) (implementation/image/Image.h:249-289).  data points to row 0;
 * strideBytes is the distance between rows.  onDevice = 1 when data is device memory of the
 * context's GPU; 0 when it is host memory.  Page-locked (or registered) host memory is drawn
 * in place through its device address: the kernels read and write it over the host link, with
 * no staging copy.  Pageable host memory is copied to a device buffer and back inside the call. */
typedef struct {
	void *data;
	int32_t width;
	int32_t height;
	int32_t strideBytes;
	int32_t packOrder;
	int32_t onDevice;
} dsrg_image;

/* Counters of the last render call (the unit of work of the benchmarks). */
typedef struct {
	uint64_t fragments;      /* (pixel, triangle) pairs inside the row intervals, before the depth test; 0 unless counting is on */
	uint64_t drawRecords;    /* triangles left after culling, clipping and the front-face test */
	uint64_t binEntries;     /* (tile, triangle) pairs */
	float milliseconds;      /* GPU time of the last render from its first kernel to its last (CUDA events) */
	float rasterMilliseconds;/* GPU time of the last render's tile raster kernel alone (CUDA events) */
	uint64_t kernelLaunches; /* kernels this library has launched in this process so far */
} dsrg_stats;

/* ---- context ---- */
int dsrg_context_create(int32_t device, dsrg_context *out);
int dsrg_context_destroy(dsrg_context context);
const char *dsrg_context_last_error(dsrg_context context);
/* The cudaStream_t all work of the context is ordered on. */
void *dsrg_context_stream(dsrg_context context);
/* counting: 1 makes render calls count fragments (and, when coverage is a device buffer of
 * width*height uint32, write the per-pixel fragment count there); 0 turns it off. */
int dsrg_context_set_counting(dsrg_context context, int32_t counting, uint32_t *deviceCoverage);
int dsrg_context_get_stats(dsrg_context context, dsrg_stats *out);
/* Fragments the tile kernels have depth-tested on this context since it was created, counted
 * whether or not counting is on (no reference counterpart).  With counting off, early depth
 * culling skips fragments that cannot win, so the difference of two readings around a render is
 * the work that render actually walked; with counting on it equals the render's fragments. */
int dsrg_context_walked_fragments(dsrg_context context, uint64_t *out);

/* ---- textures: texture_create_RgbaU8(image, resolutions) (api/textureAPI.h:450-465,
 * api/textureAPI.cpp:89-131), built on the GPU: the image is resized linearly to the next powers
 * of two (filter_resize with Sampler::Linear, api/filterAPI.cpp:852-859) into level 0, and the mip
 * pyramid is the integer 2x2 box average of texture_generatePyramid (api/textureAPI.cpp:44-87).
 * pixels: width*height RGBA bytes in memory order, host memory. ---- */
int dsrg_texture_create(dsrg_context context, const uint32_t *pixels, int32_t width, int32_t height,
                        int32_t resolutions, dsrg_texture *out);
/* dsrg_texture_create for count images at once (host or device memory, RGBA pack order, any
 * stride), with resolutions[i] levels for image i; every phase (resize, each pyramid level) runs
 * as one launch over all images.  On failure no texture is made and out[] is all null. */
int dsrg_texture_create_many(dsrg_context context, int32_t count, const dsrg_image *images, const int32_t *resolutions,
                             dsrg_texture *out);
/* A TextureRgbaU8 that already exists, as the reference holds it (implementation/image/Texture.h:42-102:
 * impl_log2width, impl_log2height, impl_maxMipLevel and the impl_buffer pyramid, smallest level
 * first): the pyramid is copied to the GPU as it is, so a texture made or edited by the reference's
 * own texture API draws the same texels.  pyramid: host memory. */
int dsrg_texture_upload(dsrg_context context, const uint32_t *pyramid, uint32_t log2width, uint32_t log2height,
                        uint32_t maxMipLevel, dsrg_texture *out);
int dsrg_texture_destroy(dsrg_texture texture);
/* Copies the pyramid (smallest level first) to host memory; fields = log2width, log2height,
 * maxMipLevel, startOffset, maxLevelMask, minWidthOrMask, minHeightOrMask, maxWidthAndMask,
 * maxHeightAndMask (implementation/image/Texture.h:42-61). Returns the texel count in *count. */
int dsrg_texture_read(dsrg_texture texture, uint32_t *pixels, int32_t maxPixels, uint32_t *fields, int32_t *count);

/* ---- models: model_create + model_addPoint/addTriangle/addQuad/setTexCoord/setVertexColor/
 * setDiffuseMap/setLightMap/setFilter (api/modelAPI.h:62-258) in one call, one part.
 * positions: pointCount x 3 floats; polygonIndices: polygonCount x 4 (index 3 = -1 for a
 * triangle); texCoords and colors: polygonCount x 4 corners x 4 floats. Host memory. ---- */
int dsrg_model_create(dsrg_context context, const float *positions, int32_t pointCount, const int32_t *polygonIndices,
                      const float *texCoords, const float *colors, int32_t polygonCount, dsrg_texture diffuse,
                      dsrg_texture light, int32_t filter, dsrg_model *out);
int dsrg_model_destroy(dsrg_model model);
/* The model's bounding box as model_getBoundingBox returns it (api/modelAPI.h:138, ModelImpl::minBound /
 * maxBound): the box the culling and occlusion tests of model_render and renderer_giveTask use.
 * dsrg_model_create sets it from the points as the reference grows it point by point; a caller
 * mirroring a reference model whose points were edited passes the reference's box here. */
int dsrg_model_set_bound(dsrg_model model, const float *minimum, const float *maximum);

/* ---- rendering ---- */
/* model_render (api/modelAPI.h:285, api/modelAPI.cpp:197-201): draws the model into the colour
 * and depth images; either may be null.  modelToWorld as in dsrg_camera.location. */
int dsrg_model_render(dsrg_context context, dsrg_model model, const float *modelToWorld, const dsrg_camera *camera,
                      const dsrg_image *color, const dsrg_image *depth);
/* model_renderDepth (api/modelAPI.h:291, api/modelAPI.cpp:202-206). */
int dsrg_model_render_depth(dsrg_context context, dsrg_model model, const float *modelToWorld,
                            const dsrg_camera *camera, const dsrg_image *depth);

/* renderer_create / renderer_begin / renderer_giveTask / renderer_end (api/rendererAPI.h:56-135,
 * api/modelAPI.h:299-301): triangles of every task are drawn at renderer_end in submission
 * order, with the same result as model_render of the tasks one after another.  Models with
 * DSRG_FILTER_ALPHA blend over the colour target in submission order and only read depth; a
 * frame mixing them with solid models runs as consecutive runs of each kind. */
int dsrg_renderer_create(dsrg_context context, dsrg_renderer *out);
int dsrg_renderer_destroy(dsrg_renderer renderer);
int dsrg_renderer_begin(dsrg_renderer renderer, const dsrg_image *color, const dsrg_image *depth);
int dsrg_renderer_give_task(dsrg_renderer renderer, dsrg_model model, const float *modelToWorld, const dsrg_camera *camera);
int dsrg_renderer_end(dsrg_renderer renderer);
/* renderer_end(renderer, debugWireframe) (api/rendererAPI.h:111-112, rendererAPI.cpp:343-415):
 * with debugWireframe, white lines (draw_line, api/drawAPI.h) along the edges of every drawn
 * triangle over the finished colour image; the silhouettes kept by occlude_from_box with
 * debugSilhouette are drawn after them, by either form of renderer_end that has a colour image
 * (without one they stay for the next frame's).  dsrg_renderer_end(r) is
 * dsrg_renderer_end_debug(r, 0). */
int dsrg_renderer_end_debug(dsrg_renderer renderer, int32_t debugWireframe);
/* renderer_takesTriangles (api/rendererAPI.h:67): 1 between begin and end. */
int dsrg_renderer_takes_triangles(dsrg_renderer renderer);
/* renderer_getColorBuffer / renderer_getDepthBuffer (api/rendererAPI.h:60-63): the images given
 * to renderer_begin while the renderer takes triangles, else images with data = NULL. */
int dsrg_renderer_get_images(dsrg_renderer renderer, dsrg_image *color, dsrg_image *depth);

/* ProjectedPoint (implementation/render/ProjectedPoint.h:33-49): camera-space position, image
 * position and the sub-pixel position (1/256 pixel) the rasterizer uses. */
typedef struct {
	float cs[3];
	float is[2];
	int64_t flat[2];
} dsrg_projected_point;
/* Camera::worldToScreen (implementation/render/Camera.h:160-190), on the host. */
int dsrg_camera_world_to_screen(const dsrg_camera *camera, const float *world, dsrg_projected_point *out);
/* renderer_giveTask_triangle (api/rendererAPI.h:82-93) for count triangles sharing textures, filter
 * and camera: corners[3 * i + k], colors[(3 * i + k) * 4] (RGBA, 1 = full) and
 * texCoords[(3 * i + k) * 4] (u1, v1 for the diffuse map, u2, v2 for the light map) give corner
 * k of triangle i, already projected with the camera.  Host memory, copied by the call. */
int dsrg_renderer_give_triangles(dsrg_renderer renderer, int32_t count, const dsrg_projected_point *corners, const float *colors,
                                 const float *texCoords, dsrg_texture diffuse, dsrg_texture light, int32_t filter,
                                 const dsrg_camera *camera);

/* The renderer's occlusion grid (api/rendererAPI.h:69-101, rendererAPI.cpp:141-477): one value per
 * 16x16-pixel cell, the farthest camera-space depth at which something in the cell may still be
 * visible.  The first occluder of a frame resets it to infinity.  While a frame has occluders,
 * renderer_give_task skips models whose bounding box is occluded, and renderer_end skips draw
 * commands behind every cell of their bound.  minimum / maximum are model-space box corners.
 *   occlude_from_box              renderer_occludeFromBox: the box's screen hull occludes at its
 *                                 farthest corner (nothing when a corner lies outside the
 *                                 narrowed view frustum).  debugSilhouette draws the hull at
 *                                 renderer_end (cyan lines).
 *   occlude_from_existing_triangles  renderer_occludeFromExistingTriangles: every solid draw
 *                                 command given so far occludes the cells it covers.
 *   occlude_from_top_rows         renderer_occludeFromTopRows: the depth image's top pixel row of
 *                                 each cell row occludes (needs a depth image).
 *   is_box_visible                renderer_isBoxVisible: *visible = 0 when the box is outside the
 *                                 view or behind every cell it covers.
 *   has_occluders                 renderer_hasOccluders: 1 once the frame has an occluder. */
int dsrg_renderer_occlude_from_box(dsrg_renderer renderer, const float *minimum, const float *maximum,
                                   const float *modelToWorld, const dsrg_camera *camera, int32_t debugSilhouette);
int dsrg_renderer_occlude_from_existing_triangles(dsrg_renderer renderer);
int dsrg_renderer_occlude_from_top_rows(dsrg_renderer renderer, const dsrg_camera *camera);
int dsrg_renderer_is_box_visible(dsrg_renderer renderer, const float *minimum, const float *maximum,
                                 const float *modelToWorld, const dsrg_camera *camera, int32_t *visible);
int dsrg_renderer_has_occluders(dsrg_renderer renderer);
/* The grid as box tests read it, gridWidth x gridHeight values row by row (no reference
 * counterpart: the reference keeps the grid private).  out may be null to query the size. */
int dsrg_renderer_get_occlusion_grid(dsrg_renderer renderer, float *out, int32_t capacity, int32_t *gridWidth,
                                     int32_t *gridHeight);

/* ---- testing the failure paths (no reference counterpart) ----
 * The device allocation `after` allocations from now (0: the next one) fails as it would on an
 * exhausted GPU (cudaErrorMemoryAllocation), once; the call that needed it returns
 * DSRG_ERROR_OUT_OF_MEMORY and leaves its context usable.  A negative value turns it off.
 * Process-wide, for tests of a caller's error handling. */
int dsrg_debug_fail_allocation(int64_t after);

/* ---- depth rendering without allocation; this entry point has no counterpart in the reference.
 *
 * For callers that must not allocate GPU memory while they render: a frame loop held to a
 * no-allocation rule after start-up (cudaMalloc and cudaFree synchronise the whole device and
 * can stall unrelated work), or a host that gives the renderer a fixed memory budget up front.
 * It draws what dsrg_model_render_depth draws and calls no cudaMalloc, cudaFree or other
 * allocating routine.  Its intermediate buffers live in one static device array of
 * DSRG_NOALLOC_SCRATCH_BYTES that every GPU loading this library keeps until the process exits.
 * The CUDA driver reserves that array when it loads the library's device code on a device (with
 * lazy module loading, at the first call that needs it), so a caller with a fixed budget makes
 * one warm-up call at start-up; later calls take no device memory.
 *   - depth must be device memory (onDevice = 1) of at most DSRG_NOALLOC_MAX_SIDE pixels on a
 *     side; the model at most DSRG_NOALLOC_MAX_POINTS points and DSRG_NOALLOC_MAX_TRIANGLES fan
 *     triangles.  Larger inputs, or a view whose visible triangles need more than
 *     DSRG_NOALLOC_MAX_ROWS pixel rows or DSRG_NOALLOC_MAX_BIN_ENTRIES (tile, triangle) pairs,
 *     are rejected with DSRG_ERROR_UNSUPPORTED and a message naming the limit.
 *   - The first call on a device looks up the array's device address (cudaGetSymbolAddress)
 *     and keeps it for the life of the process.
 *     A device reset (cudaDeviceReset) inside the process is not supported afterwards.
 *   - Each call returns with its work finished: it reads counts back to the host between its
 *     kernels and waits for them on the context's stream.
 *   - Every call on a device shares the same array and leaves its contents behind (each call
 *     clears what it needs cleared); calls whose GPU work overlaps, from any context or thread,
 *     race on it, so they must be serialised. */
#define DSRG_NOALLOC_SCRATCH_BYTES (36u * 1024u * 1024u)
#define DSRG_NOALLOC_MAX_SIDE 1024
#define DSRG_NOALLOC_MAX_POINTS 49152
#define DSRG_NOALLOC_MAX_TRIANGLES 16384
#define DSRG_NOALLOC_MAX_ROWS 2097152u
#define DSRG_NOALLOC_MAX_BIN_ENTRIES 1048576u
int dsrg_model_render_depth_noalloc(dsrg_context context, dsrg_model model, const float *modelToWorld,
                                    const dsrg_camera *camera, const dsrg_image *depth);

/* ---- batched rendering; no counterpart in the reference, which renders one target per
 * renderer_begin / renderer_end (api/rendererAPI.h:54-55).
 *
 * A batch holds many frames, each an independent renderer_begin ... renderer_end: its own
 * colour and depth images (any sizes, host or device memory) and its own tasks, drawn in the
 * order given.  dsrg_batch_render draws every frame in one pass of the kernels: triangle setup
 * and binning run over all frames' triangles at once and one persistent tile kernel pulls
 * (frame, tile) work items from a single device queue.  Each frame's result equals
 * dsrg_renderer_begin / give_task ... / end on that frame alone.  The launches of each phase are
 * kept as CUDA graphs and replayed while the batch's sizes stay the same. */
typedef struct dsrg_batch_s *dsrg_batch;
int dsrg_batch_create(dsrg_context context, dsrg_batch *out);
int dsrg_batch_destroy(dsrg_batch batch);
/* Removes every frame and task (the batch can then be filled again). */
int dsrg_batch_clear(dsrg_batch batch);
/* Adds a frame (renderer_begin, api/rendererAPI.cpp:151-168); *frameIndex receives its index. */
int dsrg_batch_add_frame(dsrg_batch batch, const dsrg_image *color, const dsrg_image *depth, int32_t *frameIndex);
/* renderer_giveTask (api/modelAPI.h:299-301) for one frame of the batch.  Alpha-filtered models
 * on a frame with a colour target are rejected with DSRG_ERROR_UNSUPPORTED (draw them with
 * dsrg_renderer_* or dsrg_model_render). */
int dsrg_batch_give_task(dsrg_batch batch, int32_t frameIndex, dsrg_model model, const float *modelToWorld,
                         const dsrg_camera *camera);
/* Draws every frame (renderer_end of each); returns when all results are in the images.  The
 * batch keeps its frames and tasks, so rendering it again redraws the same scenes. */
int dsrg_batch_render(dsrg_batch batch);

/* Launch configuration of the tile kernel, chosen per context by dsrg_batch_autotune.
 *   threadsPerTile   threads of one tile's CTA (64, 128 or 256)
 *   ctasPerSm        persistent CTAs per SM pulling tiles from the queue (1 to 1024 / threadsPerTile)
 *   smallRows/Width  triangles whose raster bound is at most smallRows x smallWidth pixels are
 *                    walked by one lane each; larger ones by a whole warp per tile
 *   graphs           1 to replay each phase's launches as a CUDA graph, 0 to launch directly
 *   resolve          how winners are shaded (same results): 0 one pixel per thread in a launch of
 *                    its own, 1 per pixel inside the tile kernel (the default), 2 one 2x2 quad
 *                    per thread in a launch of its own */
typedef struct {
	int32_t threadsPerTile;
	int32_t ctasPerSm;
	int32_t smallRows;
	int32_t smallWidth;
	int32_t graphs;
	int32_t resolve;
} dsrg_tuning;
int dsrg_context_get_tuning(dsrg_context context, dsrg_tuning *out);
int dsrg_context_set_tuning(dsrg_context context, const dsrg_tuning *tuning);
/* Renders the batch once per candidate configuration (rounds times each, each timed render
 * starting from a cold L2 cache), keeps the fastest and returns it in *best (may be null): for the
 * batch when it has a configuration of its own (dsrg_batch_set_tuning), the context's staying as
 * it was, else for the context.  The images end up holding the batch's rendered frames. */
int dsrg_batch_autotune(dsrg_batch batch, int32_t rounds, dsrg_tuning *best);

/* A tile-kernel configuration for this batch alone (no counterpart in the reference): its renders
 * use *tuning and leave the context's configuration as it is, so that batches of different
 * workloads (a frame of small triangles, shadow faces of large ones) each keep the shape that
 * suits them.  tuning = null returns the batch to the context's configuration. */
int dsrg_batch_set_tuning(dsrg_batch batch, const dsrg_tuning *tuning);

/* ---- differentiable rendering; no counterpart in the reference.
 *
 * Views of one model rendered into float RGBA images.  Coverage and the depth test are exactly
 * dsrg_model_render's (the same row intervals, 2x2 quads and depth keys; coverage is never
 * smoothed).  Shading is RgbaMultiply (shader/RgbaMultiply.h:110-173) in float without U8
 * quantisation, times a directional light:
 *   uv     = wa*uv0 + wb*uv1 + wc*uv2      the model's texture coordinates of the corners (.xy)
 *   vertex = wa*c0 + wb*c1 + wc*c2         per-point RGBA colours (parameters)
 *   texel  = bilinear sample of the float RGBA texture (parameters): the reference's 1/256
 *            sub-texel positions (api/textureAPI.h:320-430), wrapped, full resolution only
 *   light  = ambient + intensity * max(0, -dot(N, dir))   N: unit world normal of the fan triangle
 *                                                        (B - A) x (C - A); dir, intensity: parameters
 *   rgb    = texel.rgb * vertex.rgb * light,   alpha = texel.a * vertex.a
 * with (wa, wb, wc) the fragment's perspective-correct vertex weights (fillerTemplates.h:197-233)
 * and wa = 1 - (wb + wc).  Uncovered pixels are 0.  The forward pass also writes a visibility
 * buffer, the checkpoint the adjoint reads instead of rasterising again: per pixel the fan
 * triangle (0xFFFFFFFF when uncovered) and the weights wb, wc as float bits.
 * Device memory, float32, row-major: texture [textureHeight][textureWidth][4] (power-of-two
 * sides), vertex colours [pointCount][4], light [4] = dir.x, dir.y, dir.z, intensity,
 * images [views][height][width][4], visibility [views][height][width][3] (uint32). */
typedef struct dsrg_diff_s *dsrg_diff;
int dsrg_diff_create(dsrg_context context, dsrg_model model, int32_t textureWidth, int32_t textureHeight, float ambient,
                     dsrg_diff *out);
int dsrg_diff_destroy(dsrg_diff diff);
/* cameras[views]: all of the same image size. */
int dsrg_diff_forward(dsrg_diff diff, int32_t views, const dsrg_camera *cameras, const float *modelToWorld,
                      const float *texture, const float *vertexColors, const float *light, float *images,
                      uint32_t *visibility);
/* loss = sum((images - targets)^2) / count into *loss (device), gradImages = 2 (images - targets) / count. */
int dsrg_diff_l2_loss(dsrg_diff diff, int64_t count, const float *images, const float *targets, float *gradImages,
                      float *loss);
/* The adjoint of dsrg_diff_forward at fixed visibility: writes (does not accumulate) the gradients
 * of the loss with respect to the texture, the vertex colours and the light from gradImages.
 * deterministic = 0: warp-aggregated atomics (sums in a run-dependent order);
 * deterministic = 1: every contribution sorted by its target (stable radix sort) and summed per
 * target in pixel order, bit-identical from run to run. */
int dsrg_diff_adjoint(dsrg_diff diff, int32_t views, int32_t width, int32_t height, const float *modelToWorld,
                      const float *texture, const float *vertexColors, const float *light, const uint32_t *visibility,
                      const float *gradImages, float *gradTexture, float *gradVertexColors, float *gradLight,
                      int32_t deterministic);

/* ---- deferred light passes of the isometric sprite engine (SDK/SpriteEngine/lightAPI.h:27-31,
 * orthoAPI.h:41-137) and draw_higher (api/drawAPI.h:142-150).
 * Images are device memory (onDevice = 1).  RGBA images other than blend targets and draw_higher
 * images are in the standard RGBA order, like the reference's OrderedImageRgbaU8. */

/* OrthoView (orthoAPI.h:41-91) with its matrices as x, y, z axes. */
typedef struct {
	float normalToWorld[9];
	float screenDepthToLightSpace[9];
	float lightSpaceToScreenDepth[9];
	int32_t pixelOffsetPerTileX[2];
	int32_t pixelOffsetPerTileZ[2];
	int32_t yPixelsPerTile;
} dsrg_ortho_view;
/* OrthoSystem(cameraTilt, pixelsPerTile).view[index] (orthoAPI.cpp:79-123); host only, no GPU call. */
int dsrg_ortho_view_create(float cameraTilt, int32_t pixelsPerTile, int32_t index, dsrg_ortho_view *out);
/* Camera location (as dsrg_camera.location) of side 0..5 of a point light's shadow cube map, the
 * rotation ShadowCubeMapSides[side] * normalToWorld at the origin (spriteAPI.cpp:328-336, 377-381);
 * its camera is perspective with slope 1 at the cube's resolution.  Host only. */
int dsrg_shadow_side_location(const float normalToWorld[9], int32_t side, float location[12]);

/* The light passes and draw_higher take their images where the caller has them, as the
 * reference's functions take host images (lightAPI.cpp:23-323, drawAPI.cpp:872-900): device memory
 * (onDevice = 1), page-locked host memory (read and written in place through its device address) or
 * pageable host memory (copied to the GPU and the written images back inside the call).  The same
 * holds for shadow cubes and sprite sources, told apart by their pointers.
 *
 * setDirectedLight (add = 0) / addDirectedLight (add = 1) (lightAPI.cpp:23-74). */
int dsrg_light_directed(dsrg_context context, const dsrg_ortho_view *view, const dsrg_image *light, const dsrg_image *normal,
                        const float direction[3], float intensity, const int32_t color[3], int32_t add);

/* One addPointLight call (lightAPI.cpp:169-285).  shadowCube: an image of cubeWidth x 6 cubeWidth
 * floats (six reciprocal-depth faces, no row padding) or null for a light without shadows. */
typedef struct {
	float position[3]; /* relative to the camera, as the reference takes it */
	float radius;
	float intensity;
	int32_t color[3];
	const float *shadowCube;
	int32_t cubeWidth;
} dsrg_point_light;
/* addPointLight for every light of the array, all in one pass: the sum of saturated additions of
 * non-negative bytes does not depend on their order.  referenceThreads is the hardware thread count
 * whose row bands the reference's threadedSplit would use (base/threading.cpp:193-263); each band
 * restarts the reference's light-space sweep, so results depend on it.  0 = this machine's count. */
int dsrg_light_points(dsrg_context context, const dsrg_ortho_view *view, int32_t centerX, int32_t centerY,
                      const dsrg_image *light, const dsrg_image *normal, const dsrg_image *height,
                      const dsrg_point_light *lights, int32_t count, int32_t referenceThreads);
/* blendLight (lightAPI.cpp:287-323): target (any pack order) = diffuse * light / 128 per channel. */
int dsrg_light_blend(dsrg_context context, const dsrg_image *target, const dsrg_image *diffuse, const dsrg_image *light);

/* ---- dense models of the sprite engine (SDK/SpriteEngine/spriteAPI.cpp:236-262, 1143-1327) ---- */
typedef struct dsrg_dense_model_s *dsrg_dense_model;
/* DenseModel_create: the model's polygons (polygonIndices: polygonCount x 4, index 3 = -1 for a
 * triangle) as vertex-coloured triangles (colors: polygonCount x 4 corners x RGBA, 1 = full) with
 * smooth normals.  Host arrays, copied by the call. */
int dsrg_dense_model_create(dsrg_context context, const float *positions, int32_t pointCount, const int32_t *polygonIndices,
                            const float *colors, int32_t polygonCount, dsrg_dense_model *out);
int dsrg_dense_model_destroy(dsrg_dense_model model);
/* renderDenseModel<highQuality> (spriteAPI.cpp:1244-1327): the model placed by modelToWorld
 * (position, x, y, z axes, in tiles) drawn through view into device images of one size: height
 * (F32) where the model is higher, diffuse (vertex colour) and normal (RGBA, normals in normal
 * space; high quality normalizes them per pixel).  originX/Y: the world origin in target pixels. */
int dsrg_dense_render(dsrg_context context, dsrg_dense_model model, const dsrg_ortho_view *view, const dsrg_image *height,
                      const dsrg_image *diffuse, const dsrg_image *normal, float originX, float originY, const float *modelToWorld,
                      int32_t highQuality);
/* One model instance of the sprite world (drawModel, spriteAPI.cpp:325-327). */
typedef struct {
	dsrg_dense_model model;
	float originX, originY;
	float modelToWorld[12];
} dsrg_dense_instance;
/* dsrg_dense_render of every instance in order, with the same result as that many calls, in one
 * pair of launches (heights compete across the instances; among equal heights the earlier wins). */
int dsrg_dense_render_many(dsrg_context context, const dsrg_dense_instance *instances, int32_t count, const dsrg_ortho_view *view,
                           const dsrg_image *height, const dsrg_image *diffuse, const dsrg_image *normal, int32_t highQuality);

/* One draw_higher source (F32 height + two RGBA images of the same size).  onDevice = 1 when the
 * three are device memory, 0 when they are host memory (page-locked or pageable). */
typedef struct {
	const float *height;
	const uint32_t *colorA;
	const uint32_t *colorB;
	int32_t width, height_;
	int32_t heightStrideBytes, colorAStrideBytes, colorBStrideBytes;
	int32_t colorAPackOrder, colorBPackOrder;
	int32_t left, top;
	float offset;
	int32_t onDevice;
} dsrg_sprite;
/* draw_higher(targetHeight, sourceHeight, targetA, sourceA, targetB, sourceB, left, top, offset)
 * (api/drawAPI.cpp:872-900, 946-981) for every sprite in order, in one pass: a pixel ends with the
 * highest raised source height that is strictly above the target's, the earliest sprite on ties. */
int dsrg_draw_higher(dsrg_context context, const dsrg_image *targetHeight, const dsrg_image *targetA,
                     const dsrg_image *targetB, const dsrg_sprite *sprites, int32_t count);

/* One frame of the sprite engine's deferred-light pass (the frame of spriteAPI.cpp:770-816 with
 * its background cleared as BackgroundBlock::draw does, spriteAPI.cpp:525-527), in one call:
 *   1. height = clearHeight, diffuse = clearDiffuse, normal = clearNormal;
 *   2. draw_higher of every sprite into height, diffuse (colour A) and normal (colour B);
 *   3. setDirectedLight with the sun into light (sunIntensity 0 and sunColor 0 give a black light);
 *   4. the shadow batch (a depth-only batch of cube faces), its depth images cleared to 0 first
 *      (CubeMapF32::clear, spriteAPI.cpp:361-363); null for no shadows;
 *   5. addPointLight for every light (dsrg_light_points, with referenceThreads);
 *   6. blendLight(output, diffuse, light).
 * With a shadow batch, steps 1-3 run on a second stream of the context beside step 4 (they touch
 * neither the cubes nor the batch's buffers) and step 5 waits for both; otherwise every step runs
 * on the context's stream in this order.  The call waits twice: once inside the shadow batch
 * (which checks its buffers) and once at its end.  The images are those of the steps
 * above (device, page-locked or pageable host memory; each pageable image is copied in once and,
 * if written, out once).  Shadow cubes (the batch's depth images and the lights' shadowCube) must
 * be device or page-locked memory.  The result equals that of the six calls made one by one. */
typedef struct {
	const dsrg_ortho_view *view;
	int32_t centerX, centerY;
	const dsrg_image *height, *diffuse, *normal, *light, *output;
	float clearHeight;
	uint32_t clearDiffuse, clearNormal;
	const dsrg_sprite *sprites;
	int32_t spriteCount;
	float sunDirection[3];
	float sunIntensity;
	int32_t sunColor[3];
	dsrg_batch shadows;
	const dsrg_point_light *lights;
	int32_t lightCount;
	int32_t referenceThreads;
} dsrg_sprite_frame_desc;
int dsrg_sprite_frame(dsrg_context context, const dsrg_sprite_frame_desc *frame);

/* A self-check with no reference counterpart: the point lights compute the scalar build's
 * (float)sqrt((double)x) and (float)(1.0 / sqrt((double)x)) as the correctly rounded float square
 * root and reciprocal square root.  This counts, on the device, the floats x with bit patterns
 * firstBits .. firstBits + count - 1 for which either pair differs (0 expected). */
int dsrg_check_float_roots(dsrg_context context, uint32_t firstBits, uint32_t count, uint64_t *mismatches);

/* model_renderDepth semantics for every frame of a batch (1 x 1 depth walk, no colour), for
 * shadow cube maps and other depth-only views: depthOnly = 1.  Frames need depth images only. */
int dsrg_batch_set_depth_only(dsrg_batch batch, int32_t depthOnly);

#ifdef __cplusplus
}
#endif
#endif
