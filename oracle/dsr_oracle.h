/*
 * CPU oracle for the DFPSR triangle-rendering hot path -- TEST INFRASTRUCTURE ONLY.
 *
 * A plain, scalar C restatement of the reference's algorithm, used as the
 * checker for the CUDA path (tests, smoke() and bench.py's CPU-baseline leg).
 * The product never links, loads or calls it.  Every function cites the
 * reference file:line it restates (paths relative to the reference's Source/).
 *
 * Float arithmetic is IEEE binary32 in source order; the build must use
 * -ffp-contract=off so that a*b+c is never fused (the reference's exact build
 * is scalar with contraction off, see oracle/Makefile.ref).
 */
#ifndef DSR_ORACLE_H
#define DSR_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* TextureRgbaU8 (DFPSR/implementation/image/Texture.h:42-102). */
typedef struct {
	uint32_t log2width, log2height, maxMipLevel;
	uint32_t startOffset, maxLevelMask;
	uint32_t minWidthOrMask, minHeightOrMask, maxWidthAndMask, maxHeightAndMask;
	float floatMaxWidth, floatMaxHeight;
	uint32_t pixelCount;
	uint32_t *pixels; /* pyramid, smallest level first, RGBA bytes in memory order */
} or_texture;

/* A model with one part (DFPSR/implementation/render/model/Model.h:54-64,
 * Model.cpp:150-162).  polyIndices: polyCount x 4 (index 3 < 0 for triangles).
 * texCoords, colors: polyCount x 4 corners x 4 floats. */
typedef struct {
	const float *positions;
	int32_t pointCount;
	const int32_t *polyIndices;
	const float *texCoords;
	const float *colors;
	int32_t polyCount;
	const or_texture *diffuse; /* may be null */
	const or_texture *light;   /* may be null */
	int32_t filter;            /* 0 Solid, 1 Alpha */
} or_model;

/* Camera description shared by every entry point: location = position(3),
 * xAxis(3), yAxis(3), zAxis(3); slope = widthSlope (perspective) or halfWidth
 * (orthogonal). */
typedef struct {
	float location[12];
	int32_t perspective;
	float slope, nearClip, farClip;
	int32_t width, height;
} or_camera_desc;

/* Optional instrumentation collected while rendering. */
typedef struct {
	uint64_t fragments;      /* (pixel, triangle) pairs inside the row intervals, before the depth test */
	uint64_t trianglesDrawn; /* draw commands executed (after cull/clip/front-face) */
	uint32_t *coverage;      /* optional per-pixel fragment count */
	uint32_t *winner;        /* optional per-pixel order key of the last colour/depth write */
} or_stats;

/* ---- textures ---- */
int or_texture_init_empty(or_texture *t, uint32_t log2w, uint32_t log2h, uint32_t maxMipLevel);
int or_texture_create_from_image(or_texture *t, const uint32_t *level0, int32_t width, int32_t height, int32_t resolutions);
/* The same from an image in pack order packOrder (0..3, PackOrder.h:37-42). */
int or_texture_create_from_image_ordered(or_texture *t, const uint32_t *level0, int32_t width, int32_t height, int32_t resolutions,
                                         int32_t packOrder);
/* filter_resize(image, Sampler::Linear, w, h) of a dense RGBA image (api/filterAPI.cpp:852-859). */
void or_filter_resize_linear(uint32_t *dst, int32_t w, int32_t h, const uint32_t *src, int32_t sw, int32_t sh);
void or_texture_free(or_texture *t);
void or_texture_generate_pyramid(or_texture *t);
uint32_t or_texture_pixel_offset_to_layer(const or_texture *t, uint32_t mipLevel);
uint32_t or_texture_pixel_offset(const or_texture *t, uint32_t x, uint32_t y, uint32_t mipLevel);
uint32_t or_texture_read_pixel(const or_texture *t, uint32_t x, uint32_t y, uint32_t mipLevel);
void or_texture_write_pixel(or_texture *t, uint32_t x, uint32_t y, uint32_t mipLevel, uint32_t color);
uint32_t or_interpolate_color_linear(uint32_t a, uint32_t b, uint32_t weight);
uint32_t or_interpolate_color_bilinear(uint32_t a, uint32_t b, uint32_t c, uint32_t d, uint32_t wx, uint32_t wy);
uint32_t or_sample_bilinear(const or_texture *t, float u, float v, uint32_t mipLevel, int highestResolution);
uint32_t or_sample_nearest(const or_texture *t, float u, float v, uint32_t mipLevel, int highestResolution);
uint32_t or_mip_level_index(const or_texture *t, const float u[4], const float v[4]);

/* ---- geometry ---- */
void or_camera_to_screen(const or_camera_desc *cam, const float cs[3], float outIs[2], int64_t outFlat[2]);
void or_world_to_screen(const or_camera_desc *cam, const float world[3], float out[5], int64_t outFlat[2]);
int32_t or_triangle_rows(const int64_t flat[6], const int32_t clip[4], int32_t *startRow, int32_t *lefts, int32_t *rights, int32_t maxRows);

/* ---- rendering ---- */
/* model_render (DFPSR/api/modelAPI.cpp:197-201) when bands == 1, and the
 * band-split renderer_* path (renderCore.cpp:449-480) when bands > 1, run on
 * `threads` worker threads.  color (packOrder 0..3) and depth may be null. */
int or_model_render(const or_model *model, const float modelToWorld[12], const or_camera_desc *cam,
                    uint32_t *color, float *depth, int32_t packOrder, int32_t bands, int32_t threads,
                    or_stats *stats);
/* model_renderDepth (DFPSR/api/modelAPI.cpp:202-206). */
int or_model_render_depth(const or_model *model, const float modelToWorld[12], const or_camera_desc *cam,
                          float *depth, or_stats *stats);

/* ---- renderer with an occlusion grid (api/rendererAPI.cpp:141-477, modelAPI.cpp:214-275) ---- */
typedef struct or_renderer_s or_renderer;
or_renderer *or_renderer_create(void);
void or_renderer_destroy(or_renderer *r);
/* color (packOrder 0..3) and depth may be null; both are width x height without padding. */
int or_renderer_begin(or_renderer *r, uint32_t *color, float *depth, int32_t width, int32_t height, int32_t packOrder);
int or_renderer_give_task(or_renderer *r, const or_model *model, const float modelToWorld[12], const or_camera_desc *cam);
/* debugSilhouette keeps the box's hull as cyan lines drawn at renderer_end. */
int or_renderer_occlude_from_box(or_renderer *r, const float mn[3], const float mx[3], const float modelToWorld[12],
                                 const or_camera_desc *cam, int debugSilhouette);
int or_renderer_give_triangle(or_renderer *r, const float cs[9], const float is[6], const int64_t flat[6], const float colors[12],
                              const float texCoords[12], const or_texture *diffuse, const or_texture *light, int filter,
                              const or_camera_desc *cam);
int or_renderer_occlude_from_existing_triangles(or_renderer *r);
int or_renderer_occlude_from_top_rows(or_renderer *r, int perspective);
int or_renderer_is_box_visible(const or_renderer *r, const float mn[3], const float mx[3], const float modelToWorld[12],
                               const or_camera_desc *cam);
int or_renderer_has_occluders(const or_renderer *r);
int or_renderer_end(or_renderer *r, or_stats *stats, int debugWireframe);
/* draw_line (api/drawAPI.h) of a packed colour into a dense width x height image. */
void or_draw_line(uint32_t *image, int32_t width, int32_t height, int32_t x1, int32_t y1, int32_t x2, int32_t y2, uint32_t color);
int or_renderer_grid(const or_renderer *r, float *out, int32_t *gridWidth, int32_t *gridHeight);

/* ---- deferred light passes (SDK/SpriteEngine/lightAPI.h:27-31, orthoAPI.h:41-137) and draw_higher ---- */
/* OrthoView of OrthoSystem(cameraTilt, pixelsPerTile).view[index]; matrices as x, y, z axes. */
typedef struct {
	float normalToWorld[9];
	float screenDepthToLightSpace[9];
	float lightSpaceToScreenDepth[9];
	int32_t pixelOffsetPerTileX[2], pixelOffsetPerTileZ[2], yPixelsPerTile;
} or_ortho_view;
void or_ortho_view_create(float cameraTilt, int32_t pixelsPerTile, int32_t index, or_ortho_view *out);
void or_shadow_side_location(const float normalToWorld[9], int32_t side, float location[12]);
void or_directed_light(const or_ortho_view *view, uint32_t *light, int32_t lightStride, const uint32_t *normal,
                       int32_t normalStride, int32_t width, int32_t height, const float direction[3], float intensity,
                       const int32_t color[3], int32_t add);
int32_t or_point_light_bound(const or_ortho_view *view, int32_t centerX, int32_t centerY, int32_t width, int32_t height,
                             const float position[3], float radius, int32_t bound[4]);
void or_point_light(const or_ortho_view *view, int32_t centerX, int32_t centerY, uint32_t *light, int32_t lightStride,
                    const uint32_t *normal, int32_t normalStride, const float *heightImage, int32_t heightStride,
                    int32_t width, int32_t height, const float position[3], float radius, float intensity,
                    const int32_t color[3], const float *shadowCube, int32_t cubeWidth, int32_t threads);
void or_blend_light(uint32_t *target, int32_t targetStride, int32_t targetPackOrder, const uint32_t *diffuse,
                    int32_t diffuseStride, const uint32_t *lightImage, int32_t lightStride, int32_t width, int32_t height);
void or_draw_higher(float *targetHeight, int32_t thStride, uint32_t *targetA, int32_t taStride, int32_t taPack,
                    uint32_t *targetB, int32_t tbStride, int32_t tbPack, int32_t tw, int32_t th, const float *sourceHeight,
                    int32_t shStride, const uint32_t *sourceA, int32_t saStride, int32_t saPack, const uint32_t *sourceB,
                    int32_t sbStride, int32_t sbPack, int32_t sw, int32_t sh, int32_t left, int32_t top, float offset);

/* ---- dense models of the sprite engine (SDK/SpriteEngine/spriteAPI.cpp:236-262, 1143-1327) ---- */
typedef struct { float color[3][3]; float pos[3][3]; float normal[3][3]; } or_dense_triangle;
int32_t or_dense_triangle_count(const int32_t *polygons, int32_t polygonCount);
void or_dense_model_create(const float *positions, int32_t pointCount, const int32_t *polygons, const float *colors,
                           int32_t polygonCount, or_dense_triangle *out);
void or_dense_render(const or_dense_triangle *triangles, int32_t count, const or_ortho_view *view, float *height,
                     int32_t heightStride, uint32_t *diffuse, int32_t diffuseStride, uint32_t *normal, int32_t normalStride,
                     int32_t width, int32_t heightPx, float originX, float originY, const float modelToWorld[12],
                     int32_t highQuality);

#ifdef __cplusplus
}
#endif
#endif
