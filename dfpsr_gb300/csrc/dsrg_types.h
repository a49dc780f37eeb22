// Data layouts shared by the host side and the kernels of the DFPSR triangle path.
#ifndef DSRG_TYPES_H
#define DSRG_TYPES_H

#include <stddef.h>
#include <stdint.h>

#if !defined(__CUDACC__) && !defined(__align__)
#define __align__(n) alignas(n)
#endif

namespace dsrg {

// Tiles of the screen that one CTA owns while rasterising.
static const int32_t TILE_W = 16;
static const int32_t TILE_H = 16;
static const int32_t TILE_PIXELS = TILE_W * TILE_H;
// Row stride of the shared tile arrays: one word of padding keeps the 16 rows of a column in
// different shared-memory banks.
static const int32_t TILE_STRIDE = TILE_W + 1;

// A plane a*x + b*y + c*z - offset <= 0 means inside (math/FPlane3D.h:38-46).
struct Plane {
	float nx, ny, nz, offset;
};

// Everything a kernel needs from a dsr::Camera (implementation/render/Camera.h:125-218),
// precomputed on the host in the reference's order of operations.
struct CameraData {
	float position[3];
	float xAxis[3], yAxis[3], zAxis[3];
	float invWidthSlope, invHeightSlope, imageWidth, imageHeight;
	int32_t perspective;
	int32_t cullCount, clipCount;
	Plane cull[6];
	Plane clip[6];
};

// TextureRgbaU8 fields (implementation/image/Texture.h:42-61) with a device pointer to the pyramid.
struct TextureData {
	const uint32_t *pixels;
	uint32_t log2width, log2height, maxMipLevel, startOffset, maxLevelMask;
	uint32_t maxWidthAndMask, maxHeightAndMask;
	float floatMaxWidth, floatMaxHeight;
	int32_t exists;
};

// A corner given already projected (ProjectedPoint, implementation/render/ProjectedPoint.h:33-49),
// laid out as dsrg_projected_point of the C interface.
struct GivenPoint {
	float cs[3];
	float is[2];
	int64_t flat[2];
};
static_assert(sizeof(GivenPoint) == 40, "GivenPoint layout");

// Shader variant bits of processTriangle_RgbaMultiply (implementation/render/shader/RgbaMultiply.h:110-173).
enum ShadeFlags : uint32_t {
	SHADE_DIFFUSE = 1u,
	SHADE_LIGHT = 2u,
	SHADE_VERTEX_FADE = 4u,
	SHADE_COLORLESS = 8u,
	SHADE_ALPHA_FILTER = 16u,
};

// Per source triangle: scaled vertex colours and texture coordinates (shader/Shader.h:36-60,
// RgbaMultiply.h:37-58) plus the variant and its textures, computed where a pixel is shaded.
struct ShadeRecord {
	float red[3], green[3], blue[3], alpha[3];
	float u1[3], v1[3], u2[3], v2[3];
	uint32_t flags;
	int32_t diffuse; // index into the batch's texture table, -1 for none
	int32_t light;
};

// One draw command after culling, clipping and the front-face test
// (implementation/render/renderCore.h:52-70): sub-pixel corners, the row-aligned
// raster bound inside the target, and the vertex-weight projection (ITriangle2D.h:63-78).
// 96 bytes, 16-byte aligned so that it moves in six 128-bit accesses.
struct __align__(16) DrawRecord {
	int32_t flat[6];
	int32_t left, top, right, bottom; // getAlignedRasterBound against the whole target
	float start[3], dx[3], dy[3];     // pWeightStart, pWeightDx, pWeightDy
	uint32_t order;                   // submission order: triangle index * 8 + clipped sub-triangle index
	uint32_t tri;                     // fan triangle of its task (polygon data for shading)
	uint32_t task;                    // index into the batch's task table
	uint32_t frame;                   // index into the batch's frame table
	int32_t source;                   // the task's triSource entry of tri (polygon * 2 + fan), for shading
};
// The row kernel loads corners and bounds as int4 (flat[0..3]), int4 (flat[4..5], left, top) and int2 (right, bottom).
static_assert(sizeof(DrawRecord) == 96, "DrawRecord is 96 bytes");
static_assert(offsetof(DrawRecord, left) == 24 && offsetof(DrawRecord, top) == 28 && offsetof(DrawRecord, right) == 32 &&
              offsetof(DrawRecord, bottom) == 36, "DrawRecord field offsets");

} // namespace dsrg

#endif
