// Test-infrastructure harness around the UNMODIFIED DFPSR reference library.
//
// This file is part of the oracle (test infrastructure only). It is compiled
// together with the reference's own sources (built out-of-tree by
// oracle/Makefile.ref into oracle/_ref/) and exposes a small extern "C" surface
// so that Python tests can drive the reference's public API on seeded inputs:
//   * model_render / model_renderDepth        (Source/DFPSR/api/modelAPI.h:285-291)
//   * renderer_create/begin/giveTask/end      (Source/DFPSR/api/rendererAPI.h:56-135, modelAPI.h:299)
//   * texture_create_RgbaU8(image, levels)    (Source/DFPSR/api/textureAPI.h:450-465)
//   * rasterizeTriangle row intervals         (Source/DFPSR/implementation/render/ITriangle2D.h:52)
//   * addPointLight / setDirectedLight / blendLight (Source/SDK/SpriteEngine/lightAPI.h:27-31)
//   * draw_higher                              (Source/DFPSR/api/drawAPI.h:142-150)
// Nothing in the product links this file.

#include "DFPSR/includeFramework.h"
#include "DFPSR/implementation/render/ITriangle2D.h"
#include "DFPSR/implementation/render/renderCore.h"
#include "SDK/SpriteEngine/lightAPI.h"
#include "SDK/SpriteEngine/orthoAPI.h"
#include "DFPSR/base/threading.h"
#include <cstring>
#include <cstdint>
#include <vector>

using namespace dsr;

namespace {

Transform3D makeTransform(const float* t) {
	// t = position(3), xAxis(3), yAxis(3), zAxis(3)
	return Transform3D(FVector3D(t[0], t[1], t[2]),
	  FMatrix3x3(FVector3D(t[3], t[4], t[5]), FVector3D(t[6], t[7], t[8]), FVector3D(t[9], t[10], t[11])));
}

Camera makeCamera(const float* location, int perspective, float slope, int width, int height, float nearClip, float farClip) {
	if (perspective) {
		return Camera::createPerspective(makeTransform(location), float(width), float(height), slope, nearClip, farClip);
	} else {
		return Camera::createOrthogonal(makeTransform(location), float(width), float(height), slope);
	}
}

struct TextureBox { TextureRgbaU8 texture; };
struct ModelBox { Model model; };

void copyInRgba(const ImageRgbaU8& image, const uint32_t* src, int width, int height) {
	for (int y = 0; y < height; y++) {
		uint32_t* row = image_getSafePointer<uint32_t>(image, y).getUnsafe();
		std::memcpy(row, src + (size_t)y * width, sizeof(uint32_t) * width);
	}
}
void copyOutRgba(const ImageRgbaU8& image, uint32_t* dst, int width, int height) {
	for (int y = 0; y < height; y++) {
		const uint32_t* row = image_getSafePointer<uint32_t>(image, y).getUnsafe();
		std::memcpy(dst + (size_t)y * width, row, sizeof(uint32_t) * width);
	}
}
void copyInF32(const ImageF32& image, const float* src, int width, int height) {
	for (int y = 0; y < height; y++) {
		float* row = image_getSafePointer<float>(image, y).getUnsafe();
		std::memcpy(row, src + (size_t)y * width, sizeof(float) * width);
	}
}
void copyOutF32(const ImageF32& image, float* dst, int width, int height) {
	for (int y = 0; y < height; y++) {
		const float* row = image_getSafePointer<float>(image, y).getUnsafe();
		std::memcpy(dst + (size_t)y * width, row, sizeof(float) * width);
	}
}

} // namespace

extern "C" {

// Tells the reference's heap that the process is ending (base/heap.h:161), so that its
// leak report at exit stays quiet when the harness is unloaded with live allocations.
void refh_shutdown() { heap_terminatingApplication(); }

// Creates a texture pyramid from a width x height RGBA image (bytes R,G,B,A in memory).
void* refh_texture_create(const uint32_t* pixels, int width, int height, int resolutions) {
	OrderedImageRgbaU8 image = image_create_RgbaU8(width, height);
	copyInRgba(image, pixels, width, height);
	TextureBox* box = new TextureBox();
	box->texture = texture_create_RgbaU8(image, resolutions);
	return box;
}

// Reads the texture's pyramid buffer and fields.
// fields = log2width, log2height, maxMipLevel, startOffset, maxLevelMask, minWidthOrMask,
//          minHeightOrMask, maxWidthAndMask, maxHeightAndMask; returns the pixel count.
int refh_texture_info(void* handle, uint32_t* fields, uint32_t* pixels, int maxPixels) {
	TextureRgbaU8& t = ((TextureBox*)handle)->texture;
	fields[0] = t.impl_log2width; fields[1] = t.impl_log2height; fields[2] = t.impl_maxMipLevel;
	fields[3] = t.impl_startOffset; fields[4] = t.impl_maxLevelMask; fields[5] = t.impl_minWidthOrMask;
	fields[6] = t.impl_minHeightOrMask; fields[7] = t.impl_maxWidthAndMask; fields[8] = t.impl_maxHeightAndMask;
	int count = (int)(t.impl_startOffset + (uint32_t(1) << (t.impl_log2width + t.impl_log2height)));
	if (pixels) {
		const uint32_t* data = t.impl_buffer.getSafe<uint32_t>("harness").getUnsafe();
		std::memcpy(pixels, data, sizeof(uint32_t) * (count < maxPixels ? count : maxPixels));
	}
	return count;
}

// The same from an image in pack order packOrder (0..3, PackOrderIndex), created with
// image_create_RgbaU8_native as a program's own image would be; pixels are the packed values.
void* refh_texture_create_ordered(const uint32_t* pixels, int width, int height, int resolutions, int packOrder) {
	AlignedImageRgbaU8 image = image_create_RgbaU8_native(width, height, (PackOrderIndex)packOrder);
	copyInRgba(image, pixels, width, height);
	TextureBox* box = new TextureBox();
	box->texture = texture_create_RgbaU8(image, resolutions);
	return box;
}

void refh_texture_free(void* handle) { delete (TextureBox*)handle; }

// polyIndices: polyCount x 4 (index 3 = -1 for triangles); texCoords, colors: polyCount x 4 x 4 floats.
void* refh_model_create(const float* positions, int pointCount, const int* polyIndices,
                        const float* texCoords, const float* colors, int polyCount,
                        void* diffuse, void* light, int filter) {
	ModelBox* box = new ModelBox();
	box->model = model_create();
	model_setFilter(box->model, filter ? Filter::Alpha : Filter::Solid);
	int part = model_addEmptyPart(box->model, U"part");
	if (diffuse) model_setDiffuseMap(box->model, part, ((TextureBox*)diffuse)->texture);
	if (light) model_setLightMap(box->model, part, ((TextureBox*)light)->texture);
	for (int p = 0; p < pointCount; p++) {
		model_addPoint(box->model, FVector3D(positions[p * 3], positions[p * 3 + 1], positions[p * 3 + 2]));
	}
	for (int p = 0; p < polyCount; p++) {
		const int* idx = polyIndices + p * 4;
		int poly;
		int corners;
		if (idx[3] < 0) {
			poly = model_addTriangle(box->model, part, idx[0], idx[1], idx[2]);
			corners = 3;
		} else {
			poly = model_addQuad(box->model, part, idx[0], idx[1], idx[2], idx[3]);
			corners = 4;
		}
		for (int v = 0; v < corners; v++) {
			const float* tc = texCoords + (p * 4 + v) * 4;
			const float* co = colors + (p * 4 + v) * 4;
			model_setTexCoord(box->model, part, poly, v, FVector4D(tc[0], tc[1], tc[2], tc[3]));
			model_setVertexColor(box->model, part, poly, v, FVector4D(co[0], co[1], co[2], co[3]));
		}
	}
	return box;
}

void refh_model_free(void* handle) { delete (ModelBox*)handle; }

// mode 0: model_render (single thread).  mode 1: renderer_begin/giveTask/end (threaded bands).
// color may be null (depth-only target through model_render), depth may be null.
// packOrder: PackOrderIndex of the colour target (0 RGBA, 1 BGRA, 2 ARGB, 3 ABGR).
int refh_model_render(void* modelHandle, const float* modelToWorld, const float* cameraLocation,
                      int perspective, float slope, float nearClip, float farClip,
                      int width, int height, uint32_t* color, float* depth, int packOrder, int mode) {
	Model& model = ((ModelBox*)modelHandle)->model;
	Transform3D transform = makeTransform(modelToWorld);
	Camera camera = makeCamera(cameraLocation, perspective, slope, width, height, nearClip, farClip);
	ImageRgbaU8 colorImage;
	ImageF32 depthImage;
	if (color) {
		colorImage = image_create_RgbaU8_native(width, height, PackOrderIndex(packOrder));
		copyInRgba(colorImage, color, width, height);
	}
	if (depth) {
		depthImage = image_create_F32(width, height);
		copyInF32(depthImage, depth, width, height);
	}
	if (mode == 0) {
		model_render(model, transform, colorImage, depthImage, camera);
	} else {
		Renderer renderer = renderer_create();
		renderer_begin(renderer, colorImage, depthImage);
		renderer_giveTask(renderer, model, transform, camera);
		renderer_end(renderer);
	}
	if (color) copyOutRgba(colorImage, color, width, height);
	if (depth) copyOutF32(depthImage, depth, width, height);
	return 0;
}

int refh_model_render_depth(void* modelHandle, const float* modelToWorld, const float* cameraLocation,
                            int perspective, float slope, float nearClip, float farClip,
                            int width, int height, float* depth) {
	Model& model = ((ModelBox*)modelHandle)->model;
	Transform3D transform = makeTransform(modelToWorld);
	Camera camera = makeCamera(cameraLocation, perspective, slope, width, height, nearClip, farClip);
	ImageF32 depthImage = image_create_F32(width, height);
	copyInF32(depthImage, depth, width, height);
	model_renderDepth(model, transform, depthImage, camera);
	copyOutF32(depthImage, depth, width, height);
	return 0;
}

// ---- a renderer with the occlusion grid (api/rendererAPI.h:46-135, modelAPI.h:299-301)

namespace {
struct RendererBox {
	Renderer renderer;
	ImageRgbaU8 color;
	ImageF32 depth;
	uint32_t* colorOut = nullptr;
	float* depthOut = nullptr;
	int width = 0, height = 0;
};
struct CameraArgs { const float* location; int perspective; float slope, nearClip, farClip; int width, height; };
Camera makeCamera(const CameraArgs& c) { return makeCamera(c.location, c.perspective, c.slope, c.width, c.height, c.nearClip, c.farClip); }
} // namespace

void* refh_renderer_create() {
	RendererBox* box = new RendererBox();
	box->renderer = renderer_create();
	return box;
}

void refh_renderer_free(void* handle) { delete (RendererBox*)handle; }

// Images are copied in at begin and out at end (color, depth: width x height, either may be null).
void refh_renderer_begin(void* handle, uint32_t* color, float* depth, int width, int height, int packOrder) {
	RendererBox* box = (RendererBox*)handle;
	box->color = ImageRgbaU8();
	box->depth = ImageF32();
	box->colorOut = nullptr;
	box->depthOut = nullptr;
	box->width = width;
	box->height = height;
	if (color) {
		box->color = image_create_RgbaU8_native(width, height, PackOrderIndex(packOrder));
		copyInRgba(box->color, color, width, height);
		box->colorOut = color;
	}
	if (depth) {
		box->depth = image_create_F32(width, height);
		copyInF32(box->depth, depth, width, height);
		box->depthOut = depth;
	}
	renderer_begin(box->renderer, box->color, box->depth);
}

void refh_renderer_give_task(void* handle, void* modelHandle, const float* modelToWorld, const float* cameraLocation,
                             int perspective, float slope, float nearClip, float farClip, int width, int height) {
	RendererBox* box = (RendererBox*)handle;
	CameraArgs c = {cameraLocation, perspective, slope, nearClip, farClip, width, height};
	renderer_giveTask(box->renderer, ((ModelBox*)modelHandle)->model, makeTransform(modelToWorld), makeCamera(c));
}

void refh_renderer_occlude_from_box(void* handle, const float* mn, const float* mx, const float* modelToWorld,
                                    const float* cameraLocation, int perspective, float slope, float nearClip, float farClip,
                                    int width, int height, int debugSilhouette) {
	RendererBox* box = (RendererBox*)handle;
	CameraArgs c = {cameraLocation, perspective, slope, nearClip, farClip, width, height};
	renderer_occludeFromBox(box->renderer, FVector3D(mn[0], mn[1], mn[2]), FVector3D(mx[0], mx[1], mx[2]),
	                        makeTransform(modelToWorld), makeCamera(c), debugSilhouette != 0);
}

// draw_line (api/drawAPI.h) of a packed colour into a width x height RGBA image.
void refh_draw_line(uint32_t* pixels, int width, int height, int x1, int y1, int x2, int y2, uint32_t color) {
	ImageRgbaU8 image = image_create_RgbaU8(width, height);
	copyInRgba(image, pixels, width, height);
	draw_line(image, x1, y1, x2, y2, color);
	copyOutRgba(image, pixels, width, height);
}

// renderer_giveTask_triangle for one triangle: cs 3 x 3, is 3 x 2, flat 3 x 2, colors and texCoords 3 x 4.
void refh_renderer_give_triangle(void* handle, const float* cs, const float* is, const int64_t* flat, const float* colors,
                                 const float* texCoords, void* diffuse, void* light, int filter, const float* cameraLocation,
                                 int perspective, float slope, float nearClip, float farClip, int width, int height) {
	RendererBox* box = (RendererBox*)handle;
	CameraArgs c = {cameraLocation, perspective, slope, nearClip, farClip, width, height};
	ProjectedPoint p[3];
	for (int k = 0; k < 3; k++) {
		p[k] = ProjectedPoint(FVector3D(cs[3 * k], cs[3 * k + 1], cs[3 * k + 2]), FVector2D(is[2 * k], is[2 * k + 1]),
		                      LVector2D(flat[2 * k], flat[2 * k + 1]));
	}
	auto v4 = [](const float* v) { return FVector4D(v[0], v[1], v[2], v[3]); };
	TextureRgbaU8 noTexture;
	renderer_giveTask_triangle(box->renderer, p[0], p[1], p[2], v4(colors), v4(colors + 4), v4(colors + 8), v4(texCoords),
	                           v4(texCoords + 4), v4(texCoords + 8), diffuse ? ((TextureBox*)diffuse)->texture : noTexture,
	                           light ? ((TextureBox*)light)->texture : noTexture, filter ? Filter::Alpha : Filter::Solid,
	                           makeCamera(c));
}

void refh_renderer_occlude_from_existing_triangles(void* handle) {
	renderer_occludeFromExistingTriangles(((RendererBox*)handle)->renderer);
}

void refh_renderer_occlude_from_top_rows(void* handle, const float* cameraLocation, int perspective, float slope,
                                         float nearClip, float farClip, int width, int height) {
	RendererBox* box = (RendererBox*)handle;
	CameraArgs c = {cameraLocation, perspective, slope, nearClip, farClip, width, height};
	renderer_occludeFromTopRows(box->renderer, makeCamera(c));
}

int refh_renderer_is_box_visible(void* handle, const float* mn, const float* mx, const float* modelToWorld,
                                 const float* cameraLocation, int perspective, float slope, float nearClip, float farClip,
                                 int width, int height) {
	RendererBox* box = (RendererBox*)handle;
	CameraArgs c = {cameraLocation, perspective, slope, nearClip, farClip, width, height};
	return renderer_isBoxVisible(box->renderer, FVector3D(mn[0], mn[1], mn[2]), FVector3D(mx[0], mx[1], mx[2]),
	                             makeTransform(modelToWorld), makeCamera(c)) ? 1 : 0;
}

int refh_renderer_has_occluders(void* handle) { return renderer_hasOccluders(((RendererBox*)handle)->renderer) ? 1 : 0; }

// renderer_end, then copies the images out.
void refh_renderer_end(void* handle, int debugWireframe) {
	RendererBox* box = (RendererBox*)handle;
	renderer_end(box->renderer, debugWireframe != 0);
	if (box->colorOut) copyOutRgba(box->color, box->colorOut, box->width, box->height);
	if (box->depthOut) copyOutF32(box->depth, box->depthOut, box->width, box->height);
}

// Projects one camera-space point the way the reference does (Camera::cameraToScreen).
// out = is.x, is.y ; outFlat = flat.x, flat.y
void refh_camera_to_screen(const float* cameraLocation, int perspective, float slope, float nearClip, float farClip,
                           int width, int height, const float* cs, float* outIs, int64_t* outFlat) {
	Camera camera = makeCamera(cameraLocation, perspective, slope, width, height, nearClip, farClip);
	ProjectedPoint p = camera.cameraToScreen(FVector3D(cs[0], cs[1], cs[2]));
	outIs[0] = p.is.x; outIs[1] = p.is.y;
	outFlat[0] = p.flat.x; outFlat[1] = p.flat.y;
}

// Row intervals from the reference's own rasterizer for one triangle given its sub-pixel corners.
// clip = left, top, width, height. Returns the row count (or 0 if outside) and writes startRow.
int refh_triangle_rows(const int64_t* flat, const int* clip, int alignX, int alignY,
                       int* startRow, int* lefts, int* rights, int maxRows) {
	ProjectedPoint a(FVector3D(), FVector2D(), LVector2D(flat[0], flat[1]));
	ProjectedPoint b(FVector3D(), FVector2D(), LVector2D(flat[2], flat[3]));
	ProjectedPoint c(FVector3D(), FVector2D(), LVector2D(flat[4], flat[5]));
	ITriangle2D triangle(a, b, c);
	IRect clipBound(clip[0], clip[1], clip[2], clip[3]);
	int rowCount = triangle.getBufferSize(clipBound, alignX, alignY);
	if (rowCount <= 0 || rowCount > maxRows) return rowCount > maxRows ? -rowCount : 0;
	RowInterval* rows = new RowInterval[rowCount];
	triangle.getShape(*startRow, rows, clipBound, alignX, alignY);
	for (int r = 0; r < rowCount; r++) { lefts[r] = rows[r].left; rights[r] = rows[r].right; }
	delete[] rows;
	return rowCount;
}

} // extern "C"

// ---- deferred light passes and draw_higher (SDK/SpriteEngine/lightAPI.h:27-31, api/drawAPI.h:142-150)

namespace {
void storeMatrix(const FMatrix3x3& m, float* out) {
	out[0] = m.xAxis.x; out[1] = m.xAxis.y; out[2] = m.xAxis.z;
	out[3] = m.yAxis.x; out[4] = m.yAxis.y; out[5] = m.yAxis.z;
	out[6] = m.zAxis.x; out[7] = m.zAxis.y; out[8] = m.zAxis.z;
}
}

extern "C" {

// OrthoSystem(cameraTilt, pixelsPerTile).view[index]: normalToWorldSpace, screenDepthToLightSpace and
// lightSpaceToScreenDepth (27 floats) and pixelOffsetPerTileX, pixelOffsetPerTileZ, yPixelsPerTile (5 ints).
void refh_ortho_view(float cameraTilt, int pixelsPerTile, int index, float* matrices, int* ints) {
	OrthoSystem system(cameraTilt, pixelsPerTile);
	const OrthoView& v = system.view[index];
	storeMatrix(v.normalToWorldSpace, matrices);
	storeMatrix(v.screenDepthToLightSpace, matrices + 9);
	storeMatrix(v.lightSpaceToScreenDepth, matrices + 18);
	ints[0] = v.pixelOffsetPerTileX.x; ints[1] = v.pixelOffsetPerTileX.y;
	ints[2] = v.pixelOffsetPerTileZ.x; ints[3] = v.pixelOffsetPerTileZ.y;
	ints[4] = v.yPixelsPerTile;
}

// The hardware thread count that the reference's threadedSplit plans its row bands with.
int refh_thread_count() { return getThreadCount(); }

// Camera location of a shadow cube side the way PointLight::renderModelShadow builds it
// (SDK/SpriteEngine/spriteAPI.cpp:328-336, 377-381), from the reference's own matrix code.
void refh_shadow_side(const float* normalToWorld, int side, float* location) {
	static const FVector3D forward[6] = {FVector3D(1.0f, 0.0f, 0.0f), FVector3D(-1.0f, 0.0f, 0.0f), FVector3D(0.0f, 1.0f, 0.0f),
	                                     FVector3D(0.0f, -1.0f, 0.0f), FVector3D(0.0f, 0.0f, 1.0f), FVector3D(0.0f, 0.0f, -1.0f)};
	static const FVector3D up[6] = {FVector3D(0.0f, 1.0f, 0.0f), FVector3D(0.0f, 1.0f, 0.0f), FVector3D(0.0f, 0.0f, 1.0f),
	                                FVector3D(0.0f, 0.0f, 1.0f), FVector3D(0.0f, 1.0f, 0.0f), FVector3D(0.0f, 1.0f, 0.0f)};
	FMatrix3x3 n(FVector3D(normalToWorld[0], normalToWorld[1], normalToWorld[2]),
	             FVector3D(normalToWorld[3], normalToWorld[4], normalToWorld[5]),
	             FVector3D(normalToWorld[6], normalToWorld[7], normalToWorld[8]));
	FMatrix3x3 r = FMatrix3x3::makeAxisSystem(forward[side], up[side]) * n;
	location[0] = 0.0f; location[1] = 0.0f; location[2] = 0.0f;
	storeMatrix(r, location + 3);
}

// setDirectedLight (add = 0) / addDirectedLight (add = 1) on width x height RGBA images.
void refh_directed_light(float cameraTilt, int pixelsPerTile, int index, uint32_t* light, const uint32_t* normal,
                         int width, int height, const float* direction, float intensity, const int* color, int add) {
	OrthoSystem system(cameraTilt, pixelsPerTile);
	OrderedImageRgbaU8 lightImage = image_create_RgbaU8(width, height);
	OrderedImageRgbaU8 normalImage = image_create_RgbaU8(width, height);
	copyInRgba(lightImage, light, width, height);
	copyInRgba(normalImage, normal, width, height);
	FVector3D dir(direction[0], direction[1], direction[2]);
	ColorRgbI32 c(color[0], color[1], color[2]);
	if (add) addDirectedLight(system.view[index], lightImage, normalImage, dir, intensity, c);
	else setDirectedLight(system.view[index], lightImage, normalImage, dir, intensity, c);
	copyOutRgba(lightImage, light, width, height);
}

// addPointLight with a shadow cube map (cube != null: cubeWidth x 6 cubeWidth floats) or without.
void refh_point_light(float cameraTilt, int pixelsPerTile, int index, int centerX, int centerY, uint32_t* light,
                      const uint32_t* normal, const float* heightData, int width, int height, const float* position,
                      float radius, float intensity, const int* color, const float* cube, int cubeWidth) {
	OrthoSystem system(cameraTilt, pixelsPerTile);
	OrderedImageRgbaU8 lightImage = image_create_RgbaU8(width, height);
	OrderedImageRgbaU8 normalImage = image_create_RgbaU8(width, height);
	AlignedImageF32 heightImage = image_create_F32(width, height);
	copyInRgba(lightImage, light, width, height);
	copyInRgba(normalImage, normal, width, height);
	copyInF32(heightImage, heightData, width, height);
	FVector3D pos(position[0], position[1], position[2]);
	ColorRgbI32 c(color[0], color[1], color[2]);
	if (cube) {
		AlignedImageF32 cubeImage = image_create_F32(cubeWidth, cubeWidth * 6);
		copyInF32(cubeImage, cube, cubeWidth, cubeWidth * 6);
		addPointLight(system.view[index], IVector2D(centerX, centerY), lightImage, normalImage, heightImage, pos, radius, intensity, c, cubeImage);
	} else {
		addPointLight(system.view[index], IVector2D(centerX, centerY), lightImage, normalImage, heightImage, pos, radius, intensity, c);
	}
	copyOutRgba(lightImage, light, width, height);
}

// blendLight into a target of the given pack order.
void refh_blend_light(uint32_t* target, int targetPackOrder, const uint32_t* diffuse, const uint32_t* light, int width, int height) {
	AlignedImageRgbaU8 targetImage = image_create_RgbaU8_native(width, height, PackOrderIndex(targetPackOrder));
	OrderedImageRgbaU8 diffuseImage = image_create_RgbaU8(width, height);
	OrderedImageRgbaU8 lightImage = image_create_RgbaU8(width, height);
	copyInRgba(diffuseImage, diffuse, width, height);
	copyInRgba(lightImage, light, width, height);
	blendLight(targetImage, diffuseImage, lightImage);
	copyOutRgba(targetImage, target, width, height);
}

// draw_higher(F32 height, two RGBA images) with the given pack orders.
void refh_draw_higher(float* targetHeight, uint32_t* targetA, int targetAPack, uint32_t* targetB, int targetBPack, int tw, int th,
                      const float* sourceHeight, const uint32_t* sourceA, int sourceAPack, const uint32_t* sourceB, int sourceBPack,
                      int sw, int sh, int left, int top, float offset) {
	AlignedImageF32 th_ = image_create_F32(tw, th);
	AlignedImageRgbaU8 ta = image_create_RgbaU8_native(tw, th, PackOrderIndex(targetAPack));
	AlignedImageRgbaU8 tb = image_create_RgbaU8_native(tw, th, PackOrderIndex(targetBPack));
	AlignedImageF32 sh_ = image_create_F32(sw, sh);
	AlignedImageRgbaU8 sa = image_create_RgbaU8_native(sw, sh, PackOrderIndex(sourceAPack));
	AlignedImageRgbaU8 sb = image_create_RgbaU8_native(sw, sh, PackOrderIndex(sourceBPack));
	copyInF32(th_, targetHeight, tw, th); copyInRgba(ta, targetA, tw, th); copyInRgba(tb, targetB, tw, th);
	copyInF32(sh_, sourceHeight, sw, sh); copyInRgba(sa, sourceA, sw, sh); copyInRgba(sb, sourceB, sw, sh);
	ImageF32 targetHeightImage = th_;
	ImageRgbaU8 targetAImage = ta, targetBImage = tb;
	draw_higher(targetHeightImage, sh_, targetAImage, sa, targetBImage, sb, left, top, offset);
	copyOutF32(th_, targetHeight, tw, th); copyOutRgba(ta, targetA, tw, th); copyOutRgba(tb, targetB, tw, th);
}


// One frame of the sprite engine's deferred-light pass through the reference's own functions, on
// images made once: height, diffuse and normal cleared (image_fill), draw_higher of every placement,
// each light's cube map cleared and drawn with model_renderDepth of the caster on its six faces
// (the sub-images of one 6 x res image, as CubeMapF32 and PointLight::renderModelShadow do,
// spriteAPI.cpp:340-401), setDirectedLight, addPointLight per light (threadedSplit over the
// hardware threads, lightAPI.cpp:186) and blendLight (spriteAPI.cpp:770-816).  The frame runs
// `frames` times; returns the seconds of the fastest and leaves its images in the outputs.
//   types: per sprite type w, h; typeHeights / typeDiffuse / typeNormals: per type image pointers
//   placements: per sprite type, left, top and the offset's float bits
//   sun: direction xyz, intensity; lights: per light x, y, z, radius, intensity; lightColors: rgb
double refh_light_frame(float cameraTilt, int pixelsPerTile, int viewIndex, int width, int height, int centerX, int centerY,
                        float backgroundHeight, int typeCount, const int* types, const float* const* typeHeights,
                        const uint32_t* const* typeDiffuse, const uint32_t* const* typeNormals, int placementCount,
                        const int* placements, void* casterHandle, int cubeResolution, const float* sun, const int* sunColor,
                        int lightCount, const float* lights, const int* lightColors, int frames, uint32_t* output, uint32_t* lightOut,
                        float* heightOut, float* cubesOut) {
	OrthoSystem system(cameraTilt, pixelsPerTile);
	const OrthoView& view = system.view[viewIndex];
	Model& caster = ((ModelBox*)casterHandle)->model;
	std::vector<AlignedImageF32> spriteHeights;
	std::vector<OrderedImageRgbaU8> spriteDiffuse, spriteNormals;
	for (int t = 0; t < typeCount; t++) {
		const int w = types[2 * t], h = types[2 * t + 1];
		spriteHeights.push_back(image_create_F32(w, h));
		spriteDiffuse.push_back(image_create_RgbaU8(w, h));
		spriteNormals.push_back(image_create_RgbaU8(w, h));
		copyInF32(spriteHeights.back(), typeHeights[t], w, h);
		copyInRgba(spriteDiffuse.back(), typeDiffuse[t], w, h);
		copyInRgba(spriteNormals.back(), typeNormals[t], w, h);
	}
	AlignedImageF32 heightImage = image_create_F32(width, height);
	OrderedImageRgbaU8 diffuseImage = image_create_RgbaU8(width, height);
	OrderedImageRgbaU8 normalImage = image_create_RgbaU8(width, height);
	OrderedImageRgbaU8 lightImage = image_create_RgbaU8(width, height);
	AlignedImageRgbaU8 outputImage = image_create_RgbaU8_native(width, height, PackOrderIndex::RGBA);
	std::vector<AlignedImageF32> cubes;
	for (int k = 0; k < lightCount; k++) cubes.push_back(image_create_F32(cubeResolution, cubeResolution * 6));
	float normalToWorld[9];
	storeMatrix(view.normalToWorldSpace, normalToWorld);
	double best = 1e30;
	for (int f = 0; f < frames; f++) {
		const double start = time_getSeconds();
		image_fill(heightImage, backgroundHeight);
		image_fill(diffuseImage, ColorRgbaI32(0));
		image_fill(normalImage, ColorRgbaI32(0));
		for (int i = 0; i < placementCount; i++) {
			const int* p = placements + 4 * i;
			float offset;
			std::memcpy(&offset, &p[3], 4);
			ImageF32 targetHeight = heightImage;
			ImageRgbaU8 targetA = diffuseImage, targetB = normalImage;
			draw_higher(targetHeight, spriteHeights[p[0]], targetA, spriteDiffuse[p[0]], targetB, spriteNormals[p[0]], p[1], p[2], offset);
		}
		for (int k = 0; k < lightCount; k++) {
			image_fill(cubes[k], 0.0f);
			const float* l = lights + 5 * k;
			const Transform3D transform(FVector3D(-l[0], -l[1], -l[2]), FMatrix3x3());
			for (int side = 0; side < 6; side++) {
				float location[12];
				refh_shadow_side(normalToWorld, side, location);
				const Camera camera = makeCamera(location, 1, 1.0f, cubeResolution, cubeResolution, 0.01f, 1000.0f);
				ImageF32 face = image_getSubImage(cubes[k], IRect(0, side * cubeResolution, cubeResolution, cubeResolution));
				model_renderDepth(caster, transform, face, camera);
			}
		}
		setDirectedLight(view, lightImage, normalImage, FVector3D(sun[0], sun[1], sun[2]), sun[3],
		                 ColorRgbI32(sunColor[0], sunColor[1], sunColor[2]));
		for (int k = 0; k < lightCount; k++) {
			const float* l = lights + 5 * k;
			addPointLight(view, IVector2D(centerX, centerY), lightImage, normalImage, heightImage, FVector3D(l[0], l[1], l[2]), l[3], l[4],
			              ColorRgbI32(lightColors[3 * k], lightColors[3 * k + 1], lightColors[3 * k + 2]), cubes[k]);
		}
		blendLight(outputImage, diffuseImage, lightImage);
		const double seconds = time_getSeconds() - start;
		if (seconds < best) best = seconds;
	}
	if (output) copyOutRgba(outputImage, output, width, height);
	if (lightOut) copyOutRgba(lightImage, lightOut, width, height);
	if (heightOut) copyOutF32(heightImage, heightOut, width, height);
	for (int k = 0; k < lightCount && cubesOut; k++)
		copyOutF32(cubes[k], cubesOut + (size_t)k * cubeResolution * cubeResolution * 6, cubeResolution, cubeResolution * 6);
	return best;
}

} // extern "C"
