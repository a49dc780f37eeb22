// dsr::gpu: the reference's model and renderer API on the GPU, through the dsrg C ABI.
// Declarations and the contract in dsr_gpu.h.
#include "dsr_gpu.h"

#include <cstring>
#include <unordered_map>
#include <vector>

#include "DFPSR/api/imageAPI.h"
#include "DFPSR/api/textureAPI.h"
#include "dsrg.h"

namespace dsr {
namespace gpu {

namespace {

int32_t g_device = 0;
dsrg_context g_context = nullptr;

// A reference texture on the GPU, keyed by its pyramid buffer; the handle keeps the buffer alive
// (and its address unique) while the copy exists.
struct TextureCopy {
	TextureRgbaU8 texture;
	dsrg_texture gpu = nullptr;
};
std::unordered_map<const void *, TextureCopy> g_textures;

// A reference model on the GPU: one dsrg model per part, keyed by the model's implementation.
struct ModelCopy {
	Model model;
	std::vector<dsrg_model> parts;
};
std::unordered_map<const void *, ModelCopy> g_models;

dsrg_context context() {
	if (!g_context) {
		const int status = dsrg_context_create(g_device, &g_context);
		if (status != DSRG_OK) {
			g_context = nullptr;
			throwError(U"dsr::gpu: no GPU context on device ", g_device, U" (dsrg status ", status, U")\n");
		}
	}
	return g_context;
}

// A failed dsrg call becomes the reference's error: its message through throwError.
void check(int status, const char *call) {
	if (status != DSRG_OK) {
		throwError(String(call), U": ", String(dsrg_context_last_error(g_context)), U"\n");
	}
}

void toArray(const Transform3D &t, float out[12]) {
	const float values[12] = {t.position.x, t.position.y, t.position.z,
	                          t.transform.xAxis.x, t.transform.xAxis.y, t.transform.xAxis.z,
	                          t.transform.yAxis.x, t.transform.yAxis.y, t.transform.yAxis.z,
	                          t.transform.zAxis.x, t.transform.zAxis.y, t.transform.zAxis.z};
	std::memcpy(out, values, sizeof(values));
}

// Camera::createPerspective / createOrthogonal arguments of a camera (Camera.h:144-156).
dsrg_camera toCamera(const Camera &camera) {
	dsrg_camera c;
	std::memset(&c, 0, sizeof(c));
	toArray(camera.location, c.location);
	c.perspective = camera.perspective ? 1 : 0;
	c.slope = camera.widthSlope; // halfWidth of an orthogonal camera
	c.nearClip = camera.nearClip;
	c.farClip = camera.farClip;
	c.width = (int32_t)camera.imageWidth;
	c.height = (int32_t)camera.imageHeight;
	return c;
}

// An image of the reference as a dsrg_image in host memory (any stride, any start offset).
dsrg_image toImage(const ImageRgbaU8 &image) {
	dsrg_image g;
	std::memset(&g, 0, sizeof(g));
	g.data = image_getSafePointer<uint32_t>(image, 0).getUnsafe();
	g.width = image_getWidth(image);
	g.height = image_getHeight(image);
	g.strideBytes = image_getStride(image);
	g.packOrder = (int32_t)image_getPackOrderIndex(image);
	g.onDevice = 0;
	return g;
}
dsrg_image toImage(const ImageF32 &image) {
	dsrg_image g;
	std::memset(&g, 0, sizeof(g));
	g.data = image_getSafePointer<float>(image, 0).getUnsafe();
	g.width = image_getWidth(image);
	g.height = image_getHeight(image);
	g.strideBytes = image_getStride(image);
	g.packOrder = 0;
	g.onDevice = 0;
	return g;
}

// The GPU copy of a texture (null for a texture that does not exist).
dsrg_texture toTexture(const TextureRgbaU8 &texture) {
	if (!texture_exists(texture)) return nullptr;
	const void *key = texture.impl_buffer.getUnsafe();
	auto found = g_textures.find(key);
	if (found != g_textures.end()) return found->second.gpu;
	TextureCopy copy;
	copy.texture = texture;
	const uint32_t *pyramid = texture.impl_buffer.getSafe<uint32_t>("dsr::gpu texture upload").getUnsafe();
	check(dsrg_texture_upload(context(), pyramid, texture.impl_log2width, texture.impl_log2height, texture.impl_maxMipLevel,
	                          &copy.gpu), "texture upload");
	g_textures[key] = copy;
	return copy.gpu;
}

// The GPU copy of a model: its points (all of them, for every part), each part's polygons in
// order, the model's bounding box and filter (Model.h:54-64, modelAPI.h:62-258).
const std::vector<dsrg_model> &toModel(const Model &model) {
	const void *key = model.getUnsafe();
	auto found = g_models.find(key);
	if (found != g_models.end()) return found->second.parts;
	ModelCopy copy;
	copy.model = model;
	const int32_t pointCount = model_getNumberOfPoints(model);
	std::vector<float> positions((size_t)pointCount * 3);
	for (int32_t p = 0; p < pointCount; p++) {
		const FVector3D v = model_getPoint(model, p);
		positions[(size_t)p * 3] = v.x;
		positions[(size_t)p * 3 + 1] = v.y;
		positions[(size_t)p * 3 + 2] = v.z;
	}
	FVector3D minimum, maximum;
	model_getBoundingBox(model, minimum, maximum);
	const float lo[3] = {minimum.x, minimum.y, minimum.z}, hi[3] = {maximum.x, maximum.y, maximum.z};
	const int32_t filter = model_getFilter(model) == Filter::Alpha ? DSRG_FILTER_ALPHA : DSRG_FILTER_SOLID;
	Model editable = model; // model_getLightMap takes a non-const handle
	const int32_t partCount = model_getNumberOfParts(model);
	for (int32_t part = 0; part < partCount; part++) {
		const int32_t polygonCount = model_getNumberOfPolygons(model, part);
		std::vector<int32_t> indices((size_t)polygonCount * 4, -1);
		std::vector<float> texCoords((size_t)polygonCount * 16, 0.0f), colors((size_t)polygonCount * 16, 0.0f);
		for (int32_t polygon = 0; polygon < polygonCount; polygon++) {
			const int32_t corners = model_getPolygonVertexCount(model, part, polygon);
			for (int32_t k = 0; k < corners && k < 4; k++) {
				indices[(size_t)polygon * 4 + k] = model_getVertexPointIndex(model, part, polygon, k);
				const FVector4D uv = model_getTexCoord(model, part, polygon, k);
				const FVector4D rgba = model_getVertexColor(model, part, polygon, k);
				float *t = &texCoords[((size_t)polygon * 4 + k) * 4];
				float *c = &colors[((size_t)polygon * 4 + k) * 4];
				t[0] = uv.x; t[1] = uv.y; t[2] = uv.z; t[3] = uv.w;
				c[0] = rgba.x; c[1] = rgba.y; c[2] = rgba.z; c[3] = rgba.w;
			}
		}
		const dsrg_texture diffuse = toTexture(model_getDiffuseMap(model, part));
		const dsrg_texture light = toTexture(model_getLightMap(editable, part));
		dsrg_model m = nullptr;
		check(dsrg_model_create(context(), positions.data(), pointCount, indices.data(), texCoords.data(), colors.data(),
		                        polygonCount, diffuse, light, filter, &m), "model upload");
		copy.parts.push_back(m);
		check(dsrg_model_set_bound(m, lo, hi), "model upload");
	}
	return g_models.emplace(key, copy).first->second.parts;
}

} // namespace

struct RendererImpl {
	dsrg_renderer renderer = nullptr;
	ImageRgbaU8 color; // the images given to renderer_begin, returned by renderer_get*Buffer until renderer_end
	ImageF32 depth;
	~RendererImpl() {
		if (renderer) dsrg_renderer_destroy(renderer);
	}
};

void setDevice(int32_t device) { g_device = device; }

void model_forget(const Model &model) {
	auto found = g_models.find(model.getUnsafe());
	if (found == g_models.end()) return;
	for (dsrg_model m : found->second.parts) dsrg_model_destroy(m);
	g_models.erase(found);
}

void texture_forget(const TextureRgbaU8 &texture) {
	if (!texture_exists(texture)) return;
	auto found = g_textures.find(texture.impl_buffer.getUnsafe());
	if (found == g_textures.end()) return;
	dsrg_texture_destroy(found->second.gpu);
	g_textures.erase(found);
}

void forget_all() {
	for (auto &entry : g_models)
		for (dsrg_model m : entry.second.parts) dsrg_model_destroy(m);
	g_models.clear();
	for (auto &entry : g_textures) dsrg_texture_destroy(entry.second.gpu);
	g_textures.clear();
	if (g_context) dsrg_context_destroy(g_context);
	g_context = nullptr;
}

void model_render(const Model &model, const Transform3D &modelToWorldTransform, ImageRgbaU8 &colorBuffer, ImageF32 &depthBuffer,
                  const Camera &camera) {
	if (model.isNull()) return; // an empty model handle is skipped silently (modelAPI.cpp:197-201)
	const std::vector<dsrg_model> &parts = toModel(model);
	float transform[12];
	toArray(modelToWorldTransform, transform);
	const dsrg_camera cam = toCamera(camera);
	const bool hasColor = image_exists(colorBuffer), hasDepth = image_exists(depthBuffer);
	const dsrg_image color = hasColor ? toImage(colorBuffer) : dsrg_image(), depth = hasDepth ? toImage(depthBuffer) : dsrg_image();
	for (dsrg_model m : parts)
		check(dsrg_model_render(context(), m, transform, &cam, hasColor ? &color : nullptr, hasDepth ? &depth : nullptr), "model_render");
}

void model_renderDepth(const Model &model, const Transform3D &modelToWorldTransform, ImageF32 &depthBuffer, const Camera &camera) {
	if (model.isNull() || !image_exists(depthBuffer)) return;
	const std::vector<dsrg_model> &parts = toModel(model);
	float transform[12];
	toArray(modelToWorldTransform, transform);
	const dsrg_camera cam = toCamera(camera);
	const dsrg_image depth = toImage(depthBuffer);
	for (dsrg_model m : parts) check(dsrg_model_render_depth(context(), m, transform, &cam, &depth), "model_renderDepth");
}

Renderer renderer_create() {
	Renderer r = std::make_shared<RendererImpl>();
	check(dsrg_renderer_create(context(), &r->renderer), "renderer_create");
	return r;
}

bool renderer_exists(const Renderer &renderer) { return renderer != nullptr; }

static RendererImpl &existing(const Renderer &renderer, const char *call) {
	if (!renderer) throwError(U"", String(call), U": the renderer does not exist!\n"); // MUST_EXIST (rendererAPI.cpp:32)
	return *renderer;
}

void renderer_begin(Renderer &renderer, ImageRgbaU8 &colorBuffer, ImageF32 &depthBuffer) {
	RendererImpl &r = existing(renderer, "renderer_begin");
	const bool hasColor = image_exists(colorBuffer), hasDepth = image_exists(depthBuffer);
	const dsrg_image color = hasColor ? toImage(colorBuffer) : dsrg_image(), depth = hasDepth ? toImage(depthBuffer) : dsrg_image();
	check(dsrg_renderer_begin(r.renderer, hasColor ? &color : nullptr, hasDepth ? &depth : nullptr), "renderer_begin");
	r.color = colorBuffer;
	r.depth = depthBuffer;
}

ImageRgbaU8 renderer_getColorBuffer(const Renderer &renderer) { return existing(renderer, "renderer_getColorBuffer").color; }
ImageF32 renderer_getDepthBuffer(const Renderer &renderer) { return existing(renderer, "renderer_getDepthBuffer").depth; }

bool renderer_takesTriangles(const Renderer &renderer) {
	return dsrg_renderer_takes_triangles(existing(renderer, "renderer_takesTriangles").renderer) == 1;
}

void renderer_occludeFromBox(Renderer &renderer, const FVector3D &minimum, const FVector3D &maximum,
                             const Transform3D &modelToWorldTransform, const Camera &camera, bool debugSilhouette) {
	RendererImpl &r = existing(renderer, "renderer_occludeFromBox");
	const float lo[3] = {minimum.x, minimum.y, minimum.z}, hi[3] = {maximum.x, maximum.y, maximum.z};
	float transform[12];
	toArray(modelToWorldTransform, transform);
	const dsrg_camera cam = toCamera(camera);
	check(dsrg_renderer_occlude_from_box(r.renderer, lo, hi, transform, &cam, debugSilhouette ? 1 : 0), "renderer_occludeFromBox");
}

void renderer_occludeFromTopRows(Renderer &renderer, const Camera &camera) {
	RendererImpl &r = existing(renderer, "renderer_occludeFromTopRows");
	const dsrg_camera cam = toCamera(camera);
	check(dsrg_renderer_occlude_from_top_rows(r.renderer, &cam), "renderer_occludeFromTopRows");
}

bool renderer_hasOccluders(const Renderer &renderer) {
	return dsrg_renderer_has_occluders(existing(renderer, "renderer_hasOccluders").renderer) == 1;
}

bool renderer_isBoxVisible(const Renderer &renderer, const FVector3D &minimum, const FVector3D &maximum,
                           const Transform3D &modelToWorldTransform, const Camera &camera) {
	RendererImpl &r = existing(renderer, "renderer_isBoxVisible");
	const float lo[3] = {minimum.x, minimum.y, minimum.z}, hi[3] = {maximum.x, maximum.y, maximum.z};
	float transform[12];
	toArray(modelToWorldTransform, transform);
	const dsrg_camera cam = toCamera(camera);
	int32_t visible = 1;
	check(dsrg_renderer_is_box_visible(r.renderer, lo, hi, transform, &cam, &visible), "renderer_isBoxVisible");
	return visible != 0;
}

void renderer_giveTask_triangle(Renderer &renderer,
  const ProjectedPoint &posA, const ProjectedPoint &posB, const ProjectedPoint &posC,
  const FVector4D &colorA, const FVector4D &colorB, const FVector4D &colorC,
  const FVector4D &texCoordA, const FVector4D &texCoordB, const FVector4D &texCoordC,
  const TextureRgbaU8 &diffuseMap, const TextureRgbaU8 &lightMap,
  Filter filter, const Camera &camera) {
	RendererImpl &r = existing(renderer, "renderer_giveTask_triangle");
	const ProjectedPoint *points[3] = {&posA, &posB, &posC};
	const FVector4D *colors[3] = {&colorA, &colorB, &colorC}, *coords[3] = {&texCoordA, &texCoordB, &texCoordC};
	dsrg_projected_point corners[3];
	float colorValues[12], coordValues[12];
	for (int k = 0; k < 3; k++) {
		const ProjectedPoint &p = *points[k];
		corners[k].cs[0] = p.cs.x; corners[k].cs[1] = p.cs.y; corners[k].cs[2] = p.cs.z;
		corners[k].is[0] = p.is.x; corners[k].is[1] = p.is.y;
		corners[k].flat[0] = p.flat.x; corners[k].flat[1] = p.flat.y;
		colorValues[k * 4] = colors[k]->x; colorValues[k * 4 + 1] = colors[k]->y;
		colorValues[k * 4 + 2] = colors[k]->z; colorValues[k * 4 + 3] = colors[k]->w;
		coordValues[k * 4] = coords[k]->x; coordValues[k * 4 + 1] = coords[k]->y;
		coordValues[k * 4 + 2] = coords[k]->z; coordValues[k * 4 + 3] = coords[k]->w;
	}
	const dsrg_camera cam = toCamera(camera);
	check(dsrg_renderer_give_triangles(r.renderer, 1, corners, colorValues, coordValues, toTexture(diffuseMap), toTexture(lightMap),
	                                   filter == Filter::Alpha ? DSRG_FILTER_ALPHA : DSRG_FILTER_SOLID, &cam),
	      "renderer_giveTask_triangle");
}

void renderer_occludeFromExistingTriangles(Renderer &renderer) {
	check(dsrg_renderer_occlude_from_existing_triangles(existing(renderer, "renderer_occludeFromExistingTriangles").renderer),
	      "renderer_occludeFromExistingTriangles");
}

void renderer_end(Renderer &renderer, bool debugWireframe) {
	RendererImpl &r = existing(renderer, "renderer_end");
	check(dsrg_renderer_end_debug(r.renderer, debugWireframe ? 1 : 0), "renderer_end");
	r.color = ImageRgbaU8();
	r.depth = ImageF32();
}

void model_render_threaded(const Model &model, const Transform3D &modelToWorldTransform, Renderer &renderer, const Camera &camera) {
	RendererImpl &r = existing(renderer, "renderer_giveTask");
	if (model.isNull()) return; // skipped silently (modelAPI.cpp:214-222)
	const std::vector<dsrg_model> &parts = toModel(model);
	float transform[12];
	toArray(modelToWorldTransform, transform);
	const dsrg_camera cam = toCamera(camera);
	// every part carries the whole model's bounding box, so the culling and occlusion tests that the
	// reference makes once per model give each part the same answer
	for (dsrg_model m : parts) check(dsrg_renderer_give_task(r.renderer, m, transform, &cam), "renderer_giveTask");
}

void renderer_giveTask(Renderer &renderer, const Model &model, const Transform3D &modelToWorldTransform, const Camera &camera) {
	model_render_threaded(model, modelToWorldTransform, renderer, camera);
}

}
}
