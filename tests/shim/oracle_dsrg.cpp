// A test double of libdsrg.so: the dsrg C ABI entry points that dsr::gpu calls, answered by the
// CPU oracle (oracle/dsr_oracle.c) instead of the GPU.  Test infrastructure only: it lets a CPU
// test drive the compiled dsr::gpu shim with the reference's own models and images and compare
// the result with the reference's own renderer, which shows that the shim hands the C ABI what
// the reference holds (the GPU behind the same ABI is held to the oracle by the GPU tests).
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "dsrg.h"
#include "dsr_oracle.h"

struct dsrg_context_s {
	std::string lastError;
};
struct dsrg_texture_s {
	or_texture texture;
};
struct dsrg_model_s {
	std::vector<float> positions, texCoords, colors;
	std::vector<int32_t> polygons;
	dsrg_texture diffuse = nullptr, light = nullptr;
	int32_t filter = 0;
	or_model model() const {
		or_model m;
		m.positions = positions.data();
		m.pointCount = (int32_t)(positions.size() / 3);
		m.polyIndices = polygons.data();
		m.texCoords = texCoords.data();
		m.colors = colors.data();
		m.polyCount = (int32_t)(polygons.size() / 4);
		m.diffuse = diffuse ? &diffuse->texture : nullptr;
		m.light = light ? &light->texture : nullptr;
		m.filter = filter;
		return m;
	}
};

namespace {

or_camera_desc camera_of(const dsrg_camera *c) {
	or_camera_desc d;
	std::memcpy(d.location, c->location, sizeof(d.location));
	d.perspective = c->perspective;
	d.slope = c->slope;
	d.nearClip = c->nearClip;
	d.farClip = c->farClip;
	d.width = c->width;
	d.height = c->height;
	return d;
}

// A caller's image (any stride) as a dense copy the oracle draws into, written back afterwards.
template <typename T>
struct Dense {
	const dsrg_image *image = nullptr;
	std::vector<T> pixels;
	void load(const dsrg_image *im) {
		image = im;
		if (!im) return;
		pixels.resize((size_t)im->width * im->height);
		for (int32_t y = 0; y < im->height; y++)
			std::memcpy(&pixels[(size_t)y * im->width], (const char *)im->data + (size_t)y * im->strideBytes, sizeof(T) * im->width);
	}
	void store() const {
		if (!image) return;
		for (int32_t y = 0; y < image->height; y++)
			std::memcpy((char *)image->data + (size_t)y * image->strideBytes, &pixels[(size_t)y * image->width], sizeof(T) * image->width);
	}
	T *data() { return image ? pixels.data() : nullptr; }
};

int fail(dsrg_context ctx, int status, const char *message) {
	if (ctx) ctx->lastError = message;
	return status;
}

} // namespace

struct dsrg_renderer_s {
	dsrg_context context;
	or_renderer *renderer;
	dsrg_image colorImage, depthImage;
	bool hasColor = false, hasDepth = false;
	Dense<uint32_t> color;
	Dense<float> depth;
	bool receiving = false;
};

extern "C" {

int dsrg_context_create(int32_t, dsrg_context *out) {
	*out = new dsrg_context_s();
	return DSRG_OK;
}
int dsrg_context_destroy(dsrg_context ctx) {
	delete ctx;
	return DSRG_OK;
}
const char *dsrg_context_last_error(dsrg_context ctx) { return ctx ? ctx->lastError.c_str() : "null context"; }

int dsrg_texture_upload(dsrg_context ctx, const uint32_t *pyramid, uint32_t log2width, uint32_t log2height, uint32_t maxMipLevel,
                        dsrg_texture *out) {
	dsrg_texture t = new dsrg_texture_s();
	if (or_texture_init_empty(&t->texture, log2width, log2height, maxMipLevel) != 0) {
		delete t;
		return fail(ctx, DSRG_ERROR_INVALID_ARGUMENT, "dsrg_texture_upload: invalid pyramid dimensions");
	}
	std::memcpy(t->texture.pixels, pyramid, sizeof(uint32_t) * t->texture.pixelCount);
	*out = t;
	return DSRG_OK;
}
int dsrg_texture_destroy(dsrg_texture t) {
	or_texture_free(&t->texture);
	delete t;
	return DSRG_OK;
}

int dsrg_model_create(dsrg_context, const float *positions, int32_t pointCount, const int32_t *polygonIndices, const float *texCoords,
                      const float *colors, int32_t polygonCount, dsrg_texture diffuse, dsrg_texture light, int32_t filter,
                      dsrg_model *out) {
	dsrg_model m = new dsrg_model_s();
	m->positions.assign(positions, positions + (size_t)pointCount * 3);
	m->polygons.assign(polygonIndices, polygonIndices + (size_t)polygonCount * 4);
	m->texCoords.assign(texCoords, texCoords + (size_t)polygonCount * 16);
	m->colors.assign(colors, colors + (size_t)polygonCount * 16);
	m->diffuse = diffuse;
	m->light = light;
	m->filter = filter;
	*out = m;
	return DSRG_OK;
}
int dsrg_model_set_bound(dsrg_model, const float *, const float *) { return DSRG_OK; } // the oracle bounds the points itself
int dsrg_model_destroy(dsrg_model m) {
	delete m;
	return DSRG_OK;
}

int dsrg_model_render(dsrg_context, dsrg_model m, const float *modelToWorld, const dsrg_camera *camera, const dsrg_image *color,
                      const dsrg_image *depth) {
	Dense<uint32_t> c;
	Dense<float> d;
	c.load(color);
	d.load(depth);
	const or_model model = m->model();
	const or_camera_desc cam = camera_of(camera);
	or_model_render(&model, modelToWorld, &cam, c.data(), d.data(), color ? color->packOrder : 0, 1, 1, nullptr);
	c.store();
	d.store();
	return DSRG_OK;
}

int dsrg_model_render_depth(dsrg_context, dsrg_model m, const float *modelToWorld, const dsrg_camera *camera, const dsrg_image *depth) {
	Dense<float> d;
	d.load(depth);
	const or_model model = m->model();
	const or_camera_desc cam = camera_of(camera);
	or_model_render_depth(&model, modelToWorld, &cam, d.data(), nullptr);
	d.store();
	return DSRG_OK;
}

int dsrg_renderer_create(dsrg_context ctx, dsrg_renderer *out) {
	dsrg_renderer r = new dsrg_renderer_s();
	r->context = ctx;
	r->renderer = or_renderer_create();
	*out = r;
	return DSRG_OK;
}
int dsrg_renderer_destroy(dsrg_renderer r) {
	or_renderer_destroy(r->renderer);
	delete r;
	return DSRG_OK;
}
int dsrg_renderer_begin(dsrg_renderer r, const dsrg_image *color, const dsrg_image *depth) {
	if (r->receiving)
		return fail(r->context, DSRG_ERROR_CALL_ORDER, "Called renderer_begin on the same renderer twice without ending the previous batch!");
	r->hasColor = color != nullptr;
	r->hasDepth = depth != nullptr;
	if (color) r->colorImage = *color;
	if (depth) r->depthImage = *depth;
	r->color.load(color ? &r->colorImage : nullptr);
	r->depth.load(depth ? &r->depthImage : nullptr);
	const dsrg_image *any = color ? color : depth;
	or_renderer_begin(r->renderer, r->color.data(), r->depth.data(), any ? any->width : 0, any ? any->height : 0, color ? color->packOrder : 0);
	r->receiving = true;
	return DSRG_OK;
}
int dsrg_renderer_give_task(dsrg_renderer r, dsrg_model m, const float *modelToWorld, const dsrg_camera *camera) {
	const or_model model = m->model();
	const or_camera_desc cam = camera_of(camera);
	or_renderer_give_task(r->renderer, &model, modelToWorld, &cam);
	return DSRG_OK;
}
int dsrg_renderer_give_triangles(dsrg_renderer r, int32_t count, const dsrg_projected_point *corners, const float *colors,
                                 const float *texCoords, dsrg_texture diffuse, dsrg_texture light, int32_t filter,
                                 const dsrg_camera *camera) {
	const or_camera_desc cam = camera_of(camera);
	for (int32_t i = 0; i < count; i++) {
		float cs[9], is[6];
		int64_t flat[6];
		for (int k = 0; k < 3; k++) {
			const dsrg_projected_point &p = corners[3 * i + k];
			std::memcpy(cs + 3 * k, p.cs, sizeof(p.cs));
			std::memcpy(is + 2 * k, p.is, sizeof(p.is));
			std::memcpy(flat + 2 * k, p.flat, sizeof(p.flat));
		}
		or_renderer_give_triangle(r->renderer, cs, is, flat, colors + 12 * i, texCoords + 12 * i, diffuse ? &diffuse->texture : nullptr,
		                          light ? &light->texture : nullptr, filter, &cam);
	}
	return DSRG_OK;
}
int dsrg_renderer_end_debug(dsrg_renderer r, int32_t debugWireframe) {
	if (!r->receiving) return fail(r->context, DSRG_ERROR_CALL_ORDER, "Called renderer_end without renderer_begin!");
	or_renderer_end(r->renderer, nullptr, debugWireframe);
	r->color.store();
	r->depth.store();
	r->color = Dense<uint32_t>();
	r->depth = Dense<float>();
	r->hasColor = r->hasDepth = false;
	r->receiving = false;
	return DSRG_OK;
}
int dsrg_renderer_end(dsrg_renderer r) { return dsrg_renderer_end_debug(r, 0); }
int dsrg_renderer_takes_triangles(dsrg_renderer r) { return r->receiving ? 1 : 0; }
int dsrg_renderer_occlude_from_box(dsrg_renderer r, const float *mn, const float *mx, const float *modelToWorld, const dsrg_camera *camera,
                                   int32_t debugSilhouette) {
	const or_camera_desc cam = camera_of(camera);
	or_renderer_occlude_from_box(r->renderer, mn, mx, modelToWorld, &cam, debugSilhouette);
	return DSRG_OK;
}
int dsrg_renderer_occlude_from_existing_triangles(dsrg_renderer r) {
	or_renderer_occlude_from_existing_triangles(r->renderer);
	return DSRG_OK;
}
int dsrg_renderer_occlude_from_top_rows(dsrg_renderer r, const dsrg_camera *camera) {
	or_renderer_occlude_from_top_rows(r->renderer, camera->perspective);
	return DSRG_OK;
}
int dsrg_renderer_is_box_visible(dsrg_renderer r, const float *mn, const float *mx, const float *modelToWorld, const dsrg_camera *camera,
                                 int32_t *visible) {
	const or_camera_desc cam = camera_of(camera);
	*visible = or_renderer_is_box_visible(r->renderer, mn, mx, modelToWorld, &cam);
	return DSRG_OK;
}
int dsrg_renderer_has_occluders(dsrg_renderer r) { return or_renderer_has_occluders(r->renderer); }

} // extern "C"
