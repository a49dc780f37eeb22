// The renderer's occlusion grid (RendererImpl, api/rendererAPI.cpp:141-477) behind the C ABI.
//
// Box occluders and box tests are a few corners each and run on the host, on the grid's host
// copy, with the same float and integer operations as the reference.  The per-command work runs
// on the device: occludeFromExistingTriangles is a triangle-setup pass whose commands lower the
// grid with an atomic minimum, occludeFromTopRows one thread per cell, and completeOcclusion is a
// test inside the triangle setup of renderer_end, so occluded commands never become records.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <vector>

#include "dsrg_internal.h"
#include "dsrg_occlusion.h"

using namespace dsrg;

namespace {

size_t grid_cells(dsrg_renderer r) { return (size_t)r->gridAllocWidth * r->gridAllocHeight; }

// prepareForOcclusion (rendererAPI.cpp:181-191): the first occluder of a frame starts from an
// infinitely far grid, reallocated only when the frame needs more cells than it holds.
void prepare_for_occlusion(dsrg_renderer r) {
	if (!r->occluded) {
		if (!(grid_cells(r) > 0 && r->gridAllocWidth >= r->gridWidth && r->gridAllocHeight >= r->gridHeight)) {
			r->gridAllocWidth = r->gridWidth;
			r->gridAllocHeight = r->gridHeight;
		}
		r->gridHost.assign(grid_cells(r), INFINITY);
		r->gridHostValid = true;
		r->gridDeviceValid = false;
	}
	r->occluded = true;
}

// image_readPixel_clamp (api/imageAPI.h:276-282) of the grid image: 0 while no grid exists, and
// clamped to the allocated grid, which may be another frame's.
float grid_read(dsrg_renderer r, int32_t x, int32_t y) {
	if (grid_cells(r) == 0) return 0.0f;
	if (x < 0) x = 0;
	if (y < 0) y = 0;
	if (x > r->gridAllocWidth - 1) x = r->gridAllocWidth - 1;
	if (y > r->gridAllocHeight - 1) y = r->gridAllocHeight - 1;
	return r->gridHost[(size_t)y * r->gridAllocWidth + x];
}

int grid_on_host(dsrg_renderer r) {
	if (r->gridHostValid) return DSRG_OK;
	dsrg_context ctx = r->context;
	r->gridHost.resize(grid_cells(r));
	if (!r->gridHost.empty()) {
		DSRG_CUDA_TRY(ctx, cudaMemcpyAsync(r->gridHost.data(), r->gridDevice.ptr, r->gridHost.size() * sizeof(float),
		                                   cudaMemcpyDeviceToHost, ctx->stream));
		DSRG_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
	}
	r->gridHostValid = true;
	return DSRG_OK;
}

struct Hull {
	int64_t x[8], y[8];
	float z[8];
	int32_t count;
};

// getPixelBoundFromProjection (rendererAPI.cpp:92-98) as exclusive bounds.
void pixel_bound(const int64_t *x, const int64_t *y, int32_t count, int32_t *bound) {
	bound[0] = (int32_t)(x[0] / 256); bound[1] = (int32_t)(y[0] / 256);
	bound[2] = bound[0] + 1; bound[3] = bound[1] + 1;
	for (int32_t p = 1; p < count; p++) {
		const int32_t px = (int32_t)(x[p] / 256), py = (int32_t)(y[p] / 256);
		if (px < bound[0]) bound[0] = px;
		if (py < bound[1]) bound[1] = py;
		if (px + 1 > bound[2]) bound[2] = px + 1;
		if (py + 1 > bound[3]) bound[3] = py + 1;
	}
}

// jarvisConvexHullAlgorithm (rendererAPI.cpp:38-72).
bool counter_clockwise(const Projected &p, const Projected &q, const Projected &s) {
	return (q.flaty - p.flaty) * (s.flatx - q.flatx) - (q.flatx - p.flatx) * (s.flaty - q.flaty) < 0;
}
void convex_hull(const Projected *in, int32_t n, Hull &out) {
	out.count = 0;
	if (n < 3) {
		for (int32_t p = 0; p < n; p++) { out.x[p] = in[p].flatx; out.y[p] = in[p].flaty; out.z[p] = in[p].cs.z; }
		out.count = n;
		return;
	}
	int32_t l = 0;
	for (int32_t i = 1; i < n; i++) if (in[i].flatx < in[l].flatx) l = i;
	int32_t p = l;
	do {
		if (out.count >= n) return;
		out.x[out.count] = in[p].flatx; out.y[out.count] = in[p].flaty; out.z[out.count] = in[p].cs.z;
		out.count++;
		int32_t q = (p + 1) % n;
		for (int32_t i = 0; i < n; i++) if (counter_clockwise(in[p], in[i], in[q])) q = i;
		p = q;
	} while (p != l);
}

// GENERATE_BOX_CORNERS (rendererAPI.cpp:257-265).
void box_corners(const float *mn, const float *mx, Vec3 *out) {
	out[0] = vec3(mn[0], mn[1], mn[2]); out[1] = vec3(mn[0], mn[1], mx[2]);
	out[2] = vec3(mn[0], mx[1], mn[2]); out[3] = vec3(mn[0], mx[1], mx[2]);
	out[4] = vec3(mx[0], mn[1], mn[2]); out[5] = vec3(mx[0], mn[1], mx[2]);
	out[6] = vec3(mx[0], mx[1], mn[2]); out[7] = vec3(mx[0], mx[1], mx[2]);
}

// occludeFromSortedHull (rendererAPI.cpp:216-239) on the host copy.
void occlude_from_hull(dsrg_renderer r, const Hull &h) {
	int32_t bound[4];
	pixel_bound(h.x, h.y, h.count, bound);
	if (!((bound[2] - bound[0]) > OCCLUSION_CELL && (bound[3] - bound[1]) > OCCLUSION_CELL)) return;
	float distance = 0.0f;
	for (int32_t c = 0; c < h.count; c++) if (h.z[c] > distance) distance = h.z[c];
	const CellRect cells = outer_cell_bound(bound[0], bound[1], bound[2], bound[3], r->gridWidth, r->gridHeight);
	for (int32_t cy = cells.top; cy < cells.bottom; cy++) {
		for (int32_t cx = cells.left; cx < cells.right; cx++) {
			if (!cell_inside_hull(h.x, h.y, h.count, cx, cy)) continue;
			if (distance < grid_read(r, cx, cy)) r->gridHost[(size_t)cy * r->gridAllocWidth + cx] = distance;
		}
	}
}

} // namespace

int renderer_grid_on_device(dsrg_renderer r) {
	if (r->gridDeviceValid) return DSRG_OK;
	dsrg_context ctx = r->context;
	const size_t cells = grid_cells(r);
	DSRG_CUDA_TRY(ctx, r->gridDevice.reserve(cells + 1));
	if (cells) {
		r->gridHost.resize(cells, INFINITY);
		DSRG_CUDA_TRY(ctx, cudaMemcpyAsync(r->gridDevice.ptr, r->gridHost.data(), cells * sizeof(float), cudaMemcpyHostToDevice,
		                                   ctx->stream));
		DSRG_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream)); // the host copy may change right after
	}
	r->gridDeviceValid = true;
	return DSRG_OK;
}

int renderer_box_occluded(dsrg_renderer r, const float *minimum, const float *maximum, const float *modelToWorld,
                          const CameraData &camera, bool *occluded) {
	const int s = grid_on_host(r);
	if (s != DSRG_OK) return s;
	// isHullOccluded (rendererAPI.cpp:297-330)
	Vec3 local[8], cs[8];
	Projected proj[8];
	box_corners(minimum, maximum, local);
	for (int p = 0; p < 8; p++) {
		cs[p] = world_to_camera(camera, transform_point(modelToWorld, local[p]));
		proj[p] = camera_to_screen(camera, cs[p]);
	}
	for (int32_t s2 = 0; s2 < camera.cullCount; s2++) {
		bool allOutside = true;
		for (int p = 0; p < 8; p++) {
			if (plane_inside(camera.cull[s2], cs[p])) { allOutside = false; break; }
		}
		if (allOutside) { *occluded = true; return DSRG_OK; }
	}
	int64_t x[8], y[8];
	float closest = INFINITY;
	for (int p = 0; p < 8; p++) {
		x[p] = proj[p].flatx; y[p] = proj[p].flaty;
		if (proj[p].cs.z < closest) closest = proj[p].cs.z;
	}
	int32_t bound[4];
	pixel_bound(x, y, 8, bound);
	const CellRect cells = outer_cell_bound(bound[0], bound[1], bound[2], bound[3], r->gridWidth, r->gridHeight);
	for (int32_t cy = cells.top; cy < cells.bottom; cy++) {
		for (int32_t cx = cells.left; cx < cells.right; cx++) {
			if (closest < grid_read(r, cx, cy)) { *occluded = false; return DSRG_OK; }
		}
	}
	*occluded = true;
	return DSRG_OK;
}

extern "C" {

int dsrg_renderer_occlude_from_box(dsrg_renderer r, const float *minimum, const float *maximum, const float *modelToWorld,
                                   const dsrg_camera *camera, int32_t debugSilhouette) {
	if (!r) return DSRG_ERROR_INVALID_ARGUMENT;
	dsrg_context ctx = r->context;
	if (!r->receiving) return fail(ctx, DSRG_ERROR_CALL_ORDER, "Cannot call renderer_occludeFromBox without first calling renderer_begin!");
	if (!minimum || !maximum || !modelToWorld || !camera)
		return fail(ctx, DSRG_ERROR_INVALID_ARGUMENT, "renderer_occludeFromBox: null argument");
	prepare_for_occlusion(r);
	int s = grid_on_host(r);
	if (s != DSRG_OK) return s;
	const CameraData cam = make_camera(*camera);
	Vec3 local[8];
	Projected proj[8];
	box_corners(minimum, maximum, local);
	for (int p = 0; p < 8; p++) { // projectHull (rendererAPI.cpp:76-90)
		const Vec3 cs = world_to_camera(cam, transform_point(modelToWorld, local[p]));
		const Vec3 narrow = vec3(fmul(cs.x, 0.5f), fmul(cs.y, 0.5f), fmul(cs.z, 1.0f));
		for (int32_t k = 0; k < cam.cullCount; k++)
			if (!plane_inside(cam.cull[k], narrow)) return DSRG_OK;
		proj[p] = camera_to_screen(cam, cs);
	}
	Hull hull;
	convex_hull(proj, 8, hull);
	occlude_from_hull(r, hull);
	r->gridDeviceValid = false;
	if (debugSilhouette) {
		// cyan lines around the hull, drawn at renderer_end; the reference tests the depth of the
		// unsorted projection p, not of the hull corner it draws from (rendererAPI.cpp:277-291)
		for (int32_t p = 0; p < hull.count; p++) {
			const int32_t q = (p + 1) % hull.count;
			if (proj[p].cs.z > camera->nearClip) {
				r->debugLines.push_back(make_int4((int32_t)(hull.x[p] / 256), (int32_t)(hull.y[p] / 256), (int32_t)(hull.x[q] / 256),
				                                  (int32_t)(hull.y[q] / 256)));
				r->debugColors.push_back(0xFFFFFF00u); // red 0, green 255, blue 255, alpha 255
			}
		}
	}
	return DSRG_OK;
}

int dsrg_renderer_occlude_from_existing_triangles(dsrg_renderer r) {
	if (!r) return DSRG_ERROR_INVALID_ARGUMENT;
	dsrg_context ctx = r->context;
	if (!r->receiving)
		return fail(ctx, DSRG_ERROR_CALL_ORDER, "Cannot call renderer_occludeFromExistingTriangles without first calling renderer_begin!");
	prepare_for_occlusion(r);
	if (r->tasks.empty()) return DSRG_OK;
	int s = renderer_upload_given(r);
	if (s != DSRG_OK) return s;
	s = renderer_grid_on_device(r);
	if (s != DSRG_OK) return s;
	BatchJob job;
	job.tasks = r->tasks;
	job.textures = r->textures;
	job.frames.resize(1);
	renderer_frame_target(r, job.frames[0]);
	job.depthOnly = r->depthOnly;
	s = occlude_enqueue(ctx, job);
	if (s != DSRG_OK) return s;
	r->gridHostValid = false;
	return DSRG_OK;
}

int dsrg_renderer_occlude_from_top_rows(dsrg_renderer r, const dsrg_camera *camera) {
	if (!r) return DSRG_ERROR_INVALID_ARGUMENT;
	dsrg_context ctx = r->context;
	prepare_for_occlusion(r); // before the checks, as the reference orders them
	if (!r->receiving) return fail(ctx, DSRG_ERROR_CALL_ORDER, "Cannot call renderer_occludeFromTopRows without first calling renderer_begin!");
	if (!r->hasDepth)
		return fail(ctx, DSRG_ERROR_CALL_ORDER, "Cannot call renderer_occludeFromTopRows without having given a depth buffer in renderer_begin!");
	if (!camera) return fail(ctx, DSRG_ERROR_INVALID_ARGUMENT, "renderer_occludeFromTopRows: null camera");
	int s = renderer_grid_on_device(r);
	if (s != DSRG_OK) return s;
	launch_occlusion_top_rows(r->gridDevice.ptr, r->gridWidth, r->gridHeight, r->gridAllocWidth, r->deviceDepth, r->depthStride,
	                          r->width, camera->perspective != 0, ctx->stream);
	DSRG_CUDA_TRY(ctx, cudaGetLastError());
	r->gridHostValid = false;
	return DSRG_OK;
}

int dsrg_renderer_is_box_visible(dsrg_renderer r, const float *minimum, const float *maximum, const float *modelToWorld,
                                 const dsrg_camera *camera, int32_t *visible) {
	if (!r) return DSRG_ERROR_INVALID_ARGUMENT;
	dsrg_context ctx = r->context;
	if (!r->receiving)
		return fail(ctx, DSRG_ERROR_CALL_ORDER,
		            "Cannot call renderer_isBoxVisible without first calling renderer_begin and giving occluder shapes to the pass!");
	if (!minimum || !maximum || !modelToWorld || !camera || !visible)
		return fail(ctx, DSRG_ERROR_INVALID_ARGUMENT, "renderer_isBoxVisible: null argument");
	bool occluded = false; // before any occluder of the frame this reads the grid as the last frame left it
	const int s = renderer_box_occluded(r, minimum, maximum, modelToWorld, make_camera(*camera), &occluded);
	if (s != DSRG_OK) return s;
	*visible = occluded ? 0 : 1;
	return DSRG_OK;
}

int dsrg_renderer_has_occluders(dsrg_renderer r) { return (r && r->occluded) ? 1 : 0; }

int dsrg_renderer_get_occlusion_grid(dsrg_renderer r, float *out, int32_t capacity, int32_t *gridWidth, int32_t *gridHeight) {
	if (!r) return DSRG_ERROR_INVALID_ARGUMENT;
	if (gridWidth) *gridWidth = r->gridWidth;
	if (gridHeight) *gridHeight = r->gridHeight;
	if (!out) return DSRG_OK;
	if ((size_t)capacity < (size_t)r->gridWidth * r->gridHeight)
		return fail(r->context, DSRG_ERROR_INVALID_ARGUMENT, "get_occlusion_grid: output too small");
	const int s = grid_on_host(r);
	if (s != DSRG_OK) return s;
	for (int32_t y = 0; y < r->gridHeight; y++)
		for (int32_t x = 0; x < r->gridWidth; x++) out[(size_t)y * r->gridWidth + x] = grid_read(r, x, y);
	return DSRG_OK;
}

} // extern "C"
