// Host side of the dsrg C ABI: contexts, textures, models and the renderer state machine
// around the kernels in dsrg_kernels.cu.
#include <cuda_runtime.h>

#include <atomic>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "dsrg_internal.h"
#include "dsrg_occlusion.h"
#include "dsrg_shade.h"

using namespace dsrg;

#define CUDA_TRY(ctx, expr) DSRG_CUDA_TRY(ctx, expr)

namespace dsrg {

// Allocations left before the one that fails (dsrg_debug_fail_allocation); negative: none fails.
static std::atomic<int64_t> g_failAllocation(-1);

cudaError_t device_alloc(void **p, size_t bytes) {
	int64_t left = g_failAllocation.load();
	while (left >= 0) {
		if (g_failAllocation.compare_exchange_weak(left, left - 1)) {
			if (left == 0) {
				*p = nullptr;
				return cudaErrorMemoryAllocation;
			}
			break;
		}
	}
	return cudaMalloc(p, bytes);
}

} // namespace dsrg

extern "C" {

int dsrg_debug_fail_allocation(int64_t after) {
	dsrg::g_failAllocation.store(after < 0 ? -1 : after);
	return DSRG_OK;
}

int dsrg_context_create(int32_t device, dsrg_context *out) {
	if (!out) return DSRG_ERROR_INVALID_ARGUMENT;
	*out = nullptr;
	int count = 0;
	if (cudaGetDeviceCount(&count) != cudaSuccess || count <= device || device < 0) return DSRG_ERROR_CUDA;
	if (cudaSetDevice(device) != cudaSuccess) return DSRG_ERROR_CUDA;
	dsrg_context ctx = new (std::nothrow) dsrg_context_s();
	if (!ctx) return DSRG_ERROR_OUT_OF_MEMORY;
	ctx->device = device;
	memset(&ctx->stats, 0, sizeof(ctx->stats));
	// the context's stream at the device's highest priority: a sprite frame's side stream (lowest)
	// then only fills what the shadow batch on this stream leaves free
	int leastPriority = 0, greatestPriority = 0;
	if (cudaDeviceGetStreamPriorityRange(&leastPriority, &greatestPriority) != cudaSuccess) greatestPriority = 0;
	if (cudaStreamCreateWithPriority(&ctx->stream, cudaStreamNonBlocking, greatestPriority) != cudaSuccess ||
	    cudaStreamCreateWithPriority(&ctx->branchStream, cudaStreamNonBlocking, greatestPriority) != cudaSuccess ||
	    cudaEventCreateWithFlags(&ctx->branchFork, cudaEventDisableTiming) != cudaSuccess ||
	    cudaEventCreateWithFlags(&ctx->branchJoin, cudaEventDisableTiming) != cudaSuccess ||
	    cudaEventCreate(&ctx->eventStart) != cudaSuccess || cudaEventCreate(&ctx->eventStop) != cudaSuccess ||
	    cudaEventCreate(&ctx->eventRasterStart) != cudaSuccess || cudaEventCreate(&ctx->eventRasterStop) != cudaSuccess ||
	    ctx->control.reserve(16) != cudaSuccess || ctx->fragmentCounter.reserve(2) != cudaSuccess ||
	    cudaMallocHost((void **)&ctx->pinnedReadback, 16 * sizeof(uint32_t)) != cudaSuccess ||
	    cudaHostGetDevicePointer((void **)&ctx->readbackDevice, ctx->pinnedReadback, 0) != cudaSuccess) {
		delete ctx;
		return DSRG_ERROR_CUDA;
	}
	if (cudaMemsetAsync(ctx->control.ptr, 0, 4 * sizeof(uint32_t), ctx->stream) != cudaSuccess ||
	    cudaMemsetAsync(ctx->fragmentCounter.ptr, 0, 2 * sizeof(unsigned long long), ctx->stream) != cudaSuccess) {
		dsrg_context_destroy(ctx);
		return DSRG_ERROR_CUDA;
	}
	*out = ctx;
	return DSRG_OK;
}

int dsrg_renderer_destroy(dsrg_renderer renderer);

int dsrg_context_destroy(dsrg_context ctx) {
	if (!ctx) return DSRG_ERROR_INVALID_ARGUMENT;
	cudaSetDevice(ctx->device);
	cudaStreamSynchronize(ctx->stream);
	if (ctx->implicitRenderer) dsrg_renderer_destroy(ctx->implicitRenderer);
	DeviceBuffer<float> *fbufs[] = {&ctx->pointIsy, &ctx->stagingDepth};
	for (auto *b : fbufs) b->release();
	ctx->pointCsis.release(); ctx->pointFlat.release();
	DeviceBuffer<uint32_t> *ubufs[] = {&ctx->triCounts, &ctx->triOffsets, &ctx->scanScratch, &ctx->control, &ctx->binCounts,
	                                   &ctx->binOffsets, &ctx->binCursors, &ctx->binLists, &ctx->stagingColor};
	for (auto *b : ubufs) b->release();
	ctx->records.release(); ctx->tables.release(); ctx->keys.release(); ctx->denseKeys.release(); ctx->denseInstances.release();
	if (ctx->pinnedTables) cudaFreeHost(ctx->pinnedTables);
	if (ctx->pinnedReadback) cudaFreeHost(ctx->pinnedReadback);
	ctx->rowCounts.release(); ctx->rowOffsets.release(); ctx->rows.release(); ctx->textureTable.release(); ctx->fragmentCounter.release();
	ctx->lightStaging.release();
	ctx->spriteTableHost.release();
	ctx->lightTableHost.release();
	ctx->spriteKeys.release();
	ctx->spriteTables.release();
	if (ctx->sideStart) cudaEventDestroy(ctx->sideStart);
	if (ctx->sideDone) cudaEventDestroy(ctx->sideDone);
	if (ctx->sideStream) cudaStreamDestroy(ctx->sideStream);
	if (ctx->branchFork) cudaEventDestroy(ctx->branchFork);
	if (ctx->branchJoin) cudaEventDestroy(ctx->branchJoin);
	if (ctx->branchStream) cudaStreamDestroy(ctx->branchStream);
	ctx->tileList.release();
	for (PhaseGraph &g : ctx->graphs) g.reset();
	cudaEventDestroy(ctx->eventStart);
	cudaEventDestroy(ctx->eventStop);
	cudaEventDestroy(ctx->eventRasterStart);
	cudaEventDestroy(ctx->eventRasterStop);
	cudaStreamDestroy(ctx->stream);
	delete ctx;
	return DSRG_OK;
}

const char *dsrg_context_last_error(dsrg_context ctx) { return ctx ? ctx->lastError.c_str() : "null context"; }

void *dsrg_context_stream(dsrg_context ctx) { return ctx ? (void *)ctx->stream : nullptr; }

int dsrg_context_set_counting(dsrg_context ctx, int32_t counting, uint32_t *deviceCoverage) {
	if (!ctx) return DSRG_ERROR_INVALID_ARGUMENT;
	ctx->counting = counting;
	ctx->coverage = counting ? deviceCoverage : nullptr;
	return DSRG_OK;
}

int dsrg_context_walked_fragments(dsrg_context ctx, uint64_t *out) {
	if (!ctx || !out) return DSRG_ERROR_INVALID_ARGUMENT;
	unsigned long long walked = 0;
	DSRG_CUDA_TRY(ctx, cudaMemcpyAsync(&walked, ctx->fragmentCounter.ptr + 1, sizeof(walked), cudaMemcpyDeviceToHost, ctx->stream));
	DSRG_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
	*out = walked;
	return DSRG_OK;
}

int dsrg_context_get_stats(dsrg_context ctx, dsrg_stats *out) {
	if (!ctx || !out) return DSRG_ERROR_INVALID_ARGUMENT;
	if (ctx->timingPending) {
		// the last call's events completed before it returned
		float ms = 0.0f, rasterMs = 0.0f;
		cudaEventElapsedTime(&ms, ctx->eventStart, ctx->eventStop);
		if (ctx->timingHasRaster) cudaEventElapsedTime(&rasterMs, ctx->eventRasterStart, ctx->eventRasterStop);
		ctx->stats.milliseconds = ms;
		ctx->stats.rasterMilliseconds = rasterMs;
		ctx->timingPending = false;
	}
	*out = ctx->stats;
	return DSRG_OK;
}

// ------------------------------------------------------------------ textures

// texture creation, destruction and reading live in dsrg_texture.cu

// ------------------------------------------------------------------ models

int dsrg_model_create(dsrg_context ctx, const float *positions, int32_t pointCount, const int32_t *polygonIndices,
                      const float *texCoords, const float *colors, int32_t polygonCount, dsrg_texture diffuse,
                      dsrg_texture light, int32_t filter, dsrg_model *out) {
	if (!ctx || !out) return DSRG_ERROR_INVALID_ARGUMENT;
	*out = nullptr;
	if (pointCount < 0 || polygonCount < 0 || (pointCount > 0 && !positions) ||
	    (polygonCount > 0 && (!polygonIndices || !texCoords || !colors)))
		return fail(ctx, DSRG_ERROR_INVALID_ARGUMENT, "dsrg_model_create: missing arrays");
	if (filter != DSRG_FILTER_SOLID && filter != DSRG_FILTER_ALPHA)
		return fail(ctx, DSRG_ERROR_INVALID_ARGUMENT, "dsrg_model_create: unknown filter");
	std::vector<int32_t> triSource;
	triSource.reserve((size_t)polygonCount * 2);
	for (int32_t p = 0; p < polygonCount; p++) {
		const int32_t *idx = polygonIndices + p * 4;
		int corners = idx[3] < 0 ? 3 : 4;
		for (int i = 0; i < corners; i++)
			if (idx[i] < 0 || idx[i] >= pointCount)
				return fail(ctx, DSRG_ERROR_INVALID_ARGUMENT, "dsrg_model_create: polygon point index out of range");
		triSource.push_back(p * 2);
		if (corners == 4) triSource.push_back(p * 2 + 1);
	}
	dsrg_model m = new (std::nothrow) dsrg_model_s();
	if (!m) return DSRG_ERROR_OUT_OF_MEMORY;
	m->context = ctx;
	m->pointCount = pointCount;
	m->polygonCount = polygonCount;
	m->triangleCount = (int32_t)triSource.size();
	m->diffuse = diffuse;
	m->light = light;
	m->filter = filter;
	// ModelImpl::expandBound starting from a zero bound (model/Model.cpp:281-288)
	for (int i = 0; i < 3; i++) { m->minBound[i] = 0.0f; m->maxBound[i] = 0.0f; }
	for (int32_t i = 0; i < pointCount; i++) {
		for (int a = 0; a < 3; a++) {
			float v = positions[i * 3 + a];
			if (m->minBound[a] > v) m->minBound[a] = v;
			if (m->maxBound[a] < v) m->maxBound[a] = v;
		}
	}
	cudaSetDevice(ctx->device);
	size_t np = (size_t)(pointCount > 0 ? pointCount : 1), ng = (size_t)(polygonCount > 0 ? polygonCount : 1);
	bool ok = dsrg::device_alloc((void **)&m->positions, np * 3 * sizeof(float)) == cudaSuccess &&
	          dsrg::device_alloc((void **)&m->polygons, ng * 4 * sizeof(int32_t)) == cudaSuccess &&
	          dsrg::device_alloc((void **)&m->texCoords, ng * 16 * sizeof(float)) == cudaSuccess &&
	          dsrg::device_alloc((void **)&m->colors, ng * 16 * sizeof(float)) == cudaSuccess &&
	          dsrg::device_alloc((void **)&m->triSource, (triSource.size() + 1) * sizeof(int32_t)) == cudaSuccess;
	if (ok && pointCount > 0) ok = cudaMemcpy(m->positions, positions, (size_t)pointCount * 3 * sizeof(float), cudaMemcpyHostToDevice) == cudaSuccess;
	if (ok && polygonCount > 0) {
		ok = cudaMemcpy(m->polygons, polygonIndices, (size_t)polygonCount * 4 * sizeof(int32_t), cudaMemcpyHostToDevice) == cudaSuccess &&
		     cudaMemcpy(m->texCoords, texCoords, (size_t)polygonCount * 16 * sizeof(float), cudaMemcpyHostToDevice) == cudaSuccess &&
		     cudaMemcpy(m->colors, colors, (size_t)polygonCount * 16 * sizeof(float), cudaMemcpyHostToDevice) == cudaSuccess &&
		     cudaMemcpy(m->triSource, triSource.data(), triSource.size() * sizeof(int32_t), cudaMemcpyHostToDevice) == cudaSuccess;
	}
	if (!ok) {
		cudaFree(m->positions); cudaFree(m->polygons); cudaFree(m->texCoords); cudaFree(m->colors); cudaFree(m->triSource);
		delete m;
		return fail(ctx, DSRG_ERROR_OUT_OF_MEMORY, "dsrg_model_create: device allocation or copy failed");
	}
	*out = m;
	return DSRG_OK;
}

int dsrg_model_set_bound(dsrg_model m, const float *minimum, const float *maximum) {
	if (!m || !minimum || !maximum) return DSRG_ERROR_INVALID_ARGUMENT;
	for (int a = 0; a < 3; a++) { m->minBound[a] = minimum[a]; m->maxBound[a] = maximum[a]; }
	return DSRG_OK;
}

int dsrg_model_destroy(dsrg_model m) {
	if (!m) return DSRG_ERROR_INVALID_ARGUMENT;
	cudaSetDevice(m->context->device);
	cudaStreamSynchronize(m->context->stream);
	cudaFree(m->positions); cudaFree(m->polygons); cudaFree(m->texCoords); cudaFree(m->colors); cudaFree(m->triSource);
	delete m;
	return DSRG_OK;
}

// ------------------------------------------------------------------ renderer

int dsrg_renderer_create(dsrg_context ctx, dsrg_renderer *out) {
	if (!ctx || !out) return DSRG_ERROR_INVALID_ARGUMENT;
	dsrg_renderer r = new (std::nothrow) dsrg_renderer_s();
	if (!r) return DSRG_ERROR_OUT_OF_MEMORY;
	r->context = ctx;
	*out = r;
	return DSRG_OK;
}

int dsrg_renderer_destroy(dsrg_renderer r) {
	if (!r) return DSRG_ERROR_INVALID_ARGUMENT;
	delete r;
	return DSRG_OK;
}

int dsrg_renderer_takes_triangles(dsrg_renderer r) { return (r && r->receiving) ? 1 : 0; }

static bool image_valid(const dsrg_image *img, int elementSize) {
	return img && img->data && img->width > 0 && img->height > 0 && img->strideBytes >= img->width * elementSize &&
	       img->strideBytes % elementSize == 0;
}

static int begin_frame(dsrg_renderer r, const dsrg_image *color, const dsrg_image *depth, bool depthOnly) {
	dsrg_context ctx = r->context;
	// RendererImpl::beginFrame (api/rendererAPI.cpp:151-168)
	if (r->receiving) return fail(ctx, DSRG_ERROR_CALL_ORDER, "Called renderer_begin on the same renderer twice without ending the previous batch!");
	if (color && !image_valid(color, 4)) return fail(ctx, DSRG_ERROR_INVALID_ARGUMENT, "renderer_begin: invalid colour image");
	if (depth && !image_valid(depth, 4)) return fail(ctx, DSRG_ERROR_INVALID_ARGUMENT, "renderer_begin: invalid depth image");
	if (color && (color->packOrder < 0 || color->packOrder > 3)) return fail(ctx, DSRG_ERROR_INVALID_ARGUMENT, "renderer_begin: unknown pack order");
	if (color && depth && (color->width != depth->width || color->height != depth->height))
		return fail(ctx, DSRG_ERROR_INVALID_ARGUMENT, "renderer_begin: colour and depth images must have the same dimensions");
	if ((color && (color->width > 32767 || color->height > 32767)) || (depth && (depth->width > 32767 || depth->height > 32767)))
		return fail(ctx, DSRG_ERROR_UNSUPPORTED, "renderer_begin: targets are limited to 32767 x 32767 pixels");
	cudaSetDevice(ctx->device);
	r->hasColor = color != nullptr;
	r->hasDepth = depth != nullptr;
	r->depthOnly = depthOnly;
	if (color) r->color = *color;
	if (depth) r->depth = *depth;
	r->width = color ? color->width : (depth ? depth->width : 0);
	r->height = color ? color->height : (depth ? depth->height : 0);
	r->gridWidth = (r->width + (dsrg::OCCLUSION_CELL - 1)) / dsrg::OCCLUSION_CELL;
	r->gridHeight = (r->height + (dsrg::OCCLUSION_CELL - 1)) / dsrg::OCCLUSION_CELL;
	r->occluded = false;
	size_t pixels = (size_t)r->width * r->height;
	r->deviceColor = nullptr;
	r->deviceDepth = nullptr;
	r->colorDirect = r->depthDirect = false;
	void *mapped = nullptr;
	if (color) {
		if (color->onDevice) {
			r->deviceColor = (uint32_t *)color->data;
			r->colorStride = color->strideBytes / 4;
		} else if (host_mapped(color->data, &mapped)) {
			r->deviceColor = (uint32_t *)mapped;
			r->colorStride = color->strideBytes / 4;
			r->colorDirect = true;
		} else {
			CUDA_TRY(ctx, ctx->stagingColor.reserve(pixels));
			r->deviceColor = ctx->stagingColor.ptr;
			r->colorStride = r->width;
			CUDA_TRY(ctx, cudaMemcpy2DAsync(r->deviceColor, (size_t)r->width * 4, color->data, color->strideBytes,
			                                (size_t)r->width * 4, r->height, cudaMemcpyHostToDevice, ctx->stream));
		}
	}
	if (depth) {
		if (depth->onDevice) {
			r->deviceDepth = (float *)depth->data;
			r->depthStride = depth->strideBytes / 4;
		} else if (host_mapped(depth->data, &mapped)) {
			r->deviceDepth = (float *)mapped;
			r->depthStride = depth->strideBytes / 4;
			r->depthDirect = true;
		} else {
			CUDA_TRY(ctx, ctx->stagingDepth.reserve(pixels));
			r->deviceDepth = ctx->stagingDepth.ptr;
			r->depthStride = r->width;
			CUDA_TRY(ctx, cudaMemcpy2DAsync(r->deviceDepth, (size_t)r->width * 4, depth->data, depth->strideBytes,
			                                (size_t)r->width * 4, r->height, cudaMemcpyHostToDevice, ctx->stream));
		}
	}
	r->triangleCount = 0;
	r->cameraKnown = false;
	r->textures.clear();
	r->textureHandles.clear();
	r->tasks.clear();
	r->givenPoints.clear();
	r->givenPolygons.clear();
	r->givenSource.clear();
	r->givenTexCoords.clear();
	r->givenColors.clear();
	r->givenTasks.clear();
	r->givenDirty = false;
	CUDA_TRY(ctx, cudaEventRecord(ctx->eventStart, ctx->stream));
	r->receiving = true;
	return DSRG_OK;
}

int dsrg_renderer_begin(dsrg_renderer r, const dsrg_image *color, const dsrg_image *depth) {
	if (!r) return DSRG_ERROR_INVALID_ARGUMENT;
	return begin_frame(r, color, depth, false);
}

static int32_t texture_slot(dsrg_renderer r, dsrg_texture t) {
	if (!t) return -1;
	for (size_t i = 0; i < r->textureHandles.size(); i++) if (r->textureHandles[i] == t) return (int32_t)i;
	r->textureHandles.push_back(t);
	r->textures.push_back(t->data);
	return (int32_t)r->textures.size() - 1;
}

static int give_task(dsrg_renderer r, dsrg_model m, const float *modelToWorld, const dsrg_camera *camera) {
	dsrg_context ctx = r->context;
	if (!r->receiving) return fail(ctx, DSRG_ERROR_CALL_ORDER, "Cannot call renderer_giveTask before renderer_begin!");
	if (!m || !modelToWorld || !camera) return fail(ctx, DSRG_ERROR_INVALID_ARGUMENT, "renderer_giveTask: null argument");
	if (camera->width <= 0 || camera->height <= 0) return fail(ctx, DSRG_ERROR_INVALID_ARGUMENT, "renderer_giveTask: camera without image size");
	CameraData cam = make_camera(*camera);
	r->affine = !camera->perspective; // the last camera's projection (a frame may mix both)
	r->cameraKnown = true;
	if (!box_seen(cam, m->minBound, m->maxBound, modelToWorld)) return DSRG_OK;
	if (r->occluded) { // the whole model behind the occluders so far (modelAPI.cpp:228-233)
		bool occluded = false;
		const int s = renderer_box_occluded(r, m->minBound, m->maxBound, modelToWorld, cam, &occluded);
		if (s != DSRG_OK) return s;
		if (occluded) return DSRG_OK;
	}
	if (m->triangleCount == 0) return DSRG_OK;
	TaskParams task;
	memset(&task, 0, sizeof(task));
	task.positions = m->positions;
	task.polygons = m->polygons;
	task.texCoords = m->texCoords;
	task.colors = m->colors;
	task.triSource = m->triSource;
	task.pointCount = m->pointCount;
	task.triangleCount = m->triangleCount;
	task.orderBase = r->triangleCount;
	task.frame = 0;
	memcpy(task.modelToWorld, modelToWorld, sizeof(task.modelToWorld));
	task.camera = cam;
	task.filter = m->filter;
	task.diffuse = r->depthOnly ? -1 : texture_slot(r, m->diffuse);
	task.light = r->depthOnly ? -1 : texture_slot(r, m->light);
	task.depthOnly = r->depthOnly ? 1 : 0;
	r->tasks.push_back(task);
	r->triangleCount += (uint32_t)m->triangleCount;
	return DSRG_OK;
}

int dsrg_renderer_give_task(dsrg_renderer r, dsrg_model m, const float *modelToWorld, const dsrg_camera *camera) {
	if (!r) return DSRG_ERROR_INVALID_ARGUMENT;
	return give_task(r, m, modelToWorld, camera);
}

int dsrg_renderer_get_images(dsrg_renderer r, dsrg_image *color, dsrg_image *depth) {
	if (!r) return DSRG_ERROR_INVALID_ARGUMENT;
	dsrg_image none;
	memset(&none, 0, sizeof(none));
	if (color) *color = (r->receiving && r->hasColor) ? r->color : none;
	if (depth) *depth = (r->receiving && r->hasDepth) ? r->depth : none;
	return DSRG_OK;
}

int dsrg_camera_world_to_screen(const dsrg_camera *camera, const float *world, dsrg_projected_point *out) {
	if (!camera || !world || !out || camera->width <= 0 || camera->height <= 0) return DSRG_ERROR_INVALID_ARGUMENT;
	const CameraData c = make_camera(*camera);
	const Projected p = camera_to_screen(c, world_to_camera(c, vec3(world[0], world[1], world[2])));
	out->cs[0] = p.cs.x; out->cs[1] = p.cs.y; out->cs[2] = p.cs.z;
	out->is[0] = p.isx; out->is[1] = p.isy;
	out->flat[0] = p.flatx; out->flat[1] = p.flaty;
	return DSRG_OK;
}

// renderer_giveTask_triangle (api/rendererAPI.cpp:503-519): one task of pre-projected triangles,
// drawn at renderer_end in submission order with the models given around it.
int dsrg_renderer_give_triangles(dsrg_renderer r, int32_t count, const dsrg_projected_point *corners, const float *colors,
                                 const float *texCoords, dsrg_texture diffuse, dsrg_texture light, int32_t filter,
                                 const dsrg_camera *camera) {
	if (!r) return DSRG_ERROR_INVALID_ARGUMENT;
	dsrg_context ctx = r->context;
	if (!r->receiving) return fail(ctx, DSRG_ERROR_CALL_ORDER, "Cannot call renderer_giveTask before renderer_begin!");
	if (count < 0 || !camera || (count > 0 && (!corners || !colors || !texCoords)))
		return fail(ctx, DSRG_ERROR_INVALID_ARGUMENT, "renderer_giveTask_triangle: invalid argument");
	if (camera->width <= 0 || camera->height <= 0)
		return fail(ctx, DSRG_ERROR_INVALID_ARGUMENT, "renderer_giveTask_triangle: camera without image size");
	if (filter != DSRG_FILTER_SOLID && filter != DSRG_FILTER_ALPHA)
		return fail(ctx, DSRG_ERROR_INVALID_ARGUMENT, "renderer_giveTask_triangle: unknown filter");
	if ((diffuse && diffuse->context != ctx) || (light && light->context != ctx))
		return fail(ctx, DSRG_ERROR_INVALID_ARGUMENT, "renderer_giveTask_triangle: texture of another context");
	r->affine = !camera->perspective; // the last camera's projection (a frame may mix both)
	r->cameraKnown = true;
	if (count == 0 || (!r->hasColor && !r->hasDepth)) return DSRG_OK; // renderTriangleFromData: no target to draw on
	TaskParams task;
	memset(&task, 0, sizeof(task));
	task.pointCount = 3 * count;
	task.triangleCount = count;
	task.orderBase = r->triangleCount;
	task.frame = 0;
	const float identity[12] = {0, 0, 0, 1, 0, 0, 0, 1, 0, 0, 0, 1};
	memcpy(task.modelToWorld, identity, sizeof(identity));
	task.camera = make_camera(*camera);
	task.filter = filter;
	task.diffuse = r->depthOnly ? -1 : texture_slot(r, diffuse);
	task.light = r->depthOnly ? -1 : texture_slot(r, light);
	task.depthOnly = r->depthOnly ? 1 : 0;
	const uint32_t first = (uint32_t)r->givenSource.size();
	for (int32_t i = 0; i < count; i++) {
		for (int k = 0; k < 3; k++) {
			GivenPoint g;
			memcpy(&g, &corners[3 * i + k], sizeof(g));
			r->givenPoints.push_back(g);
		}
		const int32_t poly[4] = {3 * i, 3 * i + 1, 3 * i + 2, -1};
		r->givenPolygons.insert(r->givenPolygons.end(), poly, poly + 4);
		r->givenSource.push_back(2 * i); // polygon i, first fan triangle
		for (int k = 0; k < 4; k++) {
			for (int c = 0; c < 4; c++) {
				r->givenTexCoords.push_back(k < 3 ? texCoords[(3 * i + k) * 4 + c] : 0.0f);
				r->givenColors.push_back(k < 3 ? colors[(3 * i + k) * 4 + c] : 0.0f);
			}
		}
	}
	r->givenTasks.push_back(std::make_pair(r->tasks.size(), first));
	r->tasks.push_back(task);
	r->triangleCount += (uint32_t)count;
	r->givenDirty = true;
	return DSRG_OK;
}

} // extern "C"

// A page-locked host image is read and written in place through its device address (over
// NVLink-C2C on Grace-Blackwell), with no staging copy; pageable memory is staged.
bool host_mapped(const void *p, void **devicePointer) {
	cudaPointerAttributes a;
	if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
		cudaGetLastError();
		return false;
	}
	if (a.type != cudaMemoryTypeHost || !a.devicePointer) return false;
	*devicePointer = a.devicePointer;
	return true;
}

int renderer_upload_given(dsrg_renderer r) {
	if (!r->givenDirty) return DSRG_OK;
	dsrg_context ctx = r->context;
	const size_t triangles = r->givenSource.size();
	auto align = [](size_t x) { return (x + 255) & ~(size_t)255; };
	const size_t pointsAt = 0;
	const size_t polygonsAt = align(pointsAt + triangles * 3 * sizeof(GivenPoint));
	const size_t sourceAt = align(polygonsAt + triangles * 4 * sizeof(int32_t));
	const size_t texAt = align(sourceAt + triangles * sizeof(int32_t));
	const size_t colorsAt = align(texAt + triangles * 16 * sizeof(float));
	const size_t bytes = align(colorsAt + triangles * 16 * sizeof(float));
	CUDA_TRY(ctx, r->givenDevice.reserve(bytes));
	unsigned char *base = r->givenDevice.ptr;
	cudaStream_t stream = ctx->stream;
	CUDA_TRY(ctx, cudaMemcpyAsync(base + pointsAt, r->givenPoints.data(), triangles * 3 * sizeof(GivenPoint), cudaMemcpyHostToDevice, stream));
	CUDA_TRY(ctx, cudaMemcpyAsync(base + polygonsAt, r->givenPolygons.data(), triangles * 4 * sizeof(int32_t), cudaMemcpyHostToDevice, stream));
	CUDA_TRY(ctx, cudaMemcpyAsync(base + sourceAt, r->givenSource.data(), triangles * sizeof(int32_t), cudaMemcpyHostToDevice, stream));
	CUDA_TRY(ctx, cudaMemcpyAsync(base + texAt, r->givenTexCoords.data(), triangles * 16 * sizeof(float), cudaMemcpyHostToDevice, stream));
	CUDA_TRY(ctx, cudaMemcpyAsync(base + colorsAt, r->givenColors.data(), triangles * 16 * sizeof(float), cudaMemcpyHostToDevice, stream));
	for (const auto &gt : r->givenTasks) {
		TaskParams &t = r->tasks[gt.first];
		const size_t first = gt.second;
		t.given = reinterpret_cast<const GivenPoint *>(base + pointsAt) + first * 3;
		t.polygons = reinterpret_cast<const int32_t *>(base + polygonsAt) + first * 4;
		t.triSource = reinterpret_cast<const int32_t *>(base + sourceAt) + first;
		t.texCoords = reinterpret_cast<const float *>(base + texAt) + first * 16;
		t.colors = reinterpret_cast<const float *>(base + colorsAt) + first * 16;
	}
	r->givenDirty = false;
	return DSRG_OK;
}

void renderer_frame_target(dsrg_renderer r, FrameTarget &f) {
	memset(&f, 0, sizeof(f));
	f.color = r->hasColor ? r->deviceColor : nullptr;
	f.colorStride = r->colorStride;
	f.packOrder = r->hasColor ? r->color.packOrder : 0;
	f.depth = r->hasDepth ? r->deviceDepth : nullptr;
	f.depthStride = r->depthStride;
	f.width = r->width;
	f.height = r->height;
	f.affine = r->affine ? 1 : 0;
	f.coverage = r->context->counting ? r->context->coverage : nullptr;
	if (r->occluded) {
		f.occlusion = r->gridDevice.ptr;
		f.gridWidth = r->gridWidth;
		f.gridHeight = r->gridHeight;
		f.gridStride = r->gridAllocWidth;
	}
}

extern "C" {

static int end_frame(dsrg_renderer r, bool debugWireframe) {
	dsrg_context ctx = r->context;
	if (!r->receiving) return fail(ctx, DSRG_ERROR_CALL_ORDER, "Called renderer_end without renderer_begin!");
	r->receiving = false;
	const int uploaded = renderer_upload_given(r);
	if (uploaded != DSRG_OK) return uploaded;
	BatchJob &job = ctx->frameJob;
	job.tasks.swap(r->tasks);
	job.textures.swap(r->textures);
	job.frames.resize(1);
	if (r->occluded) {
		const int s = renderer_grid_on_device(r);
		if (s != DSRG_OK) {
			job.tasks.swap(r->tasks);
			job.textures.swap(r->textures);
			return s;
		}
	}
	FrameTarget &f = job.frames[0];
	renderer_frame_target(r, f);
	job.depthOnly = r->depthOnly;
	job.resolve = true;
	job.hostTargets = r->colorDirect || r->depthDirect;
	BatchTotals totals;
	int status = DSRG_OK;
	// renderer_end(debugWireframe): the edges of every drawn command, collected run by run and
	// drawn over the finished frame (rendererAPI.cpp:354-399)
	const bool wire = debugWireframe && r->hasColor;
	uint32_t wireCount = 0;
	auto enqueue = [&](BatchTotals &t) -> int {
		BatchOutputs o;
		int e = batch_enqueue(ctx, job, t, &o);
		if (e != DSRG_OK || !wire || t.records == 0 || !o.fb.records) return e;
		const size_t lines = ((size_t)wireCount + t.records) * 3;
		CUDA_TRY(ctx, r->wireLines.reserve(lines + 1, true, (size_t)wireCount * 3, ctx->stream));
		launch_wire_lines(o.fb.records, t.records, r->wireLines.ptr + (size_t)wireCount * 3, ctx->stream);
		wireCount += t.records;
		return DSRG_OK;
	};
	// Alpha-filtered tasks blend in submission order and write no depth (fillShape,
	// fillerTemplates.h:387-441), and a task seen through an orthogonal camera tests linear depth
	// with '<' where a perspective one tests 1/W with '>' (fillerTemplates.h:108-152), so a frame
	// runs as consecutive runs of tasks of one kind, each through the whole pipeline, one after
	// another on the stream.  Without a colour target an alpha-filtered task draws like a solid one.
	auto kind = [&](const TaskParams &t) {
		return ((r->hasColor && !r->depthOnly && t.filter == 1) ? 2 : 0) | (t.camera.perspective ? 0 : 1);
	};
	bool oneKind = true;
	for (const TaskParams &t : job.tasks) oneKind = oneKind && kind(t) == kind(job.tasks[0]);
	if (oneKind) {
		job.alpha = !job.tasks.empty() && (kind(job.tasks[0]) & 2) != 0;
		if (!job.tasks.empty()) f.affine = kind(job.tasks[0]) & 1;
		job.clearCounters = true;
		status = enqueue(totals);
	} else {
		std::vector<TaskParams> &all = r->runTasks;
		all.swap(job.tasks);
		size_t begin = 0;
		while (begin < all.size() && status == DSRG_OK) {
			const int k = kind(all[begin]);
			size_t end = begin + 1;
			while (end < all.size() && kind(all[end]) == k) end++;
			job.tasks.assign(all.begin() + begin, all.begin() + end);
			job.alpha = (k & 2) != 0;
			job.frames[0].affine = k & 1;
			job.clearCounters = begin == 0;
			BatchTotals run;
			status = enqueue(run);
			totals.triangles += run.triangles;
			totals.records += run.records;
			totals.rows += run.rows;
			totals.binEntries += run.binEntries;
			begin = end;
		}
		all.swap(job.tasks);
		job.alpha = false;
		job.clearCounters = true;
	}
	job.tasks.swap(r->tasks);
	job.textures.swap(r->textures);
	if (status != DSRG_OK) {
		cudaStreamSynchronize(ctx->stream);
		return status;
	}
	if (r->hasColor) {
		if (wire) launch_draw_lines(r->deviceColor, r->colorStride, r->width, r->height, r->wireLines.ptr, wireCount * 3, 0xFFFFFFFFu,
		                            ctx->stream);
		if (!r->debugLines.empty()) {
			// silhouettes kept by occludeFromBox, in the target's pack order; a launch per colour run keeps their order
			CUDA_TRY(ctx, r->debugLinesDevice.reserve(r->debugLines.size() + 1));
			CUDA_TRY(ctx, cudaMemcpyAsync(r->debugLinesDevice.ptr, r->debugLines.data(), r->debugLines.size() * sizeof(int4),
			                              cudaMemcpyHostToDevice, ctx->stream));
			size_t begin = 0;
			while (begin < r->debugLines.size()) {
				size_t end = begin + 1;
				while (end < r->debugLines.size() && r->debugColors[end] == r->debugColors[begin]) end++;
				uint32_t packed = 0; // image_saturateAndPack in the target's pack order
				for (int ch = 0; ch < 4; ch++) packed |= ((r->debugColors[begin] >> (ch * 8)) & 0xFFu) << dsrg::pack_shift(r->color.packOrder, ch);
				launch_draw_lines(r->deviceColor, r->colorStride, r->width, r->height, r->debugLinesDevice.ptr + begin,
				                  (uint32_t)(end - begin), packed, ctx->stream);
				begin = end;
			}
			CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream)); // the host list is cleared next
			r->debugLines.clear();
			r->debugColors.clear();
		}
	}
	if (r->hasColor && !r->color.onDevice && !r->colorDirect)
		CUDA_TRY(ctx, cudaMemcpy2DAsync(r->color.data, r->color.strideBytes, r->deviceColor, (size_t)r->width * 4,
		                                (size_t)r->width * 4, r->height, cudaMemcpyDeviceToHost, ctx->stream));
	if (r->hasDepth && !r->depth.onDevice && !r->depthDirect)
		CUDA_TRY(ctx, cudaMemcpy2DAsync(r->depth.data, r->depth.strideBytes, r->deviceDepth, (size_t)r->width * 4,
		                                (size_t)r->width * 4, r->height, cudaMemcpyDeviceToHost, ctx->stream));
	return batch_finish(ctx, totals);
}

int dsrg_renderer_end(dsrg_renderer r) {
	if (!r) return DSRG_ERROR_INVALID_ARGUMENT;
	return end_frame(r, false);
}

int dsrg_renderer_end_debug(dsrg_renderer r, int32_t debugWireframe) {
	if (!r) return DSRG_ERROR_INVALID_ARGUMENT;
	return end_frame(r, debugWireframe != 0);
}

// ------------------------------------------------------------------ single-call rendering

static int render_once(dsrg_context ctx, dsrg_model m, const float *modelToWorld, const dsrg_camera *camera,
                       const dsrg_image *color, const dsrg_image *depth, bool depthOnly) {
	if (!ctx) return DSRG_ERROR_INVALID_ARGUMENT;
	if (!m) return fail(ctx, DSRG_ERROR_INVALID_ARGUMENT, "model_render: null model");
	if (!color && !depth) return DSRG_OK; // renderTriangleFromData: no target buffer to draw on
	if (!ctx->implicitRenderer) {
		int s = dsrg_renderer_create(ctx, &ctx->implicitRenderer);
		if (s != DSRG_OK) return s;
	}
	dsrg_renderer r = ctx->implicitRenderer;
	int s = begin_frame(r, color, depth, depthOnly);
	if (s != DSRG_OK) return s;
	s = give_task(r, m, modelToWorld, camera);
	if (s != DSRG_OK) {
		r->receiving = false;
		cudaStreamSynchronize(ctx->stream);
		return s;
	}
	return end_frame(r, false);
}

int dsrg_model_render(dsrg_context ctx, dsrg_model m, const float *modelToWorld, const dsrg_camera *camera,
                      const dsrg_image *color, const dsrg_image *depth) {
	return render_once(ctx, m, modelToWorld, camera, color, depth, false);
}

int dsrg_model_render_depth(dsrg_context ctx, dsrg_model m, const float *modelToWorld, const dsrg_camera *camera,
                            const dsrg_image *depth) {
	if (!depth) return DSRG_OK;
	return render_once(ctx, m, modelToWorld, camera, nullptr, depth, true);
}

} // extern "C"
