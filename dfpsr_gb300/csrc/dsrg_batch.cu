// Batched rendering (dsrg_batch_*) and the tile kernel's autotuner.
//
// A batch is a list of frames, each what one renderer_begin ... renderer_end would draw
// (api/rendererAPI.cpp:151-168, 351-358), rendered by one pass of the kernels over all frames.
// The reference has no batched form; its renderer draws one target at a time.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cstdio>
#include <utility>
#include <cstring>
#include <new>
#include <string>
#include <unordered_map>
#include <vector>

#include "dsrg_internal.h"

using namespace dsrg;

struct dsrg_batch_s {
	dsrg_context context;
	struct Frame {
		dsrg_image color, depth;
		bool hasColor = false, hasDepth = false;
		int32_t width = 0, height = 0;
		uint32_t triangles = 0; // fan triangles given so far (the next task's orderBase)
	};
	std::vector<Frame> frames;
	std::vector<TaskParams> tasks;
	std::vector<TextureData> textures;
	std::unordered_map<dsrg_texture, int32_t> textureSlots;
	DeviceBuffer<uint32_t> stagingColor; // frames whose images are in pageable host memory
	DeviceBuffer<float> stagingDepth;
	std::vector<void *> mapped; // per frame: device addresses of page-locked colour and depth images
	bool depthOnly = false; // model_renderDepth semantics for every frame
	bool hasTuning = false; // the batch's own tile-kernel configuration (else the context's)
	dsrg_tuning tuning;
	BatchJob job;
	BatchJob runs; // one pass of a batch whose frames draw several runs
};

// A frame's tasks in submission order form runs of consecutive tasks of one kind: alpha-filtered
// or not (alpha-filtered tasks blend in order and write no depth, fillerTemplates.h:387-441) and
// seen through a perspective or an orthogonal camera (the depth test compares 1/W with '>' or W
// with '<', fillerTemplates.h:108-152).  Each run is drawn by the key-based passes of its kind,
// and a frame's runs follow one another, which is the reference's order.  Pass p of the batch
// draws run p of every frame that has one: the solid runs in one batch, then the alpha runs.
static int enqueue_runs(dsrg_context ctx, BatchJob &job, BatchJob &run, BatchTotals &totals) {
	const size_t frameCount = job.frames.size();
	auto kind = [&](const TaskParams &t) -> int {
		const bool alpha = !job.depthOnly && t.filter == 1 && job.frames[(size_t)t.frame].color != nullptr;
		return (alpha ? 2 : 0) | (t.camera.perspective ? 0 : 1);
	};
	// each frame's runs: [first task, end) ranges over its own task list
	std::vector<std::vector<size_t>> own(frameCount);
	for (size_t i = 0; i < job.tasks.size(); i++) own[(size_t)job.tasks[i].frame].push_back(i);
	std::vector<std::vector<std::pair<size_t, size_t>>> runs(frameCount);
	size_t passes = 0;
	bool anyAlpha = false;
	for (size_t f = 0; f < frameCount; f++) {
		const std::vector<size_t> &t = own[f];
		for (size_t begin = 0; begin < t.size();) {
			size_t end = begin + 1;
			while (end < t.size() && kind(job.tasks[t[end]]) == kind(job.tasks[t[begin]])) end++;
			runs[f].push_back(std::make_pair(begin, end));
			anyAlpha = anyAlpha || (kind(job.tasks[t[begin]]) & 2) != 0;
			begin = end;
		}
		passes = std::max(passes, runs[f].size());
		job.frames[f].affine = runs[f].empty() ? 0 : (kind(job.tasks[t[0]]) & 1);
	}
	if (passes <= 1 && !anyAlpha) {
		job.alpha = false;
		job.clearCounters = true;
		return batch_enqueue(ctx, job, totals);
	}
	run.textures.swap(job.textures);
	run.depthOnly = job.depthOnly;
	run.resolve = job.resolve;
	run.hostTargets = job.hostTargets;
	int status = DSRG_OK;
	bool first = true;
	for (size_t p = 0; p < passes && status == DSRG_OK; p++) {
		for (int alpha = 0; alpha < 2 && status == DSRG_OK; alpha++) {
			run.frames.clear();
			run.tasks.clear();
			for (size_t f = 0; f < frameCount; f++) {
				if (p >= runs[f].size()) continue;
				const std::vector<size_t> &t = own[f];
				const int k = kind(job.tasks[t[runs[f][p].first]]);
				if (((k & 2) != 0) != (alpha != 0)) continue;
				FrameTarget target = job.frames[f];
				target.affine = k & 1;
				run.frames.push_back(target);
				for (size_t i = runs[f][p].first; i < runs[f][p].second; i++) {
					TaskParams task = job.tasks[t[i]];
					task.frame = (int32_t)run.frames.size() - 1;
					run.tasks.push_back(task);
				}
			}
			if (run.frames.empty()) continue;
			run.alpha = alpha != 0;
			run.clearCounters = first;
			first = false;
			BatchTotals part;
			status = batch_enqueue(ctx, run, part);
			totals.triangles += part.triangles;
			totals.records += part.records;
			totals.rows += part.rows;
			totals.binEntries += part.binEntries;
		}
	}
	run.textures.swap(job.textures);
	return status;
}

static bool image_ok(const dsrg_image *img) {
	return img && img->data && img->width > 0 && img->height > 0 && img->strideBytes >= img->width * 4 && img->strideBytes % 4 == 0;
}

bool batch_depth_in_place(dsrg_batch b) {
	void *mappedPointer = nullptr;
	for (const auto &f : b->frames)
		if (f.hasDepth && !f.depth.onDevice && !host_mapped(f.depth.data, &mappedPointer)) return false;
	return true;
}

void batch_clear_depth(dsrg_batch b) {
	// frames whose images follow one another in memory with one width and stride (the six faces of
	// a cube map) are cleared as one rectangle
	char *first = nullptr;
	int32_t strideBytes = 0, width = 0, rows = 0;
	auto flush = [&]() {
		if (first) enqueue_fill_words(first, strideBytes / 4, width, rows, 0u, b->context->stream);
		first = nullptr;
	};
	for (const auto &f : b->frames) {
		if (!f.hasDepth) continue;
		void *at = f.depth.data;
		if (!f.depth.onDevice && !host_mapped(f.depth.data, &at)) continue; // excluded by batch_depth_in_place
		char *p = static_cast<char *>(at);
		if (first && p == first + (size_t)rows * strideBytes && f.depth.strideBytes == strideBytes && f.width == width) {
			rows += f.height;
			continue;
		}
		flush();
		first = p;
		strideBytes = f.depth.strideBytes;
		width = f.width;
		rows = f.height;
	}
	flush();
}

dsrg_context batch_context(dsrg_batch b) { return b->context; }

extern "C" {

int dsrg_batch_create(dsrg_context ctx, dsrg_batch *out) {
	if (!ctx || !out) return DSRG_ERROR_INVALID_ARGUMENT;
	dsrg_batch b = new (std::nothrow) dsrg_batch_s();
	if (!b) return DSRG_ERROR_OUT_OF_MEMORY;
	b->context = ctx;
	*out = b;
	return DSRG_OK;
}

int dsrg_batch_destroy(dsrg_batch b) {
	if (!b) return DSRG_ERROR_INVALID_ARGUMENT;
	cudaSetDevice(b->context->device);
	cudaStreamSynchronize(b->context->stream);
	b->stagingColor.release();
	b->stagingDepth.release();
	delete b;
	return DSRG_OK;
}

int dsrg_batch_clear(dsrg_batch b) {
	if (!b) return DSRG_ERROR_INVALID_ARGUMENT;
	b->frames.clear();
	b->tasks.clear();
	b->textures.clear();
	b->textureSlots.clear();
	return DSRG_OK;
}

int dsrg_batch_add_frame(dsrg_batch b, const dsrg_image *color, const dsrg_image *depth, int32_t *frameIndex) {
	if (!b) return DSRG_ERROR_INVALID_ARGUMENT;
	dsrg_context ctx = b->context;
	if (!color && !depth) return fail(ctx, DSRG_ERROR_INVALID_ARGUMENT, "dsrg_batch_add_frame: a frame needs a colour or a depth image");
	if (color && !image_ok(color)) return fail(ctx, DSRG_ERROR_INVALID_ARGUMENT, "dsrg_batch_add_frame: invalid colour image");
	if (depth && !image_ok(depth)) return fail(ctx, DSRG_ERROR_INVALID_ARGUMENT, "dsrg_batch_add_frame: invalid depth image");
	if (color && (color->packOrder < 0 || color->packOrder > 3)) return fail(ctx, DSRG_ERROR_INVALID_ARGUMENT, "dsrg_batch_add_frame: unknown pack order");
	if (color && depth && (color->width != depth->width || color->height != depth->height))
		return fail(ctx, DSRG_ERROR_INVALID_ARGUMENT, "dsrg_batch_add_frame: colour and depth images must have the same dimensions");
	const int32_t w = color ? color->width : depth->width, h = color ? color->height : depth->height;
	if (w > 32767 || h > 32767) return fail(ctx, DSRG_ERROR_UNSUPPORTED, "dsrg_batch_add_frame: targets are limited to 32767 x 32767 pixels");
	dsrg_batch_s::Frame f;
	f.hasColor = color != nullptr;
	f.hasDepth = depth != nullptr;
	if (color) f.color = *color;
	if (depth) f.depth = *depth;
	f.width = w;
	f.height = h;
	b->frames.push_back(f);
	if (frameIndex) *frameIndex = (int32_t)b->frames.size() - 1;
	return DSRG_OK;
}

int dsrg_batch_give_task(dsrg_batch b, int32_t frameIndex, dsrg_model m, const float *modelToWorld, const dsrg_camera *camera) {
	if (!b) return DSRG_ERROR_INVALID_ARGUMENT;
	dsrg_context ctx = b->context;
	if (frameIndex < 0 || frameIndex >= (int32_t)b->frames.size())
		return fail(ctx, DSRG_ERROR_INVALID_ARGUMENT, "dsrg_batch_give_task: no such frame");
	if (!m || !modelToWorld || !camera) return fail(ctx, DSRG_ERROR_INVALID_ARGUMENT, "dsrg_batch_give_task: null argument");
	if (camera->width <= 0 || camera->height <= 0) return fail(ctx, DSRG_ERROR_INVALID_ARGUMENT, "dsrg_batch_give_task: camera without image size");
	dsrg_batch_s::Frame &f = b->frames[frameIndex];
	CameraData cam = make_camera(*camera);
	// ModelImpl::render skips models whose bound is outside the view (model/Model.cpp:186-197)
	if (!box_seen(cam, m->minBound, m->maxBound, modelToWorld) || m->triangleCount == 0) return DSRG_OK;
	TaskParams task;
	memset(&task, 0, sizeof(task));
	task.positions = m->positions;
	task.polygons = m->polygons;
	task.texCoords = m->texCoords;
	task.colors = m->colors;
	task.triSource = m->triSource;
	task.pointCount = m->pointCount;
	task.triangleCount = m->triangleCount;
	task.orderBase = f.triangles;
	task.frame = frameIndex;
	memcpy(task.modelToWorld, modelToWorld, sizeof(task.modelToWorld));
	task.camera = cam;
	task.filter = m->filter;
	auto slot = [&](dsrg_texture t) -> int32_t {
		if (!t) return -1;
		auto it = b->textureSlots.find(t);
		if (it != b->textureSlots.end()) return it->second;
		const int32_t index = (int32_t)b->textures.size();
		b->textures.push_back(t->data);
		b->textureSlots[t] = index;
		return index;
	};
	task.diffuse = slot(m->diffuse);
	task.light = slot(m->light);
	task.depthOnly = 0;
	b->tasks.push_back(task);
	f.triangles += (uint32_t)m->triangleCount;
	return DSRG_OK;
}

static int batch_render_with_context_tuning(dsrg_batch b);

int dsrg_batch_render(dsrg_batch b) {
	if (!b) return DSRG_ERROR_INVALID_ARGUMENT;
	if (!b->hasTuning) return batch_render_with_context_tuning(b);
	// the batch's own configuration for this render, the context's back afterwards
	dsrg_context ctx = b->context;
	dsrg_tuning saved;
	dsrg_context_get_tuning(ctx, &saved);
	int status = dsrg_context_set_tuning(ctx, &b->tuning);
	if (status == DSRG_OK) status = batch_render_with_context_tuning(b);
	dsrg_context_set_tuning(ctx, &saved);
	return status;
}

static int batch_render_with_context_tuning(dsrg_batch b) {
	dsrg_context ctx = b->context;
	cudaSetDevice(ctx->device);
	cudaStream_t stream = ctx->stream;
	// frames in page-locked host memory are drawn in place, frames in pageable memory in staging buffers
	size_t colorPixels = 0, depthPixels = 0;
	std::vector<void *> &mapped = b->mapped;
	mapped.assign(b->frames.size() * 2, nullptr);
	for (size_t i = 0; i < b->frames.size(); i++) {
		const auto &f = b->frames[i];
		if (f.hasColor && !f.color.onDevice && !host_mapped(f.color.data, &mapped[2 * i])) colorPixels += (size_t)f.width * f.height;
		if (f.hasDepth && !f.depth.onDevice && !host_mapped(f.depth.data, &mapped[2 * i + 1])) depthPixels += (size_t)f.width * f.height;
	}
	if (colorPixels) DSRG_CUDA_TRY(ctx, b->stagingColor.reserve(colorPixels));
	if (depthPixels) DSRG_CUDA_TRY(ctx, b->stagingDepth.reserve(depthPixels));
	DSRG_CUDA_TRY(ctx, cudaEventRecord(ctx->eventStart, stream));
	BatchJob &job = b->job;
	job.frames.resize(b->frames.size());
	colorPixels = depthPixels = 0;
	for (size_t i = 0; i < b->frames.size(); i++) {
		const auto &f = b->frames[i];
		FrameTarget &t = job.frames[i];
		memset(&t, 0, sizeof(t));
		t.width = f.width;
		t.height = f.height;
		if (f.hasColor) {
			t.packOrder = f.color.packOrder;
			if (f.color.onDevice || mapped[2 * i]) {
				t.color = (uint32_t *)(f.color.onDevice ? f.color.data : mapped[2 * i]);
				t.colorStride = f.color.strideBytes / 4;
			} else {
				t.color = b->stagingColor.ptr + colorPixels;
				t.colorStride = f.width;
				colorPixels += (size_t)f.width * f.height;
				DSRG_CUDA_TRY(ctx, cudaMemcpy2DAsync(t.color, (size_t)f.width * 4, f.color.data, f.color.strideBytes, (size_t)f.width * 4,
				                                     f.height, cudaMemcpyHostToDevice, stream));
			}
		}
		if (f.hasDepth) {
			if (f.depth.onDevice || mapped[2 * i + 1]) {
				t.depth = (float *)(f.depth.onDevice ? f.depth.data : mapped[2 * i + 1]);
				t.depthStride = f.depth.strideBytes / 4;
			} else {
				t.depth = b->stagingDepth.ptr + depthPixels;
				t.depthStride = f.width;
				depthPixels += (size_t)f.width * f.height;
				DSRG_CUDA_TRY(ctx, cudaMemcpy2DAsync(t.depth, (size_t)f.width * 4, f.depth.data, f.depth.strideBytes, (size_t)f.width * 4,
				                                     f.height, cudaMemcpyHostToDevice, stream));
			}
		}
	}
	job.tasks.swap(b->tasks);
	job.textures.swap(b->textures);
	job.depthOnly = b->depthOnly;
	job.resolve = true;
	job.hostTargets = false;
	for (void *p : mapped) job.hostTargets = job.hostTargets || p != nullptr;
	if (b->depthOnly) {
		// renderTriangleFromDataDepth (renderCore.cpp:400-443): 1 x 1 walk, no shading, no colour target
		for (TaskParams &t : job.tasks) { t.depthOnly = 1; t.diffuse = -1; t.light = -1; }
		for (FrameTarget &f : job.frames) f.color = nullptr;
	} else {
		for (TaskParams &t : job.tasks) t.depthOnly = 0;
	}
	BatchTotals totals;
	const int status = enqueue_runs(ctx, job, b->runs, totals);
	job.tasks.swap(b->tasks);
	job.textures.swap(b->textures);
	if (status != DSRG_OK) {
		cudaStreamSynchronize(stream);
		return status;
	}
	for (size_t i = 0; i < b->frames.size(); i++) {
		const auto &f = b->frames[i];
		const FrameTarget &t = job.frames[i];
		if (f.hasColor && !f.color.onDevice && !mapped[2 * i])
			DSRG_CUDA_TRY(ctx, cudaMemcpy2DAsync(f.color.data, f.color.strideBytes, t.color, (size_t)f.width * 4, (size_t)f.width * 4,
			                                     f.height, cudaMemcpyDeviceToHost, stream));
		if (f.hasDepth && !f.depth.onDevice && !mapped[2 * i + 1])
			DSRG_CUDA_TRY(ctx, cudaMemcpy2DAsync(f.depth.data, f.depth.strideBytes, t.depth, (size_t)f.width * 4, (size_t)f.width * 4,
			                                     f.height, cudaMemcpyDeviceToHost, stream));
	}
	return batch_finish(ctx, totals);
}

int dsrg_batch_set_depth_only(dsrg_batch b, int32_t depthOnly) {
	if (!b) return DSRG_ERROR_INVALID_ARGUMENT;
	b->depthOnly = depthOnly != 0;
	return DSRG_OK;
}

int dsrg_context_get_tuning(dsrg_context ctx, dsrg_tuning *out) {
	if (!ctx || !out) return DSRG_ERROR_INVALID_ARGUMENT;
	out->threadsPerTile = ctx->threadsPerTile;
	out->ctasPerSm = ctx->ctasPerSm;
	out->smallRows = ctx->smallRows;
	out->smallWidth = ctx->smallWidth;
	out->graphs = ctx->useGraphs;
	out->resolve = ctx->resolveMode;
	return DSRG_OK;
}

static int check_tuning(dsrg_context ctx, const dsrg_tuning *t, const char *caller) {
	char message[200];
	const char *problem = nullptr;
	if (t->threadsPerTile != 64 && t->threadsPerTile != 128 && t->threadsPerTile != 256)
		problem = "threadsPerTile must be 64, 128 or 256";
	else if (t->ctasPerSm < 1 || t->ctasPerSm > 1024 / t->threadsPerTile)
		problem = "ctasPerSm must be between 1 and 1024 / threadsPerTile";
	else if (t->smallRows < 0 || t->smallWidth < 0 || t->smallRows > 16 || t->smallWidth > 64)
		problem = "small-triangle bound out of range (rows 0..16, width 0..64)";
	else if (t->resolve < 0 || t->resolve > 2)
		problem = "resolve must be 0 (per pixel, own pass), 1 (per pixel, in the tile kernel) or 2 (per quad)";
	if (!problem) return DSRG_OK;
	snprintf(message, sizeof(message), "%s: %s", caller, problem);
	return fail(ctx, DSRG_ERROR_INVALID_ARGUMENT, message);
}

int dsrg_context_set_tuning(dsrg_context ctx, const dsrg_tuning *t) {
	if (!ctx || !t) return DSRG_ERROR_INVALID_ARGUMENT;
	const int status = check_tuning(ctx, t, "dsrg_context_set_tuning");
	if (status != DSRG_OK) return status;
	ctx->threadsPerTile = t->threadsPerTile;
	ctx->ctasPerSm = t->ctasPerSm;
	ctx->smallRows = t->smallRows;
	ctx->smallWidth = t->smallWidth;
	ctx->useGraphs = t->graphs ? 1 : 0;
	ctx->resolveMode = t->resolve;
	return DSRG_OK;
}

int dsrg_batch_set_tuning(dsrg_batch b, const dsrg_tuning *t) {
	if (!b) return DSRG_ERROR_INVALID_ARGUMENT;
	if (!t) {
		b->hasTuning = false;
		return DSRG_OK;
	}
	const int status = check_tuning(b->context, t, "dsrg_batch_set_tuning");
	if (status != DSRG_OK) return status;
	b->tuning = *t;
	b->hasTuning = true;
	return DSRG_OK;
}

int dsrg_batch_autotune(dsrg_batch b, int32_t rounds, dsrg_tuning *best) {
	if (!b) return DSRG_ERROR_INVALID_ARGUMENT;
	dsrg_context ctx = b->context;
	if (rounds < 1) rounds = 1;
	// a batch with a configuration of its own is searched from it and keeps the result; the
	// context's configuration is then left as it was
	dsrg_tuning contextTuning;
	dsrg_context_get_tuning(ctx, &contextTuning);
	const bool own = b->hasTuning;
	if (own) dsrg_context_set_tuning(ctx, &b->tuning);
	b->hasTuning = false; // the candidates are set on the context while searching
	dsrg_tuning start;
	dsrg_context_get_tuning(ctx, &start);
	struct Restore { // whatever the search's outcome
		dsrg_batch batch; dsrg_context context; dsrg_tuning tuning; bool own;
		~Restore() {
			batch->hasTuning = own;
			if (own) dsrg_context_set_tuning(context, &tuning);
		}
	} restore{b, ctx, contextTuning, own};
	struct Shape { int32_t threads, perSm; };
	const Shape shapes[] = {{256, 4}, {256, 2}, {128, 8}, {128, 4}, {64, 16}};
	const int32_t smalls[][2] = {{8, 16}, {0, 0}, {4, 8}};
	// the launch shapes with the resolve inside the tile kernel, then the other resolves with the
	// fastest shape
	std::vector<dsrg_tuning> candidates;
	for (const Shape &s : shapes) {
		for (const auto &sm : smalls) {
			dsrg_tuning t = start;
			t.threadsPerTile = s.threads;
			t.ctasPerSm = s.perSm;
			t.smallRows = sm[0];
			t.smallWidth = sm[1];
			t.resolve = 1;
			candidates.push_back(t);
		}
	}
	const size_t shapeCount = candidates.size();
	dsrg_tuning chosen = start;
	double bestSeconds = -1.0;
	// Each timed render starts from a cold L2 (a 256 MB write first), as a batch does when other
	// work runs between batches; without it the candidates that reuse last render's lines in L2
	// would look faster than they are.
	void *flush = nullptr;
	const size_t flushBytes = (size_t)256 << 20;
	if (device_alloc(&flush, flushBytes) != cudaSuccess) {
		cudaGetLastError();
		flush = nullptr; // timed warm if the memory is not there
	}
	for (size_t c = 0; c < candidates.size(); c++) {
		const dsrg_tuning t = candidates[c];
		int status = dsrg_context_set_tuning(ctx, &t);
		if (status != DSRG_OK) {
			if (flush) cudaFree(flush);
			return status;
		}
		status = dsrg_batch_render(b); // warm-up: scratch sizes and graphs for this shape
		if (status != DSRG_OK) {
			if (flush) cudaFree(flush);
			dsrg_context_set_tuning(ctx, &start);
			return status;
		}
		double seconds = -1.0;
		for (int32_t r = 0; r < rounds; r++) {
			if (flush) {
				cudaMemsetAsync(flush, r + 1, flushBytes, ctx->stream);
				cudaStreamSynchronize(ctx->stream);
			}
			const auto t0 = std::chrono::steady_clock::now();
			status = dsrg_batch_render(b);
			const auto t1 = std::chrono::steady_clock::now();
			if (status != DSRG_OK) {
				if (flush) cudaFree(flush);
				dsrg_context_set_tuning(ctx, &start);
				return status;
			}
			const double d = std::chrono::duration<double>(t1 - t0).count();
			if (seconds < 0.0 || d < seconds) seconds = d;
		}
		if (bestSeconds < 0.0 || seconds < bestSeconds) {
			bestSeconds = seconds;
			chosen = t;
		}
		if (c + 1 == shapeCount) {
			for (const int32_t resolve : {0, 2}) {
				dsrg_tuning t = chosen;
				t.resolve = resolve;
				candidates.push_back(t);
			}
		}
	}
	if (flush) cudaFree(flush);
	if (own) b->tuning = chosen; // the context gets its own configuration back (Restore)
	else dsrg_context_set_tuning(ctx, &chosen);
	if (best) *best = chosen;
	return DSRG_OK;
}

} // extern "C"
