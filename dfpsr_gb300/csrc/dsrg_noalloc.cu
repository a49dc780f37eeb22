// dsrg_model_render_depth_noalloc: model_renderDepth for callers that must not allocate GPU
// memory while they render, such as a frame loop that runs under a strict no-allocation
// policy after start-up (cudaMalloc and cudaFree synchronise the whole device and can stall
// other work), or a host that hands the renderer a fixed memory budget up front.
//
// Every buffer the depth path needs between its kernels (projected points, draw records,
// row intervals, tile lists, depth keys, counters) is carved out of one file-scope device
// array of DSRG_NOALLOC_SCRATCH_BYTES, which every GPU that loads the library holds until the
// process exits.  The caller passes the inputs (a model created earlier) and the output
// (a depth image in device memory).
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "dsrg_internal.h"

using namespace dsrg;

static __device__ __align__(256) unsigned char g_noallocScratch[DSRG_NOALLOC_SCRATCH_BYTES];

namespace {

// Per-device device address of g_noallocScratch, looked up once per device.
std::mutex g_scratchMutex;
void *g_scratchAddress[64] = {};

int scratch_address(dsrg_context ctx, unsigned char **out) {
	if (ctx->device < 0 || ctx->device >= 64) return fail(ctx, DSRG_ERROR_UNSUPPORTED, "dsrg_model_render_depth_noalloc: device index above 63");
	std::lock_guard<std::mutex> lock(g_scratchMutex);
	if (!g_scratchAddress[ctx->device]) {
		// The array's name is only a host-side stand-in; its device address must be asked for,
		// with the device current.
		void *p = nullptr;
		cudaError_t e = cudaGetSymbolAddress(&p, g_noallocScratch);
		if (e != cudaSuccess || !p)
			return fail(ctx, DSRG_ERROR_CUDA, std::string("dsrg_model_render_depth_noalloc: cudaGetSymbolAddress failed: ") + cudaGetErrorString(e));
		g_scratchAddress[ctx->device] = p;
	}
	*out = (unsigned char *)g_scratchAddress[ctx->device];
	return DSRG_OK;
}

// Bump allocator over the static array (nothing is ever freed; the layout is rebuilt per call).
struct Carver {
	unsigned char *base;
	size_t used;
	template <typename T>
	T *take(size_t count) {
		size_t at = (used + 255) & ~(size_t)255;
		used = at + count * sizeof(T);
		return (T *)(base + at);
	}
};

const uint32_t MAX_RECORDS = 7u * DSRG_NOALLOC_MAX_TRIANGLES; // a clipped triangle is a fan of at most 7
const uint32_t MAX_TILES = (uint32_t)((DSRG_NOALLOC_MAX_SIDE + 15) / 16) * (uint32_t)((DSRG_NOALLOC_MAX_SIDE + 15) / 16);
const size_t TABLE_BYTES = 4096; // task, frame and base tables of a batch of one

} // namespace

extern "C" int dsrg_model_render_depth_noalloc(dsrg_context ctx, dsrg_model m, const float *modelToWorld,
                                               const dsrg_camera *camera, const dsrg_image *depth) {
	if (!ctx) return DSRG_ERROR_INVALID_ARGUMENT;
	if (!m || !modelToWorld || !camera || !depth || !depth->data)
		return fail(ctx, DSRG_ERROR_INVALID_ARGUMENT, "dsrg_model_render_depth_noalloc: null argument");
	if (!depth->onDevice)
		return fail(ctx, DSRG_ERROR_INVALID_ARGUMENT, "dsrg_model_render_depth_noalloc: the depth image must be device memory (onDevice = 1)");
	if (depth->width <= 0 || depth->height <= 0 || depth->strideBytes < depth->width * 4 || depth->strideBytes % 4 != 0)
		return fail(ctx, DSRG_ERROR_INVALID_ARGUMENT, "dsrg_model_render_depth_noalloc: invalid depth image");
	if (depth->width > DSRG_NOALLOC_MAX_SIDE || depth->height > DSRG_NOALLOC_MAX_SIDE)
		return fail(ctx, DSRG_ERROR_UNSUPPORTED, "dsrg_model_render_depth_noalloc: depth image larger than DSRG_NOALLOC_MAX_SIDE (1024) pixels on a side");
	if (m->pointCount > DSRG_NOALLOC_MAX_POINTS)
		return fail(ctx, DSRG_ERROR_UNSUPPORTED, "dsrg_model_render_depth_noalloc: model has more than DSRG_NOALLOC_MAX_POINTS (49152) points");
	if (m->triangleCount > DSRG_NOALLOC_MAX_TRIANGLES)
		return fail(ctx, DSRG_ERROR_UNSUPPORTED, "dsrg_model_render_depth_noalloc: model has more than DSRG_NOALLOC_MAX_TRIANGLES (16384) triangles");
	if (camera->width <= 0 || camera->height <= 0)
		return fail(ctx, DSRG_ERROR_INVALID_ARGUMENT, "dsrg_model_render_depth_noalloc: camera without image size");
	DSRG_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
	unsigned char *base = nullptr;
	int status = scratch_address(ctx, &base);
	if (status != DSRG_OK) return status;

	CameraData cam = make_camera(*camera);
	if (!box_seen(cam, m->minBound, m->maxBound, modelToWorld)) return DSRG_OK; // ModelImpl::renderDepth (Model.cpp:199-211)
	if (m->triangleCount == 0) return DSRG_OK;
	cudaStream_t stream = ctx->stream;
	const int32_t width = depth->width, height = depth->height;

	// carve the scratch
	Carver carve{base, 0};
	const size_t np = (size_t)DSRG_NOALLOC_MAX_POINTS;
	FrameBuffers fb;
	memset(&fb, 0, sizeof(fb));
	fb.points.csis = carve.take<float4>(np); fb.points.isy = carve.take<float>(np); fb.points.flat = carve.take<longlong2>(np);
	fb.triCounts = carve.take<uint32_t>(DSRG_NOALLOC_MAX_TRIANGLES + 2);
	fb.triOffsets = carve.take<uint32_t>(DSRG_NOALLOC_MAX_TRIANGLES + 2);
	fb.records = carve.take<DrawRecord>(MAX_RECORDS);
	uint32_t *rowCounts = carve.take<uint32_t>(MAX_RECORDS + 2);
	fb.rowOffsets = carve.take<uint32_t>(MAX_RECORDS + 2);
	fb.rows = carve.take<uint32_t>(DSRG_NOALLOC_MAX_ROWS);
	uint32_t *control = carve.take<uint32_t>(4); // [0] tile queue, [1] error flag
	fb.errorFlag = (int32_t *)(control + 1);
	fb.scanScratchElems = scan_scratch_elems(MAX_RECORDS + 2);
	fb.scanScratch = carve.take<uint32_t>(fb.scanScratchElems);
	TileBins bins;
	memset(&bins, 0, sizeof(bins)); // no deferred big-record list: every record is binned in one launch
	bins.counts = carve.take<uint32_t>(2 * MAX_TILES + 1);
	bins.offsets = carve.take<uint32_t>(2 * MAX_TILES + 1);
	bins.cursors = carve.take<uint32_t>(2 * MAX_TILES + 1);
	bins.lists = carve.take<uint32_t>(DSRG_NOALLOC_MAX_BIN_ENTRIES);
	bins.listCapacity = DSRG_NOALLOC_MAX_BIN_ENTRIES;
	unsigned long long *keys = carve.take<unsigned long long>((size_t)DSRG_NOALLOC_MAX_SIDE * DSRG_NOALLOC_MAX_SIDE);
	unsigned char *tables = carve.take<unsigned char>(TABLE_BYTES);
	if (carve.used > (size_t)DSRG_NOALLOC_SCRATCH_BYTES)
		return fail(ctx, DSRG_ERROR_DEVICE, "dsrg_model_render_depth_noalloc: scratch layout exceeds DSRG_NOALLOC_SCRATCH_BYTES");

	// the task and frame tables of a batch of one (renderTriangleFromDataDepth, renderCore.cpp:400-443)
	TaskParams task;
	memset(&task, 0, sizeof(task));
	task.positions = m->positions;
	task.polygons = m->polygons;
	task.texCoords = m->texCoords;
	task.colors = m->colors;
	task.triSource = m->triSource;
	task.pointCount = m->pointCount;
	task.triangleCount = m->triangleCount;
	memcpy(task.modelToWorld, modelToWorld, sizeof(task.modelToWorld));
	task.camera = cam;
	task.diffuse = -1;
	task.light = -1;
	task.depthOnly = 1;
	FrameTarget frame;
	memset(&frame, 0, sizeof(frame));
	frame.depth = (float *)depth->data;
	frame.depthStride = depth->strideBytes / 4;
	frame.width = width;
	frame.height = height;
	frame.affine = camera->perspective ? 0 : 1;
	BatchParams params;
	memset(&params, 0, sizeof(params));
	BatchTotals totals;
	alignas(16) unsigned char hostTables[TABLE_BYTES];
	const size_t tableBytes = layout_tables(&task, 1, &frame, 1, nullptr, 0, true, keys, hostTables, tables, params, totals);
	if (tableBytes > TABLE_BYTES) return fail(ctx, DSRG_ERROR_DEVICE, "dsrg_model_render_depth_noalloc: table layout exceeds its scratch");
	params.smallRows = ctx->smallRows;
	params.smallWidth = ctx->smallWidth;
	params.tileQueue = control;
	// pageable source: the copy is staged before the call returns, so the stack array may go
	DSRG_CUDA_TRY(ctx, cudaMemcpyAsync(tables, hostTables, tableBytes, cudaMemcpyHostToDevice, stream));
	// the counters start at zero on every call: the array keeps whatever the previous call left
	DSRG_CUDA_TRY(ctx, cudaMemsetAsync(control, 0, 4 * sizeof(uint32_t), stream));
	launch_project(params, fb, stream);
	launch_setup_count(params, fb, stream);
	uint32_t recordCount = 0;
	DSRG_CUDA_TRY(ctx, cudaMemcpyAsync(&recordCount, fb.triOffsets + totals.triangles, sizeof(uint32_t), cudaMemcpyDeviceToHost, stream));
	DSRG_CUDA_TRY(ctx, cudaStreamSynchronize(stream));
	if (recordCount > MAX_RECORDS) return fail(ctx, DSRG_ERROR_DEVICE, "dsrg_model_render_depth_noalloc: more draw records than its scratch holds");

	// records, row intervals and tile lists
	launch_setup_write(params, fb, MAX_RECORDS, stream);
	launch_row_offsets(fb, recordCount, rowCounts, stream);
	launch_bin_count(params, fb, recordCount, bins, stream);
	uint32_t totalsRead[3] = {0, 0, 0};
	DSRG_CUDA_TRY(ctx, cudaMemcpyAsync(&totalsRead[0], fb.rowOffsets + recordCount, sizeof(uint32_t), cudaMemcpyDeviceToHost, stream));
	DSRG_CUDA_TRY(ctx, cudaMemcpyAsync(&totalsRead[1], bins.offsets + 2 * (size_t)totals.tiles, sizeof(uint32_t), cudaMemcpyDeviceToHost, stream));
	DSRG_CUDA_TRY(ctx, cudaMemcpyAsync(&totalsRead[2], control + 1, sizeof(uint32_t), cudaMemcpyDeviceToHost, stream));
	DSRG_CUDA_TRY(ctx, cudaStreamSynchronize(stream));
	if (totalsRead[2] != 0) return fail(ctx, DSRG_ERROR_DEVICE, "dsrg_model_render_depth_noalloc: triangle setup reported device error bits " + std::to_string(totalsRead[2]));
	if (totalsRead[0] > DSRG_NOALLOC_MAX_ROWS)
		return fail(ctx, DSRG_ERROR_UNSUPPORTED, "dsrg_model_render_depth_noalloc: the visible triangles span more than DSRG_NOALLOC_MAX_ROWS (2097152) pixel rows");
	if (totalsRead[1] > DSRG_NOALLOC_MAX_BIN_ENTRIES)
		return fail(ctx, DSRG_ERROR_UNSUPPORTED, "dsrg_model_render_depth_noalloc: the visible triangles touch more than DSRG_NOALLOC_MAX_BIN_ENTRIES (1048576) tiles in total");
	launch_rows(fb, recordCount, false, stream);
	launch_bin_fill(params, fb, recordCount, bins, stream);

	// depth raster (executeTriangleDrawingDepth, renderCore.cpp:343-387) and resolve
	RasterConfig config;
	config.threadsPerTile = ctx->threadsPerTile;
	config.ctasPerSm = ctx->ctasPerSm;
	config.resolveMode = 0; // depth only: the per-pixel depth resolve
	launch_raster(params, fb, bins, config, true, stream);
	DSRG_CUDA_TRY(ctx, take_enqueue_error());
	DSRG_CUDA_TRY(ctx, cudaGetLastError());
	uint32_t errorBits = 0;
	DSRG_CUDA_TRY(ctx, cudaMemcpyAsync(&errorBits, control + 1, sizeof(uint32_t), cudaMemcpyDeviceToHost, stream));
	DSRG_CUDA_TRY(ctx, cudaStreamSynchronize(stream));
	if (errorBits != 0) return fail(ctx, DSRG_ERROR_DEVICE, "dsrg_model_render_depth_noalloc: device error bits " + std::to_string(errorBits));
	return DSRG_OK;
}
