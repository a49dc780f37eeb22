// Host side of one batch through the kernels: table layout, scratch sizing and the three
// launch phases, shared by the renderer (one frame), the batch API (many frames) and the
// differentiable renderer.  Between the phases the host reads two totals (draw records, then
// row intervals and tile-list entries) to size the next phase's buffers exactly.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <string>

#include "dsrg_internal.h"

namespace dsrg {

static size_t align16(size_t x) { return (x + 15) & ~(size_t)15; }

size_t layout_tables(TaskParams *tasks, size_t taskCount, FrameTarget *frames, size_t frameCount, const TextureData *textures,
                     size_t textureCount, bool depthOnly, unsigned long long *keysBase, unsigned char *host,
                     unsigned char *deviceBase, BatchParams &params, BatchTotals &totals) {
	// bases
	uint32_t points = 0, triangles = 0, tiles = 0;
	size_t pixels = 0;
	for (size_t i = 0; i < taskCount; i++) {
		TaskParams &t = tasks[i];
		t.pointBase = points;
		t.triangleBase = triangles;
		points += (uint32_t)t.pointCount;
		triangles += (uint32_t)t.triangleCount;
	}
	for (size_t i = 0; i < frameCount; i++) {
		FrameTarget &f = frames[i];
		f.tilesX = (f.width + TILE_W - 1) / TILE_W;
		f.tilesY = (f.height + TILE_H - 1) / TILE_H;
		f.tileBase = tiles;
		tiles += (uint32_t)(f.tilesX * f.tilesY);
		f.keys = keysBase ? keysBase + pixels : nullptr;
		pixels += (size_t)f.width * f.height;
	}
	totals.points = points;
	totals.triangles = triangles;
	totals.tiles = tiles;
	totals.pixels = pixels;
	// layout
	const size_t taskOffset = 0;
	const size_t pointBaseOffset = align16(taskOffset + taskCount * sizeof(TaskParams));
	const size_t triangleBaseOffset = align16(pointBaseOffset + (taskCount + 1) * sizeof(uint32_t));
	const size_t frameOffset = align16(triangleBaseOffset + (taskCount + 1) * sizeof(uint32_t));
	const size_t frameTileOffset = align16(frameOffset + frameCount * sizeof(FrameTarget));
	const size_t textureOffset = align16(frameTileOffset + (frameCount + 1) * sizeof(uint32_t));
	const size_t bytes = align16(textureOffset + (textureCount + 1) * sizeof(TextureData));
	if (host) {
		memset(host, 0, bytes);
		if (taskCount) memcpy(host + taskOffset, tasks, taskCount * sizeof(TaskParams));
		uint32_t *pointBase = (uint32_t *)(host + pointBaseOffset), *triangleBase = (uint32_t *)(host + triangleBaseOffset);
		for (size_t i = 0; i < taskCount; i++) { pointBase[i] = tasks[i].pointBase; triangleBase[i] = tasks[i].triangleBase; }
		pointBase[taskCount] = points;
		triangleBase[taskCount] = triangles;
		if (frameCount) memcpy(host + frameOffset, frames, frameCount * sizeof(FrameTarget));
		uint32_t *frameTile = (uint32_t *)(host + frameTileOffset);
		for (size_t i = 0; i < frameCount; i++) frameTile[i] = frames[i].tileBase;
		frameTile[frameCount] = tiles;
		if (textureCount) memcpy(host + textureOffset, textures, textureCount * sizeof(TextureData));
	}
	params.tasks = (const TaskParams *)(deviceBase + taskOffset);
	params.taskPointBase = (const uint32_t *)(deviceBase + pointBaseOffset);
	params.taskTriangleBase = (const uint32_t *)(deviceBase + triangleBaseOffset);
	params.taskCount = (int32_t)taskCount;
	params.frames = (const FrameTarget *)(deviceBase + frameOffset);
	params.frameTileBase = (const uint32_t *)(deviceBase + frameTileOffset);
	params.frameCount = (int32_t)frameCount;
	params.textures = (const TextureData *)(deviceBase + textureOffset);
	params.totalPoints = points;
	params.totalTriangles = triangles;
	params.totalTiles = tiles;
	params.depthOnly = depthOnly ? 1 : 0;
	params.oddDepthFrames = 0;
	params.maxTilesX = 0;
	for (size_t i = 0; i < frameCount; i++) {
		if ((frames[i].height & 1) && frames[i].depth) params.oddDepthFrames++;
		params.maxTilesX = std::max(params.maxTilesX, frames[i].tilesX);
	}
	return bytes;
}

size_t layout_tables(BatchJob &job, unsigned long long *keysBase, unsigned char *host, unsigned char *deviceBase,
                     BatchParams &params, BatchTotals &totals) {
	return layout_tables(job.tasks.data(), job.tasks.size(), job.frames.data(), job.frames.size(), job.textures.data(),
	                     job.textures.size(), job.depthOnly, keysBase, host, deviceBase, params, totals);
}

#define TRY(expr) DSRG_CUDA_TRY(ctx, expr)

// Launch parameters of one phase; compared byte for byte, so it is cleared before it is filled.
struct PhaseKey {
	int32_t phase;
	int32_t resolve;
	int32_t alpha;
	uint32_t recordCount;
	uint32_t entries;
	AlphaBuffers alphaBuffers;
	RasterConfig config;
	BatchParams params;
	FrameBuffers fb;
	TileBins bins;
	uint32_t *rowCounts;
};

// Runs one phase's launches on the context's stream, through its graph when the phase repeats.
template <typename Launches>
static cudaError_t run_phase(dsrg_context ctx, PhaseGraph &g, const PhaseKey &key, Launches launches) {
	const unsigned char *k = reinterpret_cast<const unsigned char *>(&key);
	const bool same = g.key.size() == sizeof(key) && memcmp(g.key.data(), k, sizeof(key)) == 0;
	if (!ctx->useGraphs || !same) {
		if (!same) {
			if (g.exec) cudaGraphExecDestroy(g.exec);
			g.exec = nullptr;
			g.key.assign(k, k + sizeof(key));
		}
		launches();
		const cudaError_t enqueued = take_enqueue_error();
		const cudaError_t launched = cudaGetLastError();
		return enqueued != cudaSuccess ? enqueued : launched;
	}
	if (g.exec) {
		add_launches(g.launches);
		return cudaGraphLaunch(g.exec, ctx->stream);
	}
	const uint64_t before = launch_count();
	cudaError_t e = cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal);
	if (e != cudaSuccess) return e;
	launches();
	const cudaError_t enqueued = take_enqueue_error();
	const cudaError_t refused = cudaGetLastError(); // a launch refused while capturing
	const cudaError_t launched = enqueued != cudaSuccess ? enqueued : refused;
	cudaGraph_t graph = nullptr;
	e = cudaStreamEndCapture(ctx->stream, &graph);
	if (e != cudaSuccess) return e;
	if (launched != cudaSuccess) {
		cudaGraphDestroy(graph);
		return launched;
	}
	g.launches = launch_count() - before;
	e = cudaGraphInstantiate(&g.exec, graph, 0);
	cudaGraphDestroy(graph);
	if (e != cudaSuccess) {
		g.exec = nullptr;
		return e;
	}
	return cudaGraphLaunch(g.exec, ctx->stream);
}

static int enqueue_phases(dsrg_context ctx, BatchJob &job, BatchTotals &totals, BatchOutputs *outputs) {
	cudaStream_t stream = ctx->stream;
	ctx->stopRecorded = false;
	totals = BatchTotals();
	BatchParams params;
	memset(&params, 0, sizeof(params));
	// sizes first, then the buffers, then the tables with their final device addresses
	const size_t tableBytes = layout_tables(job, nullptr, nullptr, nullptr, params, totals);
	if (totals.pixels > 0) TRY(ctx->keys.reserve(totals.pixels));
	TRY(ctx->tables.reserve(tableBytes));
	TRY(ctx->tileList.reserve((size_t)totals.tiles + 1));
	if (ctx->pinnedCapacity < tableBytes) {
		if (ctx->pinnedTables) cudaFreeHost(ctx->pinnedTables);
		ctx->pinnedTables = nullptr;
		ctx->pinnedCapacity = 0;
		size_t capacity = 4096;
		while (capacity < tableBytes) capacity *= 2;
		TRY(cudaMallocHost((void **)&ctx->pinnedTables, capacity));
		ctx->pinnedCapacity = capacity;
	}
	layout_tables(job, ctx->keys.ptr, ctx->pinnedTables, ctx->tables.ptr, params, totals);
	TRY(cudaMemcpyAsync(ctx->tables.ptr, ctx->pinnedTables, tableBytes, cudaMemcpyHostToDevice, stream));
	// without the resolve pass the caller reads every key, also where no tile was drawn
	if (!job.resolve && totals.pixels > 0) TRY(cudaMemsetAsync(ctx->keys.ptr, 0, totals.pixels * sizeof(unsigned long long), stream));
	params.smallRows = ctx->smallRows;
	params.smallWidth = ctx->smallWidth;
	params.tileQueue = ctx->control.ptr;
	// depth-only batches (shadow-cube faces) are mostly empty tiles: their tile kernel pulls only
	// the listed ones.  Colour frames pull every tile in order, which measured faster for them
	// (the listed order is not the tile order, and the list costs a wider totals launch).
	params.tileList = job.depthOnly ? ctx->tileList.ptr : nullptr;
	params.tileListCount = job.depthOnly ? ctx->control.ptr + 9 : nullptr;
	params.fragments = nullptr;
	params.walked = ctx->fragmentCounter.ptr + 1;
	if (ctx->counting && !job.clearCounters) {
		params.fragments = ctx->fragmentCounter.ptr;
	} else if (ctx->counting) {
		TRY(cudaMemsetAsync(ctx->fragmentCounter.ptr, 0, sizeof(unsigned long long), stream));
		params.fragments = ctx->fragmentCounter.ptr;
		for (const FrameTarget &f : job.frames)
			if (f.coverage) TRY(cudaMemsetAsync(f.coverage, 0, (size_t)f.width * f.height * sizeof(uint32_t), stream));
	}
	if (totals.triangles == 0) return DSRG_OK; // nothing reaches the tiles: the targets stay as they are
	params.errorFlag = (const int32_t *)(ctx->control.ptr + 1);
	RasterConfig config;
	config.threadsPerTile = ctx->threadsPerTile;
	config.ctasPerSm = ctx->ctasPerSm;
	// fewer triangles than one per 8 pixels: tall triangles, whose rows are balanced by row
	const bool tallTriangles = (uint64_t)totals.triangles * 8u <= (uint64_t)totals.pixels;
	// how winners are shaded (the context's tuning); targets in host memory take the per-pixel
	// stores inside the tile kernel (2x2 quads scatter small writes over the link)
	config.resolveMode = ctx->resolveMode == 2 && job.hostTargets ? 1 : ctx->resolveMode;

	// Buffers whose sizes depend on earlier phases are sized from the context's capacities (the
	// largest totals seen, with slack); the phases then run back to back with no host round trip.
	// A total above its capacity sets an overflow bit, the tile and resolve kernels return at once,
	// and batch_enqueue redoes the batch with the capacities the totals asked for.
	const size_t np = totals.points, nt = totals.triangles;
	const uint32_t recordCap = (uint32_t)std::max<uint64_t>(ctx->recordCapacity, nt + nt / 8 + 1024);
	const uint32_t rowCap = (uint32_t)std::max<uint64_t>(ctx->rowCapacity, (uint64_t)recordCap * 4);
	const uint32_t binCap = (uint32_t)std::max<uint64_t>(ctx->binCapacity, (uint64_t)recordCap * 2);
	TRY(ctx->pointCsis.reserve(np)); TRY(ctx->pointIsy.reserve(np)); TRY(ctx->pointFlat.reserve(np));
	TRY(ctx->triCounts.reserve(nt + 1));
	TRY(ctx->triOffsets.reserve(nt + 1));
	TRY(ctx->records.reserve((size_t)recordCap + 1));
	TRY(ctx->rowCounts.reserve((size_t)recordCap + 1));
	TRY(ctx->rowOffsets.reserve((size_t)recordCap + 1));
	TRY(ctx->rows.reserve((size_t)rowCap + 2));
	TRY(ctx->binCounts.reserve(2 * (size_t)totals.tiles + 1));
	TRY(ctx->binOffsets.reserve(2 * (size_t)totals.tiles + 1));
	TRY(ctx->binCursors.reserve(2 * (size_t)totals.tiles + 1));
	TRY(ctx->binLists.reserve((size_t)binCap + 1));
	TRY(ctx->bigList.reserve((size_t)recordCap + 1));
	const uint64_t largest = std::max<uint64_t>(std::max<uint64_t>(nt, recordCap), 2 * (uint64_t)totals.tiles);
	// the row and tile-list scans share one launch pair, with both arrays' chunk sums in the scratch
	TRY(ctx->scanScratch.reserve(std::max(scan_scratch_elems((uint32_t)largest + 1),
	                                      scan_scratch_elems(recordCap + 1) + scan_scratch_elems(2 * (uint32_t)totals.tiles + 1))));
	FrameBuffers fb;
	memset(&fb, 0, sizeof(fb));
	fb.points.csis = ctx->pointCsis.ptr; fb.points.isy = ctx->pointIsy.ptr; fb.points.flat = ctx->pointFlat.ptr;
	fb.triCounts = ctx->triCounts.ptr;
	fb.triOffsets = ctx->triOffsets.ptr;
	fb.records = ctx->records.ptr;
	fb.rowOffsets = ctx->rowOffsets.ptr;
	fb.rows = ctx->rows.ptr;
	fb.errorFlag = (int32_t *)(ctx->control.ptr + 1);
	fb.scanScratch = ctx->scanScratch.ptr;
	fb.scanScratchElems = ctx->scanScratch.capacity;
	fb.recordCountDevice = fb.triOffsets + nt;
	fb.rowCapacity = rowCap;
	TileBins bins;
	memset(&bins, 0, sizeof(bins));
	bins.counts = ctx->binCounts.ptr;
	bins.offsets = ctx->binOffsets.ptr;
	bins.cursors = ctx->binCursors.ptr;
	bins.lists = ctx->binLists.ptr;
	bins.listCapacity = binCap;
	bins.bigList = ctx->bigList.ptr;
	bins.bigCount = ctx->control.ptr + 8;
	bins.cleared = 1; // by the first launch of phase A
	uint32_t *rowCounts = ctx->rowCounts.ptr;
	uint32_t *gathered = ctx->readbackDevice; // records, rows, bin entries, error bits: written into host memory
	PhaseKey key;
	memset(&key, 0, sizeof(key));
	key.resolve = job.resolve ? 1 : 0;
	key.alpha = job.alpha ? 1 : 0;
	key.config = config;
	key.params = params;
	key.fb = fb;
	key.bins = bins;
	key.rowCounts = rowCounts;
	key.recordCount = recordCap;
	key.phase = 0;
	// phases A (projection, record counts), B (records, row offsets, tile counts) and C (row
	// intervals, tile lists) as one graph, then D (tiles and resolve) for solid batches as another
	TRY(run_phase(ctx, ctx->graphs[0], key, [&] {
		launch_clear_tiles(params, bins, fb.errorFlag, stream);
		launch_project(params, fb, stream);
		launch_setup_count(params, fb, stream);
		// the row offsets and intervals on a second branch right after the records, the tile counts,
		// offsets and lists on this one: neither needs the other; joined before the totals
		launch_setup_write_counting(params, fb, recordCap, rowCounts, bins, stream, ctx->branchStream, ctx->branchFork);
		launch_rows(fb, recordCap, tallTriangles, ctx->branchStream);
		launch_bin_fill(params, fb, recordCap, bins, stream);
		enqueue_join(ctx->branchStream, stream, ctx->branchJoin);
		launch_gather_totals(fb.triOffsets, (uint32_t)nt, fb.rowOffsets, recordCap, bins.offsets, totals.tiles, fb.errorFlag,
		                     gathered, params.tileList, params.tileListCount, stream);
	}));
	if (!job.alpha) {
		// phase D right behind, timed on the stream between the two graphs; after an overflow its
		// kernels return at once and the targets stay untouched
		TRY(cudaEventRecord(ctx->eventRasterStart, stream));
		key.phase = 1;
		TRY(run_phase(ctx, ctx->graphs[1], key, [&] { launch_raster(params, fb, bins, config, job.resolve, stream); }));
		TRY(cudaEventRecord(ctx->eventRasterStop, stream));
		// the batch's own work ends here: the one host wait below also completes the timing events
		TRY(cudaEventRecord(ctx->eventStop, stream));
		if (ctx->counting)
			TRY(cudaMemcpyAsync(ctx->pinnedReadback + 4, ctx->fragmentCounter.ptr, sizeof(unsigned long long), cudaMemcpyDeviceToHost,
			                    stream));
	}
	TRY(cudaStreamSynchronize(stream));
	ctx->stopRecorded = !job.alpha;
	totals.records = ctx->pinnedReadback[0];
	totals.rows = ctx->pinnedReadback[1];
	totals.binEntries = ctx->pinnedReadback[2];
	const uint32_t errorBits = ctx->pinnedReadback[3];
	if (errorBits & ERROR_OVERFLOW_BITS) {
		// the capacities the totals ask for; a total counted past an overflowed buffer is a lower bound
		const bool recordsOver = totals.records > recordCap;
		ctx->recordCapacity = std::max<uint64_t>(ctx->recordCapacity, (uint64_t)totals.records + totals.records / 4 + 1024);
		if (!recordsOver) {
			ctx->rowCapacity = std::max<uint64_t>(ctx->rowCapacity, (uint64_t)totals.rows + totals.rows / 4 + 1024);
			ctx->binCapacity = std::max<uint64_t>(ctx->binCapacity, (uint64_t)totals.binEntries + totals.binEntries / 4 + 1024);
		}
		return DSRG_RETRY;
	}
	if (errorBits != 0) return fail(ctx, DSRG_ERROR_DEVICE, "triangle setup reported device error bits " + std::to_string(errorBits));
	if (job.alpha) {
		// blending in submission order: sorted tile lists, one thread per pixel (needs the entry count)
		TRY(cudaEventRecord(ctx->eventRasterStart, stream));
		const uint64_t n = totals.binEntries;
		const uint32_t blocks = sort_blocks(n);
		TRY(ctx->alphaEntryTile.reserve(n + 1)); TRY(ctx->alphaTileKeys.reserve(n + 1)); TRY(ctx->alphaRecords.reserve(n + 1));
		TRY(ctx->sortKeysA.reserve(n + 1)); TRY(ctx->sortKeysB.reserve(n + 1));
		TRY(ctx->sortIdsA.reserve(n + 1)); TRY(ctx->sortIdsB.reserve(n + 1));
		TRY(ctx->sortHist.reserve((size_t)256 * blocks + 1)); TRY(ctx->sortOffsets.reserve((size_t)256 * blocks + 1));
		TRY(ctx->scanScratch.reserve(scan_scratch_elems((uint32_t)((size_t)256 * blocks) + 1)));
		AlphaBuffers a;
		memset(&a, 0, sizeof(a));
		a.entryTile = ctx->alphaEntryTile.ptr; a.tileKeys = ctx->alphaTileKeys.ptr; a.records = ctx->alphaRecords.ptr;
		a.sort.keysA = ctx->sortKeysA.ptr; a.sort.keysB = ctx->sortKeysB.ptr;
		a.sort.idsA = ctx->sortIdsA.ptr; a.sort.idsB = ctx->sortIdsB.ptr;
		a.sort.hist = ctx->sortHist.ptr; a.sort.offsets = ctx->sortOffsets.ptr;
		a.sort.scanScratch = ctx->scanScratch.ptr; a.sort.scanScratchElems = ctx->scanScratch.capacity;
		key.phase = 3;
		key.entries = totals.binEntries;
		key.alphaBuffers = a;
		key.recordCount = totals.records;
		TRY(run_phase(ctx, ctx->graphs[3], key, [&] { launch_alpha(params, fb, bins, totals.binEntries, totals.records, a, stream); }));
		TRY(cudaEventRecord(ctx->eventRasterStop, stream));
	}
	if (outputs) {
		outputs->params = params;
		outputs->fb = fb;
	}
	return DSRG_OK;
}

int batch_enqueue(dsrg_context ctx, BatchJob &job, BatchTotals &totals, BatchOutputs *outputs) {
	if (outputs) memset(outputs, 0, sizeof(*outputs));
	int status = DSRG_RETRY;
	// a batch whose totals outgrow the capacities is redone once per buffer that was too small
	for (int attempt = 0; attempt < 4 && status == DSRG_RETRY; attempt++) status = enqueue_phases(ctx, job, totals, outputs);
	if (status == DSRG_RETRY) return fail(ctx, DSRG_ERROR_DEVICE, "batch buffers kept overflowing");
	if (status == DSRG_OK && !ctx->stopRecorded) TRY(cudaEventRecord(ctx->eventStop, ctx->stream));
	return status;
}

int occlude_enqueue(dsrg_context ctx, BatchJob &job) {
	cudaStream_t stream = ctx->stream;
	BatchTotals totals;
	BatchParams params;
	memset(&params, 0, sizeof(params));
	const size_t tableBytes = layout_tables(job, nullptr, nullptr, nullptr, params, totals);
	if (totals.triangles == 0) return DSRG_OK;
	TRY(ctx->tables.reserve(tableBytes));
	if (ctx->pinnedCapacity < tableBytes) {
		if (ctx->pinnedTables) cudaFreeHost(ctx->pinnedTables);
		ctx->pinnedTables = nullptr;
		ctx->pinnedCapacity = 0;
		size_t capacity = 4096;
		while (capacity < tableBytes) capacity *= 2;
		TRY(cudaMallocHost((void **)&ctx->pinnedTables, capacity));
		ctx->pinnedCapacity = capacity;
	}
	layout_tables(job, nullptr, ctx->pinnedTables, ctx->tables.ptr, params, totals);
	TRY(cudaMemcpyAsync(ctx->tables.ptr, ctx->pinnedTables, tableBytes, cudaMemcpyHostToDevice, stream));
	const size_t np = totals.points;
	TRY(ctx->pointCsis.reserve(np)); TRY(ctx->pointIsy.reserve(np)); TRY(ctx->pointFlat.reserve(np));
	FrameBuffers fb;
	memset(&fb, 0, sizeof(fb));
	fb.points.csis = ctx->pointCsis.ptr; fb.points.isy = ctx->pointIsy.ptr; fb.points.flat = ctx->pointFlat.ptr;
	fb.errorFlag = (int32_t *)(ctx->control.ptr + 1);
	launch_project(params, fb, stream);
	launch_setup_occlude(params, fb, stream);
	TRY(take_enqueue_error());
	TRY(cudaGetLastError());
	// the page-locked tables are rewritten by the next batch: wait for their copy (and the grid)
	TRY(cudaStreamSynchronize(stream));
	return DSRG_OK;
}

// Only the setup, row and binning kernels raise error bits, and enqueue_phases has read them
// after those (gather_totals_kernel): what is left is the fragment count and one wait for the
// work the caller queued after the batch (image copies, overlays), if any.
int batch_finish(dsrg_context ctx, const BatchTotals &totals) {
	cudaStream_t stream = ctx->stream;
	unsigned long long fragments = 0;
	uint32_t *readback = ctx->pinnedReadback + 4;
	if (ctx->counting && !ctx->stopRecorded)
		TRY(cudaMemcpyAsync(readback, ctx->fragmentCounter.ptr, sizeof(fragments), cudaMemcpyDeviceToHost, stream));
	TRY(cudaStreamSynchronize(stream));
	if (ctx->counting) memcpy(&fragments, readback, sizeof(fragments));
	ctx->stopRecorded = false;
	ctx->timingPending = true;
	ctx->timingHasRaster = totals.triangles > 0;
	ctx->stats.fragments = fragments;
	ctx->stats.drawRecords = totals.records;
	ctx->stats.binEntries = totals.binEntries;
	ctx->stats.kernelLaunches = launch_count();
	return DSRG_OK;
}

} // namespace dsrg
