// Launch interface of the kernels of the DFPSR triangle path (host side).
//
// Every launch covers a whole batch: any number of frames (target image pairs), each drawn by
// any number of tasks (models with a transform and a camera).  model_render is a batch of one
// frame with one task, renderer_begin/giveTask/end one frame with several tasks.
#ifndef DSRG_KERNELS_H
#define DSRG_KERNELS_H

#include <cuda_runtime.h>
#include <stdint.h>
#include "dsrg_types.h"

namespace dsrg {

// One model submitted to a frame: model_render / renderer_giveTask (api/modelAPI.cpp:197-281).
struct TaskParams {
	const float *positions;   // pointCount x 3
	const int32_t *polygons;  // polygonCount x 4
	const float *texCoords;   // polygonCount x 4 x 4
	const float *colors;      // polygonCount x 4 x 4
	const int32_t *triSource; // per fan triangle: polygon * 2 + fan index
	int32_t pointCount;
	int32_t triangleCount;
	uint32_t pointBase;       // this task's first projected point in the batch
	uint32_t triangleBase;    // this task's first fan triangle in the batch
	uint32_t orderBase;       // fan triangles submitted earlier to the same frame
	int32_t frame;            // the frame this task draws into
	float modelToWorld[12];
	CameraData camera;
	int32_t filter;           // 0 Solid, 1 Alpha
	int32_t diffuse, light;   // indices into the batch's texture table, -1 for none
	int32_t depthOnly;        // model_renderDepth: 1x1 alignment, no shading (renderCore.cpp:343-443)
	const GivenPoint *given;  // renderer_giveTask_triangle: the corners come projected (positions unused)
};

// One frame of a batch: its target images, its key image and its range of tiles.
struct FrameTarget {
	uint32_t *color;          // device pointer or null
	int32_t colorStride;      // in pixels
	int32_t packOrder;
	float *depth;             // device pointer or null
	int32_t depthStride;
	int32_t width, height;
	int32_t affine;           // orthogonal camera: depth test '<' on linear depth
	unsigned long long *keys; // width * height winning (depth, record) keys, written by the tile pass
	uint32_t *coverage;       // optional per-pixel fragment counts (width * height, dense)
	uint32_t tileBase;        // the frame's first tile in the batch
	int32_t tilesX, tilesY;
	float *occlusion;         // the renderer's occlusion grid (gridWidth x gridHeight cells) or null
	int32_t gridWidth, gridHeight, gridStride;
};

// Device tables of a batch.
struct BatchParams {
	const TaskParams *tasks;
	const uint32_t *taskPointBase;    // taskCount + 1 prefix sums of point counts
	const uint32_t *taskTriangleBase; // taskCount + 1 prefix sums of fan-triangle counts
	int32_t taskCount;
	const FrameTarget *frames;
	const uint32_t *frameTileBase;    // frameCount + 1 prefix sums of tile counts
	int32_t frameCount;
	uint32_t totalPoints, totalTriangles, totalTiles;
	const TextureData *textures;
	unsigned long long *fragments;    // optional fragment total
	unsigned long long *walked;       // optional running total of the fragments the tile kernels depth-tested
	int32_t smallRows;                // records whose raster bound is at most smallRows x smallWidth pixels
	int32_t smallWidth;               // are walked by one lane each instead of by the whole warp
	int32_t depthOnly;                // the whole batch is model_renderDepth (1x1 walk)
	int32_t oddDepthFrames;           // frames of odd height with a depth buffer (their last row: odd_row_kernel)
	int32_t maxTilesX;                // the widest frame's tile columns
	uint32_t *tileQueue;              // work counter of the persistent tile kernel
	uint32_t *tileList;               // the tiles that have list entries (written at the end of phase C), or null: every tile
	uint32_t *tileListCount;          // their number
	const int32_t *errorFlag;         // device error bits; tile and resolve kernels return when an overflow is set
};

// Projected corners (implementation/render/ProjectedPoint.h:33-49): the camera-space position and
// the image x in one 16-byte vector, the image y, and both sub-pixel coordinates in one 16-byte
// vector, so that the triangle setup gathers a corner with three loads.
struct ProjectedPoints {
	float4 *csis;     // cs.x, cs.y, cs.z, is.x
	float *isy;       // is.y
	longlong2 *flat;  // flat x, flat y
};

struct FrameBuffers {
	ProjectedPoints points;
	uint32_t *triCounts;      // per fan triangle: draw records it emits
	uint32_t *triOffsets;     // exclusive scan of triCounts, total at [totalTriangles]
	DrawRecord *records;
	uint32_t *rowOffsets;     // per record: first entry of its rows in `rows` (+ total at [recordCount])
	uint32_t *rows;           // row intervals of every record, left | right << 16
	int32_t *errorFlag;       // device error bits
	uint32_t *scanScratch;
	size_t scanScratchElems;
	// when set, the record count is read on the device (at most the host count given to the
	// launches, which then bounds the grids), and rows hold at most rowCapacity entries
	const uint32_t *recordCountDevice;
	uint32_t rowCapacity;
	// when rowCounts is set, the record-writing setup pass also writes every record's row count and
	// counts its tiles (bins of up to four tiles; larger records go to bigList for bin_big_kernel)
	struct {
		uint32_t *rowCounts;
		uint32_t *binCounts;
		uint32_t *bigList;
		uint32_t *bigCount;
		int32_t smallRows, smallWidth, depthOnly;
	} counts;
};

// Two lists per tile: slot 2 * tile holds the records walked one lane each (small), slot
// 2 * tile + 1 the ones walked by a whole warp (large).
struct TileBins {
	uint32_t *counts;   // 2 * totalTiles
	uint32_t *offsets;  // 2 * totalTiles + 1
	uint32_t *cursors;  // 2 * totalTiles
	uint32_t *lists;
	size_t listCapacity;
	// records over more than four tiles, binned by whole warps in a second launch (room for every
	// record; the count pass fills the list, the fill pass reads it); null: binned in the same launch
	uint32_t *bigList;
	uint32_t *bigCount;
	// counts, cursors, bigCount, the tile queue and the error bits are zeroed by launch_clear_tiles
	// at the start of the batch's phases (0: each launcher zeroes what it uses with memsets)
	int32_t cleared;
};

// True when one lane walks the whole record inside a tile (small-triangle path).
__host__ __device__ inline bool record_is_small(const DrawRecord &r, int32_t smallRows, int32_t smallWidth) {
	return (r.bottom - r.top) <= smallRows && (r.right - r.left) <= smallWidth;
}

enum ErrorBits : int32_t {
	ERROR_RECORD_OVERFLOW = 1,
	ERROR_COORDINATE_RANGE = 2,
	ERROR_BIN_OVERFLOW = 4,
	ERROR_ROW_OVERFLOW = 8,
	ERROR_INTERNAL = 16,
	// a buffer sized before its count was known was too small: the frame is redone with larger
	// buffers, and the kernels that would read past them or write the targets return at once
	ERROR_OVERFLOW_BITS = ERROR_RECORD_OVERFLOW | ERROR_BIN_OVERFLOW | ERROR_ROW_OVERFLOW,
};

// Phase A: projection and the count of draw records per fan triangle, scanned so that the record
// count ends at triOffsets[totalTriangles].
void launch_project(const BatchParams &b, const FrameBuffers &fb, cudaStream_t stream);
void launch_setup_count(const BatchParams &b, const FrameBuffers &fb, cudaStream_t stream);
// Phase B: the records, in submission order (per frame: the order of its tasks, then of their
// triangles), row offsets (total at rowOffsets[recordCount]) and tile counts (total at offsets[2 * totalTiles]).
void launch_setup_write(const BatchParams &b, const FrameBuffers &fb, uint32_t recordCapacity, cudaStream_t stream);
// launch_setup_write with the row and tile counting folded in (fb.counts is filled from rowCounts and
// bins here), then the big records' tile counts and the scans of row counts and tile counts: the
// work of launch_setup_write + launch_row_offsets + launch_bin_count in one pass over the records.
void launch_clear_tiles(const BatchParams &b, const TileBins &bins, int32_t *errorFlag, cudaStream_t stream);
// With rowStream, the row-offset scan runs there (forked with `fork` right after the records) and
// the caller's row-interval launch on rowStream follows it; the tile counts stay on `stream`.
void launch_setup_write_counting(const BatchParams &b, FrameBuffers fb, uint32_t recordCapacity, uint32_t *rowCounts, TileBins &bins,
                                 cudaStream_t stream, cudaStream_t rowStream = nullptr, cudaEvent_t fork = nullptr);
// occludeFromExistingTriangles (api/rendererAPI.cpp:240-255): every solid draw command of the batch
// whose bound exceeds one cell lowers the occlusion grid of its frame over the cells it covers.
void launch_setup_occlude(const BatchParams &b, const FrameBuffers &fb, cudaStream_t stream);
// occludeFromTopRows (api/rendererAPI.cpp:417-476) from a device depth image.
void launch_occlusion_top_rows(float *grid, int32_t gridWidth, int32_t gridHeight, int32_t gridStride, const float *depth,
                               int32_t depthStride, int32_t width, bool perspective, cudaStream_t stream);
void launch_row_offsets(const FrameBuffers &fb, uint32_t recordCount, uint32_t *rowCounts, cudaStream_t stream);
void launch_bin_count(const BatchParams &b, const FrameBuffers &fb, uint32_t recordCount, TileBins &bins, cudaStream_t stream);
// Phase C: row intervals, tile lists, the persistent tile raster and the per-pixel resolve.
// tallRecords: records average many rows (large triangles); rows are then balanced by row, not by record.
void launch_rows(const FrameBuffers &fb, uint32_t recordCount, bool tallRecords, cudaStream_t stream);
void launch_bin_fill(const BatchParams &b, const FrameBuffers &fb, uint32_t recordCount, TileBins &bins, cudaStream_t stream);
// Launch shape of the persistent tile kernel.
struct RasterConfig {
	int32_t threadsPerTile; // 64, 128 or 256
	int32_t ctasPerSm;      // resident CTAs per SM pulling tiles (at most 1024 / threadsPerTile)
	int32_t resolveMode;    // 0 one pixel per thread in a pass of its own, 1 per pixel inside the tile
	                        // kernel, 2 one 2x2 quad per thread in a pass of its own (same results)
};
// resolve = false leaves the winners in the key images (the differentiable renderer reads them).
void launch_raster(const BatchParams &b, const FrameBuffers &fb, const TileBins &bins, const RasterConfig &config, bool resolve,
                   cudaStream_t stream);
// Buffers of launch_stable_sort for n items: keys and ids twice n; hist and offsets
// 256 * sort_blocks(n) + 1; scan scratch for 256 * sort_blocks(n) + 1 values.
struct SortBuffers {
	uint32_t *keysA, *keysB, *idsA, *idsB, *hist, *offsets;
	uint32_t *scanScratch;
	size_t scanScratchElems;
};
uint32_t sort_blocks(uint64_t n);
// Stable LSD radix sort of the ids (the item indices when ids is null) by the low keyBits bits of
// their keys; *sortedKeys and *sortedIds point at the buffers holding the result (the inputs when n is 0).
void launch_stable_sort(const uint32_t *keys, const uint32_t *ids, uint64_t n, int keyBits, const SortBuffers &b,
                        cudaStream_t stream, const uint32_t **sortedKeys, const uint32_t **sortedIds);
// Scratch of launch_alpha for `entries` list entries: entryTile, tileKeys and records hold
// `entries` values each; sort as launch_stable_sort needs for `entries` items.
struct AlphaBuffers {
	uint32_t *entryTile, *tileKeys, *records;
	SortBuffers sort;
};
// The alpha filter over the binned records (in place of launch_raster): colour blends in
// submission order, depth read only.
void launch_alpha(const BatchParams &b, const FrameBuffers &fb, const TileBins &bins, uint32_t entries, uint32_t recordCount,
                  const AlphaBuffers &a, cudaStream_t stream);
// Debug overlays: the three edges of every record as lines in pixels (flat / 256), and draw_line
// (api/drawAPI.cpp:176-279) of many lines of one packed colour into a device image.
void launch_wire_lines(const DrawRecord *records, uint32_t count, int4 *lines, cudaStream_t stream);
void launch_draw_lines(uint32_t *image, int32_t stride, int32_t width, int32_t height, const int4 *lines, uint32_t count,
                       uint32_t color, cudaStream_t stream);
// out[0..3] = record count, row count, tile-list entry count, error bits of a batch.
void launch_gather_totals(const uint32_t *triOffsets, uint32_t triangles, const uint32_t *rowOffsets, uint32_t recordCapacity,
                          const uint32_t *binOffsets, uint32_t tiles, const int32_t *errorFlag, uint32_t *out, uint32_t *tileList,
                          uint32_t *tileListCount, cudaStream_t stream);
// Exclusive scan of n uint32 values into out (out[n] = total); two launches, scratch of
// scan_scratch_elems(n) values.
void launch_scan(const uint32_t *in, uint32_t *out, uint32_t n, uint32_t *scratch, size_t scratchElems, cudaStream_t stream);
// The same for a length written on the device (*nDevice, at most capacity; scratch for capacity).
void launch_scan_device(const uint32_t *in, uint32_t *out, const uint32_t *nDevice, uint32_t capacity, uint32_t *scratch,
                        size_t scratchElems, cudaStream_t stream);
size_t scan_scratch_elems(uint32_t n);
// The first memset the launchers above failed to enqueue on this thread since the last call
// (cudaSuccess if none), cleared by the call; callers check it with cudaGetLastError after launching.
cudaError_t take_enqueue_error();
// Makes `to` wait for what `from` has queued so far (an event recorded on `from`); inside a stream
// capture this forks or joins branches of the graph.  A failure is kept for take_enqueue_error.
void enqueue_join(cudaStream_t from, cudaStream_t to, cudaEvent_t event);
// Kernels launched by this library in this process (host-side count).
uint64_t launch_count();
// Adds kernels launched through a replayed CUDA graph to that count.
void add_launches(uint64_t n);
int32_t sm_count();

} // namespace dsrg

#endif
