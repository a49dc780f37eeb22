// Launch interface of the kernels of the DFPSR triangle path (host side).
#ifndef DSRG_KERNELS_H
#define DSRG_KERNELS_H

#include <cuda_runtime.h>
#include <stdint.h>
#include "dsrg_types.h"

namespace dsrg {

// One model submitted for one frame: model_render / renderer_giveTask (api/modelAPI.cpp:197-281).
struct TaskParams {
	const float *positions;   // pointCount x 3
	const int32_t *polygons;  // polygonCount x 4
	const float *texCoords;   // polygonCount x 4 x 4
	const float *colors;      // polygonCount x 4 x 4
	const int32_t *triSource; // per fan triangle: polygon * 2 + fan index
	int32_t pointCount;
	int32_t triangleCount;
	uint32_t orderBase;       // fan triangles submitted earlier in the same frame
	uint32_t taskIndex;       // this task's entry in the frame's TaskData table
	float modelToWorld[12];
	CameraData camera;
	int32_t width, height;
	int32_t hasColor, hasDepth;
	int32_t filter;           // 0 Solid, 1 Alpha
	int32_t diffuse, light;   // indices into the frame's texture table, -1 for none
	int32_t depthOnly;        // model_renderDepth: 1x1 alignment, no shading (renderCore.cpp:343-443)
};

struct FrameBuffers {
	ProjectedPoints points;
	uint32_t *triCounts;      // per fan triangle: draw records it emits
	uint32_t *triOffsets;     // exclusive scan of triCounts (+ running record count at [triangleCount])
	DrawRecord *records;
	uint32_t *rowOffsets;     // per record: first entry of its rows in `rows` (+ total at [recordCount])
	uint32_t *rows;           // row intervals of every record, left | right << 16
	uint32_t *recordCount;    // device counter of records in the frame
	int32_t *errorFlag;       // device error bits
	uint32_t *scanScratch;
	size_t scanScratchElems;
};

struct TileBins {
	int32_t tilesX, tilesY;
	uint32_t *counts;   // tilesX * tilesY
	uint32_t *offsets;  // tilesX * tilesY + 1
	uint32_t *cursors;  // tilesX * tilesY
	uint32_t *lists;
	size_t listCapacity;
};

struct TargetParams {
	uint32_t *color;          // device pointer or null
	int32_t colorStride;      // in pixels
	int32_t packOrder;
	float *depth;             // device pointer or null
	int32_t depthStride;
	int32_t width, height;
	int32_t affine;           // orthogonal camera: depth test '<' on linear depth
	uint32_t *coverage;       // optional per-pixel fragment counts (width * height, dense)
	unsigned long long *fragments; // optional fragment total
	unsigned long long *keys; // width * height winning (depth, record) keys, written by the tile pass
	const uint32_t *rowOffsets; // see FrameBuffers
	const uint32_t *rows;
	int32_t smallRows;        // records whose raster bound is at most smallRows x smallWidth pixels are
	int32_t smallWidth;       // walked by one lane each instead of by the whole warp
};

// True when one lane walks the whole record inside a tile (small-triangle path).
__host__ __device__ inline bool record_is_small(const DrawRecord &r, int32_t smallRows, int32_t smallWidth) {
	return (r.bottom - r.top) <= smallRows && (r.right - r.left) <= smallWidth;
}

enum ErrorBits : int32_t {
	ERROR_RECORD_OVERFLOW = 1,
	ERROR_COORDINATE_RANGE = 2,
	ERROR_BIN_OVERFLOW = 4,
};

void launch_project(const TaskParams &task, const FrameBuffers &fb, cudaStream_t stream);
// Counts draw records per fan triangle, scans them and writes the records in submission order.
void launch_setup(const TaskParams &task, const FrameBuffers &fb, uint32_t recordCapacity, cudaStream_t stream);
// Bins the first *recordCount records into tiles.  Returns the number of list entries needed
// (reads it back, synchronising the stream) so that the caller can grow the list buffer.
// Counts the (tile, record) pairs and scans them into bins.offsets (total at offsets[tiles]).
void launch_bin_count(const FrameBuffers &fb, uint32_t recordCount, TileBins &bins, int32_t smallRows, int32_t smallWidth,
                      cudaStream_t stream);
// Row counts of the records scanned into fb.rowOffsets (total at rowOffsets[recordCount]).
void launch_row_offsets(const FrameBuffers &fb, uint32_t recordCount, uint32_t *rowCounts, cudaStream_t stream);
// The row intervals of every record (rasterizeTriangle, ITriangle2D.cpp:150-176) into fb.rows.
void launch_rows(const FrameBuffers &fb, uint32_t recordCount, cudaStream_t stream);
void launch_bin_fill(const FrameBuffers &fb, uint32_t recordCount, TileBins &bins, int32_t smallRows, int32_t smallWidth,
                     cudaStream_t stream);
// One CTA per tile rasterises, depth-tests and shades every record binned to it.
void launch_raster(const FrameBuffers &fb, const TaskData *tasks, const TextureData *textures, const TileBins &bins,
                   const TargetParams &target, cudaStream_t stream);
void launch_raster_depth_only(const FrameBuffers &fb, const TileBins &bins, const TargetParams &target, cudaStream_t stream);
// Exclusive scan of n uint32 values into out (out[n] = total).
void launch_scan(const uint32_t *in, uint32_t *out, uint32_t n, uint32_t *scratch, size_t scratchElems, cudaStream_t stream);
size_t scan_scratch_elems(uint32_t n);
// Kernels launched by this library in this process (host-side count).
uint64_t launch_count();

} // namespace dsrg

#endif
