// The renderer's debug overlays (endFrame, api/rendererAPI.cpp:354-415): white lines around every
// drawn command with renderer_end(debugWireframe), and the cyan silhouettes kept by
// renderer_occludeFromBox(debugSilhouette), drawn with draw_line (api/drawAPI.cpp:176-279).
//
// draw_line walks the longer axis with an integer error term: after k steps the shorter axis has
// moved floor((k * tilt + maxError) / (2 * maxError)) pixels (tilt = 2 * shorter extent, maxError =
// longer extent), so every pixel of a line is independent.  One warp draws one line, its lanes
// taking the steps whose longer-axis coordinate lies inside the image.  All lines of one launch
// have the same colour, so their order does not matter.
#include <cuda_runtime.h>
#include <stdint.h>

#include "dsrg_kernels.h"

namespace dsrg {

namespace {

__global__ void wire_lines_kernel(const DrawRecord *__restrict__ records, uint32_t count, int4 *lines) {
	for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
		const DrawRecord &r = records[i];
		int32_t x[3], y[3];
		for (int c = 0; c < 3; c++) { x[c] = r.flat[2 * c] / 256; y[c] = r.flat[2 * c + 1] / 256; } // flat / unitsPerPixel
		for (int e = 0; e < 3; e++) {
			const int n = (e + 1) % 3;
			lines[(size_t)i * 3 + e] = make_int4(x[e], y[e], x[n], y[n]);
		}
	}
}

__device__ __forceinline__ void put(uint32_t *image, int32_t stride, int32_t width, int32_t height, int32_t x, int32_t y, uint32_t color) {
	if (x >= 0 && y >= 0 && x < width && y < height) image[(size_t)y * stride + x] = color;
}

__global__ void draw_lines_kernel(uint32_t *image, int32_t stride, int32_t width, int32_t height, const int4 *__restrict__ lines,
                                  uint32_t count, uint32_t color) {
	const int lane = threadIdx.x & 31;
	const uint32_t warps = (gridDim.x * blockDim.x) >> 5;
	for (uint32_t w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; w < count; w += warps) {
		int32_t x1 = lines[w].x, y1 = lines[w].y, x2 = lines[w].z, y2 = lines[w].w;
		if ((x1 < 0 && x2 < 0) || (y1 < 0 && y2 < 0) || (x1 >= width && x2 >= width) || (y1 >= height && y2 >= height)) continue;
		const int64_t adx = x2 > x1 ? (int64_t)x2 - x1 : (int64_t)x1 - x2, ady = y2 > y1 ? (int64_t)y2 - y1 : (int64_t)y1 - y2;
		if (y1 == y2 || x1 == x2 || ady >= adx) {
			// along y (a horizontal run when y1 == y2 walks x below)
			if (y1 == y2) {
				const int32_t l = max(min(x1, x2), 0), r = min(max(x1, x2), width - 1);
				for (int32_t x = l + lane; x <= r; x += 32) put(image, stride, width, height, x, y1, color);
				continue;
			}
			if (y2 < y1) { int32_t t = x1; x1 = x2; x2 = t; t = y1; y1 = y2; y2 = t; }
			const int32_t step = x2 > x1 ? 1 : (x2 < x1 ? -1 : 0);
			const int64_t tilt = 2 * adx, maxError = (int64_t)y2 - y1;
			const int64_t k0 = y1 < 0 ? -(int64_t)y1 : 0, k1 = min((int64_t)y2, (int64_t)height - 1) - y1;
			for (int64_t k = k0 + lane; k <= k1; k += 32) {
				const int64_t moved = (k * tilt + maxError) / (2 * maxError);
				put(image, stride, width, height, (int32_t)(x1 + step * moved), (int32_t)(y1 + k), color);
			}
		} else {
			if (x2 < x1) { int32_t t = x1; x1 = x2; x2 = t; t = y1; y1 = y2; y2 = t; }
			const int32_t step = y2 > y1 ? 1 : -1;
			const int64_t tilt = 2 * ady, maxError = (int64_t)x2 - x1;
			const int64_t k0 = x1 < 0 ? -(int64_t)x1 : 0, k1 = min((int64_t)x2, (int64_t)width - 1) - x1;
			for (int64_t k = k0 + lane; k <= k1; k += 32) {
				const int64_t moved = (k * tilt + maxError) / (2 * maxError);
				put(image, stride, width, height, (int32_t)(x1 + k), (int32_t)(y1 + step * moved), color);
			}
		}
	}
}

int grid_of(uint64_t threads) {
	const uint64_t blocks = (threads + 255) / 256;
	const uint64_t cap = (uint64_t)sm_count() * 8;
	return (int)(blocks < 1 ? 1 : (blocks < cap ? blocks : cap));
}

} // namespace

void launch_wire_lines(const DrawRecord *records, uint32_t count, int4 *lines, cudaStream_t stream) {
	if (count == 0) return;
	wire_lines_kernel<<<grid_of(count), 256, 0, stream>>>(records, count, lines);
	add_launches(1);
}

void launch_draw_lines(uint32_t *image, int32_t stride, int32_t width, int32_t height, const int4 *lines, uint32_t count,
                       uint32_t color, cudaStream_t stream) {
	if (count == 0 || width <= 0 || height <= 0) return;
	draw_lines_kernel<<<grid_of((uint64_t)count * 32), 256, 0, stream>>>(image, stride, width, height, lines, count, color);
	add_launches(1);
}

} // namespace dsrg
