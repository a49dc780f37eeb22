// CUDA kernels of the DFPSR triangle path for sm_103a.
//
// Every launch covers a whole batch of frames (see dsrg_kernels.h).  Per batch:
//   A  project_kernel       Camera::worldToScreen for every model point (implementation/render/Camera.h:157-190)
//      setup_kernel<false>  per fan triangle: cull, clip, front-face; counts its draw records
//      scan                 record offsets, so that records land in submission order
//      setup_kernel<true>   writes the DrawRecords (bound, sub-pixel corners, projection)
//   B  row_count_kernel     + scan: where each record's row intervals go
//      bin_kernel<false>    + scan: (tile, record) pair counts per tile
//   C  rows_kernel          row intervals of every record (rasterizeTriangle)
//      bin_kernel<true>     per-tile record lists
//      raster_kernel        persistent CTAs pull tiles from a queue; every fragment competes for
//                           64-bit depth keys in shared memory; the winners go to the key image
//      resolve_kernel       every pixel re-evaluates and shades its winning fragment
//
// Why the depth test can run out of order: the reference writes a fragment when its depth is
// strictly greater (1/W, perspective) or smaller (linear, orthogonal) than the stored one
// (implementation/render/shader/fillerTemplates.h:108-152).  After any sequence of opaque
// triangles the stored value is the extreme depth over all fragments that beat the initial
// value, and the colour is the earliest fragment reaching it.  Packing (depth, ~record index)
// into one 64-bit key and taking the maximum reproduces exactly that, in any order, because
// the records of a frame are stored in submission order.
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <utility>

#include "dsrg_exact.h"
#include "dsrg_geometry.h"
#include "dsrg_shade.h"
#include "dsrg_kernels.h"
#include "dsrg_raster.cuh"
#include "dsrg_occlusion.h"

namespace dsrg {

static uint64_t g_launches = 0;

// The first failed enqueue of a memset inside the launchers of this thread, reported to the caller
// of the launches by take_enqueue_error (the launchers themselves return nothing).
static thread_local cudaError_t t_enqueueError = cudaSuccess;

static void memset_async(void *p, int value, size_t bytes, cudaStream_t stream) {
	const cudaError_t e = cudaMemsetAsync(p, value, bytes, stream);
	if (e != cudaSuccess && t_enqueueError == cudaSuccess) t_enqueueError = e;
}

void enqueue_join(cudaStream_t from, cudaStream_t to, cudaEvent_t event) {
	cudaError_t e = cudaEventRecord(event, from);
	if (e == cudaSuccess) e = cudaStreamWaitEvent(to, event, 0);
	if (e != cudaSuccess && t_enqueueError == cudaSuccess) t_enqueueError = e;
}

cudaError_t take_enqueue_error() {
	const cudaError_t e = t_enqueueError;
	t_enqueueError = cudaSuccess;
	return e;
}
uint64_t launch_count() { return g_launches; }
void add_launches(uint64_t n) { g_launches += n; }
#define COUNT_LAUNCH() (g_launches++)

int32_t sm_count() {
	static int32_t count = 0;
	if (count == 0) {
		int device = 0, value = 0;
		cudaGetDevice(&device);
		cudaDeviceGetAttribute(&value, cudaDevAttrMultiProcessorCount, device);
		count = value > 0 ? value : 1;
	}
	return count;
}

// Grid of a grid-stride kernel over n items: enough CTAs to fill the GPU, never more than needed.
static int grid_for(uint64_t n, int threads) {
	uint64_t blocks = (n + threads - 1) / threads;
	const uint64_t cap = (uint64_t)sm_count() * 16;
	if (blocks > cap) blocks = cap;
	return (int)(blocks > 0 ? blocks : 1);
}

// Programmatic dependent launch.  A kernel launched with launch_chained may be scheduled while
// the kernel before it on the stream is still running: that kernel lets it in once all of its
// CTAs have started (the release in chain_enter), and chain_enter, the first statement of every
// chained kernel, holds its threads until the predecessor has completed with its writes visible.
// Captured into a graph the pair becomes a programmatic edge, so the launch of each dependent
// kernel overlaps the last CTAs of the one before.  Kernels launched the ordinary way pass the
// wait at once.  Every CTA of a chained kernel runs chain_enter before anything else, so a kernel
// completes only after its predecessor did and the chain stays ordered end to end.
__device__ __forceinline__ void chain_enter() {
	asm volatile("griddepcontrol.wait;" ::: "memory");
	asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

template <typename... Params, typename... Args>
static void launch_chained(void (*kernel)(Params...), dim3 grid, uint32_t block, cudaStream_t stream, Args &&...args) {
	cudaLaunchAttribute attribute[1];
	attribute[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
	attribute[0].val.programmaticStreamSerializationAllowed = 1;
	cudaLaunchConfig_t config;
	memset(&config, 0, sizeof(config));
	config.gridDim = grid;
	config.blockDim = dim3(block);
	config.stream = stream;
	config.attrs = attribute;
	config.numAttrs = 1;
	cudaLaunchKernelEx(&config, kernel, std::forward<Args>(args)...);
}

// A count written on the device, bounded by the capacity the host sized the buffers for.
__device__ __forceinline__ uint32_t device_count(uint32_t capacity, const uint32_t *countDevice) {
	if (!countDevice) return capacity;
	const uint32_t n = *countDevice;
	return n < capacity ? n : capacity;
}

__device__ __forceinline__ bool overflowed(const BatchParams &b) {
	return b.errorFlag && (*(volatile const int32_t *)b.errorFlag & ERROR_OVERFLOW_BITS) != 0;
}

// ------------------------------------------------------------------ projection

__global__ void project_kernel(BatchParams b, ProjectedPoints out) {
	chain_enter();
	for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < b.totalPoints; i += gridDim.x * blockDim.x) {
		const TaskParams &task = b.tasks[find_segment(b.taskPointBase, b.taskCount, i)];
		const uint32_t local = i - task.pointBase;
		if (task.given) { // renderer_giveTask_triangle: projected by the caller
			const GivenPoint &g = task.given[local];
			out.csis[i] = make_float4(g.cs[0], g.cs[1], g.cs[2], g.is[0]);
			out.isy[i] = g.is[1];
			out.flat[i] = make_longlong2(g.flat[0], g.flat[1]);
			continue;
		}
		Vec3 p = vec3(task.positions[local * 3], task.positions[local * 3 + 1], task.positions[local * 3 + 2]);
		Projected pr = camera_to_screen(task.camera, world_to_camera(task.camera, transform_point(task.modelToWorld, p)));
		out.csis[i] = make_float4(pr.cs.x, pr.cs.y, pr.cs.z, pr.isx);
		out.isy[i] = pr.isy;
		out.flat[i] = make_longlong2(pr.flatx, pr.flaty);
	}
}

void launch_project(const BatchParams &b, const FrameBuffers &fb, cudaStream_t stream) {
	if (b.totalPoints == 0) return;
	COUNT_LAUNCH();
	launch_chained(project_kernel, grid_for(b.totalPoints, 256), 256, stream, b, fb.points);
}

// ------------------------------------------------------------------ triangle setup

struct Corner {
	Vec3 cs;
	float isx, isy;
	int64_t fx, fy;
};

// Emits one draw command (renderCore.cpp:203-217 executeTriangleDrawing against the whole target):
// the triangle bound cut to the target with rows aligned to pairs (ITriangle2D.cpp:70-75).
enum SetupMode { SETUP_COUNT = 0, SETUP_WRITE = 1, SETUP_OCCLUDE = 2 };

// Lowers a frame's occlusion grid to the command's farthest corner over the cells its triangle
// covers (occludeFromSortedHull with the triangle as the hull, rendererAPI.cpp:216-239, 240-255).
// Cells only ever decrease, so the order of the commands does not matter.
__device__ void occlude_cells(const FrameTarget &f, const int64_t *fx, const int64_t *fy, const int32_t *bd, const Corner *c) {
	if (!((bd[2] - bd[0]) > OCCLUSION_CELL && (bd[3] - bd[1]) > OCCLUSION_CELL)) return;
	float distance = 0.0f;
	for (int i = 0; i < 3; i++) if (c[i].cs.z > distance) distance = c[i].cs.z;
	const CellRect cells = outer_cell_bound(bd[0], bd[1], bd[2], bd[3], f.gridWidth, f.gridHeight);
	for (int32_t cy = cells.top; cy < cells.bottom; cy++) {
		for (int32_t cx = cells.left; cx < cells.right; cx++) {
			if (!cell_inside_hull(fx, fy, 3, cx, cy)) continue;
			// float minimum by compare-and-swap; it stops as soon as the cell holds a smaller value
			int *cell = reinterpret_cast<int *>(f.occlusion + (size_t)cy * f.gridStride + cx);
			int old = *cell;
			while (distance < __int_as_float(old)) {
				const int seen = atomicCAS(cell, old, __float_as_int(distance));
				if (seen == old) break;
				old = seen;
			}
		}
	}
}

template <int MODE>
__device__ void emit_record(const TaskParams &task, uint32_t taskIndex, const FrameTarget &frame, const FrameBuffers &fb,
                            uint32_t recordCapacity, const Corner *c, const float *subB, const float *subC, uint32_t order,
                            uint32_t tri, uint32_t base, uint32_t &emitted) {
	const int32_t width = frame.width, height = frame.height;
	int64_t fx[3] = {c[0].fx, c[1].fx, c[2].fx}, fy[3] = {c[0].fy, c[1].fy, c[2].fy};
	int32_t bd[4];
	triangle_bound(fx, fy, bd);
	if (MODE == SETUP_OCCLUDE) {
		if (task.filter == 0 && frame.occlusion) occlude_cells(frame, fx, fy, bd, c);
		return;
	}
	// completeOcclusion: commands behind every cell of the grid are not drawn
	if (frame.occlusion &&
	    !command_survives(frame.occlusion, frame.gridWidth, frame.gridHeight, frame.gridStride, bd,
	                      nearest_corner(c[0].cs.z, c[1].cs.z, c[2].cs.z)))
		return;
	if (!(bd[0] < width && bd[2] > 0 && bd[1] < height && bd[3] > 0)) return;
	if (MODE == SETUP_WRITE) {
		const uint32_t index = base + emitted;
		if (index >= recordCapacity) {
			atomicOr(fb.errorFlag, ERROR_RECORD_OVERFLOW);
		} else {
			DrawRecord r;
			bool inRange = true;
			for (int i = 0; i < 3; i++) {
				if (fx[i] < -(1ll << 30) || fx[i] > (1ll << 30) || fy[i] < -(1ll << 30) || fy[i] > (1ll << 30)) inRange = false;
				r.flat[i * 2] = (int32_t)fx[i];
				r.flat[i * 2 + 1] = (int32_t)fy[i];
			}
			if (!inRange) atomicOr(fb.errorFlag, ERROR_COORDINATE_RANGE);
			r.left = bd[0] > 0 ? bd[0] : 0;
			r.top = (bd[1] > 0 ? bd[1] : 0) & ~1;                           // roundDown(top, 2)
			r.right = bd[2] < width ? bd[2] : width;
			r.bottom = ((bd[3] < height ? bd[3] : height) + 1) & ~1;        // roundUp(bottom, 2)
			float isx[3] = {c[0].isx, c[1].isx, c[2].isx}, isy[3] = {c[0].isy, c[1].isy, c[2].isy};
			float csz[3] = {c[0].cs.z, c[1].cs.z, c[2].cs.z};
			triangle_projection(isx, isy, csz, subB, subC, task.camera.perspective != 0, r.start, r.dx, r.dy);
			r.order = order;
			r.tri = tri;
			r.task = taskIndex;
			r.frame = (uint32_t)task.frame;
			r.source = task.triSource[tri];
			fb.records[index] = r;
			if (fb.counts.rowCounts) {
				// the record's rows, and its tiles as bin_kernel<false> counts them
				fb.counts.rowCounts[index] = (uint32_t)(r.bottom - r.top);
				const uint32_t large = (fb.counts.depthOnly || !record_is_small(r, fb.counts.smallRows, fb.counts.smallWidth)) ? 1u : 0u;
				const int32_t tx0 = r.left >> 4, ty0 = r.top >> 4;
				const int32_t tx1 = min((r.right - 1) >> 4, frame.tilesX - 1), ty1 = min((r.bottom - 1) >> 4, frame.tilesY - 1);
				const int32_t w = tx1 - tx0 + 1, h = ty1 - ty0 + 1;
				const int32_t tiles = (w > 0 && h > 0) ? w * h : 0;
				if (tiles > 4) {
					fb.counts.bigList[atomicAdd(fb.counts.bigCount, 1u)] = index;
				} else {
					for (int32_t i = 0; i < tiles; i++)
						atomicAdd(&fb.counts.binCounts[2u * (frame.tileBase + (uint32_t)((ty0 + i / w) * frame.tilesX + tx0 + i % w)) + large], 1u);
				}
			}
		}
	}
	emitted++;
}

// renderTriangleFromData / renderTriangleFromDataDepth for one fan triangle (renderCore.cpp:220-341, 400-443).
template <int MODE>
__global__ void __launch_bounds__(256) setup_kernel(BatchParams b, FrameBuffers fb, uint32_t recordCapacity) {
	chain_enter();
	const bool WRITE = MODE == SETUP_WRITE;
	for (uint32_t g = blockIdx.x * blockDim.x + threadIdx.x; g < b.totalTriangles; g += gridDim.x * blockDim.x) {
		const uint32_t k = (uint32_t)find_segment(b.taskTriangleBase, b.taskCount, g);
		const TaskParams &task = b.tasks[k];
		const FrameTarget &frame = b.frames[task.frame];
		const bool hasTarget = frame.color != nullptr || frame.depth != nullptr;
		const uint32_t t = g - task.triangleBase;
		uint32_t emitted = 0;
		const uint32_t base = WRITE ? fb.triOffsets[g] : 0u;
		if (WRITE && fb.triOffsets[g + 1] == base) continue; // the count pass emitted nothing for it
		const int32_t src = task.triSource[t];
		const int32_t p = src >> 1, fan = src & 1;
		const int corner[3] = {0, 1 + fan, 2 + fan}; // fan 0-1-2, 0-2-3 (model/Model.cpp:135-162, 164-183)
		Corner c[3];
		for (int i = 0; i < 3; i++) {
			const uint32_t pi = task.pointBase + (uint32_t)task.polygons[p * 4 + corner[i]];
			const float4 a = fb.points.csis[pi];
			const longlong2 f = fb.points.flat[pi];
			c[i].cs = vec3(a.x, a.y, a.z);
			c[i].isx = a.w; c[i].isy = fb.points.isy[pi];
			c[i].fx = f.x; c[i].fy = f.y;
		}
		const uint32_t order = (task.orderBase + t) * 8u;
		bool visible = triangle_visibility(task.camera, c[0].cs, c[1].cs, c[2].cs, false) != 0;
		if (visible && !task.depthOnly && task.filter == 1) {
			// renderTriangleFromData skips alpha-filtered triangles whose three alphas are almost zero (renderCore.cpp:319)
			const float *col = task.colors + p * 16;
			if (almost_zero(col[corner[0] * 4 + 3]) && almost_zero(col[corner[1] * 4 + 3]) && almost_zero(col[corner[2] * 4 + 3]))
				visible = false;
		}
		if (visible && hasTarget) {
			const float defaultB[3] = {0.0f, 1.0f, 0.0f}, defaultC[3] = {0.0f, 0.0f, 1.0f};
			const float zero3[3] = {0.0f, 0.0f, 0.0f};
			if (triangle_visibility(task.camera, c[0].cs, c[1].cs, c[2].cs, true) == 1) {
				int64_t fx[3] = {c[0].fx, c[1].fx, c[2].fx}, fy[3] = {c[0].fy, c[1].fy, c[2].fy};
				if (is_frontfacing(fx, fy)) {
					emit_record<MODE>(task, k, frame, fb, recordCapacity, c, task.depthOnly ? zero3 : defaultB,
					                   task.depthOnly ? zero3 : defaultC, order, t, base, emitted);
				}
			} else {
				ClippedPolygon poly;
				poly.count = 3;
				for (int i = 0; i < 3; i++) { poly.v[i].cs = c[i].cs; poly.v[i].state = 0; poly.v[i].value = 0.0f; }
				poly.v[0].subB = 0.0f; poly.v[0].subC = 0.0f;
				poly.v[1].subB = 1.0f; poly.v[1].subC = 0.0f;
				poly.v[2].subB = 0.0f; poly.v[2].subC = 1.0f;
				for (int s = 0; s < task.camera.clipCount; s++) poly.clip(task.camera.clip[s]);
				for (int f = 0; f < poly.count - 2; f++) {
					const SubVertex *sv[3] = {&poly.v[0], &poly.v[1 + f], &poly.v[2 + f]};
					Corner sc[3];
					for (int i = 0; i < 3; i++) {
						Projected pr = camera_to_screen(task.camera, sv[i]->cs);
						sc[i].cs = pr.cs; sc[i].isx = pr.isx; sc[i].isy = pr.isy; sc[i].fx = pr.flatx; sc[i].fy = pr.flaty;
					}
					int64_t fx[3] = {sc[0].fx, sc[1].fx, sc[2].fx}, fy[3] = {sc[0].fy, sc[1].fy, sc[2].fy};
					if (is_frontfacing(fx, fy)) {
						float sb[3] = {sv[0]->subB, sv[1]->subB, sv[2]->subB};
						float scc[3] = {sv[0]->subC, sv[1]->subC, sv[2]->subC};
						emit_record<MODE>(task, k, frame, fb, recordCapacity, sc, task.depthOnly ? zero3 : sb,
						                   task.depthOnly ? zero3 : scc, order + (uint32_t)f, t, base, emitted);
					}
				}
			}
		}
		if (MODE == SETUP_COUNT) fb.triCounts[g] = emitted;
	}
}

void launch_setup_count(const BatchParams &b, const FrameBuffers &fb, cudaStream_t stream) {
	if (b.totalTriangles == 0) {
		memset_async(fb.triOffsets, 0, sizeof(uint32_t), stream);
		return;
	}
	COUNT_LAUNCH();
	launch_chained(setup_kernel<SETUP_COUNT>, grid_for(b.totalTriangles, 256), 256, stream, b, fb, 0u);
	launch_scan(fb.triCounts, fb.triOffsets, b.totalTriangles, fb.scanScratch, fb.scanScratchElems, stream);
}

void launch_setup_write(const BatchParams &b, const FrameBuffers &fb, uint32_t recordCapacity, cudaStream_t stream) {
	if (b.totalTriangles == 0) return;
	COUNT_LAUNCH();
	launch_chained(setup_kernel<SETUP_WRITE>, grid_for(b.totalTriangles, 256), 256, stream, b, fb, recordCapacity);
}

void launch_setup_occlude(const BatchParams &b, const FrameBuffers &fb, cudaStream_t stream) {
	if (b.totalTriangles == 0) return;
	COUNT_LAUNCH();
	launch_chained(setup_kernel<SETUP_OCCLUDE>, grid_for(b.totalTriangles, 256), 256, stream, b, fb, 0u);
}

// One thread per cell of the grid: the cell's run of the top pixel row of its cell row.  The
// reference's runs are [0, 15) for the first cell and [16 g - 1, 16 g + 15) after it, cut at the
// image's width; perspective depth holds 1 / distance, orthogonal depth the distance itself.
__global__ void occlusion_top_rows_kernel(float *grid, int32_t gridWidth, int32_t gridHeight, int32_t gridStride,
                                          const float *__restrict__ depth, int32_t depthStride, int32_t width, int32_t perspective) {
	const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= gridWidth * gridHeight) return;
	const int32_t gx = i % gridWidth, gy = i / gridWidth;
	const float *row = depth + (size_t)(gy * OCCLUSION_CELL) * depthStride;
	const int32_t start = gx == 0 ? 0 : gx * OCCLUSION_CELL - 1;
	int32_t end = gx * OCCLUSION_CELL + OCCLUSION_CELL - 1;
	if (end >= width) end = width;
	float value;
	if (perspective) {
		float maxInv = __int_as_float(0x7F800000);
		for (int32_t x = start; x < end; x++) if (row[x] < maxInv) maxInv = row[x];
		value = __fdiv_rn(1.0f, maxInv);
	} else {
		value = 0.0f;
		for (int32_t x = start; x < end; x++) if (row[x] > value) value = row[x];
	}
	float &cell = grid[(size_t)gy * gridStride + gx];
	if (value < cell) cell = value;
}

void launch_occlusion_top_rows(float *grid, int32_t gridWidth, int32_t gridHeight, int32_t gridStride, const float *depth,
                               int32_t depthStride, int32_t width, bool perspective, cudaStream_t stream) {
	const int32_t cells = gridWidth * gridHeight;
	if (cells <= 0) return;
	COUNT_LAUNCH();
	occlusion_top_rows_kernel<<<(cells + 127) / 128, 128, 0, stream>>>(grid, gridWidth, gridHeight, gridStride, depth, depthStride,
	                                                                 width, perspective ? 1 : 0);
}

// ------------------------------------------------------------------ scan

// Exclusive scan in two launches and no host round trip: the first writes one sum per chunk of
// SCAN_CHUNK values, the second gives every chunk the sum of the chunk sums before it (read by
// the whole block) and scans the chunk through shared memory.  The length may live on the
// device (a count written by an earlier kernel), with `capacity` bounding it for the grid.
static const int SCAN_THREADS = 256;
static const int SCAN_PER_THREAD = 16;
static const uint32_t SCAN_CHUNK = SCAN_THREADS * SCAN_PER_THREAD;

__device__ __forceinline__ uint32_t scan_length(uint32_t n, const uint32_t *nDevice, uint32_t capacity) {
	if (!nDevice) return n;
	const uint32_t d = *nDevice;
	return d < capacity ? d : capacity;
}

__device__ __forceinline__ uint32_t block_sum(uint32_t v, uint32_t *shared) {
	for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xFFFFFFFFu, v, o);
	if ((threadIdx.x & 31) == 0) shared[threadIdx.x >> 5] = v;
	__syncthreads();
	uint32_t total = 0;
	for (int w = 0; w < SCAN_THREADS / 32; w++) total += shared[w];
	__syncthreads();
	return total;
}

__global__ void __launch_bounds__(SCAN_THREADS) scan_reduce_kernel(const uint32_t *__restrict__ in, uint32_t n, const uint32_t *nDevice,
                                                                   uint32_t capacity, uint32_t *chunkSums) {
	chain_enter();
	__shared__ uint32_t warpSums[SCAN_THREADS / 32];
	const uint32_t count = scan_length(n, nDevice, capacity);
	const uint32_t begin = blockIdx.x * SCAN_CHUNK;
	uint32_t v = 0;
	for (uint32_t i = begin + threadIdx.x; i < begin + SCAN_CHUNK && i < count; i += SCAN_THREADS) v += in[i];
	const uint32_t total = block_sum(v, warpSums);
	if (threadIdx.x == 0) chunkSums[blockIdx.x] = total;
}

__global__ void __launch_bounds__(SCAN_THREADS) scan_apply_kernel(const uint32_t *__restrict__ in, uint32_t *out, uint32_t n,
                                                                  const uint32_t *nDevice, uint32_t capacity,
                                                                  const uint32_t *__restrict__ chunkSums) {
	chain_enter();
	__shared__ uint32_t values[SCAN_CHUNK + SCAN_CHUNK / 32]; // one padding word per 32: a thread's 16 values hit 16 banks
	__shared__ uint32_t warpSums[SCAN_THREADS / 32];
	const uint32_t count = scan_length(n, nDevice, capacity);
	const uint32_t begin = blockIdx.x * SCAN_CHUNK;
	if (begin > count || (begin == count && count != 0)) return;
	// the sum of every chunk before this one
	uint32_t p = 0;
	for (uint32_t c = threadIdx.x; c < blockIdx.x; c += SCAN_THREADS) p += chunkSums[c];
	const uint32_t prefix = block_sum(p, warpSums);
	for (int k = 0; k < SCAN_PER_THREAD; k++) {
		const uint32_t i = begin + k * SCAN_THREADS + threadIdx.x;
		const uint32_t at = k * SCAN_THREADS + threadIdx.x;
		values[at + (at >> 5)] = i < count ? in[i] : 0u;
	}
	__syncthreads();
	uint32_t local[SCAN_PER_THREAD];
	uint32_t mine = 0;
	for (int k = 0; k < SCAN_PER_THREAD; k++) {
		local[k] = mine;
		const uint32_t at = threadIdx.x * SCAN_PER_THREAD + k;
		mine += values[at + (at >> 5)];
	}
	// exclusive scan of the threads' sums
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
	uint32_t x = mine;
	for (int o = 1; o < 32; o <<= 1) {
		const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, o);
		if (lane >= o) x += y;
	}
	if (lane == 31) warpSums[warp] = x;
	__syncthreads();
	uint32_t before = prefix + x - mine;
	for (int w = 0; w < warp; w++) before += warpSums[w];
	for (int k = 0; k < SCAN_PER_THREAD; k++) {
		const uint32_t at = threadIdx.x * SCAN_PER_THREAD + k;
		values[at + (at >> 5)] = before + local[k];
	}
	__syncthreads();
	for (int k = 0; k < SCAN_PER_THREAD; k++) {
		const uint32_t i = begin + k * SCAN_THREADS + threadIdx.x;
		const uint32_t at = k * SCAN_THREADS + threadIdx.x;
		if (i < count) out[i] = values[at + (at >> 5)];
	}
	// the total after the last value, by the block holding it
	if (threadIdx.x == SCAN_THREADS - 1 && (count == 0 || (count - 1) / SCAN_CHUNK == blockIdx.x)) {
		uint32_t total = prefix;
		for (int w = 0; w < SCAN_THREADS / 32; w++) total += warpSums[w];
		out[count] = total;
	}
}

size_t scan_scratch_elems(uint32_t n) { return (size_t)(n / SCAN_CHUNK) + 16; }

static void scan_launch(const uint32_t *in, uint32_t *out, uint32_t n, const uint32_t *nDevice, uint32_t *scratch, size_t scratchElems,
                        cudaStream_t stream) {
	const uint32_t blocks = n / SCAN_CHUNK + 1; // n = the length, or the capacity bounding a device length
	if (blocks > scratchElems) {
		memset_async(out, 0xFF, sizeof(uint32_t), stream); // never reached: callers size the scratch
		return;
	}
	COUNT_LAUNCH();
	launch_chained(scan_reduce_kernel, blocks, SCAN_THREADS, stream, in, n, nDevice, n, scratch);
	COUNT_LAUNCH();
	launch_chained(scan_apply_kernel, blocks, SCAN_THREADS, stream, in, out, n, nDevice, n, scratch);
}


void launch_scan(const uint32_t *in, uint32_t *out, uint32_t n, uint32_t *scratch, size_t scratchElems, cudaStream_t stream) {
	scan_launch(in, out, n, nullptr, scratch, scratchElems, stream);
}

void launch_scan_device(const uint32_t *in, uint32_t *out, const uint32_t *nDevice, uint32_t capacity, uint32_t *scratch,
                        size_t scratchElems, cudaStream_t stream) {
	scan_launch(in, out, capacity, nDevice, scratch, scratchElems, stream);
}

// The totals a batch's host side reads once its phases ran: records, rows, tile-list entries and
// the error bits, gathered into one small block for a single copy.  The same launch lists the
// tiles that have entries (one thread per tile, warp-aggregated appends), so that the persistent
// tile kernel pulls only those: frames that are mostly empty (shadow-cube faces) no longer send
// every CTA through thousands of empty tiles.
__global__ void gather_totals_kernel(const uint32_t *triOffsets, uint32_t triangles, const uint32_t *rowOffsets, uint32_t recordCapacity,
                                     const uint32_t *binOffsets, uint32_t tiles, const int32_t *errorFlag, uint32_t *out,
                                     uint32_t *tileList, uint32_t *tileListCount) {
	chain_enter();
	if (blockIdx.x == 0 && threadIdx.x == 0) {
		const uint32_t records = triOffsets[triangles];
		out[0] = records;
		out[1] = rowOffsets[records < recordCapacity ? records : recordCapacity];
		out[2] = binOffsets[2 * tiles];
		out[3] = (uint32_t)*errorFlag;
	}
	if (!tileList) return;
	const uint32_t lane = threadIdx.x & 31u;
	for (uint32_t first = blockIdx.x * blockDim.x; first < tiles; first += gridDim.x * blockDim.x) { // uniform per block
		const uint32_t t = first + threadIdx.x;
		const bool drawn = t < tiles && binOffsets[2 * t] != binOffsets[2 * t + 2];
		const uint32_t mask = __ballot_sync(0xFFFFFFFFu, drawn);
		if (!mask) continue;
		const uint32_t leader = __ffs(mask) - 1;
		uint32_t at = 0;
		if (lane == leader) at = atomicAdd(tileListCount, (uint32_t)__popc(mask));
		at = __shfl_sync(0xFFFFFFFFu, at, leader);
		if (drawn) tileList[at + __popc(mask & ((1u << lane) - 1u))] = t;
	}
}

void launch_gather_totals(const uint32_t *triOffsets, uint32_t triangles, const uint32_t *rowOffsets, uint32_t recordCapacity,
                          const uint32_t *binOffsets, uint32_t tiles, const int32_t *errorFlag, uint32_t *out, uint32_t *tileList,
                          uint32_t *tileListCount, cudaStream_t stream) {
	COUNT_LAUNCH();
	launch_chained(gather_totals_kernel, tileList ? grid_for(tiles, 256) : 1u, tileList ? 256u : 1u, stream, triOffsets, triangles, rowOffsets,
	               recordCapacity, binOffsets, tiles, errorFlag, out, tileList, tileListCount);
}

// ------------------------------------------------------------------ row intervals

__global__ void row_count_kernel(const DrawRecord *__restrict__ records, uint32_t capacity, const uint32_t *countDevice,
                                 uint32_t *counts) {
	chain_enter();
	const uint32_t recordCount = device_count(capacity, countDevice);
	for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < recordCount; i += gridDim.x * blockDim.x)
		counts[i] = (uint32_t)(records[i].bottom - records[i].top);
}

void launch_row_offsets(const FrameBuffers &fb, uint32_t recordCount, uint32_t *rowCounts, cudaStream_t stream) {
	if (recordCount > 0) {
		COUNT_LAUNCH();
		launch_chained(row_count_kernel, grid_for(recordCount, 256), 256, stream, fb.records, recordCount, fb.recordCountDevice, rowCounts);
	}
	if (fb.recordCountDevice)
		launch_scan_device(rowCounts, fb.rowOffsets, fb.recordCountDevice, recordCount, fb.scanScratch, fb.scanScratchElems, stream);
	else
		launch_scan(rowCounts, fb.rowOffsets, recordCount, fb.scanScratch, fb.scanScratchElems, stream);
}

// Row interval of row y for corners held in registers (row_interval without the corner array).
__device__ __forceinline__ void row_interval_regs(int32_t x0, int32_t y0, int32_t x1, int32_t y1, int32_t x2, int32_t y2,
                                                  int32_t y, int32_t L, int32_t R, int32_t &left, int32_t &right) {
	if ((x0 == x1 && y0 == y1) || (x1 == x2 && y1 == y2) || (x2 == x0 && y2 == y0)) { left = R; right = L; return; }
	left = L; right = R;
	cut_row(make_edge(x0, y0, x1, y1), y, L, R, left, right);
	cut_row(make_edge(x1, y1, x2, y2), y, L, R, left, right);
	cut_row(make_edge(x2, y2, x0, y0), y, L, R, left, right);
}

// The row intervals of every record (rasterizeTriangle, ITriangle2D.cpp:150-176), balanced by rows:
// each CTA takes ROWS_CHUNK consecutive rows of the concatenation of all records' rows (one warp
// finds the records they belong to with a 32-way search over the row offsets), stages those
// records' corners in shared memory, gives each thread ROWS_PER_THREAD consecutive rows and
// writes the chunk back coalesced.  Every record has at least two rows (raster bounds cover row
// pairs), so a chunk spans at most ROWS_CHUNK / 2 + 2 records.
static const int ROWS_THREADS = 256;
static const int ROWS_PER_THREAD = 4;
static const uint32_t ROWS_CHUNK = ROWS_THREADS * ROWS_PER_THREAD;
static const uint32_t ROWS_MAX_RECORDS = ROWS_CHUNK / 2 + 2;

// The largest r in [0, n) with offsets[r] <= v (offsets non-decreasing, offsets[0] = 0 <= v), by one warp.
__device__ __forceinline__ uint32_t warp_search(const uint32_t *offsets, uint32_t n, uint32_t v) {
	const uint32_t lane = threadIdx.x & 31;
	uint32_t lo = 0, hi = n;
	while (hi - lo > 32) {
		const uint32_t step = (hi - lo + 31) / 32;
		const uint32_t probe = lo + lane * step;
		const bool below = probe < hi && offsets[probe] <= v;
		const uint32_t k = 31 - __clz(__ballot_sync(0xFFFFFFFFu, below));
		lo += k * step;
		hi = min(lo + step, hi);
	}
	const uint32_t probe = lo + lane;
	const bool below = probe < hi && offsets[probe] <= v;
	return lo + (31 - __clz(__ballot_sync(0xFFFFFFFFu, below)));
}

__global__ void __launch_bounds__(ROWS_THREADS) rows_chunk_kernel(const DrawRecord *__restrict__ records, uint32_t capacity,
                                                            const uint32_t *countDevice, const uint32_t *__restrict__ rowOffsets,
                                                            uint32_t *rows, uint32_t rowCapacity, int32_t *errorFlag) {
	chain_enter();
	__shared__ uint32_t first, last;
	__shared__ uint32_t offsets[ROWS_MAX_RECORDS + 1];
	__shared__ int4 cornersA[ROWS_MAX_RECORDS];   // flat 0..3
	__shared__ int4 cornersB[ROWS_MAX_RECORDS];   // flat 4..5, left, top
	__shared__ int32_t rights[ROWS_MAX_RECORDS];
	__shared__ uint32_t out[ROWS_CHUNK + ROWS_CHUNK / 32];
	const uint32_t n = device_count(capacity, countDevice);
	if (n == 0) return;
	const uint32_t total = rowOffsets[n];
	for (uint32_t begin = blockIdx.x * ROWS_CHUNK; begin < total; begin += gridDim.x * ROWS_CHUNK) {
		const uint32_t end = min(begin + ROWS_CHUNK, total);
		if (threadIdx.x < 32) {
			const uint32_t f = warp_search(rowOffsets, n, begin);
			const uint32_t l = warp_search(rowOffsets, n, end - 1);
			if (threadIdx.x == 0) { first = f; last = l; }
		}
		__syncthreads();
		uint32_t count = last - first + 1;
		if (count > ROWS_MAX_RECORDS) { // only records without rows could do this, and none are made
			if (threadIdx.x == 0) atomicOr(errorFlag, ERROR_INTERNAL);
			count = ROWS_MAX_RECORDS;
		}
		for (uint32_t k = threadIdx.x; k < count; k += ROWS_THREADS) {
			const DrawRecord &r = records[first + k];
			cornersA[k] = __ldg(reinterpret_cast<const int4 *>(&r.flat[0]));
			cornersB[k] = __ldg(reinterpret_cast<const int4 *>(&r.flat[4]));
			rights[k] = r.right;
			offsets[k] = rowOffsets[first + k];
		}
		if (threadIdx.x == 0) offsets[count] = rowOffsets[first + count];
		__syncthreads();
		// this thread's rows: [j0, j0 + ROWS_PER_THREAD) within the chunk
		const uint32_t j0 = begin + threadIdx.x * ROWS_PER_THREAD;
		if (j0 < end) {
			uint32_t lo = 0, hi = count; // the record holding row j0
			while (hi - lo > 1) {
				const uint32_t mid = (lo + hi) >> 1;
				if (offsets[mid] <= j0) lo = mid; else hi = mid;
			}
			uint32_t k = lo;
			const uint32_t jEnd = min(j0 + (uint32_t)ROWS_PER_THREAD, end);
			if (offsets[k + 1] >= jEnd) {
				// all of this thread's rows belong to one record: stepped from the first (two divisions
				// per edge instead of one per edge and row; rows past jEnd are stepped but not kept)
				const int4 a = cornersA[k], c = cornersB[k];
				const int32_t flat[6] = {a.x, a.y, a.z, a.w, c.x, c.y};
				int32_t lefts[ROWS_PER_THREAD], rightsOut[ROWS_PER_THREAD];
				row_intervals_stepped(flat, c.w + (int32_t)(j0 - offsets[k]), ROWS_PER_THREAD, c.z, rights[k], lefts, rightsOut);
#pragma unroll
				for (int i = 0; i < ROWS_PER_THREAD; i++) {
					const uint32_t j = j0 + i;
					if (j >= jEnd) break;
					const uint32_t at = j - begin;
					out[at + (at >> 5)] = (uint32_t)(lefts[i] & 0xFFFF) | ((uint32_t)rightsOut[i] << 16);
				}
			} else {
				for (int i = 0; i < ROWS_PER_THREAD; i++) {
					const uint32_t j = j0 + i;
					if (j >= end) break;
					while (offsets[k + 1] <= j) k++;
					const int4 a = cornersA[k], c = cornersB[k];
					int32_t left, right;
					row_interval_regs(a.x, a.y, a.z, a.w, c.x, c.y, c.w + (int32_t)(j - offsets[k]), c.z, rights[k], left, right);
					const uint32_t at = j - begin;
					out[at + (at >> 5)] = (uint32_t)(left & 0xFFFF) | ((uint32_t)right << 16);
				}
			}
		}
		__syncthreads();
		for (uint32_t at = threadIdx.x; at < end - begin; at += ROWS_THREADS) {
			const uint32_t j = begin + at;
			if (j < rowCapacity) rows[j] = out[at + (at >> 5)];
			else atomicOr(errorFlag, ERROR_ROW_OVERFLOW);
		}
		__syncthreads();
	}
}

static const int32_t ROWS_STEPPED_MAX = 16; // records of at most this many rows are stepped by one lane each

// The row intervals of every record, stepped exactly (row_intervals_stepped: two floor divisions
// per edge start a segment of rows, then one carry step per edge and row).  Each warp takes 32
// records.  When all of them have at most ROWS_STEPPED_MAX rows (dense meshes) each lane steps its
// own record; otherwise the records are cut into segments of up to ROWS_STEPPED_MAX rows that are
// spread over the lanes (a lane finds its record by a search over the warp's prefix sums of
// segment counts and fetches its corners with shuffles), so tall triangles keep every lane busy.
__global__ void __launch_bounds__(256, 3) rows_group_kernel(const DrawRecord *__restrict__ records, uint32_t capacity,
                                                   const uint32_t *countDevice, const uint32_t *__restrict__ rowOffsets,
                                                   uint32_t *rows, uint32_t rowCapacity, int32_t *errorFlag) {
	chain_enter();
	const uint32_t recordCount = device_count(capacity, countDevice);
	const int lane = threadIdx.x & 31;
	const uint32_t warps = (gridDim.x * blockDim.x) >> 5;
	for (uint32_t w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; w * 32u < recordCount; w += warps) {
		const uint32_t i = w * 32u + (uint32_t)lane;
		int32_t count = 0, top = 0, L = 0, R = 0;
		int32_t f0 = 0, f1 = 0, f2 = 0, f3 = 0, f4 = 0, f5 = 0;
		uint32_t out = 0;
		if (i < recordCount) {
			const int4 a = __ldg(reinterpret_cast<const int4 *>(&records[i].flat[0]));   // flat[0..3]
			const int4 b = __ldg(reinterpret_cast<const int4 *>(&records[i].flat[4]));   // flat[4..5], left, top
			const int2 c = __ldg(reinterpret_cast<const int2 *>(&records[i].right));     // right, bottom
			f0 = a.x; f1 = a.y; f2 = a.z; f3 = a.w; f4 = b.x; f5 = b.y;
			L = b.z; top = b.w; R = c.x;
			count = c.y - top;
			out = rowOffsets[i];
		}
		const bool short_ = __all_sync(0xFFFFFFFFu, count <= ROWS_STEPPED_MAX);
		const int32_t segments = short_ ? 1 : (count + ROWS_STEPPED_MAX - 1) / ROWS_STEPPED_MAX;
		int32_t inclusive = segments, total = 32;
		if (!short_) {
			for (int o = 1; o < 32; o <<= 1) {
				const int32_t v = __shfl_up_sync(0xFFFFFFFFu, inclusive, o);
				if (lane >= o) inclusive += v;
			}
			total = __shfl_sync(0xFFFFFFFFu, inclusive, 31);
		}
		for (int32_t base = 0; base < total; base += 32) {
			// this lane's segment: the rows [first, first + rowsHere) of the record held by lane k
			int32_t x0 = f0, y0 = f1, x1 = f2, y1 = f3, x2 = f4, y2 = f5, kTop = top, kL = L, kR = R, kCount = count;
			uint32_t kOut = out;
			int32_t first = 0;
			const int32_t j = base + lane;
			if (!short_) {
				int k = 0; // first lane whose inclusive sum exceeds j
				for (int step = 16; step >= 1; step >>= 1)
					if (__shfl_sync(0xFFFFFFFFu, inclusive, k + step - 1) <= j) k += step;
				const int32_t start = __shfl_sync(0xFFFFFFFFu, inclusive, k) - __shfl_sync(0xFFFFFFFFu, segments, k);
				x0 = __shfl_sync(0xFFFFFFFFu, f0, k); y0 = __shfl_sync(0xFFFFFFFFu, f1, k);
				x1 = __shfl_sync(0xFFFFFFFFu, f2, k); y1 = __shfl_sync(0xFFFFFFFFu, f3, k);
				x2 = __shfl_sync(0xFFFFFFFFu, f4, k); y2 = __shfl_sync(0xFFFFFFFFu, f5, k);
				kTop = __shfl_sync(0xFFFFFFFFu, top, k); kL = __shfl_sync(0xFFFFFFFFu, L, k);
				kR = __shfl_sync(0xFFFFFFFFu, R, k); kCount = __shfl_sync(0xFFFFFFFFu, count, k);
				kOut = __shfl_sync(0xFFFFFFFFu, out, k);
				first = (j - start) * ROWS_STEPPED_MAX;
			}
			if (j >= total) continue;
			const int32_t rowsHere = min(ROWS_STEPPED_MAX, kCount - first);
			if (rowsHere <= 0) continue;
			const bool degenerate = (x0 == x1 && y0 == y1) || (x1 == x2 && y1 == y2) || (x2 == x0 && y2 == y0);
			EdgeStepper st[3];
			if (!degenerate) {
				st[0] = edge_stepper(make_edge(x0, y0, x1, y1), kTop + first);
				st[1] = edge_stepper(make_edge(x1, y1, x2, y2), kTop + first);
				st[2] = edge_stepper(make_edge(x2, y2, x0, y0), kTop + first);
			}
			for (int32_t r = 0; r < rowsHere; r++) {
				int32_t left = kR, right = kL;
				if (!degenerate) {
					left = kL; right = kR;
					edge_step(st[0], kL, kR, left, right);
					edge_step(st[1], kL, kR, left, right);
					edge_step(st[2], kL, kR, left, right);
				}
				const uint32_t at = kOut + (uint32_t)(first + r);
				if (at < rowCapacity) rows[at] = (uint32_t)(left & 0xFFFF) | ((uint32_t)right << 16);
				else atomicOr(errorFlag, ERROR_ROW_OVERFLOW);
			}
		}
	}
}

void launch_rows(const FrameBuffers &fb, uint32_t recordCount, bool tallRecords, cudaStream_t stream) {
	if (recordCount == 0) return;
	COUNT_LAUNCH();
	const uint32_t rowCapacity = fb.rowCapacity ? fb.rowCapacity : 0xFFFFFFFFu;
	if (tallRecords)
		launch_chained(rows_chunk_kernel, sm_count() * 6, ROWS_THREADS, stream, fb.records, recordCount, fb.recordCountDevice, fb.rowOffsets,
		                                                               fb.rows, rowCapacity, fb.errorFlag);
	else
		launch_chained(rows_group_kernel, grid_for((uint64_t)((recordCount + 31) / 32) * 32, 256), 256, stream,
			fb.records, recordCount, fb.recordCountDevice, fb.rowOffsets, fb.rows, rowCapacity, fb.errorFlag);
}

// ------------------------------------------------------------------ binning

// Conservative test of whether any pixel of the tile whose top-left pixel is (px0, py0) can be
// inside the record's row intervals: a pixel (x, y) passes edge i of cutConvexEdge when
//   (128 + 256x - sx)*nx + (128 + 256y - sy)*ny <= threshold      (ITriangle2D.cpp:96-146)
// and that linear function is largest at a corner of any rectangle, so a tile is out when one
// edge rejects all four corners of the tile grown by two pixels (the growth covers the rows
// where the reference's truncating division admits a pixel just outside an edge).
__device__ __forceinline__ bool tile_may_overlap(const DrawRecord &r, int32_t px0, int32_t py0) {
	const int64_t X0 = 128 + 256 * (int64_t)(px0 - 2), X1 = 128 + 256 * (int64_t)(px0 + TILE_W + 1);
	const int64_t Y0 = 128 + 256 * (int64_t)(py0 - 2), Y1 = 128 + 256 * (int64_t)(py0 + TILE_H + 1);
	for (int i = 0; i < 3; i++) {
		const int j = (i + 1) % 3;
		const Edge e = make_edge(r.flat[i * 2], r.flat[i * 2 + 1], r.flat[j * 2], r.flat[j * 2 + 1]);
		const int64_t a = (X0 - e.sx) * e.nx, bb = (X1 - e.sx) * e.nx;
		const int64_t c = (Y0 - e.sy) * e.ny, d = (Y1 - e.sy) * e.ny;
		const int64_t lowest = (a < bb ? a : bb) + (c < d ? c : d);
		if (lowest > e.threshold) return false;
	}
	return true;
}

// The corner test above is exact only when no row of the record makes the reference cast a
// quotient beyond 32 bits (a nearly horizontal edge whose row crossings lie 2^30 pixels away),
// because such a row's interval comes from the wrapped value, not from the edge.
__device__ __forceinline__ bool tile_test_is_exact(const DrawRecord &r) {
	for (int i = 0; i < 3; i++) {
		const int j = (i + 1) % 3;
		const Edge e = make_edge(r.flat[i * 2], r.flat[i * 2 + 1], r.flat[j * 2], r.flat[j * 2 + 1]);
		if (e.nx == 0) continue;
		const float den = fabsf(i64_to_float(e.nx * 256));
		for (int k = 0; k < 2; k++) {
			const int64_t y = k ? (int64_t)r.bottom : (int64_t)r.top;
			const int64_t limit = e.threshold - (128 - e.sx) * e.nx - (128 + 256 * y - e.sy) * e.ny;
			if (fabsf(i64_to_float(limit)) >= 5.0e8f * den) return false;
		}
	}
	return true;
}

// Counts (FILL = false) or writes (FILL = true) the (tile, record) pairs.  Every tile has two lists,
// slot 2 * tile for the records the tile kernel walks one lane each (small) and slot 2 * tile + 1
// for the ones it walks with a whole warp (large).  Records touching at most 4 tiles are binned by
// their own thread, with the atomics of threads that hit the same slot merged into one; larger
// ones by the whole warp, tested tile by tile.  A list keeps submission order only per warp, which
// the order-free depth keys do not need.
template <bool FILL>
__global__ void bin_kernel(BatchParams b, const DrawRecord *__restrict__ records, uint32_t capacity, const uint32_t *countDevice,
                           TileBins bins, int32_t *errorFlag) {
	chain_enter();
	const uint32_t recordCount = device_count(capacity, countDevice);
	const uint32_t lane = threadIdx.x & 31;
	const uint32_t stride = gridDim.x * blockDim.x;
	for (uint32_t r0 = blockIdx.x * blockDim.x; r0 < recordCount; r0 += stride) {
		const uint32_t r = r0 + threadIdx.x;
		int32_t tx0 = 0, tx1 = -1, ty0 = 0, ty1 = -1, tilesX = 0;
		uint32_t tileBase = 0, large = 1;
		if (r < recordCount) {
			const DrawRecord rec = records[r];
			const FrameTarget &f = b.frames[rec.frame];
			large = (b.depthOnly || !record_is_small(rec, b.smallRows, b.smallWidth)) ? 1u : 0u;
			tilesX = f.tilesX;
			tileBase = f.tileBase;
			tx0 = rec.left >> 4; tx1 = (rec.right - 1) >> 4;
			ty0 = rec.top >> 4; ty1 = (rec.bottom - 1) >> 4;
			if (tx1 >= f.tilesX) tx1 = f.tilesX - 1;
			if (ty1 >= f.tilesY) ty1 = f.tilesY - 1;
		}
		const int32_t w = tx1 - tx0 + 1, h = ty1 - ty0 + 1;
		const int32_t tiles = (w > 0 && h > 0) ? w * h : 0;
		const bool big = tiles > 4;
		for (int32_t i = 0; i < 4; i++) {
			const bool active = !big && i < tiles;
			const uint32_t tile = active ? 2u * (tileBase + (uint32_t)((ty0 + i / w) * tilesX + tx0 + i % w)) + large : 0xFFFFFFFFu;
			const uint32_t peers = __match_any_sync(0xFFFFFFFFu, tile);
			if (active) {
				const uint32_t leader = __ffs(peers) - 1;
				const uint32_t rank = __popc(peers & ((1u << lane) - 1u));
				uint32_t baseSlot = 0;
				if (lane == leader) baseSlot = atomicAdd(FILL ? &bins.cursors[tile] : &bins.counts[tile], (uint32_t)__popc(peers));
				baseSlot = __shfl_sync(peers, baseSlot, leader);
				if (FILL) {
					const uint32_t slot = bins.offsets[tile] + baseSlot + rank;
					if (slot < bins.listCapacity) bins.lists[slot] = r; else atomicOr(errorFlag, ERROR_BIN_OVERFLOW);
				}
			}
		}
		uint32_t bigMask = __ballot_sync(0xFFFFFFFFu, big);
		if (bins.bigList) {
			// deferred to bin_big_kernel, which gives every big record a warp of its own
			if (!FILL && bigMask) {
				const uint32_t leader = __ffs(bigMask) - 1;
				uint32_t base = 0;
				if (lane == leader) base = atomicAdd(bins.bigCount, (uint32_t)__popc(bigMask));
				base = __shfl_sync(0xFFFFFFFFu, base, leader);
				if (big) bins.bigList[base + __popc(bigMask & ((1u << lane) - 1u))] = r;
			}
			continue;
		}
		while (bigMask) {
			const uint32_t src = __ffs(bigMask) - 1;
			bigMask &= bigMask - 1;
			const int32_t bx0 = __shfl_sync(0xFFFFFFFFu, tx0, src), by0 = __shfl_sync(0xFFFFFFFFu, ty0, src);
			const int32_t bw = __shfl_sync(0xFFFFFFFFu, w, src), bt = __shfl_sync(0xFFFFFFFFu, tiles, src);
			const int32_t btx = __shfl_sync(0xFFFFFFFFu, tilesX, src);
			const uint32_t bbase = __shfl_sync(0xFFFFFFFFu, tileBase, src);
			const uint32_t br = __shfl_sync(0xFFFFFFFFu, r, src);
			const uint32_t blarge = __shfl_sync(0xFFFFFFFFu, large, src);
			const DrawRecord rec = records[br];
			const bool exact = tile_test_is_exact(rec);
			for (int32_t i = (int32_t)lane; i < bt; i += 32) {
				const int32_t tx = bx0 + i % bw, ty = by0 + i / bw;
				if (exact && !tile_may_overlap(rec, tx * TILE_W, ty * TILE_H)) continue;
				const uint32_t tile = 2u * (bbase + (uint32_t)(ty * btx + tx)) + blarge;
				uint32_t slot = atomicAdd(FILL ? &bins.cursors[tile] : &bins.counts[tile], 1u);
				if (FILL) {
					slot += bins.offsets[tile];
					if (slot < bins.listCapacity) bins.lists[slot] = br; else atomicOr(errorFlag, ERROR_BIN_OVERFLOW);
				}
			}
		}
	}
}

// The records bin_kernel deferred.  A block takes BIG_GROUP of them at a time and its threads share
// the (record, tile) pairs of their bounds evenly, so that one record spanning a whole frame is
// spread over the block instead of keeping a single warp busy while the rest of the grid idles.
static const int BIG_GROUP = 8;

struct BigRecord {
	DrawRecord rec;
	uint32_t index, tileBase, large;
	int32_t tx0, ty0, bw, tilesX, exact;
};

template <bool FILL>
__global__ void __launch_bounds__(256) bin_big_kernel(BatchParams b, const DrawRecord *__restrict__ records, TileBins bins,
                                                      int32_t *errorFlag) {
	chain_enter();
	__shared__ BigRecord held[BIG_GROUP];
	__shared__ int32_t firstPair[BIG_GROUP + 1];
	const uint32_t count = *bins.bigCount;
	for (uint32_t first = blockIdx.x * BIG_GROUP; first < count; first += gridDim.x * BIG_GROUP) { // uniform per block
		if (threadIdx.x < BIG_GROUP) {
			const uint32_t w = first + threadIdx.x;
			int32_t pairs = 0;
			if (w < count) {
				BigRecord &h = held[threadIdx.x];
				h.index = bins.bigList[w];
				h.rec = records[h.index];
				const FrameTarget &f = b.frames[h.rec.frame];
				h.large = (b.depthOnly || !record_is_small(h.rec, b.smallRows, b.smallWidth)) ? 1u : 0u;
				h.tx0 = h.rec.left >> 4;
				h.ty0 = h.rec.top >> 4;
				const int32_t tx1 = min((h.rec.right - 1) >> 4, f.tilesX - 1), ty1 = min((h.rec.bottom - 1) >> 4, f.tilesY - 1);
				h.bw = tx1 - h.tx0 + 1;
				h.tilesX = f.tilesX;
				h.tileBase = f.tileBase;
				h.exact = tile_test_is_exact(h.rec) ? 1 : 0;
				pairs = (h.bw > 0 && ty1 >= h.ty0) ? h.bw * (ty1 - h.ty0 + 1) : 0;
			}
			// prefix sums of the group's pair counts within the first BIG_GROUP lanes
			int32_t inclusive = pairs;
			for (int o = 1; o < BIG_GROUP; o <<= 1) {
				const int32_t v = __shfl_up_sync((1u << BIG_GROUP) - 1u, inclusive, o);
				if ((int)threadIdx.x >= o) inclusive += v;
			}
			firstPair[threadIdx.x + 1] = inclusive;
			if (threadIdx.x == 0) firstPair[0] = 0;
		}
		__syncthreads();
		const int32_t total = firstPair[BIG_GROUP];
		for (int32_t i = (int32_t)threadIdx.x; i < total; i += (int32_t)blockDim.x) {
			int k = 0;
			while (firstPair[k + 1] <= i) k++;
			const BigRecord &h = held[k];
			const int32_t local = i - firstPair[k];
			const int32_t tx = h.tx0 + local % h.bw, ty = h.ty0 + local / h.bw;
			if (h.exact && !tile_may_overlap(h.rec, tx * TILE_W, ty * TILE_H)) continue;
			const uint32_t tile = 2u * (h.tileBase + (uint32_t)(ty * h.tilesX + tx)) + h.large;
			uint32_t slot = atomicAdd(FILL ? &bins.cursors[tile] : &bins.counts[tile], 1u);
			if (FILL) {
				slot += bins.offsets[tile];
				if (slot < bins.listCapacity) bins.lists[slot] = h.index; else atomicOr(errorFlag, ERROR_BIN_OVERFLOW);
			}
		}
		__syncthreads(); // the group is done with before the next one is loaded
	}
}

// Zeroes a batch's tile counters (per-tile counts and cursors, the big-record count, the tile
// queue) and its error bits in one launch at the start of its phases, so that no memset node sits
// in the chain of dependent launches behind it.
__global__ void clear_tiles_kernel(TileBins bins, uint32_t slots, uint32_t *tileQueue, uint32_t *tileListCount, int32_t *errorFlag) {
	chain_enter();
	for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < slots; i += gridDim.x * blockDim.x) {
		bins.counts[i] = 0u;
		bins.cursors[i] = 0u;
	}
	if (blockIdx.x == 0 && threadIdx.x == 0) {
		if (bins.bigCount) *bins.bigCount = 0u;
		if (tileQueue) *tileQueue = 0u;
		if (tileListCount) *tileListCount = 0u;
		if (errorFlag) *errorFlag = 0;
	}
}

void launch_clear_tiles(const BatchParams &b, const TileBins &bins, int32_t *errorFlag, cudaStream_t stream) {
	const uint32_t slots = 2 * b.totalTiles;
	COUNT_LAUNCH();
	launch_chained(clear_tiles_kernel, grid_for(slots, 256), 256, stream, bins, slots, b.tileQueue, b.tileListCount, errorFlag);
}

void launch_setup_write_counting(const BatchParams &b, FrameBuffers fb, uint32_t recordCapacity, uint32_t *rowCounts, TileBins &bins,
                                 cudaStream_t stream, cudaStream_t rowStream, cudaEvent_t fork) {
	if (!bins.cleared) {
		memset_async(bins.counts, 0, sizeof(uint32_t) * 2 * b.totalTiles, stream);
		memset_async(bins.bigCount, 0, sizeof(uint32_t), stream);
	}
	fb.counts.rowCounts = rowCounts;
	fb.counts.binCounts = bins.counts;
	fb.counts.bigList = bins.bigList;
	fb.counts.bigCount = bins.bigCount;
	fb.counts.smallRows = b.smallRows;
	fb.counts.smallWidth = b.smallWidth;
	fb.counts.depthOnly = b.depthOnly;
	launch_setup_write(b, fb, recordCapacity, stream);
	const uint32_t rowBlocks = recordCapacity / SCAN_CHUNK + 1, tileBlocks = (2 * b.totalTiles) / SCAN_CHUNK + 1;
	if (rowStream && (size_t)rowBlocks + tileBlocks <= fb.scanScratchElems) {
		// the row offsets on the second stream right after the records (each scan with its own part
		// of the scratch), the big records' tile counts and the tile-list offsets on this one
		enqueue_join(stream, rowStream, fork);
		scan_launch(rowCounts, fb.rowOffsets, recordCapacity, fb.recordCountDevice, fb.scanScratch, rowBlocks, rowStream);
	}
	if (recordCapacity > 0) {
		COUNT_LAUNCH();
		launch_chained(bin_big_kernel<false>, sm_count() * 8, 256, stream, b, fb.records, bins, fb.errorFlag);
	}
	if (rowStream && (size_t)rowBlocks + tileBlocks <= fb.scanScratchElems) {
		scan_launch(bins.counts, bins.offsets, 2 * b.totalTiles, nullptr, fb.scanScratch + rowBlocks, fb.scanScratchElems - rowBlocks, stream);
		return;
	}
	// one after the other on this stream, sharing the scratch (rowStream, if given, waits for both)
	scan_launch(rowCounts, fb.rowOffsets, recordCapacity, fb.recordCountDevice, fb.scanScratch, fb.scanScratchElems, stream);
	scan_launch(bins.counts, bins.offsets, 2 * b.totalTiles, nullptr, fb.scanScratch, fb.scanScratchElems, stream);
	if (rowStream) enqueue_join(stream, rowStream, fork);
}

void launch_bin_count(const BatchParams &b, const FrameBuffers &fb, uint32_t recordCount, TileBins &bins, cudaStream_t stream) {
	if (!bins.cleared) {
		memset_async(bins.counts, 0, sizeof(uint32_t) * 2 * b.totalTiles, stream);
		if (bins.bigCount) memset_async(bins.bigCount, 0, sizeof(uint32_t), stream);
	}
	if (recordCount > 0) {
		COUNT_LAUNCH();
		launch_chained(bin_kernel<false>, grid_for(recordCount, 256), 256, stream, b, fb.records, recordCount, fb.recordCountDevice, bins,
		                                                                  fb.errorFlag);
		if (bins.bigList) {
			COUNT_LAUNCH();
			launch_chained(bin_big_kernel<false>, sm_count() * 8, 256, stream, b, fb.records, bins, fb.errorFlag);
		}
	}
	launch_scan(bins.counts, bins.offsets, 2 * b.totalTiles, fb.scanScratch, fb.scanScratchElems, stream);
}

void launch_bin_fill(const BatchParams &b, const FrameBuffers &fb, uint32_t recordCount, TileBins &bins, cudaStream_t stream) {
	if (!bins.cleared) memset_async(bins.cursors, 0, sizeof(uint32_t) * 2 * b.totalTiles, stream);
	if (recordCount > 0) {
		COUNT_LAUNCH();
		launch_chained(bin_kernel<true>, grid_for(recordCount, 256), 256, stream, b, fb.records, recordCount, fb.recordCountDevice, bins,
		                                                                 fb.errorFlag);
		if (bins.bigList) {
			COUNT_LAUNCH();
			launch_chained(bin_big_kernel<true>, sm_count() * 8, 256, stream, b, fb.records, bins, fb.errorFlag);
		}
	}
}

// RgbaMultiply_data and its variant (shader/RgbaMultiply.h:37-58, 110-173) for the fan triangle whose
// triSource entry is `src` (polygon * 2 + fan).
__device__ __forceinline__ void make_shade(const TaskParams &task, int32_t src, ShadeRecord &s) {
	const int32_t p = src >> 1, k = src & 1;
	const int corner[3] = {0, 1 + k, 2 + k};
	float scale = 255.0f;
	if (task.diffuse >= 0) scale = fmul(scale, 1.0f / 255.0f);
	if (task.light >= 0) scale = fmul(scale, 1.0f / 255.0f);
	for (int i = 0; i < 3; i++) {
		const float4 col = *reinterpret_cast<const float4 *>(task.colors + (p * 4 + corner[i]) * 4);
		const float4 tc = *reinterpret_cast<const float4 *>(task.texCoords + (p * 4 + corner[i]) * 4);
		s.red[i] = fmul(col.x, scale); s.green[i] = fmul(col.y, scale);
		s.blue[i] = fmul(col.z, scale); s.alpha[i] = fmul(col.w, scale);
		s.u1[i] = tc.x; s.v1[i] = tc.y; s.u2[i] = tc.z; s.v2[i] = tc.w;
	}
	bool fade = !(almost_same3(s.red) && almost_same3(s.green) && almost_same3(s.blue) && almost_same3(s.alpha));
	bool colorless = almost_one3(s.red) && almost_one3(s.green) && almost_one3(s.blue) && almost_one3(s.alpha);
	const bool hasDiffuse = task.diffuse >= 0, hasLight = task.light >= 0;
	if (fade || (hasDiffuse == hasLight)) colorless = false;
	s.flags = (hasDiffuse ? SHADE_DIFFUSE : 0u) | (hasLight ? SHADE_LIGHT : 0u) | (fade ? SHADE_VERTEX_FADE : 0u) |
	          (colorless ? SHADE_COLORLESS : 0u) | (task.filter == 1 ? SHADE_ALPHA_FILTER : 0u);
	s.diffuse = task.diffuse;
	s.light = task.light;
}

// ------------------------------------------------------------------ tiles

// Depth test of one fragment against the tile's shared keys.
__device__ __forceinline__ void tile_fragment(unsigned long long *keys, const float *initialDepth, uint32_t *coverage,
                                              bool counting, int pix, float z, uint32_t record, bool depthTest,
                                              bool affine, uint32_t &fragments) {
	fragments++;
	if (counting) atomicAdd(&coverage[pix], 1u);
	const bool pass = !depthTest || (affine ? (z < initialDepth[pix]) : (z > initialDepth[pix]));
	if (pass) {
		const unsigned long long key = make_key(z, record, depthTest, affine);
		if (key > keys[pix]) atomicMax(&keys[pix], key);
	}
}

// Early depth culling.  A fragment can only change a pixel when its key beats the pixel's key
// and its depth passes the test against the initial depth buffer.  In key order (the upper 32
// bits of make_key) the pixel therefore has a threshold max(key hi, initial depth hi), and a
// record whose best key hi anywhere in the tile is below the smallest threshold of the tile's
// pixels cannot change the tile.  Keys only grow while a tile is drawn, so a threshold read
// early (or read while other warps write) is smaller than the true one: culling stays safe.

// Smallest threshold over the tile's pixels inside the frame, reduced over the warp.
__device__ __forceinline__ uint32_t warp_tile_threshold(const unsigned long long *keys, const float *initialDepth, int lane,
                                                        int32_t validW, int32_t validH, bool affine) {
	uint32_t m = 0xFFFFFFFFu;
#pragma unroll
	for (int k = 0; k < TILE_W * TILE_H / 32; k++) {
		const int p = lane + 32 * k;
		const int row = p >> 4, col = p & 15;
		if (col < validW && row < validH) {
			const int at = row * TILE_STRIDE + col;
			const uint32_t keyHi = (uint32_t)(keys[at] >> 32);
			uint32_t initialHi = ordered_depth(initialDepth[at]);
			if (affine) initialHi = ~initialHi;
			m = min(m, max(keyHi, initialHi));
		}
	}
	for (int o = 16; o > 0; o >>= 1) m = min(m, __shfl_xor_sync(0xFFFFFFFFu, m, o));
	return m;
}

// Largest key hi any fragment of the record can have inside the tile.  The reference
// accumulates depth along rows (start + dx*(x0 + 0.5) + dy*(y + 0.5), then one addition per
// quad or per pixel), so a fragment's depth differs from the plane's value at its centre by at
// most (3 + steps) roundings of at most 2^-24 * M each, where M bounds every partial sum and
// steps is the length of the row walk.  The plane's extreme over the pixel centres of the tile
// and record bounds lies at a corner; widening it by four times that error bound is conservative.
// Returns 0xFFFFFFFF (never culled) for non-finite planes.
__device__ __forceinline__ uint32_t record_best_hi(const DrawRecord &r, int32_t tx0, int32_t ty0, bool affine, bool pixelSteps) {
	const int32_t left = r.left, top = r.top, right = r.right, bottom = r.bottom;
	const float s = r.start[0], dx = r.dx[0], dy = r.dy[0];
	const int32_t xa = max(tx0, left), xb = min(tx0 + TILE_W, right) - 1;
	const int32_t ya = max(ty0, top), yb = min(ty0 + TILE_H, bottom) - 1;
	const float fxa = (float)xa + 0.5f, fxb = (float)xb + 0.5f, fya = (float)ya + 0.5f, fyb = (float)yb + 0.5f;
	const bool up = !affine; // perspective: the largest 1/W wins; orthogonal: the smallest W
	const float px = (dx >= 0.0f) == up ? fxb : fxa;
	const float py = (dy >= 0.0f) == up ? fyb : fya;
	const float extreme = __fadd_rn(__fadd_rn(s, __fmul_rn(dx, px)), __fmul_rn(dy, py));
	const float bound = __fadd_rn(__fadd_rn(fabsf(s), __fmul_rn(fabsf(dx), (float)(abs(right) + abs(left) + 2))),
	                              __fmul_rn(fabsf(dy), (float)(abs(bottom) + abs(top) + 2)));
	const int32_t steps = (pixelSteps ? (right - left) : ((right - left) >> 1)) + 16;
	const float margin = __fmul_rn(__fmul_rn(bound, (float)steps), 2.384185791015625e-7f); // 2^-22 per step
	const float best = up ? __fadd_rn(extreme, margin) : __fsub_rn(extreme, margin);
	if (!isfinite(best) || !isfinite(margin)) return 0xFFFFFFFFu;
	const uint32_t hi = ordered_depth(best);
	return affine ? ~hi : hi;
}

// Lane `lane` of the record's quad at (x, y1), shaded and written to pixel (px, py): the
// reference's running sums of the quad (quad_lanes), the vertex weights, RgbaMultiply and the
// packed colour and depth.
__device__ __forceinline__ void write_lane(const BatchParams &b, const FrameTarget &f, const DrawRecord &r, const RowPair &pair,
                                           int32_t y1, int32_t x, int lane, int32_t px, int32_t py, bool affine) {
	float w[3][4];
	const int components = f.color ? 3 : 1;
	for (int c = 0; c < components; c++) quad_lanes(r.start[c], r.dx[c], r.dy[c], pair, y1, x, w[c]);
	const float depthValue = (lane == 0) ? w[0][0] : (lane == 1) ? w[0][1] : (lane == 2) ? w[0][2] : w[0][3];
	if (f.color) {
		float wa[4], wb[4], wc[4];
		lane_weights(w, affine, wa, wb, wc);
		ShadeRecord shade;
		make_shade(b.tasks[r.task], r.source, shade);
		float rgba[4];
		shade_lane_inline(shade, b.textures, wa, wb, wc, lane, rgba);
		f.color[(size_t)py * f.colorStride + px] = pack_saturated(rgba, f.packOrder);
	}
	if (f.depth) f.depth[(size_t)py * f.depthStride + px] = depthValue;
}

// The depth model_renderDepth leaves at (px, py) when record ri wins the pixel: the reference's
// 1 x 1 walk from its row's left end (executeTriangleDrawingDepth, renderCore.cpp:343-387).
__device__ __forceinline__ float depth_walk_value(const DrawRecord *__restrict__ records, const uint32_t *__restrict__ rowOffsets,
                                                  const uint32_t *__restrict__ rows, uint32_t ri, int32_t px, int32_t py) {
	const DrawRecord r = records[ri];
	int32_t left, right;
	unpack_row(rows[rowOffsets[ri] + (py - r.top)], left, right);
	const float value = fadd(fadd(r.start[0], fmul(r.dx[0], (float)left + 0.5f)), fmul(r.dy[0], (float)py + 0.5f));
	return chain_add(value, r.dx[0], px - left);
}

// The depth of a depth-only winner from its key: the key's upper word is the ordered bits of the
// very value the walk wrote (make_key), so it decodes to that value, except that +0 and -0 share
// one key word; that word is walked again.
__device__ __forceinline__ float depth_from_key(unsigned long long key, bool affine, const DrawRecord *__restrict__ records,
                                                const uint32_t *__restrict__ rowOffsets, const uint32_t *__restrict__ rows,
                                                int32_t px, int32_t py) {
	uint32_t hi = (uint32_t)(key >> 32);
	if (affine) hi = ~hi;
	if (hi == 0x80000000u) return depth_walk_value(records, rowOffsets, rows, key_record(key, true), px, py);
	return bitsf((hi & 0x80000000u) ? (hi & 0x7FFFFFFFu) : ~hi);
}

// The winner of one pixel, shaded and written: the reference's running sums of its quad
// (quad_lanes), the vertex weights, RgbaMultiply and the packed colour and depth.  On the last row
// of an odd-height target the depth-tested pixels are left to odd_row_kernel (their result depends
// on the order of the triangles); without a depth buffer the last triangle drawn wins there as
// anywhere, with its lower lane's value where the pixel lies in its run of full quads.
__device__ __forceinline__ void resolve_pixel(const BatchParams &b, const FrameTarget &f, const DrawRecord *__restrict__ records,
                                              const uint32_t *__restrict__ rowOffsets, const uint32_t *__restrict__ rows,
                                              int32_t px, int32_t py, unsigned long long key) {
	const bool depthTest = f.depth != nullptr, affine = f.affine != 0;
	const bool oddRow = odd_last_row(py, f.height);
	if (oddRow && depthTest) return;
	const uint32_t ri = key_record(key, depthTest);
	const DrawRecord r = records[ri];
	const int32_t y1 = py & ~1, x = px & ~1;
	const RowPair pair = record_row_pair(r, rows + rowOffsets[ri], y1, f.height);
	const int lane4 = ((py & 1) << 1) | (px & 1) | ((oddRow && full_quad(pair, x)) ? 2 : 0);
	write_lane(b, f, r, pair, y1, x, lane4, px, py, affine);
}

// The winner of pixel (px, py) when all four pixels of its 2x2 quad have that winner, evaluated by
// the four lanes of the quad together (lanes 4q..4q+3 of `quadLanes` hold quad q, lane l4 its
// position): each lane computes the running sums of its own position only (quad_lane), and the
// vertex weights of positions 0..2, which every position's mip level needs, come from the other
// lanes by shuffles.  The values are those of resolve_pixel; the quad's sums are evaluated once
// instead of four times.
__device__ __forceinline__ void resolve_shared_quad(const BatchParams &b, const FrameTarget &f, const DrawRecord *__restrict__ records,
                                                    const uint32_t *__restrict__ rowOffsets, const uint32_t *__restrict__ rows,
                                                    int32_t px, int32_t py, unsigned long long key, int l4, unsigned quadLanes) {
	const bool depthTest = f.depth != nullptr, affine = f.affine != 0;
	const uint32_t ri = key_record(key, depthTest);
	const DrawRecord r = records[ri];
	const int32_t y1 = py & ~1, x = px & ~1;
	const RowPair pair = record_row_pair(r, rows + rowOffsets[ri], y1, f.height);
	const float depthValue = quad_lane(r.start[0], r.dx[0], r.dy[0], pair, y1, x, l4);
	if (f.color) {
		float a, bw, c;
		lane_weight(depthValue, quad_lane(r.start[1], r.dx[1], r.dy[1], pair, y1, x, l4),
		            quad_lane(r.start[2], r.dx[2], r.dy[2], pair, y1, x, l4), affine, a, bw, c);
		const int base = (int)(threadIdx.x & 31u) & ~3;
		float wa[4], wb[4], wc[4];
		for (int l = 0; l < 3; l++) {
			wa[l] = __shfl_sync(quadLanes, a, base + l);
			wb[l] = __shfl_sync(quadLanes, bw, base + l);
			wc[l] = __shfl_sync(quadLanes, c, base + l);
		}
		wa[3] = a; wb[3] = bw; wc[3] = c; // position 3 reads only its own weights
		ShadeRecord shade;
		make_shade(b.tasks[r.task], r.source, shade);
		float rgba[4];
		shade_lane_inline(shade, b.textures, wa, wb, wc, l4, rgba);
		f.color[(size_t)py * f.colorStride + px] = pack_saturated(rgba, f.packOrder);
	}
	if (f.depth) f.depth[(size_t)py * f.depthStride + px] = depthValue;
}

// Persistent CTAs pull 16x16 tiles of the batch from a device queue.  The binning split every
// tile's list into small and large records.  Both are dealt round-robin over the warps (warp w of
// W takes entries w, w + W, ...): the quads of a warp's 32 small records inside the tile are spread
// over its lanes, one quad each (the reference's running sums at that quad, quad_lanes); large
// records are rasterised by the whole warp, one lane per (row pair, position in the 2x2 quad),
// which evaluates the running sums once at the tile's left edge and then walks on.
// All fragments compete for the tile's shared keys; the winners go to the frame's key image.
// Tiles that nothing covers write nothing: the resolve pass skips them too.
static const int SHARED_FRAMES = 256;

template <bool DEPTH_ONLY_1X1, int THREADS, bool RESOLVE>
__global__ void __launch_bounds__(THREADS, 1024 / THREADS) raster_kernel(BatchParams b, const DrawRecord *__restrict__ records,
                                                                         TileBins bins, const uint32_t *__restrict__ rowOffsets,
                                                                         const uint32_t *__restrict__ rows) {
	chain_enter();
	constexpr int WARPS = THREADS / 32;
	if (overflowed(b)) return; // the lists or rows are incomplete: the frame is redone
	constexpr int PIXELS = TILE_W * TILE_H / THREADS; // tile pixels owned by each thread
	__shared__ unsigned long long keys[TILE_H * TILE_STRIDE];
	__shared__ float initialDepth[TILE_H * TILE_STRIDE];
	__shared__ uint32_t coverage[TILE_H * TILE_STRIDE];
	__shared__ uint32_t sharedTile;
	__shared__ unsigned long long fragmentSum;
	__shared__ uint32_t frameBases[SHARED_FRAMES]; // the frames' first tiles, for batches of up to SHARED_FRAMES frames
	const int tid = threadIdx.x;
	const int warp = tid >> 5, lane = tid & 31;
	const bool framesShared = b.frameCount <= SHARED_FRAMES;
	if (framesShared)
		for (int i = tid; i < b.frameCount; i += THREADS) frameBases[i] = b.frameTileBase[i];
	const uint32_t listed = (tid == 0 && b.tileList) ? *b.tileListCount : 0u;
	for (;;) {
		if (tid == 0) {
			// the listed tiles (those with entries), or every tile.  (A ticket taken one tile ahead
			// hides the atomic's round trip but holds a tile back from idle CTAs: slower overall.)
			const uint32_t ticket = atomicAdd(b.tileQueue, 1u);
			sharedTile = !b.tileList ? ticket : (ticket < listed ? b.tileList[ticket] : 0xFFFFFFFFu);
			fragmentSum = 0ull;
		}
		__syncthreads();
		const uint32_t tile = sharedTile;
		if (tile >= b.totalTiles) break;
		const uint32_t smallBegin = bins.offsets[2 * tile], smallEnd = bins.offsets[2 * tile + 1], end = bins.offsets[2 * tile + 2];
		if (smallBegin == end) { __syncthreads(); continue; }
		const FrameTarget &f = b.frames[framesShared ? find_segment_shared(frameBases, b.frameCount, tile)
		                                             : find_segment(b.frameTileBase, b.frameCount, tile)];
		const int32_t width = f.width, height = f.height;
		const float *depthImage = f.depth;
		const bool depthTest = depthImage != nullptr;
		const bool affine = f.affine != 0;
		uint32_t *coverageImage = f.coverage;
		const bool counting = coverageImage != nullptr;
		unsigned long long *keyImage = f.keys;
		const int32_t local = (int32_t)(tile - f.tileBase);
		const int32_t tx0 = (local % f.tilesX) * TILE_W, ty0 = (local / f.tilesX) * TILE_H;
		for (int k = 0; k < PIXELS; k++) {
			const int p = tid + k * THREADS;
			const int32_t px = tx0 + (p & 15), py = ty0 + (p >> 4);
			const int me = (p >> 4) * TILE_STRIDE + (p & 15); // the pixel in the padded tile arrays
			initialDepth[me] = (depthTest && px < width && py < height) ? depthImage[(size_t)py * f.depthStride + px] : 0.0f;
			keys[me] = 0ull;
			coverage[me] = 0u;
		}
		__syncthreads();

		uint32_t fragments = 0;
		// early depth culling needs a depth buffer and is off while fragments are being counted; the
		// 1x1 depth walk of depth-only frames is cheaper than the culling test itself
		const bool cull = depthTest && b.fragments == nullptr && !DEPTH_ONLY_1X1;
		const int32_t validW = min(TILE_W, width - tx0), validH = min(TILE_H, height - ty0);
		uint32_t tileMin = 0u; // this warp's view of the tile's depth threshold (0: nothing culled yet)
		// small records: dealt round-robin over the warps (warp w of W takes entries w, w + W, ...).
		// A warp's 32 records are cut into their quads inside the tile, (row pair, quad column)
		// slots of each record's bound, and the slots are spread evenly over the lanes: a lane finds
		// its record by a search over the warp's prefix sums, builds the row pair from the record's
		// two rows and evaluates the reference's running sums at its quad (quad_lanes), so records
		// of different sizes no longer keep lanes idle.  Small records are not culled early: in dense
		// meshes a tile's small list is walked about once per pixel, and the bound test per record
		// cost more than it saved (large records keep the culling; a scene of small triangles with
		// heavy overdraw can send every record down that path with a small bound of 0 x 0).
		for (uint32_t chunk = smallBegin; chunk < smallEnd; chunk += (uint32_t)THREADS) {
			const uint32_t e = chunk + (uint32_t)warp + (uint32_t)WARPS * (uint32_t)lane;
			uint32_t ri = 0, rowOffset = 0;
			int32_t slots = 0, cols = 1, rowStart = 0, colStart = 0, top = 0, colsRecip = 65536;
			float s0 = 0.0f, dx0 = 0.0f, dy0 = 0.0f;
			if (e < smallEnd) {
				ri = bins.lists[e];
				const DrawRecord &r = records[ri];
				const int32_t left = r.left, right = r.right;
				top = r.top;
				const int32_t bottom = r.bottom;
				s0 = r.start[0]; dx0 = r.dx[0]; dy0 = r.dy[0];
				rowOffset = rowOffsets[ri];
				rowStart = max(top, ty0);
				const int32_t rowEnd = min(bottom, ty0 + TILE_H);
				colStart = max(left & ~1, tx0);
				const int32_t colEnd = min((right + 1) & ~1, tx0 + TILE_W);
				if (rowEnd > rowStart && colEnd > colStart) {
					cols = (colEnd - colStart) >> 1;
					slots = ((rowEnd - rowStart) >> 1) * cols;
				}
				colsRecip = (65536 + cols - 1) / cols;
			}
			int32_t inclusive = slots;
			for (int o = 1; o < 32; o <<= 1) {
				const int32_t v = __shfl_up_sync(0xFFFFFFFFu, inclusive, o);
				if (lane >= o) inclusive += v;
			}
			const int32_t total = __shfl_sync(0xFFFFFFFFu, inclusive, 31);
			for (int32_t base = 0; base < total; base += 32) {
				const int32_t j = base + lane;
				int k = 0; // the first lane whose inclusive sum exceeds j
				for (int step = 16; step >= 1; step >>= 1)
					if (__shfl_sync(0xFFFFFFFFu, inclusive, k + step - 1) <= j) k += step;
				const int32_t first = __shfl_sync(0xFFFFFFFFu, inclusive, k) - __shfl_sync(0xFFFFFFFFu, slots, k);
				const int32_t kCols = __shfl_sync(0xFFFFFFFFu, cols, k), kRecip = __shfl_sync(0xFFFFFFFFu, colsRecip, k);
				const int32_t kRowStart = __shfl_sync(0xFFFFFFFFu, rowStart, k), kColStart = __shfl_sync(0xFFFFFFFFu, colStart, k);
				const int32_t kTop = __shfl_sync(0xFFFFFFFFu, top, k);
				const uint32_t kRecord = __shfl_sync(0xFFFFFFFFu, ri, k), kRowOffset = __shfl_sync(0xFFFFFFFFu, rowOffset, k);
				const float kS = __shfl_sync(0xFFFFFFFFu, s0, k), kDx = __shfl_sync(0xFFFFFFFFu, dx0, k);
				const float kDy = __shfl_sync(0xFFFFFFFFu, dy0, k);
				if (j >= total) continue;
				const int32_t slot = j - first;
				const int32_t pairIndex = (slot * kRecip) >> 16; // slot / kCols: slots < 64, columns <= 8
				const int32_t y1 = kRowStart + 2 * pairIndex, x = kColStart + 2 * (slot - pairIndex * kCols);
				// the record's rows y1 and y1 + 1 (row offsets are even: one 8-byte load)
				const uint2 two = *reinterpret_cast<const uint2 *>(rows + kRowOffset + (uint32_t)(y1 - kTop));
				int32_t uL, uR, lL, lR;
				unpack_row(two.x, uL, uR);
				unpack_row(two.y, lL, lR);
				const RowPair pair = make_row_pair(uL, uR, lL, lR, y1 + 1, height);
				if (!pair.any || x < pair.obs || x >= pair.obe) continue;
				const bool edge = pair.ibe <= pair.ibs || x < pair.ibs || x >= pair.ibe;
				float v[4];
				quad_lanes(kS, kDx, kDy, pair, y1, x, v);
				for (int l = 0; l < 4; l++) {
					const int32_t xx = x + (l & 1), yy = y1 + (l >> 1);
					if (yy >= height || xx >= width) continue;
					if (!lane_covered(pair, x, edge, l)) continue;
					tile_fragment(keys, initialDepth, coverage, counting, (yy - ty0) * TILE_STRIDE + (xx - tx0), v[l], kRecord,
					              depthTest, affine, fragments);
				}
			}
		}
		// large records: dealt round-robin over the warps (warp w of W takes entries w, w + W, ...),
		// each rasterised by the whole warp
		for (uint32_t chunk = smallEnd; chunk < end; chunk += 32u * WARPS) {
			const uint32_t e = chunk + (uint32_t)warp + (uint32_t)WARPS * (uint32_t)lane;
			const bool valid = e < end;
			const uint32_t myRecord = valid ? bins.lists[e] : 0u;
			bool culled = false;
			uint32_t myBest = 0u;
			if (cull) tileMin = warp_tile_threshold(keys, initialDepth, lane, validW, validH, affine);
			if (valid && cull) {
				myBest = record_best_hi(records[myRecord], tx0, ty0, affine, DEPTH_ONLY_1X1);
				culled = myBest < tileMin;
			}
			uint32_t largeMask = __ballot_sync(0xFFFFFFFFu, valid && !culled);
			int sinceRefresh = 0;
			while (largeMask) {
				const int src = __ffs(largeMask) - 1;
				largeMask &= largeMask - 1;
				if (cull) {
					// the threshold only rises while the tile is drawn: refresh it every few records
					if (++sinceRefresh == 4) {
						sinceRefresh = 0;
						tileMin = warp_tile_threshold(keys, initialDepth, lane, validW, validH, affine);
					}
					if (__shfl_sync(0xFFFFFFFFu, myBest, src) < tileMin) continue;
				}
				const uint32_t ri = __shfl_sync(0xFFFFFFFFu, myRecord, src);
				const DrawRecord r = records[ri];
				// every lane reads one of the tile's 16 rows (lanes 16..31 repeat 0..15)
				int32_t rowLeft = 0, rowRight = 0;
				const int32_t ry = ty0 + (lane & 15);
				if (ry >= r.top && ry < r.bottom) unpack_row(rows[rowOffsets[ri] + (ry - r.top)], rowLeft, rowRight);
				if (DEPTH_ONLY_1X1) {
					// executeTriangleDrawingDepth (renderCore.cpp:343-387): depth starts at the row's left
					// pixel and grows by dx one pixel at a time.
					if (ry >= r.top && ry < r.bottom && ry < height && rowRight > rowLeft) {
						const int32_t xs = tx0 + (lane >> 4) * 8;
						const int32_t x0 = max(xs, rowLeft), x1 = min(xs + 8, rowRight);
						if (x0 < x1) {
							float value = fadd(fadd(r.start[0], fmul(r.dx[0], (float)rowLeft + 0.5f)), fmul(r.dy[0], (float)ry + 0.5f));
							value = chain_add(value, r.dx[0], x0 - rowLeft);
							for (int32_t x = x0; x < x1; x++) {
								tile_fragment(keys, initialDepth, coverage, counting, (ry - ty0) * TILE_STRIDE + (x - tx0), value, ri, true,
								              affine, fragments);
								value = fadd(value, r.dx[0]);
							}
						}
					}
					continue;
				}
				// lane = (row pair, position in the 2x2 quad); it walks its position across the tile's quads
				const int rp = lane >> 2, pos = lane & 3;
				const int32_t y1 = ty0 + 2 * rp;
				const int32_t uL = __shfl_sync(0xFFFFFFFFu, rowLeft, 2 * rp), uR = __shfl_sync(0xFFFFFFFFu, rowRight, 2 * rp);
				const int32_t lL = __shfl_sync(0xFFFFFFFFu, rowLeft, 2 * rp + 1), lR = __shfl_sync(0xFFFFFFFFu, rowRight, 2 * rp + 1);
				if (y1 < r.top || y1 >= r.bottom) continue;
				const RowPair pair = make_row_pair(uL, uR, lL, lR, y1 + 1, height);
				if (!pair.any) continue;
				const int32_t x0 = max(tx0, pair.obs), x1 = min(tx0 + TILE_W, pair.obe);
				if (x0 >= x1) continue;
				const int32_t yy = y1 + (pos >> 1);
				if (yy >= height) continue;
				const bool odd = (pos & 1) != 0;
				const int32_t rowL = (pos < 2) ? pair.upperLeft : pair.lowerLeft, rowR = (pos < 2) ? pair.upperRight : pair.lowerRight;
				const float dx = r.dx[0], d2 = fmul(dx, 2.0f);
				const float P0 = fadd(fadd(r.start[0], fmul(dx, (float)pair.obs + 0.5f)), fmul(r.dy[0], (float)y1 + 0.5f));
				const float R0 = (pos < 2) ? P0 : fadd(P0, r.dy[0]);
				const bool allEdge = pair.ibe <= pair.ibs;
				const int32_t nL = (pair.ibs - pair.obs) >> 1;
				const float m = fmul(d2, (float)((pair.ibe - pair.ibs) >> 1));
				// state of the reference's running sums at quad x0 (fillerTemplates.h:328-373)
				int region; // 0 left edge, 1 full quads, 2 right edge
				float R, V = 0.0f, Rb = 0.0f;
				if (allEdge || x0 < pair.ibs) {
					region = 0;
					R = chain_add_short(R0, d2, (x0 - pair.obs) >> 1);
				} else {
					Rb = chain_add_short(R0, d2, nL);
					if (x0 < pair.ibe) {
						region = 1;
						R = Rb;
						V = chain_add_short(odd ? fadd(Rb, dx) : Rb, d2, (x0 - pair.ibs) >> 1);
					} else {
						region = 2;
						R = chain_add_short(fadd(Rb, m), d2, (x0 - pair.ibe) >> 1);
					}
				}
				const int pixRow = (yy - ty0) * TILE_STRIDE;
				for (int32_t x = x0; x < x1; x += 2) {
					const int32_t xx = x + (odd ? 1 : 0);
					const float z = (region == 1) ? V : (odd ? fadd(R, dx) : R);
					const bool covered = (region == 1) || (xx >= rowL && xx < rowR);
					if (covered && xx < width)
						tile_fragment(keys, initialDepth, coverage, counting, pixRow + (xx - tx0), z, ri, depthTest, affine, fragments);
					if (region == 0) {
						R = fadd(R, d2);
						if (!allEdge && x + 2 == pair.ibs) { region = 1; Rb = R; V = odd ? fadd(R, dx) : R; }
					} else if (region == 1) {
						V = fadd(V, d2);
						if (x + 2 == pair.ibe) { region = 2; R = fadd(Rb, m); }
					} else {
						R = fadd(R, d2);
					}
				}
			}
		}
		if (b.fragments || b.walked) {
			for (int o = 16; o > 0; o >>= 1) fragments += __shfl_xor_sync(0xFFFFFFFFu, fragments, o);
			if (lane == 0) atomicAdd(&fragmentSum, (unsigned long long)fragments);
		}
		__syncthreads();
#pragma unroll 1
		for (int k = 0; k < PIXELS; k++) { // one copy of the (inlined) resolve code, not PIXELS
			// quad-major: lanes 4q..4q+3 hold the four pixels of quad q, and a warp holds a 16 x 2 strip
			const int p = tid + k * THREADS, q = p >> 2, l4 = p & 3;
			const int lx = 2 * (q & 7) + (l4 & 1), ly = 2 * (q >> 3) + (l4 >> 1);
			const int32_t px = tx0 + lx, py = ty0 + ly;
			const int me = ly * TILE_STRIDE + lx;
			const bool inside = px < width && py < height;
			const unsigned long long key = inside ? keys[me] : 0ull;
			if (inside) {
				if (counting) coverageImage[(size_t)py * width + px] += coverage[me]; // zeroed before a frame's first run
				if (!RESOLVE) keyImage[(size_t)py * width + px] = key;
				// model_renderDepth: the winner's depth straight from its key, written by the tile pass itself
				else if (DEPTH_ONLY_1X1 && key != 0ull)
					f.depth[(size_t)py * f.depthStride + px] = depth_from_key(key, affine, records, rowOffsets, rows, px, py);
			}
			if (!RESOLVE || DEPTH_ONLY_1X1) continue;
			// the tile's winners shaded right away (resolve_pixels_kernel fused into the tile pass): a
			// warp whose quads each have one winner (or none) shares each quad's sums among its lanes;
			// other warps, and every quad touching the image's edge or an odd height's last row (whose
			// missing pixels have no key), resolve pixel by pixel
			const int same = key == __shfl_sync(0xFFFFFFFFu, key, lane & ~3) ? 1 : 0;
			const bool quadSame = (same & __shfl_xor_sync(0xFFFFFFFFu, same, 1) & __shfl_xor_sync(0xFFFFFFFFu, same, 2) &
			                       __shfl_xor_sync(0xFFFFFFFFu, same, 3)) != 0;
			const unsigned drawn = __ballot_sync(0xFFFFFFFFu, key != 0ull);
			if (__all_sync(0xFFFFFFFFu, quadSame || key == 0ull)) {
				if (key != 0ull) resolve_shared_quad(b, f, records, rowOffsets, rows, px, py, key, l4, drawn);
			} else if (key != 0ull) {
				resolve_pixel(b, f, records, rowOffsets, rows, px, py, key);
			}
		}
		if (tid == 0 && fragmentSum) {
			if (b.fragments) atomicAdd(b.fragments, fragmentSum);
			if (b.walked) atomicAdd(b.walked, fragmentSum);
		}
		__syncthreads();
	}
}

// One thread per pixel: the winning fragment's quad is re-evaluated exactly (its row pair's
// intervals and the reference's running sums at that quad) and the pixel is shaded.  Used for
// frames of small triangles, where the pixels of a quad mostly have different winners.  One CTA
// of 256 threads per 16x16 tile.
__global__ void __launch_bounds__(256, 4) resolve_pixels_kernel(BatchParams b, const DrawRecord *__restrict__ records,
                                                                const uint32_t *__restrict__ binOffsets,
                                                                const uint32_t *__restrict__ rowOffsets, const uint32_t *__restrict__ rows) {
	chain_enter();
	if (overflowed(b)) return;
	const uint32_t tile = blockIdx.x;
	if (binOffsets[2 * tile] == binOffsets[2 * tile + 2]) return;
	const FrameTarget &f = b.frames[find_segment(b.frameTileBase, b.frameCount, tile)];
	const int32_t local = (int32_t)(tile - f.tileBase);
	const int32_t px = (local % f.tilesX) * TILE_W + (threadIdx.x & 15), py = (local / f.tilesX) * TILE_H + (threadIdx.x >> 4);
	if (px >= f.width || py >= f.height) return;
	const unsigned long long key = f.keys[(size_t)py * f.width + px];
	if (key != 0ull) resolve_pixel(b, f, records, rowOffsets, rows, px, py, key);
}

// One thread per 2x2 quad: the winners of its pixels are grouped by record, and for each record
// the reference's running sums of the quad (its row pair's intervals and chains), the vertex
// weights, the shader inputs and the mip level are evaluated once for all the pixels it won
// (deferred shading: only winners are shaded).  Used for frames of larger triangles, where a
// quad's pixels mostly share their winner.  One CTA of 64 threads per 16x16 tile.
__global__ void __launch_bounds__(64) resolve_quads_kernel(BatchParams b, const DrawRecord *__restrict__ records,
                                                     const uint32_t *__restrict__ binOffsets,
                                                     const uint32_t *__restrict__ rowOffsets, const uint32_t *__restrict__ rows) {
	chain_enter();
	if (overflowed(b)) return;
	const uint32_t tile = blockIdx.x;
	if (binOffsets[2 * tile] == binOffsets[2 * tile + 2]) return;
	const FrameTarget &f = b.frames[find_segment(b.frameTileBase, b.frameCount, tile)];
	const int32_t local = (int32_t)(tile - f.tileBase);
	const int32_t x = (local % f.tilesX) * TILE_W + 2 * (threadIdx.x & 7), y1 = (local / f.tilesX) * TILE_H + 2 * (threadIdx.x >> 3);
	const int32_t width = f.width, height = f.height;
	if (x >= width || y1 >= height) return;
	const bool depthTest = f.depth != nullptr, affine = f.affine != 0;
	uint32_t record[4];
	uint32_t pending = 0;
	for (int l = 0; l < 4; l++) {
		const int32_t px = x + (l & 1), py = y1 + (l >> 1);
		record[l] = 0;
		// depth-tested pixels of an odd-height target's last row: odd_row_kernel
		if (px < width && py < height && !(depthTest && odd_last_row(py, height))) {
			const unsigned long long key = f.keys[(size_t)py * width + px];
			if (key != 0ull) {
				record[l] = key_record(key, depthTest);
				pending |= 1u << l;
			}
		}
	}
	while (pending) {
		const int first = __ffs(pending) - 1;
		const uint32_t ri = record[first];
		uint32_t mask = 0;
		for (int l = first; l < 4; l++)
			if ((pending & (1u << l)) && record[l] == ri) mask |= 1u << l;
		pending &= ~mask;
		const DrawRecord r = records[ri];
		const RowPair pair = record_row_pair(r, rows + rowOffsets[ri], y1, height);
		float w[3][4];
		const int components = f.color ? 3 : 1;
		for (int c = 0; c < components; c++) quad_lanes(r.start[c], r.dx[c], r.dy[c], pair, y1, x, w[c]);
		if (f.color) {
			float wa[4], wb[4], wc[4];
			lane_weights(w, affine, wa, wb, wc);
			ShadeRecord shade;
			make_shade(b.tasks[r.task], r.source, shade);
			float u[4], v[4];
			const uint32_t mip = quad_diffuse_coordinates(shade, b.textures, wa, wb, wc, u, v);
			// no depth buffer, last row of an odd height: the lower lanes of full quads are written last
			const int lower = (odd_last_row(y1, height) && full_quad(pair, x)) ? 2 : 0;
#pragma unroll
			for (int l = 0; l < 4; l++) {
				if (!(mask & (1u << l))) continue;
				float rgba[4];
				shade_quad_lane(shade, b.textures, wa, wb, wc, u, v, mip, l + lower, rgba);
				f.color[(size_t)(y1 + (l >> 1)) * f.colorStride + x + (l & 1)] = pack_saturated(rgba, f.packOrder);
			}
		}
		if (depthTest)
			for (int l = 0; l < 4; l++)
				if (mask & (1u << l)) f.depth[(size_t)(y1 + (l >> 1)) * f.depthStride + x + (l & 1)] = w[0][l];
	}
}

// ------------------------------------------------------------------ last row of odd heights

// Records one odd_row_kernel window holds (candidates of all 16 columns in shared memory).
static const int ODD_WINDOW = 320;
static const int ODD_SORT = 512; // ODD_WINDOW rounded up to a power of two, for the bitonic sort

// Whether a record can touch row y of the 16 columns from tx0 (its bound, which holds every pixel
// it writes, the lower lanes of the last row's full quads included).
__device__ __forceinline__ bool odd_row_relevant(const DrawRecord *__restrict__ records, uint32_t ri, int32_t y, int32_t tx0) {
	const int4 bound = *reinterpret_cast<const int4 *>(&records[ri].flat[4]); // flat[4], flat[5], left, top
	const int2 rb = *reinterpret_cast<const int2 *>(&records[ri].right);
	return bound.w <= y && rb.y > y && bound.z < tx0 + TILE_W && rb.x > tx0;
}

// Relevant records of the tile's list with index in [lo, hi): counted, and the largest one.
__device__ __forceinline__ void odd_row_count(const DrawRecord *__restrict__ records, const uint32_t *__restrict__ lists,
                                              uint32_t begin, uint32_t end, uint32_t lo, uint32_t hi, int32_t y, int32_t tx0,
                                              uint32_t *count, uint32_t *largest) {
	__syncthreads(); // every thread has read the previous totals
	if (threadIdx.x == 0) { *count = 0u; *largest = 0u; }
	__syncthreads();
	uint32_t n = 0, m = 0;
	for (uint32_t e = begin + threadIdx.x; e < end; e += blockDim.x) {
		const uint32_t ri = lists[e];
		if (ri >= lo && ri < hi && odd_row_relevant(records, ri, y, tx0)) { n++; m = max(m, ri); }
	}
	if (n) { atomicAdd(count, n); atomicMax(largest, m); }
	__syncthreads();
}

// The last row of a depth-tested frame of odd height, in submission order (odd_last_row).  Along
// the run of full quads of that row pair a triangle writes its lower lane's value over its upper
// lane's whenever the lower lane passes the depth test, even where the upper lane is nearer, so
// the row's result is not the nearest fragment and the max-key argument of the tile pass does not
// hold: the tile pass leaves the row alone and this kernel replays it.  One CTA per tile of the
// frame's bottom tile row (blockIdx.x the tile column, blockIdx.y the frame).  The tile's records
// that reach the row are taken in windows of at most ODD_WINDOW in increasing record index (the
// submission order); a window is sorted in shared memory, every (record, column) pair evaluates its
// upper and lower candidates in parallel (quad_lanes, as the tile pass does), and one thread per
// column folds them in order with the reference's strict tests: the lower lane if it beats the
// stored depth, else the upper one if it does.  The winner is shaded once at the end.
__global__ void __launch_bounds__(256) odd_row_kernel(BatchParams b, const DrawRecord *__restrict__ records,
                                                      const uint32_t *__restrict__ binOffsets, const uint32_t *__restrict__ lists,
                                                      const uint32_t *__restrict__ rowOffsets, const uint32_t *__restrict__ rows) {
	chain_enter();
	if (overflowed(b)) return;
	__shared__ uint32_t ids[ODD_SORT];
	__shared__ float2 candidates[ODD_WINDOW * TILE_W];
	__shared__ uint32_t count, largest;
	// every condition that skips a frame or tile is the same for the whole CTA
	for (int32_t frame = (int32_t)blockIdx.y; frame < b.frameCount; frame += (int32_t)gridDim.y) {
		const FrameTarget &f = b.frames[frame];
		if (!(f.height & 1) || f.depth == nullptr || (int32_t)blockIdx.x >= f.tilesX) continue;
		const uint32_t tile = f.tileBase + (uint32_t)((f.tilesY - 1) * f.tilesX) + blockIdx.x;
		const uint32_t begin = binOffsets[2 * tile], end = binOffsets[2 * tile + 2];
		if (begin == end) continue;
		const int32_t y = f.height - 1, tx0 = (int32_t)blockIdx.x * TILE_W, width = f.width;
		const bool affine = f.affine != 0;
		const int tid = threadIdx.x;
		// fold state of column tid (threads 0..15); orthogonal depths are negated so that the nearer
		// one is always the greater (x < y exactly when -x > -y, and NaN fails both)
		const int32_t px = tx0 + tid;
		float stored = 0.0f;
		uint32_t winner = 0xFFFFFFFFu;
		int winnerLower = 0;
		if (tid < TILE_W && px < width) {
			stored = f.depth[(size_t)y * f.depthStride + px];
			if (affine) stored = -stored;
		}
		uint32_t lo = 0;
		for (;;) {
			odd_row_count(records, lists, begin, end, lo, 0xFFFFFFFFu, y, tx0, &count, &largest);
			uint32_t n = count;
			if (n == 0) break;
			uint32_t hi = 0xFFFFFFFFu;
			if (n > (uint32_t)ODD_WINDOW) {
				// the largest hi whose window [lo, hi) holds at most ODD_WINDOW records (bisection;
				// [lo, lo + 1) holds at most one, [lo, largest + 1) too many)
				uint32_t good = lo + 1, bad = largest + 1;
				while (bad - good > 1) {
					const uint32_t mid = good + (bad - good) / 2;
					odd_row_count(records, lists, begin, end, lo, mid, y, tx0, &count, &largest);
					if (count <= (uint32_t)ODD_WINDOW) good = mid; else bad = mid;
				}
				hi = good;
			}
			// gather the window (any order), then sort it ascending
			__syncthreads();
			if (tid == 0) count = 0u;
			__syncthreads();
			for (uint32_t e = begin + tid; e < end; e += blockDim.x) {
				const uint32_t ri = lists[e];
				if (ri >= lo && ri < hi && odd_row_relevant(records, ri, y, tx0)) {
					const uint32_t slot = atomicAdd(&count, 1u);
					if (slot < (uint32_t)ODD_WINDOW) ids[slot] = ri; // always true: the window was sized by the same test
				}
			}
			__syncthreads();
			n = min(count, (uint32_t)ODD_WINDOW);
			for (uint32_t i = n + tid; i < (uint32_t)ODD_SORT; i += blockDim.x) ids[i] = 0xFFFFFFFFu;
			__syncthreads();
			for (uint32_t k = 2; k <= (uint32_t)ODD_SORT; k <<= 1) {
				for (uint32_t j = k >> 1; j > 0; j >>= 1) {
					for (uint32_t i = tid; i < (uint32_t)ODD_SORT; i += blockDim.x) {
						const uint32_t partner = i ^ j;
						if (partner > i) {
							const uint32_t a = ids[i], c = ids[partner];
							const bool ascending = (i & k) == 0;
							if ((a > c) == ascending) { ids[i] = c; ids[partner] = a; }
						}
					}
					__syncthreads();
				}
			}
			// candidates of every (record, column): upper lane where covered, lower lane in full quads
			for (uint32_t p = tid; p < n * TILE_W; p += blockDim.x) {
				const uint32_t j = p >> 4;
				const int32_t cx = tx0 + (int32_t)(p & 15);
				const float none = __int_as_float(0x7FC00000); // quiet NaN: fails every depth test
				float2 cand = make_float2(none, none);
				if (cx < width) {
					const uint32_t ri = ids[j];
					const DrawRecord r = records[ri];
					const RowPair pair = record_row_pair(r, rows + rowOffsets[ri], y, f.height);
					const int32_t x = cx & ~1;
					if (pair.any && x >= pair.obs && x < pair.obe) {
						float v[4];
						quad_lanes(r.start[0], r.dx[0], r.dy[0], pair, y, x, v);
						const bool full = full_quad(pair, x);
						const int l = cx & 1;
						if (lane_covered(pair, x, !full, l)) cand.x = affine ? -v[l] : v[l];
						if (full) cand.y = affine ? -v[l + 2] : v[l + 2];
					}
				}
				candidates[p] = cand;
			}
			__syncthreads();
			if (tid < TILE_W) {
				for (uint32_t j = 0; j < n; j++) {
					const float2 cand = candidates[j * TILE_W + tid];
					if (cand.y > stored) { stored = cand.y; winner = ids[j]; winnerLower = 1; }
					else if (cand.x > stored) { stored = cand.x; winner = ids[j]; winnerLower = 0; }
				}
			}
			__syncthreads();
			if (hi == 0xFFFFFFFFu) break;
			lo = hi;
		}
		if (tid < TILE_W && px < width && winner != 0xFFFFFFFFu) {
			const DrawRecord r = records[winner];
			const int32_t x = px & ~1;
			const RowPair pair = record_row_pair(r, rows + rowOffsets[winner], y, f.height);
			write_lane(b, f, r, pair, y, x, (px & 1) + (winnerLower ? 2 : 0), px, y, affine);
		}
		__syncthreads(); // the next frame reuses the shared arrays
	}
}

// ------------------------------------------------------------------ alpha filter

// Tile of every list entry (the entries of tile t are [offsets[2t], offsets[2t + 2])).
__global__ void entry_tile_kernel(const uint32_t *__restrict__ binOffsets, uint32_t *entryTile) {
	const uint32_t tile = blockIdx.x;
	const uint32_t begin = binOffsets[2 * tile], end = binOffsets[2 * tile + 2];
	for (uint32_t e = begin + threadIdx.x; e < end; e += blockDim.x) entryTile[e] = tile;
}

// After the sort by record: the tile of each sorted entry (key of the second sort) and its record.
__global__ void tile_keys_kernel(const uint32_t *__restrict__ entryTile, const uint32_t *__restrict__ sortedRecords,
                                 const uint32_t *__restrict__ sortedEntries, uint32_t n, uint32_t *tileKeys, uint32_t *records) {
	for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
		tileKeys[i] = entryTile[sortedEntries[i]];
		records[i] = sortedRecords[i];
	}
}

// Alpha-filtered triangles (fillQuadSuper with Filter::Alpha, fillerTemplates.h:160-186, read-only
// depth: fillerTemplates.h:386-441): every covered fragment that passes the depth test blends its
// colour over the pixel, source * (alpha / 255) + target * (1 - alpha / 255), packed with
// saturation after each blend, and writes no depth.  The order matters, so one thread per pixel
// takes the tile's records in submission order (lists sorted by record).  The fragment's value is
// re-evaluated exactly as the resolve pass does.  One CTA of 256 threads per 16x16 tile.
__global__ void __launch_bounds__(256) alpha_kernel(BatchParams b, const DrawRecord *__restrict__ records,
                                                    const uint32_t *__restrict__ binOffsets, const uint32_t *__restrict__ sorted,
                                                    const uint32_t *__restrict__ rowOffsets, const uint32_t *__restrict__ rows) {
	if (overflowed(b)) return;
	const uint32_t tile = blockIdx.x;
	const uint32_t begin = binOffsets[2 * tile], end = binOffsets[2 * tile + 2];
	if (begin == end) return;
	const FrameTarget &f = b.frames[find_segment(b.frameTileBase, b.frameCount, tile)];
	const int32_t local = (int32_t)(tile - f.tileBase);
	const int32_t px = (local % f.tilesX) * TILE_W + (threadIdx.x & 15), py = (local / f.tilesX) * TILE_H + (threadIdx.x >> 4);
	if (px >= f.width || py >= f.height || !f.color) return;
	const bool depthTest = f.depth != nullptr, affine = f.affine != 0;
	const float stored = depthTest ? f.depth[(size_t)py * f.depthStride + px] : 0.0f;
	uint32_t *target = f.color + (size_t)py * f.colorStride + px;
	uint32_t packed = *target;
	const int32_t y1 = py & ~1, x = px & ~1;
	const int lane4 = ((py & 1) << 1) | (px & 1);
	const bool oddRow = odd_last_row(py, f.height);
	uint32_t fragments = 0;
	for (uint32_t e = begin; e < end; e++) {
		const uint32_t ri = sorted[e];
		const DrawRecord r = records[ri];
		if (py < r.top || py >= r.bottom || px < r.left || px >= r.right) continue;
		int32_t left, right;
		unpack_row(rows[rowOffsets[ri] + (py - r.top)], left, right);
		if (px < left || px >= right) continue;
		fragments++;
		const RowPair pair = record_row_pair(r, rows + rowOffsets[ri], y1, f.height);
		float w[3][4];
		for (int c = 0; c < 3; c++) quad_lanes(r.start[c], r.dx[c], r.dy[c], pair, y1, x, w[c]);
		const float z = (lane4 == 0) ? w[0][0] : (lane4 == 1) ? w[0][1] : (lane4 == 2) ? w[0][2] : w[0][3];
		int lane = lane4;
		if (oddRow && full_quad(pair, x)) {
			// the lower lane reads the same target colour and is written after the upper one: it
			// decides the pixel when it passes the depth test (odd_last_row)
			const float zl = w[0][lane4 + 2];
			if (!depthTest || (affine ? (zl < stored) : (zl > stored))) lane = lane4 + 2;
		}
		if (lane == lane4 && depthTest && !(affine ? (z < stored) : (z > stored))) continue;
		float wa[4], wb[4], wc[4];
		lane_weights(w, affine, wa, wb, wc);
		ShadeRecord shade;
		make_shade(b.tasks[r.task], r.source, shade);
		float rgba[4];
		shade_lane_inline(shade, b.textures, wa, wb, wc, lane, rgba);
		const float opacity = fmul(rgba[3], 1.0f / 255.0f);
		const float keep = fsub(1.0f, opacity);
		float blended[4];
		for (int c = 0; c < 4; c++) {
			const float t = (float)((packed >> pack_shift(f.packOrder, c)) & 0xFFu);
			blended[c] = fadd(fmul(rgba[c], opacity), fmul(t, keep));
		}
		packed = pack_saturated(blended, f.packOrder);
	}
	*target = packed;
	if (f.coverage) f.coverage[(size_t)py * f.width + px] += fragments;
	if (b.fragments && fragments) atomicAdd(b.fragments, (unsigned long long)fragments);
	if (b.walked && fragments) atomicAdd(b.walked, (unsigned long long)fragments);
}

void launch_alpha(const BatchParams &b, const FrameBuffers &fb, const TileBins &bins, uint32_t entries, uint32_t recordCount,
                  const AlphaBuffers &a, cudaStream_t stream) {
	if (b.totalTiles == 0) return;
	const uint32_t *sorted = bins.lists;
	if (entries > 1) {
		// every tile's list in submission order: a stable sort of the entries by record, then a
		// stable sort of that order by tile (a tile's entries keep their offsets, which only
		// depend on the tile's count)
		COUNT_LAUNCH();
		entry_tile_kernel<<<b.totalTiles, 128, 0, stream>>>(bins.offsets, a.entryTile);
		int recordBits = 1, tileBits = 1;
		while ((1ull << recordBits) < (uint64_t)recordCount) recordBits++;
		while ((1ull << tileBits) < (uint64_t)b.totalTiles) tileBits++;
		const uint32_t *records = nullptr, *order = nullptr;
		launch_stable_sort(bins.lists, nullptr, entries, recordBits, a.sort, stream, &records, &order);
		COUNT_LAUNCH();
		tile_keys_kernel<<<grid_for(entries, 256), 256, 0, stream>>>(a.entryTile, records, order, entries, a.tileKeys, a.records);
		const uint32_t *tiles = nullptr;
		launch_stable_sort(a.tileKeys, a.records, entries, tileBits, a.sort, stream, &tiles, &sorted);
	}
	COUNT_LAUNCH();
	alpha_kernel<<<b.totalTiles, 256, 0, stream>>>(b, fb.records, bins.offsets, sorted, fb.rowOffsets, fb.rows);
}

void launch_odd_rows(const BatchParams &b, const FrameBuffers &fb, const TileBins &bins, cudaStream_t stream) {
	if (b.depthOnly || b.oddDepthFrames == 0 || b.totalTiles == 0) return;
	COUNT_LAUNCH();
	const unsigned frames = (unsigned)std::min<int32_t>(b.frameCount, 65535);
	launch_chained(odd_row_kernel, dim3((unsigned)b.maxTilesX, frames), 256, stream, b, fb.records, bins.offsets,
	               bins.lists, fb.rowOffsets, fb.rows);
}

void launch_raster(const BatchParams &b, const FrameBuffers &fb, const TileBins &bins, const RasterConfig &config, bool resolve,
                   cudaStream_t stream) {
	if (b.totalTiles == 0) return;
	if (!bins.cleared) memset_async(b.tileQueue, 0, sizeof(uint32_t), stream);
	const int threads = config.threadsPerTile == 64 ? 64 : (config.threadsPerTile == 128 ? 128 : 256);
	const int maxPerSm = 1024 / threads;
	const int perSm = config.ctasPerSm < 1 ? 1 : (config.ctasPerSm > maxPerSm ? maxPerSm : config.ctasPerSm);
	uint32_t ctas = (uint32_t)sm_count() * (uint32_t)perSm;
	if (ctas > b.totalTiles) ctas = b.totalTiles;
	COUNT_LAUNCH();
	// small triangles resolve per pixel inside the tile pass; the keys then never leave the chip
	const bool fused = resolve && !b.depthOnly && config.resolveMode == 1;
#define DSRG_RASTER(T)                                                                                            \
	if (b.depthOnly && resolve) launch_chained(raster_kernel<true, T, true>, ctas, T, stream, b, fb.records, bins, fb.rowOffsets, fb.rows); \
	else if (b.depthOnly) launch_chained(raster_kernel<true, T, false>, ctas, T, stream, b, fb.records, bins, fb.rowOffsets, fb.rows); \
	else if (fused) launch_chained(raster_kernel<false, T, true>, ctas, T, stream, b, fb.records, bins, fb.rowOffsets, fb.rows); \
	else launch_chained(raster_kernel<false, T, false>, ctas, T, stream, b, fb.records, bins, fb.rowOffsets, fb.rows);
	if (threads == 64) { DSRG_RASTER(64) }
	else if (threads == 128) { DSRG_RASTER(128) }
	else { DSRG_RASTER(256) }
#undef DSRG_RASTER
	if (!resolve) return;
	if (!fused && !b.depthOnly) { // depth-only batches resolve inside the tile pass (depth_from_key)
		COUNT_LAUNCH();
		if (config.resolveMode == 2) launch_chained(resolve_quads_kernel, b.totalTiles, 64, stream, b, fb.records, bins.offsets, fb.rowOffsets, fb.rows);
		else launch_chained(resolve_pixels_kernel, b.totalTiles, 256, stream, b, fb.records, bins.offsets, fb.rowOffsets, fb.rows);
	}
	// the last rows of depth-tested odd-height frames, which every resolve above leaves alone
	launch_odd_rows(b, fb, bins, stream);
}

} // namespace dsrg
