// Internal declarations shared by the host-side translation units of libdsrg
// (objects behind the C ABI handles and host helpers); not part of the public ABI.
#ifndef DSRG_INTERNAL_H
#define DSRG_INTERNAL_H

#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/dsrg.h"
#include "dsrg_geometry.h"
#include "dsrg_kernels.h"

namespace dsrg {

// Every device allocation of the library (cudaMalloc), so that a test can make the k-th one fail
// as an exhausted device would (dsrg_debug_fail_allocation).
cudaError_t device_alloc(void **p, size_t bytes);

template <typename T>
struct DeviceBuffer {
	T *ptr = nullptr;
	size_t capacity = 0;
	cudaError_t reserve(size_t n, bool keep = false, size_t keepCount = 0, cudaStream_t stream = 0) {
		if (n <= capacity) return cudaSuccess;
		size_t newCapacity = capacity ? capacity : 1024;
		while (newCapacity < n) newCapacity *= 2;
		T *fresh = nullptr;
		cudaError_t err = device_alloc((void **)&fresh, newCapacity * sizeof(T));
		if (err != cudaSuccess) return err;
		if (keep && ptr && keepCount) {
			err = cudaMemcpyAsync(fresh, ptr, keepCount * sizeof(T), cudaMemcpyDeviceToDevice, stream);
			if (err != cudaSuccess) { cudaFree(fresh); return err; }
			cudaStreamSynchronize(stream);
		}
		if (ptr) cudaFree(ptr);
		ptr = fresh;
		capacity = newCapacity;
		return cudaSuccess;
	}
	void release() {
		if (ptr) cudaFree(ptr);
		ptr = nullptr;
		capacity = 0;
	}
};

// Page-locked host memory that a call fills and copies to the device asynchronously: a copy from
// pageable memory would first wait for everything queued on the stream.  Grown as needed; the
// call that filled it must be finished before the next one refills it.
struct HostStaging {
	unsigned char *ptr = nullptr;
	size_t capacity = 0;
	cudaError_t reserve(size_t n) {
		if (n <= capacity) return cudaSuccess;
		if (ptr) cudaFreeHost(ptr);
		ptr = nullptr;
		capacity = 0;
		size_t c = 4096;
		while (c < n) c *= 2;
		const cudaError_t e = cudaMallocHost((void **)&ptr, c);
		if (e == cudaSuccess) capacity = c;
		return e;
	}
	void release() {
		if (ptr) cudaFreeHost(ptr);
		ptr = nullptr;
		capacity = 0;
	}
};

// Camera::createPerspective / createOrthogonal and ViewFrustum (implementation/render/Camera.h:55-156),
// computed on the host in the reference's order (this file is built with -ffp-contract=off).
inline Plane make_plane(float x, float y, float z, float offset) {
	Plane p;
	float l = sqrtf(x * x + y * y + z * z);
	if (l == 0.0f) { p.nx = 0.0f; p.ny = 0.0f; p.nz = 1.0f; }
	else { p.nx = x / l; p.ny = y / l; p.nz = z / l; }
	p.offset = offset;
	return p;
}

inline int frustum_perspective(Plane *planes, float nearClip, float farClip, float ws, float hs) {
	planes[0] = make_plane(-1.0f, 0.0f, -ws, 0.0f);
	planes[1] = make_plane(1.0f, 0.0f, -ws, 0.0f);
	planes[2] = make_plane(0.0f, 1.0f, -hs, 0.0f);
	planes[3] = make_plane(0.0f, -1.0f, -hs, 0.0f);
	planes[4] = make_plane(0.0f, 0.0f, -1.0f, -nearClip);
	planes[5] = make_plane(0.0f, 0.0f, 1.0f, farClip);
	return std::isinf(farClip) && farClip > 0 ? 5 : 6;
}

inline int frustum_orthogonal(Plane *planes, float hw, float hh) {
	planes[0] = make_plane(-1.0f, 0.0f, 0.0f, hw);
	planes[1] = make_plane(1.0f, 0.0f, 0.0f, hw);
	planes[2] = make_plane(0.0f, 1.0f, 0.0f, hh);
	planes[3] = make_plane(0.0f, -1.0f, 0.0f, hh);
	return 4;
}

inline CameraData make_camera(const dsrg_camera &d) {
	CameraData c;
	memset(&c, 0, sizeof(c));
	for (int i = 0; i < 3; i++) {
		c.position[i] = d.location[i];
		c.xAxis[i] = d.location[3 + i];
		c.yAxis[i] = d.location[6 + i];
		c.zAxis[i] = d.location[9 + i];
	}
	c.imageWidth = (float)d.width;
	c.imageHeight = (float)d.height;
	c.perspective = d.perspective ? 1 : 0;
	float ws = d.slope;
	float hs = ws * c.imageHeight / c.imageWidth;
	if (d.perspective) {
		c.cullCount = frustum_perspective(c.cull, d.nearClip, d.farClip, ws * 1.0001f, hs * 1.0001f);
		c.clipCount = frustum_perspective(c.clip, d.nearClip, d.farClip, ws * 2.0f, hs * 2.0f);
	} else {
		c.cullCount = frustum_orthogonal(c.cull, ws * 1.0001f, hs * 1.0001f);
		c.clipCount = frustum_orthogonal(c.clip, ws * 2.0f, hs * 2.0f);
	}
	c.invWidthSlope = 0.5f / ws;
	c.invHeightSlope = 0.5f / hs;
	return c;
}

// Camera::isBoxSeen (implementation/render/Camera.h:202-217).
inline bool box_seen(const CameraData &c, const float *mn, const float *mx, const float *modelToWorld) {
	const float corners[8][3] = {{mn[0], mn[1], mn[2]}, {mx[0], mn[1], mn[2]}, {mn[0], mx[1], mn[2]}, {mx[0], mx[1], mn[2]},
	                             {mn[0], mn[1], mx[2]}, {mx[0], mn[1], mx[2]}, {mn[0], mx[1], mx[2]}, {mx[0], mx[1], mx[2]}};
	Vec3 cs[8];
	for (int i = 0; i < 8; i++) cs[i] = world_to_camera(c, transform_point(modelToWorld, vec3(corners[i][0], corners[i][1], corners[i][2])));
	for (int s = 0; s < c.cullCount; s++) {
		bool anyInside = false;
		for (int i = 0; i < 8; i++) if (plane_inside(c.cull[s], cs[i])) anyInside = true;
		if (!anyInside) return false;
	}
	return true;
}


// One batch for the kernels: frames (targets in device memory) and the tasks drawing into them.
// The tasks of one frame must appear in submission order; their orderBase counts the fan
// triangles given to the same frame before them.
struct BatchJob {
	std::vector<TaskParams> tasks;
	std::vector<FrameTarget> frames;  // color, depth, strides, packOrder, size, affine and coverage set by the caller
	std::vector<TextureData> textures;
	bool depthOnly = false;
	bool resolve = true;
	bool alpha = false;         // every task is alpha-filtered and every frame has a colour target
	bool clearCounters = true;  // false for the later runs of one frame: fragment counts accumulate
	bool hostTargets = false;   // a target is page-locked host memory drawn in place: resolve per pixel,
	                            // whose stores run along rows, even where the tuning asks for quads
};

// The launches of one phase between two host synchronisations, kept as a CUDA graph.  A phase
// whose launch parameters (key) repeat those of the previous call is captured on the repeat and
// replayed from then on; a phase whose parameters change every call is launched directly.
struct PhaseGraph {
	std::vector<unsigned char> key;
	cudaGraphExec_t exec = nullptr;
	uint64_t launches = 0; // kernels in the graph
	void reset() {
		if (exec) cudaGraphExecDestroy(exec);
		exec = nullptr;
		key.clear();
		launches = 0;
	}
};

struct BatchTotals {
	uint32_t points = 0, triangles = 0, tiles = 0;
	size_t pixels = 0;
	uint32_t records = 0, rows = 0, binEntries = 0;
};

} // namespace dsrg

using dsrg::DeviceBuffer;
using dsrg::HostStaging;
using dsrg::DrawRecord;
using dsrg::TaskParams;
using dsrg::FrameTarget;
using dsrg::BatchParams;
using dsrg::TextureData;
using dsrg::CameraData;

struct dsrg_context_s {
	int device = 0;
	cudaStream_t stream = nullptr;
	std::string lastError;
	// frame scratch, grown on demand and reused
	DeviceBuffer<float4> pointCsis;      // projected points (ProjectedPoints)
	DeviceBuffer<float> pointIsy;
	DeviceBuffer<longlong2> pointFlat;
	DeviceBuffer<uint32_t> triCounts, triOffsets, scanScratch;
	DeviceBuffer<unsigned long long> denseKeys; // per-pixel winners of dsrg_dense_render
	DeviceBuffer<unsigned char> denseInstances; // the instance table of one dense-model call
	DeviceBuffer<DrawRecord> records;
	DeviceBuffer<unsigned char> tables;  // the batch's task, frame and texture tables
	unsigned char *pinnedTables = nullptr; // host staging of the tables (page-locked)
	size_t pinnedCapacity = 0;
	DeviceBuffer<uint32_t> control;      // [0] tile queue, [1] error flag, [4..7] a batch's gathered totals, [9] listed tiles
	DeviceBuffer<uint32_t> tileList;     // the tiles of a batch that have tile-list entries
	uint32_t *pinnedReadback = nullptr;  // page-locked: the gathered totals (written there by the GPU), the fragment count,
	                                     // [8] the entries a deterministic adjoint's sums keep
	uint32_t *readbackDevice = nullptr;  // its device address
	bool timingPending = false;          // stats' times not yet read from the events of the last call
	bool timingHasRaster = false;
	bool stopRecorded = false;           // the last batch recorded eventStop before its host wait
	// capacities of the buffers sized before their totals are known (largest totals seen, with slack)
	uint64_t recordCapacity = 0, rowCapacity = 0, binCapacity = 0;
	DeviceBuffer<uint32_t> binCounts, binOffsets, binCursors, binLists;
	DeviceBuffer<uint32_t> bigList;      // records binned a warp each (their count lives in control[8])
	DeviceBuffer<TextureData> textureTable;
	DeviceBuffer<uint32_t> stagingColor;
	DeviceBuffer<uint32_t> textureStaging;      // texture creation: host images and two-step resize halves
	DeviceBuffer<unsigned char> textureTables;  // texture creation: work tables
	DeviceBuffer<float> stagingDepth;
	DeviceBuffer<uint32_t> lightStaging;        // light passes and draw_higher: pageable host images and sprites
	HostStaging spriteTableHost, lightTableHost; // draw_higher's sprite table and the point lights' table on their way to the GPU
	DeviceBuffer<unsigned long long> spriteKeys; // draw_higher's per-pixel keys and its sprite table, apart from the
	DeviceBuffer<unsigned char> spriteTables;    // pipeline's, so that a sprite frame can draw sprites beside its shadows
	cudaStream_t sideStream = nullptr;           // a sprite frame's second stream (created on first use)
	cudaStream_t branchStream = nullptr;         // a batch's second branch: the row intervals beside the tile lists
	cudaEvent_t branchFork = nullptr, branchJoin = nullptr;
	cudaEvent_t sideStart = nullptr, sideDone = nullptr;
	DeviceBuffer<unsigned long long> fragmentCounter;
	DeviceBuffer<unsigned long long> keys;
	DeviceBuffer<uint32_t> rowCounts, rowOffsets, rows;
	DeviceBuffer<uint32_t> alphaEntryTile, alphaTileKeys, alphaRecords; // the alpha filter's list order
	DeviceBuffer<uint32_t> sortKeysA, sortKeysB, sortIdsA, sortIdsB, sortHist, sortOffsets;
	int32_t smallRows = 8, smallWidth = 16; // one lane walks records whose raster bound is at most 8 x 16 pixels
	int32_t ctasPerSm = 4;                  // resident CTAs per SM of the persistent tile kernel
	int32_t threadsPerTile = 256;           // threads of one tile's CTA
	int32_t useGraphs = 1;                  // replay unchanged phases as CUDA graphs
	int32_t resolveMode = 1;                // 0 per pixel in its own pass, 1 per pixel in the tile kernel, 2 per quad
	dsrg::PhaseGraph graphs[4];             // phases A, B, C (lists) and D (raster)
	int32_t counting = 0;
	uint32_t *coverage = nullptr;
	dsrg_stats stats;
	cudaEvent_t eventStart = nullptr, eventStop = nullptr, eventRasterStart = nullptr, eventRasterStop = nullptr;
	dsrg_renderer implicitRenderer = nullptr;
	dsrg::BatchJob frameJob;                // reused by renderer_end
};

struct dsrg_texture_s {
	dsrg_context context;
	uint32_t *pixels = nullptr;
	uint32_t fields[9];
	uint32_t pixelCount = 0;
	TextureData data;
};

struct dsrg_model_s {
	dsrg_context context;
	float *positions = nullptr;
	int32_t *polygons = nullptr;
	float *texCoords = nullptr;
	float *colors = nullptr;
	int32_t *triSource = nullptr;
	int32_t pointCount = 0, polygonCount = 0, triangleCount = 0;
	float minBound[3], maxBound[3];
	dsrg_texture diffuse = nullptr, light = nullptr;
	int32_t filter = 0;
};

struct dsrg_renderer_s {
	dsrg_context context;
	bool receiving = false;
	dsrg_image color, depth;
	bool hasColor = false, hasDepth = false;
	int32_t width = 0, height = 0;
	uint32_t *deviceColor = nullptr;
	float *deviceDepth = nullptr;
	bool colorDirect = false, depthDirect = false; // page-locked host images used in place
	int32_t colorStride = 0, depthStride = 0;
	uint32_t triangleCount = 0;   // fan triangles submitted this frame
	bool depthOnly = false;
	bool affine = false;
	bool cameraKnown = false;
	std::vector<TextureData> textures;
	std::vector<dsrg_texture> textureHandles;
	std::vector<TaskParams> tasks;
	std::vector<TaskParams> runTasks; // the frame's tasks while it runs as alpha-filtered and other runs
	// renderer_giveTask_triangle data of this frame, uploaded before the tasks run (given tasks
	// point into the device copy; givenTasks lists them with their first triangle)
	std::vector<dsrg::GivenPoint> givenPoints;
	std::vector<int32_t> givenPolygons, givenSource;
	std::vector<float> givenTexCoords, givenColors;
	std::vector<std::pair<size_t, uint32_t>> givenTasks;
	bool givenDirty = false;
	DeviceBuffer<unsigned char> givenDevice;
	// occlusion grid (RendererImpl::depthGrid, api/rendererAPI.cpp:141-191): one float per 16x16
	// cell, kept on the host for box occluders and box tests and on the device for the per-command
	// work; whichever copy is stale is refreshed from the other before it is used
	bool occluded = false;
	int32_t gridWidth = 0, gridHeight = 0;           // cells covering this frame's target
	int32_t gridAllocWidth = 0, gridAllocHeight = 0; // the grid image, grown but never shrunk; its row stride
	std::vector<float> gridHost;
	DeviceBuffer<float> gridDevice;
	bool gridHostValid = false, gridDeviceValid = false;
	// debug overlays (DebugLine, rendererAPI.cpp:132-137): silhouettes kept until a renderer_end
	// with a colour target draws them (colour as RGBA bytes), and the frame's wireframe lines
	std::vector<int4> debugLines;
	std::vector<uint32_t> debugColors;
	DeviceBuffer<int4> wireLines;
	DeviceBuffer<int4> debugLinesDevice;
};

// Uploads the frame's renderer_giveTask_triangle data and points its tasks at it.
int renderer_upload_given(dsrg_renderer r);
// The device address of page-locked (or registered) host memory, which kernels then read and write
// in place; false for pageable memory, which is staged through device buffers.
bool host_mapped(const void *p, void **devicePointer);
// Queues a fill of a rectangle of 32-bit words (device or mapped memory) with one value.
void enqueue_fill_words(void *image, int32_t strideWords, int32_t width, int32_t height, uint32_t value, cudaStream_t stream);
// Whether every depth image of a batch is reachable by kernels without staging (device or page-locked memory).
bool batch_depth_in_place(dsrg_batch b);
// Queues zeroing of every depth image of a batch (CubeMapF32::clear for a batch of cube faces).
void batch_clear_depth(dsrg_batch b);
// The context a batch belongs to.
dsrg_context batch_context(dsrg_batch b);
// The frame target of a renderer's current frame (images, size, occlusion grid when in use).
void renderer_frame_target(dsrg_renderer r, dsrg::FrameTarget &f);
// Uploads the occlusion grid when the device copy is stale.
int renderer_grid_on_device(dsrg_renderer r);
// isBoxOccluded (api/rendererAPI.cpp:297-341) against the current grid; sets *occluded.
int renderer_box_occluded(dsrg_renderer r, const float *minimum, const float *maximum, const float *modelToWorld,
                          const dsrg::CameraData &camera, bool *occluded);

#define DSRG_CUDA_TRY(ctx, expr)                                                                      \
	do {                                                                                         \
		cudaError_t _e = (expr);                                                                 \
		if (_e != cudaSuccess) {                                                                 \
			(ctx)->lastError = std::string("CUDA error in " #expr ": ") + cudaGetErrorString(_e); \
			return _e == cudaErrorMemoryAllocation ? DSRG_ERROR_OUT_OF_MEMORY : DSRG_ERROR_CUDA; \
		}                                                                                        \
	} while (0)

// Internal status of a batch attempt whose buffers were too small (never returned to callers).
const int DSRG_RETRY = 100;

inline int fail(dsrg_context ctx, int code, const std::string &message) {
	if (ctx) ctx->lastError = message;
	return code;
}

namespace dsrg {


// Fills the tasks' point and triangle bases and the frames' tile ranges and key images
// (keysBase + the frame's first pixel), and lays the tables out for a device copy at deviceBase:
// writes them to `host` when it is not null and points `params` at their device addresses.
// Returns the bytes the tables take.
size_t layout_tables(BatchJob &job, unsigned long long *keysBase, unsigned char *host, unsigned char *deviceBase,
                     BatchParams &params, BatchTotals &totals);
size_t layout_tables(TaskParams *tasks, size_t taskCount, FrameTarget *frames, size_t frameCount, const TextureData *textures,
                     size_t textureCount, bool depthOnly, unsigned long long *keysBase, unsigned char *host,
                     unsigned char *deviceBase, BatchParams &params, BatchTotals &totals);

// Where the kernels of an enqueued batch left their results (all null when nothing was drawn).
struct BatchOutputs {
	BatchParams params;
	FrameBuffers fb;
};

// Runs the phases of the batch on the context's stream (growing its scratch as needed) and
// returns with the raster queued; the caller queues its copies and then calls batch_finish.
// Without the resolve pass (job.resolve = false) every frame's key image is complete: zero where
// nothing was drawn.
int batch_enqueue(dsrg_context ctx, BatchJob &job, BatchTotals &totals, BatchOutputs *outputs = nullptr);
// Waits for the stream, checks the device error bits and fills the context's statistics.
int batch_finish(dsrg_context ctx, const BatchTotals &totals);
// occludeFromExistingTriangles for the job's tasks: projection and triangle setup, the setup's
// commands lowering their frame's occlusion grid instead of becoming records; waits for the GPU.
int occlude_enqueue(dsrg_context ctx, BatchJob &job);

} // namespace dsrg


#endif
