// Differentiable rendering (dsrg_diff_*): a float-target forward pass over the same coverage
// and depth test as dsrg_model_render, a visibility buffer as its checkpoint, and the
// hand-written adjoint that scatters dL/dpixel into the texture, the vertex colours and the
// light, by warp-aggregated atomics or by a deterministic sort-by-target segmented sum.
// The reference has no differentiable renderer; the shading model is stated in include/dsrg.h.
#include <cuda_runtime.h>

#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "dsrg_internal.h"
#include "dsrg_raster.cuh"
#include "dsrg_shade.h"

using namespace dsrg;

namespace {

const uint32_t NO_TRIANGLE = 0xFFFFFFFFu;

struct DiffModel {
	const float *positions;   // pointCount x 3
	const int32_t *polygons;  // polygonCount x 4
	const float *texCoords;   // polygonCount x 4 x 4 (.xy used)
	const int32_t *triSource; // per fan triangle: polygon * 2 + fan index
	int32_t pointCount, triangleCount;
};

struct DiffParams {
	const float *texture;      // [texH][texW][4]
	const float *vertexColors; // [pointCount][4]
	const float *light;        // dir.xyz, intensity
	const float *normals;      // [triangleCount][3], world space, unit
	int32_t log2W, log2H;
	float ambient;
};

// The three corners of fan triangle `tri`: point indices and polygon-corner slots (model/Model.cpp:135-162).
__device__ __forceinline__ void fan_corners(const DiffModel &m, uint32_t tri, int32_t *point, int32_t *slot) {
	const int32_t src = m.triSource[tri];
	const int32_t p = src >> 1, fan = src & 1;
	const int corner[3] = {0, 1 + fan, 2 + fan};
	for (int i = 0; i < 3; i++) {
		slot[i] = p * 4 + corner[i];
		point[i] = m.polygons[slot[i]];
	}
}

// Texel indices and weights of the bilinear sample at (u, v): the sub-texel position of
// texture_sample_bilinear (api/textureAPI.h:320-430) at full resolution, weights w/256.
__device__ __forceinline__ void bilinear_taps(float u, float v, int32_t log2W, int32_t log2H, uint32_t *index, float *weight) {
	const uint32_t scaleU = 256u << log2W, scaleV = 256u << log2H;
	const uint32_t maskX = (1u << log2W) - 1u, maskY = (1u << log2H) - 1u;
	const uint32_t sx = trunc_u32(fmul(fadd(u, 256.0f), (float)scaleU)) - 128u;
	const uint32_t sy = trunc_u32(fmul(fadd(v, 256.0f), (float)scaleV)) - 128u;
	const float fx = fmul((float)(sx & 0xFFu), 0.00390625f), fy = fmul((float)(sy & 0xFFu), 0.00390625f);
	const uint32_t left = (sx >> 8) & maskX, right = ((sx >> 8) + 1u) & maskX;
	const uint32_t top = (sy >> 8) & maskY, bottom = ((sy >> 8) + 1u) & maskY;
	index[0] = (top << log2W) | left;
	index[1] = (top << log2W) | right;
	index[2] = (bottom << log2W) | left;
	index[3] = (bottom << log2W) | right;
	const float gx = 1.0f - fx, gy = 1.0f - fy;
	weight[0] = fmul(gx, gy);
	weight[1] = fmul(fx, gy);
	weight[2] = fmul(gx, fy);
	weight[3] = fmul(fx, fy);
}

// Everything the shading of one visible pixel depends on.
struct PixelShade {
	int32_t point[3];
	float w[3];        // wa, wb, wc
	uint32_t taps[4];
	float tapWeight[4];
	float4 texel, vertex;
	float normalDotLight; // -dot(N, dir)
	float light;          // ambient + intensity * max(0, normalDotLight)
};

__device__ __forceinline__ float4 load4(const float *p) { return *reinterpret_cast<const float4 *>(p); }

__device__ __forceinline__ void shade_pixel(const DiffModel &m, const DiffParams &q, uint32_t tri, float wb, float wc,
                                            PixelShade &s) {
	int32_t slot[3];
	fan_corners(m, tri, s.point, slot);
	s.w[0] = 1.0f - fadd(wb, wc);
	s.w[1] = wb;
	s.w[2] = wc;
	float uv[3][2];
	for (int i = 0; i < 3; i++) {
		uv[i][0] = m.texCoords[slot[i] * 4];
		uv[i][1] = m.texCoords[slot[i] * 4 + 1];
	}
	const float u = fadd(fadd(fmul(uv[0][0], s.w[0]), fmul(uv[1][0], s.w[1])), fmul(uv[2][0], s.w[2]));
	const float v = fadd(fadd(fmul(uv[0][1], s.w[0]), fmul(uv[1][1], s.w[1])), fmul(uv[2][1], s.w[2]));
	bilinear_taps(u, v, q.log2W, q.log2H, s.taps, s.tapWeight);
	float4 t = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
	for (int k = 0; k < 4; k++) {
		const float4 c = load4(q.texture + (size_t)s.taps[k] * 4);
		t.x = fadd(t.x, fmul(c.x, s.tapWeight[k]));
		t.y = fadd(t.y, fmul(c.y, s.tapWeight[k]));
		t.z = fadd(t.z, fmul(c.z, s.tapWeight[k]));
		t.w = fadd(t.w, fmul(c.w, s.tapWeight[k]));
	}
	s.texel = t;
	float4 c = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
	for (int i = 0; i < 3; i++) {
		const float4 vc = load4(q.vertexColors + (size_t)s.point[i] * 4);
		c.x = fadd(c.x, fmul(vc.x, s.w[i]));
		c.y = fadd(c.y, fmul(vc.y, s.w[i]));
		c.z = fadd(c.z, fmul(vc.z, s.w[i]));
		c.w = fadd(c.w, fmul(vc.w, s.w[i]));
	}
	s.vertex = c;
	const float *n = q.normals + (size_t)tri * 3;
	s.normalDotLight = -fadd(fadd(fmul(n[0], q.light[0]), fmul(n[1], q.light[1])), fmul(n[2], q.light[2]));
	s.light = fadd(q.ambient, fmul(q.light[3], s.normalDotLight > 0.0f ? s.normalDotLight : 0.0f));
}

// Unit world-space normal (B - A) x (C - A) of every fan triangle.
__global__ void normals_kernel(DiffModel m, const float *__restrict__ modelToWorld, float *normals) {
	__shared__ float t[12];
	if (threadIdx.x < 12) t[threadIdx.x] = modelToWorld[threadIdx.x];
	__syncthreads();
	for (uint32_t tri = blockIdx.x * blockDim.x + threadIdx.x; tri < (uint32_t)m.triangleCount; tri += gridDim.x * blockDim.x) {
		int32_t point[3], slot[3];
		fan_corners(m, tri, point, slot);
		Vec3 p[3];
		for (int i = 0; i < 3; i++)
			p[i] = transform_point(t, vec3(m.positions[point[i] * 3], m.positions[point[i] * 3 + 1], m.positions[point[i] * 3 + 2]));
		const float ax = p[1].x - p[0].x, ay = p[1].y - p[0].y, az = p[1].z - p[0].z;
		const float bx = p[2].x - p[0].x, by = p[2].y - p[0].y, bz = p[2].z - p[0].z;
		const float nx = fmul(ay, bz) - fmul(az, by), ny = fmul(az, bx) - fmul(ax, bz), nz = fmul(ax, by) - fmul(ay, bx);
		const float len = __fsqrt_rn(fadd(fadd(fmul(nx, nx), fmul(ny, ny)), fmul(nz, nz)));
		const float inv = len > 0.0f ? frcp(len) : 0.0f;
		normals[tri * 3] = fmul(nx, inv);
		normals[tri * 3 + 1] = fmul(ny, inv);
		normals[tri * 3 + 2] = fmul(nz, inv);
	}
}

// One thread per pixel of every view: the winning fragment's vertex weights, re-evaluated
// exactly as the resolve pass does, then the float shading and the visibility buffer.
__global__ void __launch_bounds__(256) diff_forward_kernel(BatchParams b, const DrawRecord *__restrict__ records,
                                                           const uint32_t *__restrict__ rowOffsets, const uint32_t *__restrict__ rows,
                                                           const unsigned long long *__restrict__ keys, DiffModel m, DiffParams q,
                                                           int32_t width, int32_t height, uint64_t pixels, float4 *images,
                                                           uint32_t *visibility) {
	for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < pixels; i += (uint64_t)gridDim.x * blockDim.x) {
		const uint64_t hw = (uint64_t)width * height;
		const uint32_t view = (uint32_t)(i / hw);
		const uint32_t rem = (uint32_t)(i - (uint64_t)view * hw);
		const int32_t py = (int32_t)(rem / (uint32_t)width), px = (int32_t)(rem - (uint32_t)py * (uint32_t)width);
		const unsigned long long key = keys ? keys[i] : 0ull;
		if (key == 0ull) {
			images[i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
			visibility[i * 3] = NO_TRIANGLE;
			visibility[i * 3 + 1] = 0u;
			visibility[i * 3 + 2] = 0u;
			continue;
		}
		const uint32_t ri = key_record(key, true);
		const DrawRecord r = records[ri];
		const bool affine = b.frames[view].affine != 0;
		const int32_t y1 = py & ~1, x = px & ~1;
		const int lane4 = ((py & 1) << 1) | (px & 1);
		const RowPair pair = record_row_pair(r, rows + rowOffsets[ri], y1, height);
		float w[3][4], wa[4], wb[4], wc[4];
		for (int c = 0; c < 3; c++) quad_lanes(r.start[c], r.dx[c], r.dy[c], pair, y1, x, w[c]);
		lane_weights(w, affine, wa, wb, wc);
		const float pb = lane4 == 0 ? wb[0] : lane4 == 1 ? wb[1] : lane4 == 2 ? wb[2] : wb[3];
		const float pc = lane4 == 0 ? wc[0] : lane4 == 1 ? wc[1] : lane4 == 2 ? wc[2] : wc[3];
		PixelShade s;
		shade_pixel(m, q, r.tri, pb, pc, s);
		images[i] = make_float4(fmul(fmul(s.texel.x, s.vertex.x), s.light), fmul(fmul(s.texel.y, s.vertex.y), s.light),
		                        fmul(fmul(s.texel.z, s.vertex.z), s.light), fmul(s.texel.w, s.vertex.w));
		visibility[i * 3] = r.tri;
		visibility[i * 3 + 1] = fbits(pb);
		visibility[i * 3 + 2] = fbits(pc);
	}
}

// ------------------------------------------------------------------ loss

__global__ void l2_loss_kernel(const float *__restrict__ images, const float *__restrict__ targets, float *grad, uint64_t count,
                               float scale, float *blockSums) {
	__shared__ float partial[8];
	float sum = 0.0f;
	for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < count; i += (uint64_t)gridDim.x * blockDim.x) {
		const float d = images[i] - targets[i];
		grad[i] = fmul(fmul(2.0f, d), scale);
		sum = fadd(sum, fmul(d, d));
	}
	for (int o = 16; o > 0; o >>= 1) sum = fadd(sum, __shfl_xor_sync(0xFFFFFFFFu, sum, o));
	if ((threadIdx.x & 31) == 0) partial[threadIdx.x >> 5] = sum;
	__syncthreads();
	if (threadIdx.x == 0) {
		float s = 0.0f;
		for (int w = 0; w < 8; w++) s = fadd(s, partial[w]);
		blockSums[blockIdx.x] = s;
	}
}

// Sums block partials in a fixed order (deterministic), times scale.
__global__ void fixed_order_sum_kernel(const float *blockSums, int32_t blocks, int32_t width, float scale, float *out) {
	// width interleaved sums: out[j] = scale * sum over blocks of blockSums[block * width + j]
	__shared__ float partial[256];
	for (int32_t j = 0; j < width; j++) {
		float s = 0.0f;
		for (int32_t k = threadIdx.x; k < blocks; k += blockDim.x) s = fadd(s, blockSums[(size_t)k * width + j]);
		partial[threadIdx.x] = s;
		__syncthreads();
		for (int o = blockDim.x >> 1; o > 0; o >>= 1) {
			if ((int)threadIdx.x < o) partial[threadIdx.x] = fadd(partial[threadIdx.x], partial[threadIdx.x + o]);
			__syncthreads();
		}
		if (threadIdx.x == 0) out[j] = fmul(partial[0], scale);
		__syncthreads();
	}
}

// ------------------------------------------------------------------ adjoint

// Adds `value` to base[key] (a float4) once per run of consecutive lanes holding the same key:
// a segmented scan over the run (shuffles up, only within the run) and one vector atomic from
// its last lane.  Consecutive pixels mostly share their triangle's corners and often a texel, so
// runs catch nearly all repeats; equal keys in separate runs each add their own sum.
__device__ __forceinline__ void warp_run_add(float4 *base, uint32_t key, float4 value, bool active) {
	const uint32_t k = active ? key : 0xFFFFFFFFu;
	const int lane = threadIdx.x & 31;
	const uint32_t previous = __shfl_up_sync(0xFFFFFFFFu, k, 1);
	const bool head = lane == 0 || previous != k;
	const uint32_t heads = __ballot_sync(0xFFFFFFFFu, head);
	const int start = 31 - __clz(heads & (0xFFFFFFFFu >> (31 - lane))); // this lane's run begins here
	if (heads != 0xFFFFFFFFu) { // some run holds more than one lane
		for (int d = 1; d < 32; d <<= 1) {
			const float ox = __shfl_up_sync(0xFFFFFFFFu, value.x, d), oy = __shfl_up_sync(0xFFFFFFFFu, value.y, d);
			const float oz = __shfl_up_sync(0xFFFFFFFFu, value.z, d), ow = __shfl_up_sync(0xFFFFFFFFu, value.w, d);
			if (lane - d >= start) {
				value.x = fadd(value.x, ox); value.y = fadd(value.y, oy);
				value.z = fadd(value.z, oz); value.w = fadd(value.w, ow);
			}
		}
	}
	const bool last = lane == 31 || ((heads >> (lane + 1)) & 1u) != 0;
	if (active && last) atomicAdd(base + key, value);
}

// Per-pixel gradients: texture (4 taps), vertex colours (3 corners) and light.
struct PixelGrad {
	float4 tex[4], vertex[3];
	float light[4]; // dir.xyz, intensity
};

__device__ __forceinline__ bool pixel_gradient(const DiffModel &m, const DiffParams &q, const uint32_t *visibility, uint64_t i,
                                               float4 g, PixelShade &s, PixelGrad &out) {
	const uint32_t tri = visibility[i * 3];
	if (tri >= (uint32_t)m.triangleCount) return false; // uncovered (or not a triangle of this model)
	shade_pixel(m, q, tri, bitsf(visibility[i * 3 + 1]), bitsf(visibility[i * 3 + 2]), s);
	// d out / d texel: vertex colour times light (alpha unlit)
	const float4 gt = make_float4(fmul(fmul(g.x, s.vertex.x), s.light), fmul(fmul(g.y, s.vertex.y), s.light),
	                              fmul(fmul(g.z, s.vertex.z), s.light), fmul(g.w, s.vertex.w));
	for (int k = 0; k < 4; k++)
		out.tex[k] = make_float4(fmul(gt.x, s.tapWeight[k]), fmul(gt.y, s.tapWeight[k]), fmul(gt.z, s.tapWeight[k]), fmul(gt.w, s.tapWeight[k]));
	const float4 gc = make_float4(fmul(fmul(g.x, s.texel.x), s.light), fmul(fmul(g.y, s.texel.y), s.light),
	                              fmul(fmul(g.z, s.texel.z), s.light), fmul(g.w, s.texel.w));
	for (int c = 0; c < 3; c++)
		out.vertex[c] = make_float4(fmul(gc.x, s.w[c]), fmul(gc.y, s.w[c]), fmul(gc.z, s.w[c]), fmul(gc.w, s.w[c]));
	// d out / d light factor, then through max(0, -dot(N, dir))
	const float dLight = fadd(fadd(fmul(fmul(g.x, s.texel.x), s.vertex.x), fmul(fmul(g.y, s.texel.y), s.vertex.y)),
	                          fmul(fmul(g.z, s.texel.z), s.vertex.z));
	if (s.normalDotLight > 0.0f) {
		const float *n = q.normals + (size_t)tri * 3;
		const float k = -fmul(dLight, q.light[3]);
		out.light[0] = fmul(k, n[0]);
		out.light[1] = fmul(k, n[1]);
		out.light[2] = fmul(k, n[2]);
		out.light[3] = fmul(dLight, s.normalDotLight);
	} else {
		out.light[0] = out.light[1] = out.light[2] = out.light[3] = 0.0f;
	}
	return true;
}

// Block partial sums of the light gradient, written per block (reduced in a fixed order later).
__device__ __forceinline__ void block_light_sums(const float *light, float *blockSums) {
	__shared__ float partial[8][4];
	float v[4] = {light[0], light[1], light[2], light[3]};
	for (int j = 0; j < 4; j++)
		for (int o = 16; o > 0; o >>= 1) v[j] = fadd(v[j], __shfl_xor_sync(0xFFFFFFFFu, v[j], o));
	if ((threadIdx.x & 31) == 0)
		for (int j = 0; j < 4; j++) partial[threadIdx.x >> 5][j] = v[j];
	__syncthreads();
	if (threadIdx.x < 4) {
		float s = 0.0f;
		for (int w = 0; w < 8; w++) s = fadd(s, partial[w][threadIdx.x]);
		blockSums[blockIdx.x * 4 + threadIdx.x] = s;
	}
	__syncthreads();
}

__global__ void __launch_bounds__(256) adjoint_atomic_kernel(DiffModel m, DiffParams q, const uint32_t *__restrict__ visibility,
                                                             const float4 *__restrict__ grad, uint64_t pixels, float4 *gradTexture,
                                                             float4 *gradVertex, float *blockLight) {
	float light[4] = {0.0f, 0.0f, 0.0f, 0.0f};
	for (uint64_t base = blockIdx.x * (uint64_t)blockDim.x; base < pixels; base += (uint64_t)gridDim.x * blockDim.x) {
		const uint64_t i = base + threadIdx.x;
		PixelShade s;
		PixelGrad pg;
		const bool active = i < pixels && pixel_gradient(m, q, visibility, i, grad[i < pixels ? i : 0], s, pg);
		for (int k = 0; k < 4; k++) warp_run_add(gradTexture, active ? s.taps[k] : 0u, pg.tex[k], active);
		for (int c = 0; c < 3; c++) warp_run_add(gradVertex, active ? (uint32_t)s.point[c] : 0u, pg.vertex[c], active);
		if (active)
			for (int j = 0; j < 4; j++) light[j] = fadd(light[j], pg.light[j]);
	}
	block_light_sums(light, blockLight);
}

// Deterministic mode, step 1: every contribution as (target, value) in pixel order.
__global__ void __launch_bounds__(256) adjoint_emit_kernel(DiffModel m, DiffParams q, const uint32_t *__restrict__ visibility,
                                                           const float4 *__restrict__ grad, uint64_t pixels, uint32_t texKeyEnd,
                                                           uint32_t vertexKeyEnd, uint32_t *texKeys, float4 *texValues,
                                                           uint32_t *vertexKeys, float4 *vertexValues, float *blockLight) {
	float light[4] = {0.0f, 0.0f, 0.0f, 0.0f};
	for (uint64_t base = blockIdx.x * (uint64_t)blockDim.x; base < pixels; base += (uint64_t)gridDim.x * blockDim.x) {
		const uint64_t i = base + threadIdx.x;
		if (i >= pixels) continue;
		PixelShade s;
		PixelGrad pg;
		const bool active = pixel_gradient(m, q, visibility, i, grad[i], s, pg);
		for (int k = 0; k < 4; k++) {
			texKeys[i * 4 + k] = active ? s.taps[k] : texKeyEnd;
			texValues[i * 4 + k] = active ? pg.tex[k] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
		}
		for (int c = 0; c < 3; c++) {
			vertexKeys[i * 3 + c] = active ? (uint32_t)s.point[c] : vertexKeyEnd;
			vertexValues[i * 3 + c] = active ? pg.vertex[c] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
		}
		if (active)
			for (int j = 0; j < 4; j++) light[j] = fadd(light[j], pg.light[j]);
	}
	block_light_sums(light, blockLight);
}

// One warp per target key k: the values of the ids sorted into [segment[k], segment[k + 1]),
// lane l summing entries l, l + 32, ... in order, then a butterfly over the lanes.  Float
// addition is commutative, so every lane of the butterfly ends with the same bits; the shape of
// the sum depends only on the segment's length, which makes the result run-independent.
__global__ void segment_sum_kernel(const uint32_t *__restrict__ segment, const uint32_t *__restrict__ sortedIds,
                                   const float4 *__restrict__ values, uint32_t keys, float4 *out) {
	const uint32_t lane = threadIdx.x & 31;
	const uint32_t warps = (gridDim.x * blockDim.x) >> 5;
	for (uint32_t k = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; k < keys; k += warps) {
		float4 s = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
		const uint32_t end = segment[k + 1];
		for (uint32_t j = segment[k] + lane; j < end; j += 32) {
			const float4 v = values[sortedIds[j]];
			s.x = fadd(s.x, v.x); s.y = fadd(s.y, v.y); s.z = fadd(s.z, v.z); s.w = fadd(s.w, v.w);
		}
		for (int o = 16; o > 0; o >>= 1) {
			s.x = fadd(s.x, __shfl_xor_sync(0xFFFFFFFFu, s.x, o));
			s.y = fadd(s.y, __shfl_xor_sync(0xFFFFFFFFu, s.y, o));
			s.z = fadd(s.z, __shfl_xor_sync(0xFFFFFFFFu, s.z, o));
			s.w = fadd(s.w, __shfl_xor_sync(0xFFFFFFFFu, s.w, o));
		}
		if (lane == 0) out[k] = s;
	}
}

__global__ void key_count_kernel(const uint32_t *__restrict__ keys, uint64_t n, uint32_t keyEnd, uint32_t *counts) {
	for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
		const uint32_t k = keys[i];
		if (k < keyEnd) atomicAdd(&counts[k], 1u);
	}
}

int grid_for(uint64_t n, int threads) {
	uint64_t blocks = (n + threads - 1) / threads;
	const uint64_t cap = (uint64_t)sm_count() * 16;
	if (blocks > cap) blocks = cap;
	return (int)(blocks > 0 ? blocks : 1);
}

} // namespace

struct dsrg_diff_s {
	dsrg_context context;
	dsrg_model model;
	int32_t texW, texH, log2W, log2H;
	float ambient;
	DeviceBuffer<float> depth, normals, blockSums, transform;
	DeviceBuffer<uint32_t> keysA, keysB, idsA, idsB, hist, offsets, counts, segments, emitted;
	DeviceBuffer<float4> texValues, vertexValues;
	BatchJob job;
	int32_t views = 0, width = 0, height = 0;
};

static DiffModel diff_model(dsrg_diff d) {
	DiffModel m;
	m.positions = d->model->positions;
	m.polygons = d->model->polygons;
	m.texCoords = d->model->texCoords;
	m.triSource = d->model->triSource;
	m.pointCount = d->model->pointCount;
	m.triangleCount = d->model->triangleCount;
	return m;
}

#define TRY(expr) DSRG_CUDA_TRY(ctx, expr)

// Scratch of segmented_sum for n entries and keys below keyEnd, reserved before any launch.
static int reserve_segmented_sum(dsrg_diff d, uint64_t n, uint32_t keyEnd) {
	dsrg_context ctx = d->context;
	const uint32_t blocks = sort_blocks(n);
	TRY(d->keysA.reserve(n)); TRY(d->keysB.reserve(n)); TRY(d->idsA.reserve(n)); TRY(d->idsB.reserve(n));
	TRY(d->hist.reserve((size_t)256 * blocks + 1));
	TRY(d->offsets.reserve((size_t)256 * blocks + 1));
	TRY(d->counts.reserve((size_t)keyEnd + 1));
	TRY(d->segments.reserve((size_t)keyEnd + 1));
	const size_t scanElems = scan_scratch_elems((uint32_t)((size_t)256 * blocks > keyEnd ? (size_t)256 * blocks : keyEnd) + 1);
	TRY(ctx->scanScratch.reserve(scanElems));
	return DSRG_OK;
}

// Entries a block of compact_count_kernel / compact_write_kernel takes (256 threads x 16).
static const int COMPACT_ITEMS = 16;
static const uint64_t COMPACT_CHUNK = 256 * COMPACT_ITEMS;

// The entries of each block's chunk with a key below keyEnd (the others are pixels without a
// triangle), counted.
__global__ void __launch_bounds__(256) compact_count_kernel(const uint32_t *__restrict__ keys, uint64_t n, uint32_t keyEnd,
                                                            uint32_t *blockCounts) {
	__shared__ uint32_t warpSums[8];
	const uint64_t begin = (uint64_t)blockIdx.x * COMPACT_CHUNK;
	uint32_t c = 0;
	for (int r = 0; r < COMPACT_ITEMS; r++) {
		const uint64_t i = begin + (uint64_t)r * 256 + threadIdx.x;
		if (i < n && keys[i] < keyEnd) c++;
	}
	for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xFFFFFFFFu, c, o);
	if ((threadIdx.x & 31) == 0) warpSums[threadIdx.x >> 5] = c;
	__syncthreads();
	if (threadIdx.x == 0) {
		uint32_t total = 0;
		for (int w = 0; w < 8; w++) total += warpSums[w];
		blockCounts[blockIdx.x] = total;
	}
}

// Those entries as (key, entry index) pairs, in entry order, each block from its scanned offset.
__global__ void __launch_bounds__(256) compact_write_kernel(const uint32_t *__restrict__ keys, uint64_t n, uint32_t keyEnd,
                                                            const uint32_t *__restrict__ blockOffsets, uint32_t *outKeys,
                                                            uint32_t *outIds) {
	__shared__ uint32_t warpCounts[8];
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
	const uint64_t begin = (uint64_t)blockIdx.x * COMPACT_CHUNK;
	uint32_t running = blockOffsets[blockIdx.x];
	for (int r = 0; r < COMPACT_ITEMS; r++) {
		const uint64_t i = begin + (uint64_t)r * 256 + threadIdx.x;
		const uint32_t k = i < n ? keys[i] : keyEnd;
		const bool keep = k < keyEnd;
		const uint32_t kept = __ballot_sync(0xFFFFFFFFu, keep);
		if (lane == 0) warpCounts[warp] = __popc(kept);
		__syncthreads();
		uint32_t before = running, total = 0;
		for (int w = 0; w < 8; w++) {
			if (w < warp) before += warpCounts[w];
			total += warpCounts[w];
		}
		if (keep) {
			const uint32_t at = before + __popc(kept & ((1u << lane) - 1u));
			outKeys[at] = k;
			outIds[at] = (uint32_t)i;
		}
		running += total;
		__syncthreads(); // warpCounts is read before the next round writes it
	}
}

// Sums `values` per key in [0, keyEnd) into out (keyEnd float4), in the order of the entries:
// count and scan the keys, keep the entries with a key (in entry order), stable-sort their ids by
// key, then one ordered sum per key.  Its scratch must have been reserved (reserve_segmented_sum).
static int segmented_sum(dsrg_diff d, const uint32_t *keys, const float4 *values, uint64_t n, uint32_t keyEnd, float4 *out) {
	dsrg_context ctx = d->context;
	cudaStream_t stream = ctx->stream;
	int bits = 1;
	while ((1ull << bits) <= (uint64_t)keyEnd) bits++;
	// segment starts per key
	TRY(cudaMemsetAsync(d->counts.ptr, 0, sizeof(uint32_t) * keyEnd, stream));
	key_count_kernel<<<grid_for(n, 256), 256, 0, stream>>>(keys, n, keyEnd, d->counts.ptr);
	add_launches(1);
	launch_scan(d->counts.ptr, d->segments.ptr, keyEnd, ctx->scanScratch.ptr, ctx->scanScratch.capacity, stream);
	// the entries with a key, in entry order, into the sort's second buffers (its first pass reads
	// them from there); their number comes back to the host for the sort's launch shape
	const uint32_t blocks = (uint32_t)((n + COMPACT_CHUNK - 1) / COMPACT_CHUNK);
	uint32_t kept = 0;
	if (blocks > 0) {
		compact_count_kernel<<<blocks, 256, 0, stream>>>(keys, n, keyEnd, d->hist.ptr);
		launch_scan(d->hist.ptr, d->offsets.ptr, blocks, ctx->scanScratch.ptr, ctx->scanScratch.capacity, stream);
		compact_write_kernel<<<blocks, 256, 0, stream>>>(keys, n, keyEnd, d->offsets.ptr, d->keysB.ptr, d->idsB.ptr);
		add_launches(2);
		TRY(cudaGetLastError());
		TRY(cudaMemcpyAsync(ctx->pinnedReadback + 8, d->offsets.ptr + blocks, sizeof(uint32_t), cudaMemcpyDeviceToHost, stream));
		TRY(cudaStreamSynchronize(stream));
		kept = ctx->pinnedReadback[8];
	}
	// the kept entries' ids sorted by key, entries of one key in entry order
	SortBuffers sb;
	sb.keysA = d->keysA.ptr; sb.keysB = d->keysB.ptr; sb.idsA = d->idsA.ptr; sb.idsB = d->idsB.ptr;
	sb.hist = d->hist.ptr; sb.offsets = d->offsets.ptr;
	sb.scanScratch = ctx->scanScratch.ptr; sb.scanScratchElems = ctx->scanScratch.capacity;
	const uint32_t *sortedKeys = nullptr, *iin = nullptr;
	launch_stable_sort(d->keysB.ptr, d->idsB.ptr, kept, bits, sb, stream, &sortedKeys, &iin);
	segment_sum_kernel<<<grid_for((uint64_t)keyEnd * 32, 256), 256, 0, stream>>>(d->segments.ptr, iin, values, keyEnd, out);
	add_launches(1);
	TRY(cudaGetLastError());
	return DSRG_OK;
}

static int compute_normals(dsrg_diff d, const float *modelToWorld) {
	dsrg_context ctx = d->context;
	TRY(d->normals.reserve((size_t)d->model->triangleCount * 3 + 3));
	TRY(d->transform.reserve(16));
	TRY(cudaMemcpyAsync(d->transform.ptr, modelToWorld, 12 * sizeof(float), cudaMemcpyHostToDevice, ctx->stream));
	if (d->model->triangleCount > 0) {
		normals_kernel<<<grid_for(d->model->triangleCount, 256), 256, 0, ctx->stream>>>(diff_model(d), d->transform.ptr, d->normals.ptr);
		add_launches(1);
	}
	TRY(cudaGetLastError());
	return DSRG_OK;
}

extern "C" {

int dsrg_diff_create(dsrg_context ctx, dsrg_model model, int32_t textureWidth, int32_t textureHeight, float ambient, dsrg_diff *out) {
	if (!ctx || !out) return DSRG_ERROR_INVALID_ARGUMENT;
	*out = nullptr;
	if (!model) return fail(ctx, DSRG_ERROR_INVALID_ARGUMENT, "dsrg_diff_create: null model");
	int32_t lw = 0, lh = 0;
	while ((1 << lw) < textureWidth) lw++;
	while ((1 << lh) < textureHeight) lh++;
	if (textureWidth < 1 || textureHeight < 1 || (1 << lw) != textureWidth || (1 << lh) != textureHeight || lw > 15 || lh > 15)
		return fail(ctx, DSRG_ERROR_UNSUPPORTED, "dsrg_diff_create: texture sides must be powers of two up to 32768");
	dsrg_diff d = new (std::nothrow) dsrg_diff_s();
	if (!d) return DSRG_ERROR_OUT_OF_MEMORY;
	d->context = ctx;
	d->model = model;
	d->texW = textureWidth;
	d->texH = textureHeight;
	d->log2W = lw;
	d->log2H = lh;
	d->ambient = ambient;
	*out = d;
	return DSRG_OK;
}

int dsrg_diff_destroy(dsrg_diff d) {
	if (!d) return DSRG_ERROR_INVALID_ARGUMENT;
	cudaSetDevice(d->context->device);
	cudaStreamSynchronize(d->context->stream);
	DeviceBuffer<float> *f[] = {&d->depth, &d->normals, &d->blockSums, &d->transform};
	for (auto *b : f) b->release();
	DeviceBuffer<uint32_t> *u[] = {&d->keysA, &d->keysB, &d->idsA, &d->idsB, &d->hist, &d->offsets, &d->counts, &d->segments, &d->emitted};
	for (auto *b : u) b->release();
	d->texValues.release();
	d->vertexValues.release();
	delete d;
	return DSRG_OK;
}

int dsrg_diff_forward(dsrg_diff d, int32_t views, const dsrg_camera *cameras, const float *modelToWorld, const float *texture,
                      const float *vertexColors, const float *light, float *images, uint32_t *visibility) {
	if (!d) return DSRG_ERROR_INVALID_ARGUMENT;
	dsrg_context ctx = d->context;
	if (views < 1 || !cameras || !modelToWorld || !texture || !vertexColors || !light || !images || !visibility)
		return fail(ctx, DSRG_ERROR_INVALID_ARGUMENT, "dsrg_diff_forward: null argument or no views");
	const int32_t width = cameras[0].width, height = cameras[0].height;
	for (int32_t v = 0; v < views; v++)
		if (cameras[v].width != width || cameras[v].height != height || width <= 0 || height <= 0)
			return fail(ctx, DSRG_ERROR_INVALID_ARGUMENT, "dsrg_diff_forward: every view needs the same positive image size");
	cudaSetDevice(ctx->device);
	cudaStream_t stream = ctx->stream;
	dsrg_model m = d->model;
	const uint64_t hw = (uint64_t)width * height, pixels = hw * (uint64_t)views;
	TRY(d->depth.reserve(pixels));
	TRY(cudaMemsetAsync(d->depth.ptr, 0, pixels * sizeof(float), stream)); // depth cleared to 0: infinitely far for 1/W
	int status = compute_normals(d, modelToWorld);
	if (status != DSRG_OK) return status;
	TRY(cudaEventRecord(ctx->eventStart, stream));
	BatchJob &job = d->job;
	job.frames.assign(views, FrameTarget());
	job.tasks.clear();
	job.textures.clear();
	job.depthOnly = false;
	job.resolve = false;
	for (int32_t v = 0; v < views; v++) {
		FrameTarget &f = job.frames[v];
		memset(&f, 0, sizeof(f));
		f.depth = d->depth.ptr + hw * v;
		f.depthStride = width;
		f.width = width;
		f.height = height;
		f.affine = cameras[v].perspective ? 0 : 1;
		CameraData cam = make_camera(cameras[v]);
		// ModelImpl::render's bound test (model/Model.cpp:186-197)
		if (m->triangleCount == 0 || !box_seen(cam, m->minBound, m->maxBound, modelToWorld)) continue;
		TaskParams t;
		memset(&t, 0, sizeof(t));
		t.positions = m->positions;
		t.polygons = m->polygons;
		t.texCoords = m->texCoords;
		t.colors = m->colors;
		t.triSource = m->triSource;
		t.pointCount = m->pointCount;
		t.triangleCount = m->triangleCount;
		t.frame = v;
		memcpy(t.modelToWorld, modelToWorld, sizeof(t.modelToWorld));
		t.camera = cam;
		t.filter = 0;
		t.diffuse = -1;
		t.light = -1;
		job.tasks.push_back(t);
	}
	BatchTotals totals;
	BatchOutputs outputs;
	status = batch_enqueue(ctx, job, totals, &outputs);
	if (status != DSRG_OK) {
		cudaStreamSynchronize(stream);
		return status;
	}
	DiffParams q;
	q.texture = texture;
	q.vertexColors = vertexColors;
	q.light = light;
	q.normals = d->normals.ptr;
	q.log2W = d->log2W;
	q.log2H = d->log2H;
	q.ambient = d->ambient;
	const unsigned long long *keys = totals.pixels ? ctx->keys.ptr : nullptr;
	diff_forward_kernel<<<grid_for(pixels, 256), 256, 0, stream>>>(outputs.params, outputs.fb.records, outputs.fb.rowOffsets,
	                                                               outputs.fb.rows, keys, diff_model(d), q, width, height, pixels,
	                                                               reinterpret_cast<float4 *>(images), visibility);
	add_launches(1);
	TRY(cudaGetLastError());
	d->views = views;
	d->width = width;
	d->height = height;
	return batch_finish(ctx, totals);
}

int dsrg_diff_l2_loss(dsrg_diff d, int64_t count, const float *images, const float *targets, float *gradImages, float *loss) {
	if (!d) return DSRG_ERROR_INVALID_ARGUMENT;
	dsrg_context ctx = d->context;
	if (count < 1 || !images || !targets || !gradImages || !loss) return fail(ctx, DSRG_ERROR_INVALID_ARGUMENT, "dsrg_diff_l2_loss: null argument");
	cudaSetDevice(ctx->device);
	const int blocks = grid_for((uint64_t)count, 256);
	TRY(d->blockSums.reserve((size_t)blocks));
	float *sums = d->blockSums.ptr;
	const float scale = 1.0f / (float)count;
	l2_loss_kernel<<<blocks, 256, 0, ctx->stream>>>(images, targets, gradImages, (uint64_t)count, scale, sums);
	fixed_order_sum_kernel<<<1, 256, 0, ctx->stream>>>(sums, blocks, 1, scale, loss);
	add_launches(2);
	TRY(cudaGetLastError());
	TRY(cudaStreamSynchronize(ctx->stream));
	return DSRG_OK;
}

int dsrg_diff_adjoint(dsrg_diff d, int32_t views, int32_t width, int32_t height, const float *modelToWorld, const float *texture,
                      const float *vertexColors, const float *light, const uint32_t *visibility, const float *gradImages,
                      float *gradTexture, float *gradVertexColors, float *gradLight, int32_t deterministic) {
	if (!d) return DSRG_ERROR_INVALID_ARGUMENT;
	dsrg_context ctx = d->context;
	if (views < 1 || width < 1 || height < 1 || !modelToWorld || !texture || !vertexColors || !light || !visibility || !gradImages ||
	    !gradTexture || !gradVertexColors || !gradLight)
		return fail(ctx, DSRG_ERROR_INVALID_ARGUMENT, "dsrg_diff_adjoint: null argument or empty image");
	cudaSetDevice(ctx->device);
	cudaStream_t stream = ctx->stream;
	int status = compute_normals(d, modelToWorld);
	if (status != DSRG_OK) return status;
	DiffParams q;
	q.texture = texture;
	q.vertexColors = vertexColors;
	q.light = light;
	q.normals = d->normals.ptr;
	q.log2W = d->log2W;
	q.log2H = d->log2H;
	q.ambient = d->ambient;
	const uint64_t pixels = (uint64_t)width * height * (uint64_t)views;
	const uint32_t texels = (uint32_t)(d->texW * d->texH), points = (uint32_t)d->model->pointCount;
	const int blocks = grid_for(pixels, 256);
	TRY(d->blockSums.reserve((size_t)blocks * 4));
	float *blockLight = d->blockSums.ptr;
	const float4 *grad = reinterpret_cast<const float4 *>(gradImages);
	if (!deterministic) {
		TRY(cudaMemsetAsync(gradTexture, 0, sizeof(float) * 4 * texels, stream));
		TRY(cudaMemsetAsync(gradVertexColors, 0, sizeof(float) * 4 * points, stream));
		adjoint_atomic_kernel<<<blocks, 256, 0, stream>>>(diff_model(d), q, visibility, grad, pixels,
		                                                  reinterpret_cast<float4 *>(gradTexture),
		                                                  reinterpret_cast<float4 *>(gradVertexColors), blockLight);
		add_launches(1);
	} else {
		TRY(d->texValues.reserve(pixels * 4));
		TRY(d->vertexValues.reserve(pixels * 3));
		TRY(d->emitted.reserve(pixels * 7));
		status = reserve_segmented_sum(d, pixels * 4, texels > points ? texels : points);
		if (status != DSRG_OK) return status;
		uint32_t *texKeys = d->emitted.ptr, *vertexKeys = d->emitted.ptr + pixels * 4;
		adjoint_emit_kernel<<<blocks, 256, 0, stream>>>(diff_model(d), q, visibility, grad, pixels, texels, points, texKeys,
		                                                d->texValues.ptr, vertexKeys, d->vertexValues.ptr, blockLight);
		add_launches(1);
		TRY(cudaGetLastError());
		status = segmented_sum(d, texKeys, d->texValues.ptr, pixels * 4, texels, reinterpret_cast<float4 *>(gradTexture));
		if (status == DSRG_OK)
			status = segmented_sum(d, vertexKeys, d->vertexValues.ptr, pixels * 3, points, reinterpret_cast<float4 *>(gradVertexColors));
		if (status != DSRG_OK) {
			cudaStreamSynchronize(stream);
			return status;
		}
	}
	fixed_order_sum_kernel<<<1, 256, 0, stream>>>(blockLight, blocks, 4, 1.0f, gradLight);
	add_launches(1);
	TRY(cudaGetLastError());
	TRY(cudaStreamSynchronize(stream));
	return DSRG_OK;
}

} // extern "C"
