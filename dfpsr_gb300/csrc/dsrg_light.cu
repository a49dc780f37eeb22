// Deferred light passes of the isometric sprite engine and draw_higher, on the GPU.
//
//   light_directed_kernel   setDirectedLight / addDirectedLight (SDK/SpriteEngine/lightAPI.cpp:23-74)
//   light_points_kernel     addPointLight for many lights in one pass (lightAPI.cpp:76-285)
//   light_blend_kernel      blendLight (lightAPI.cpp:287-323)
//   higher_keys_kernel      draw_higher for many sprites: the winning (height, sprite) per pixel ...
//   higher_resolve_kernel   ... and the copy of its height and colours (api/drawAPI.cpp:872-900)
//
// The reference's scalar build works on 4-lane float vectors (base/simd.h:4196-4207).  The point
// light sweeps light space along each row with running sums: every lane starts at the band's first
// row (F32xXx3::createGradient), adds the screen's y axis once per row and the x axis times four once
// per 4-pixel step.  Each pixel here reproduces its own lane's sums with chain_add, so the values
// are the reference's bit for bit.  Rows are cut into the bands of the reference's threadedSplit,
// which restart the sweep.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <map>
#include <new>
#include <string>
#include <thread>
#include <tuple>
#include <vector>

#include "dsrg_internal.h"
#include "dsrg_shade.h"

using namespace dsrg;

namespace {

// ------------------------------------------------------------------ host: ortho views (host code is built with
// -ffp-contract=off, so every expression below is the reference's sequence of binary32 operations)

struct M3 { Vec3 x, y, z; };

Vec3 v3(float x, float y, float z) { return vec3(x, y, z); }

// normalize (math/FVector.h:113-119)
Vec3 normalize_ref(Vec3 v) {
	const float l = sqrtf(v.x * v.x + v.y * v.y + v.z * v.z);
	if (l == 0.0f) return v3(0.0f, 0.0f, 1.0f);
	return v3(v.x / l, v.y / l, v.z / l);
}
Vec3 cross_ref(Vec3 a, Vec3 b) { return v3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }

// FMatrix3x3::makeAxisSystem (math/FMatrix3x3.h:24-30)
M3 axis_system(Vec3 forward, Vec3 up) {
	M3 r;
	const Vec3 f = normalize_ref(forward);
	r.z = f;
	r.x = normalize_ref(cross_ref(normalize_ref(up), f));
	r.y = normalize_ref(cross_ref(f, r.x));
	return r;
}
Vec3 transform_ref(const M3 &m, Vec3 p) { // FMatrix3x3.h:31-37
	return v3(p.x * m.x.x + p.y * m.y.x + p.z * m.z.x, p.x * m.x.y + p.y * m.y.y + p.z * m.z.y, p.x * m.x.z + p.y * m.y.z + p.z * m.z.z);
}
Vec3 transform_transposed_ref(const M3 &m, Vec3 p) { // FMatrix3x3.h:38-44
	return v3(p.x * m.x.x + p.y * m.x.y + p.z * m.x.z, p.x * m.y.x + p.y * m.y.y + p.z * m.y.z, p.x * m.z.x + p.y * m.z.y + p.z * m.z.z);
}
M3 inverse_ref(const M3 &m) { // FMatrix3x3.h:54-80
	const float det = m.x.x * m.y.y * m.z.z + m.z.x * m.x.y * m.y.z + m.y.x * m.z.y * m.x.z - m.x.x * m.z.y * m.y.z -
	                  m.y.x * m.x.y * m.z.z - m.z.x * m.y.y * m.x.z;
	const float invDet = 1.0f / det;
	M3 r;
	r.x.x = invDet * (m.y.y * m.z.z - m.y.z * m.z.y);
	r.x.y = -invDet * (m.x.y * m.z.z - m.x.z * m.z.y);
	r.x.z = invDet * (m.x.y * m.y.z - m.x.z * m.y.y);
	r.y.x = -invDet * (m.y.x * m.z.z - m.y.z * m.z.x);
	r.y.y = invDet * (m.x.x * m.z.z - m.x.z * m.z.x);
	r.y.z = -invDet * (m.x.x * m.y.z - m.x.z * m.y.x);
	r.z.x = invDet * (m.y.x * m.z.y - m.y.y * m.z.x);
	r.z.y = -invDet * (m.x.x * m.z.y - m.x.y * m.z.x);
	r.z.z = invDet * (m.x.x * m.y.y - m.x.y * m.y.x);
	return r;
}
void store_m3(const M3 &m, float *out) {
	const float v[9] = {m.x.x, m.x.y, m.x.z, m.y.x, m.y.y, m.y.z, m.z.x, m.z.y, m.z.z};
	memcpy(out, v, sizeof(v));
}
M3 load_m3(const float *in) {
	M3 m;
	m.x = v3(in[0], in[1], in[2]);
	m.y = v3(in[3], in[4], in[5]);
	m.z = v3(in[6], in[7], in[8]);
	return m;
}

// ------------------------------------------------------------------ device

// truncated, clamped channels packed as the reference's packOrder_packBytes(r, g, b) (alpha 0)
__device__ __forceinline__ uint32_t light_channel(float v) { return trunc_u32((255.1f < v) ? 255.1f : v); }

__device__ __forceinline__ float vmin_ref(float left, float right) { return (right < left) ? right : left; } // simd.h:2198-2216
__device__ __forceinline__ float vmax_ref(float left, float right) { return (right > left) ? right : left; } // simd.h:2217-2235

__device__ __forceinline__ uint32_t sat_add_bytes(uint32_t a, uint32_t b) { // saturatedAddition (simd.h:2670-2690)
	uint32_t out = 0;
	for (int i = 0; i < 4; i++) {
		const uint32_t s = ((a >> (8 * i)) & 0xFFu) + ((b >> (8 * i)) & 0xFFu);
		out |= (s > 255u ? 255u : s) << (8 * i);
	}
	return out;
}

struct DirectedParams {
	float rev[3]; // -normalize(N^T dir) * intensity * 2
	float color[3];
	int32_t add;
};

__global__ void light_directed_kernel(uint32_t *light, int32_t lightStride, const uint32_t *__restrict__ normal, int32_t normalStride,
                                      int32_t width, int32_t height, DirectedParams p) {
	const int32_t x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
	if (x >= width || y >= height) return;
	const uint32_t c = normal[(size_t)y * normalStride + x];
	const float nx = fadd((float)(c & 0xFFu), -128.0f), ny = fadd((float)((c >> 8) & 0xFFu), -128.0f);
	const float nz = fadd((float)((c >> 16) & 0xFFu), -128.0f);
	const float dot = fadd(fadd(fmul(nx, p.rev[0]), fmul(ny, p.rev[1])), fmul(nz, p.rev[2]));
	const float i = vmax_ref(0.0f, dot);
	const uint32_t bytes = light_channel(fmul(i, p.color[0])) | (light_channel(fmul(i, p.color[1])) << 8) |
	                       (light_channel(fmul(i, p.color[2])) << 16);
	uint32_t *q = light + (size_t)y * lightStride + x;
	*q = p.add ? sat_add_bytes(*q, bytes) : bytes;
}

// One point light, as prepared on the host (calculateBound and the uniforms of addPointLightSuper).
struct PointLightParams {
	int32_t left, top, right, bottom; // bound, left and right aligned to 4 pixels
	int32_t jobs;                     // threadedSplit bands of the bound's rows
	float source[3];                  // light-space position
	float color[3];
	float reciprocalRadius;
	const float *cube;                // shadow cube map or null
	int32_t cubeWidth;
	float cubeCenter;
};

struct PointFrame {
	float toLight[9];     // screenDepthToLightSpace (x, y, z axes)
	int32_t centerX, centerY;
	int32_t lightCount;
	const PointLightParams *lights;
};

// getShadowTransparency (lightAPI.cpp:104-138)
__device__ __forceinline__ float shadow_transparency(const float *cube, int32_t width, float halfWidth, float ox, float oy, float oz) {
	const float absX = ox < 0.0f ? -ox : ox, absY = oy < 0.0f ? -oy : oy, absZ = oz < 0.0f ? -oz : oz;
	const bool xIsLongest = absX > absY && absX > absZ;
	const bool yIsLongerThanZ = absY > absZ;
	float depth = xIsLongest ? ox : (yIsLongerThanZ ? oy : oz);
	const float slopeUp = (yIsLongerThanZ && !xIsLongest) ? oz : oy;
	float slopeSide = xIsLongest ? -oz : (yIsLongerThanZ ? -ox : ox);
	int32_t viewOffset = width * (xIsLongest ? 0 : (yIsLongerThanZ ? 2 : 4));
	if (depth < 0.0f) {
		depth = -depth;
		slopeSide = -slopeSide;
		viewOffset += width;
	}
	const float reciDepth = frcp(depth);
	const float scale = fmul(halfWidth, reciDepth);
	int32_t sampleX = (int32_t)fadd(halfWidth, fmul(slopeSide, scale));
	int32_t sampleY = (int32_t)fsub(halfWidth, fmul(slopeUp, scale));
	const int32_t maxPixel = width - 1;
	sampleX = sampleX < 0 ? 0 : (sampleX > maxPixel ? maxPixel : sampleX);
	sampleY = sampleY < 0 ? 0 : (sampleY > maxPixel ? maxPixel : sampleY);
	const float shadowReciDepth = __ldg(&cube[(size_t)(sampleY + viewOffset) * width + sampleX]);
	return fmul(reciDepth, 1.02f) > shadowReciDepth ? 1.0f : 0.0f;
}

// Contribution bytes (r, g, b) of one light at one pixel from its light-space offset o.
__device__ __forceinline__ void point_light_bytes(const PointLightParams &p, const float *o, uint32_t normalWord, uint32_t *sum) {
	const float negN[3] = {fmul(fadd((float)(normalWord & 0xFFu), -128.0f), -0.0078125f),
	                       fmul(fadd((float)((normalWord >> 8) & 0xFFu), -128.0f), -0.0078125f),
	                       fmul(fadd((float)((normalWord >> 16) & 0xFFu), -128.0f), -0.0078125f)};
	const float squareLength = fadd(fadd(fmul(o[0], o[0]), fmul(o[1], o[1])), fmul(o[2], o[2]));
	// squareRoot and reciprocalSquareRoot of the scalar build go through the double overload of sqrt
	// (simd.h:4084-4146): (float)sqrt((double)x) and (float)(1.0 / sqrt((double)x)).  Both equal the
	// correctly rounded single-precision results, so no double arithmetic is needed: the square root
	// because rounding first to 53 and then to 24 bits is innocuous for sqrt (53 >= 2 * 24 + 2), the
	// reciprocal square root as checked for every float of [1, 4) on the device (dsrg_check_float_roots;
	// both sides scale exactly by 2 when x scales by 4).
	const float length = __fsqrt_rn(squareLength);
	const float ratio = vmin_ref(1.0f, fmul(length, p.reciprocalRadius));
	const float distanceIntensity = fadd(fsub(1.0f, fmul(2.0f, ratio)), fmul(ratio, ratio));
	const float rs = __frsqrt_rn(squareLength);
	const float angle = vmax_ref(0.0f, fadd(fadd(fmul(fmul(o[0], rs), negN[0]), fmul(fmul(o[1], rs), negN[1])),
	                                        fmul(fmul(o[2], rs), negN[2])));
	float intensity = fmul(angle, distanceIntensity);
	if (p.cube) intensity = fmul(intensity, shadow_transparency(p.cube, p.cubeWidth, p.cubeCenter, o[0], o[1], o[2]));
	for (int c = 0; c < 3; c++) sum[c] += light_channel(fmul(intensity, p.color[c]));
}

// Every thread owns one lane (x mod 4) of one row and eight of its 4-pixel groups, spread 8 groups
// apart so that a warp's loads for one step are 32 consecutive pixels: the reference's running
// sums are evaluated with chain_add once per light at the first group, then advanced 8 steps of
// dx*4 at a time with plain additions.  The bytes of every light whose bound holds a pixel are
// summed and added to the pixel with saturation (equal to the reference's saturated additions
// light after light, because every added byte is non-negative).  Blocks of 32 x 8 threads cover
// 256 x 8 pixels.
__global__ void __launch_bounds__(256) light_points_kernel(uint32_t *light, int32_t lightStride, const uint32_t *__restrict__ normal,
                                                           int32_t normalStride, const float *__restrict__ heightImage,
                                                           int32_t heightStride, int32_t width, int32_t height, PointFrame f) {
	const int32_t lane = threadIdx.x & 3, seg = (threadIdx.x >> 2) & 7;
	const int32_t y = blockIdx.y * 8 + (threadIdx.x >> 5);
	const int32_t g0 = blockIdx.x * 64 + seg; // first group; the thread's groups are g0, g0 + 8, ..., g0 + 56
	if (y >= height) return;
	uint32_t sum[8][3];
	for (int j = 0; j < 8; j++) sum[j][0] = sum[j][1] = sum[j][2] = 0u;
	uint32_t touched = 0;
	const float *m = f.toLight;
	for (int32_t k = 0; k < f.lightCount; k++) {
		const PointLightParams &p = f.lights[k];
		if (y < p.top || y >= p.bottom) continue;
		const int32_t gl = p.left >> 2, gr = p.right >> 2; // groups of the bound (left and right are multiples of 4)
		// the thread's groups inside [gl, gr): j from jFirst while g0 + 8j < gr
		int32_t jFirst = gl > g0 ? (gl - g0 + 7) >> 3 : 0;
		if (jFirst > 7 || g0 + 8 * jFirst >= gr) continue;
		// the band holding this row (splitStartIndex, base/threading.cpp:209-221)
		const int32_t rows = p.bottom - p.top;
		int32_t bandTop = p.top;
		for (int32_t b = 1; b < p.jobs; b++) {
			const int32_t start = (b * rows) / p.jobs + p.top;
			if (start <= y) bandTop = start;
		}
		// lightBaseRow = screenDepthToLightSpace.transform((0.5 - cx + left, 0.5 - cy + bandTop, 0)) - source
		const float px = fadd(fsub(0.5f, (float)f.centerX), (float)p.left);
		const float py = fadd(fsub(0.5f, (float)f.centerY), (float)bandTop);
		float value[3], stepX[3];
		for (int c = 0; c < 3; c++) {
			const float base = fsub(fadd(fadd(fmul(px, m[c]), fmul(py, m[3 + c])), fmul(0.0f, m[6 + c])), p.source[c]);
			const float dx = m[c], dy = m[3 + c];
			// F32x4::createGradient (base/simd.h:474-476), then one += dy per row of the band
			const float start = lane == 0 ? base : fadd(base, lane == 1 ? dx : fmul(dx, (float)lane));
			const float row = chain_add(start, dy, y - bandTop);
			stepX[c] = fmul(dx, 4.0f);
			value[c] = chain_add(row, stepX[c], g0 + 8 * jFirst - gl);
		}
		for (int32_t j = jFirst; j < 8; j++) {
			const int32_t g = g0 + 8 * j;
			if (g >= gr) break;
			if (j > jFirst)
				for (int c = 0; c < 3; c++)
					for (int s = 0; s < 8; s++) value[c] = fadd(value[c], stepX[c]);
			const int32_t x = 4 * g + lane;
			if (x >= width) continue;
			const float depthOffset = heightImage[(size_t)y * heightStride + x];
			const float o[3] = {fadd(value[0], fmul(m[6], depthOffset)), fadd(value[1], fmul(m[7], depthOffset)),
			                    fadd(value[2], fmul(m[8], depthOffset))};
			point_light_bytes(p, o, normal[(size_t)y * normalStride + x], sum[j]);
			touched |= 1u << j;
		}
	}
	for (int32_t j = 0; j < 8; j++) {
		if (!(touched & (1u << j))) continue;
		const int32_t x = 4 * (g0 + 8 * j) + lane;
		uint32_t *q = light + (size_t)y * lightStride + x;
		uint32_t v = *q;
		for (int c = 0; c < 3; c++) {
			const uint32_t s = ((v >> (8 * c)) & 0xFFu) + sum[j][c];
			v = (v & ~(0xFFu << (8 * c))) | ((s > 255u ? 255u : s) << (8 * c));
		}
		*q = v;
	}
}

__global__ void light_blend_kernel(uint32_t *target, int32_t targetStride, int32_t packOrder, const uint32_t *__restrict__ diffuse,
                                   int32_t diffuseStride, const uint32_t *__restrict__ light, int32_t lightStride, int32_t width,
                                   int32_t height) {
	const int32_t x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
	if (x >= width || y >= height) return;
	const uint32_t d = diffuse[(size_t)y * diffuseStride + x], l = light[(size_t)y * lightStride + x];
	uint32_t out = 0;
	for (int c = 0; c < 3; c++) {
		const float v = fmul(fmul((float)((d >> (8 * c)) & 0xFFu), (float)((l >> (8 * c)) & 0xFFu)), 0.0078125f);
		out |= light_channel(v) << pack_shift(packOrder, c);
	}
	target[(size_t)y * targetStride + x] = out;
}

struct SpriteData {
	const float *height;
	const uint32_t *colorA, *colorB;
	int32_t width, height_;
	int32_t heightStride, aStride, bStride; // in elements
	int32_t aPack, bPack;
	int32_t left, top;
	float offset;
};

__device__ __forceinline__ uint32_t ordered_height(float h) {
	uint32_t bits = fbits(h);
	if (bits == 0x80000000u) bits = 0u; // -0 equals +0
	return (bits & 0x80000000u) ? ~bits : (bits | 0x80000000u);
}

// Every source pixel raised above the initial target height bids (height, ~sprite) for its pixel.
// Blocks of 64 x 4 threads: columns over threadIdx.x, rows over threadIdx.y and the sprite's blocks
// (blockIdx.x; blockIdx.y is the sprite).  Keys only grow, so a bid that a key already in place
// beats (read without the atomic; a stale read is only smaller) is dropped before the atomic.
__global__ void __launch_bounds__(256) higher_keys_kernel(const SpriteData *__restrict__ sprites, int32_t first, int32_t count,
                                                          const float *__restrict__ targetHeight, int32_t thStride, int32_t width,
                                                          int32_t height, unsigned long long *keys) {
	const int32_t s = first + (int32_t)blockIdx.y;
	if (s >= count) return;
	const SpriteData sp = sprites[s];
	const unsigned long long low = (unsigned long long)(~(uint32_t)s);
	for (int32_t sy = (int32_t)(blockIdx.x * blockDim.y + threadIdx.y); sy < sp.height_; sy += (int32_t)(gridDim.x * blockDim.y)) {
		const int32_t y = sp.top + sy;
		if (y < 0 || y >= height) continue;
		for (int32_t sx = (int32_t)threadIdx.x; sx < sp.width; sx += (int32_t)blockDim.x) {
			const int32_t x = sp.left + sx;
			if (x < 0 || x >= width) continue;
			float h = sp.height[(size_t)sy * sp.heightStride + sx];
			if (!(h > -INFINITY)) continue;
			h = fadd(h, sp.offset);
			if (!(h > targetHeight[(size_t)y * thStride + x])) continue;
			const unsigned long long key = ((unsigned long long)ordered_height(h) << 32) | low;
			unsigned long long *slot = &keys[(size_t)y * width + x];
			if (key > *slot) atomicMax(slot, key);
		}
	}
}

// Byte index of red, green, blue, alpha in memory for a PackOrderIndex (image/PackOrder.h:61-92).
__device__ __forceinline__ int pack_index(int32_t order, int channel) {
	const int table[4][4] = {{0, 1, 2, 3}, {2, 1, 0, 3}, {1, 2, 3, 0}, {3, 2, 1, 0}};
	return table[order & 3][channel];
}

__device__ __forceinline__ uint32_t reorder(uint32_t source, int32_t from, int32_t to) {
	uint32_t out = 0;
	for (int c = 0; c < 4; c++) out |= ((source >> (8 * pack_index(from, c))) & 0xFFu) << (8 * pack_index(to, c));
	return out;
}

__global__ void higher_resolve_kernel(const SpriteData *__restrict__ sprites, const unsigned long long *__restrict__ keys,
                                      float *targetHeight, int32_t thStride, uint32_t *targetA, int32_t taStride, int32_t taPack,
                                      uint32_t *targetB, int32_t tbStride, int32_t tbPack, int32_t width, int32_t height) {
	const int32_t x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
	if (x >= width || y >= height) return;
	const unsigned long long key = keys[(size_t)y * width + x];
	if (key == 0ull) return;
	const SpriteData sp = sprites[~(uint32_t)(key & 0xFFFFFFFFull)];
	const int32_t sx = x - sp.left, sy = y - sp.top;
	targetHeight[(size_t)y * thStride + x] = fadd(sp.height[(size_t)sy * sp.heightStride + sx], sp.offset);
	targetA[(size_t)y * taStride + x] = reorder(sp.colorA[(size_t)sy * sp.aStride + sx], sp.aPack, taPack);
	targetB[(size_t)y * tbStride + x] = reorder(sp.colorB[(size_t)sy * sp.bStride + sx], sp.bPack, tbPack);
}

// The scalar build's float square roots through double precision against the correctly rounded
// single-precision operations, for `count` consecutive float bit patterns from firstBits: counts
// the inputs where either differs (NaN results compare equal to NaN).
__global__ void root_check_kernel(uint32_t firstBits, uint32_t count, unsigned long long *mismatches) {
	unsigned long long bad = 0;
	for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
		const float x = __uint_as_float(firstBits + i);
		const double root = __dsqrt_rn((double)x);
		const float viaDouble[2] = {__double2float_rn(root), __double2float_rn(__ddiv_rn(1.0, root))};
		const float single[2] = {__fsqrt_rn(x), __frsqrt_rn(x)};
		for (int k = 0; k < 2; k++) {
			const bool bothNaN = viaDouble[k] != viaDouble[k] && single[k] != single[k];
			if (!bothNaN && __float_as_uint(viaDouble[k]) != __float_as_uint(single[k])) bad++;
		}
	}
	if (bad) atomicAdd(mismatches, bad);
}

// A rectangle of 32-bit words set to one value (the frame's clears).
__global__ void fill_words_kernel(uint32_t *image, int32_t stride, int32_t width, int32_t height, uint32_t value) {
	const int32_t x = (int32_t)(blockIdx.x * blockDim.x + threadIdx.x), y = (int32_t)blockIdx.y;
	if (x < width && y < height) image[(size_t)y * stride + x] = value;
}

bool sprite_ok(const dsrg_sprite &s) {
	return s.height && s.colorA && s.colorB && s.width >= 0 && s.height_ >= 0 && s.heightStrideBytes >= s.width * 4 &&
	       s.colorAStrideBytes >= s.width * 4 && s.colorBStrideBytes >= s.width * 4 && s.heightStrideBytes % 4 == 0 &&
	       s.colorAStrideBytes % 4 == 0 && s.colorBStrideBytes % 4 == 0 && s.colorAPackOrder >= 0 && s.colorAPackOrder <= 3 &&
	       s.colorBPackOrder >= 0 && s.colorBPackOrder <= 3;
}

bool valid_image(const dsrg_image *img) {
	return img && img->data && img->width > 0 && img->height > 0 && img->strideBytes >= img->width * 4 && img->strideBytes % 4 == 0;
}

// Memory the kernels of one call reach: device memory as given, page-locked host memory through
// its device address (read and written in place over the host link), pageable host memory through
// a copy in the context's staging buffer, copied back after the kernels when the call writes it.
// The reference's light passes and draw_higher take host images (lightAPI.cpp:23-323,
// drawAPI.cpp:872-900); this lets the same images come straight from the caller.
struct CallMemory {
	const void *host = nullptr; // the caller's pointer
	size_t rowBytes = 0, strideBytes = 0, rows = 0;
	bool onDevice = false, written = false;
	void *device = nullptr;     // where the kernels find it
	size_t stagedAt = SIZE_MAX; // 4-byte offset into the staging buffer, for pageable memory
};

CallMemory call_image(const dsrg_image *img, bool written) {
	CallMemory m;
	m.host = img->data;
	m.rowBytes = (size_t)img->width * 4;
	m.strideBytes = (size_t)img->strideBytes;
	m.rows = (size_t)img->height;
	m.onDevice = img->onDevice != 0;
	m.written = written;
	return m;
}

// Resolves where each block lives, stages the pageable ones (one buffer for the call) and copies them in.
int place(dsrg_context ctx, std::vector<CallMemory> &blocks) {
	size_t staged = 0;
	for (CallMemory &m : blocks) {
		if (m.onDevice || m.rowBytes * m.rows == 0) {
			m.device = const_cast<void *>(m.host);
		} else if (!host_mapped(m.host, &m.device)) {
			m.stagedAt = staged;
			staged += (m.rowBytes * m.rows + 3) / 4;
		}
	}
	if (staged == 0) return DSRG_OK;
	DSRG_CUDA_TRY(ctx, ctx->lightStaging.reserve(staged));
	for (CallMemory &m : blocks) {
		if (m.stagedAt == SIZE_MAX) continue;
		m.device = ctx->lightStaging.ptr + m.stagedAt;
		DSRG_CUDA_TRY(ctx, cudaMemcpy2DAsync(m.device, m.rowBytes, m.host, m.strideBytes, m.rowBytes, m.rows, cudaMemcpyHostToDevice,
		                                     ctx->stream));
		m.strideBytes = m.rowBytes; // the staged copy has no row padding
	}
	return DSRG_OK;
}

// Copies the staged blocks the call wrote back to the caller's memory, and waits for the call.
// Inside a sprite frame (wait = false) every image comes placed already, so nothing is staged and
// the frame waits once at its end.
int finish(dsrg_context ctx, const std::vector<CallMemory> &blocks, const dsrg_image *const *images, bool wait = true) {
	if (!wait) {
		for (const CallMemory &m : blocks)
			if (m.stagedAt != SIZE_MAX) return fail(ctx, DSRG_ERROR_CUDA, "sprite frame: an image of a step was not placed");
		return DSRG_OK;
	}
	for (size_t i = 0; i < blocks.size(); i++) {
		const CallMemory &m = blocks[i];
		if (m.stagedAt == SIZE_MAX || !m.written) continue;
		DSRG_CUDA_TRY(ctx, cudaMemcpy2DAsync(const_cast<void *>(m.host), (size_t)images[i]->strideBytes, m.device, m.rowBytes, m.rowBytes,
		                                     m.rows, cudaMemcpyDeviceToHost, ctx->stream));
	}
	DSRG_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
	return DSRG_OK;
}

int32_t stride_of(const CallMemory &m) { return (int32_t)(m.strideBytes / 4); }

int32_t hardware_threads() {
	const unsigned n = std::thread::hardware_concurrency();
	return n > 0 ? (int32_t)n : 1;
}

int light_directed_impl(dsrg_context ctx, const dsrg_ortho_view *view, const dsrg_image *light, const dsrg_image *normal,
                        const float direction[3], float intensity, const int32_t color[3], int32_t add, bool wait) {
	if (!ctx) return DSRG_ERROR_INVALID_ARGUMENT;
	if (!view || !direction || !color) return fail(ctx, DSRG_ERROR_INVALID_ARGUMENT, "dsrg_light_directed: null argument");
	if (!valid_image(light) || !valid_image(normal) || light->width != normal->width || light->height != normal->height)
		return fail(ctx, DSRG_ERROR_INVALID_ARGUMENT, "dsrg_light_directed: light and normal must be images of one size");
	cudaSetDevice(ctx->device);
	std::vector<CallMemory> mem = {call_image(light, true), call_image(normal, false)};
	const dsrg_image *const images[2] = {light, normal};
	const int placed = place(ctx, mem);
	if (placed != DSRG_OK) return placed;
	const M3 n = load_m3(view->normalToWorld);
	const Vec3 d = normalize_ref(transform_transposed_ref(n, v3(direction[0], direction[1], direction[2])));
	DirectedParams p;
	p.rev[0] = -d.x * intensity * 2.0f;
	p.rev[1] = -d.y * intensity * 2.0f;
	p.rev[2] = -d.z * intensity * 2.0f;
	for (int c = 0; c < 3; c++) {
		const float v = (float)color[c] / 255.0f;
		p.color[c] = 0.0f > v ? 0.0f : v;
	}
	p.add = add ? 1 : 0;
	const dim3 grid((light->width + 255) / 256, light->height);
	light_directed_kernel<<<grid, 256, 0, ctx->stream>>>((uint32_t *)mem[0].device, stride_of(mem[0]), (const uint32_t *)mem[1].device,
	                                                     stride_of(mem[1]), light->width, light->height, p);
	add_launches(1);
	DSRG_CUDA_TRY(ctx, cudaGetLastError());
	return finish(ctx, mem, images, wait);
}

int light_points_impl(dsrg_context ctx, const dsrg_ortho_view *view, int32_t centerX, int32_t centerY, const dsrg_image *light,
                      const dsrg_image *normal, const dsrg_image *height, const dsrg_point_light *lights, int32_t count,
                      int32_t referenceThreads, bool wait) {
	if (!ctx) return DSRG_ERROR_INVALID_ARGUMENT;
	if (!view || (count > 0 && !lights) || count < 0) return fail(ctx, DSRG_ERROR_INVALID_ARGUMENT, "dsrg_light_points: null argument");
	if (!valid_image(light) || !valid_image(normal) || !valid_image(height) || light->width != normal->width ||
	    light->height != normal->height || light->width != height->width || light->height != height->height)
		return fail(ctx, DSRG_ERROR_INVALID_ARGUMENT, "dsrg_light_points: light, normal and height must be images of one size");
	cudaSetDevice(ctx->device);
	const int32_t width = light->width, imageHeight = light->height;
	const int32_t threads = referenceThreads > 0 ? referenceThreads : hardware_threads();
	const M3 n = load_m3(view->normalToWorld), fromLight = load_m3(view->lightSpaceToScreenDepth);
	std::vector<PointLightParams> params;
	for (int32_t k = 0; k < count; k++) {
		const dsrg_point_light &l = lights[k];
		if (l.shadowCube && l.cubeWidth < 1) return fail(ctx, DSRG_ERROR_INVALID_ARGUMENT, "dsrg_light_points: shadow cube without a width");
		// calculateBound (lightAPI.cpp:76-102)
		const Vec3 source = transform_transposed_ref(n, v3(l.position[0], l.position[1], l.position[2]));
		const Vec3 rotated = transform_ref(fromLight, source);
		const int32_t pcx = (int32_t)rotated.x + centerX, pcy = (int32_t)rotated.y + centerY;
		const int32_t pixelRadius = (int32_t)(l.radius * fromLight.x.x);
		if (pcx < -pixelRadius || pcx > width + pixelRadius || pcy < -pixelRadius || pcy > imageHeight + pixelRadius) continue;
		const int32_t side = (int32_t)((float)pixelRadius * 2.0f);
		const int32_t bl = pcx - pixelRadius, bt = pcy - pixelRadius, br = bl + side, bb = bt + side;
		if (!(0 < br && width > bl && 0 < bb && imageHeight > bt)) continue; // IRect::overlaps (IRect.h:77-79)
		const int32_t left = bl > 0 ? bl : 0, top = bt > 0 ? bt : 0;
		const int32_t right = br < width ? br : width, bottom = bb < imageHeight ? bb : imageHeight;
		if (right - left <= 0 || bottom - top <= 0) continue;
		PointLightParams p;
		p.left = left - (left % 4);                  // roundDown(left, 4) for left >= 0
		p.right = right + 3 - ((right - 1) % 4);     // roundUp(right, 4) for right >= 1
		p.top = top;
		p.bottom = bottom;
		const int32_t rows = bottom - top;
		int32_t jobs = threads * 2; // getJobCount (base/threading.cpp:193-206) with 128 rows per job, 2 jobs per thread
		if (jobs > rows / 128) jobs = rows / 128;
		if (jobs < 1) jobs = 1;
		p.jobs = jobs;
		p.source[0] = source.x; p.source[1] = source.y; p.source[2] = source.z;
		for (int c = 0; c < 3; c++) {
			const float v = (float)l.color[c] * l.intensity;
			p.color[c] = 0.0f > v ? 0.0f : v;
		}
		p.reciprocalRadius = 1.0f / l.radius;
		p.cube = l.shadowCube;
		p.cubeWidth = l.cubeWidth;
		p.cubeCenter = (float)l.cubeWidth * 0.5f;
		params.push_back(p);
	}
	if (params.empty()) return DSRG_OK;
	// the images and the shadow cubes where the kernel reaches them
	std::vector<CallMemory> mem = {call_image(light, true), call_image(normal, false), call_image(height, false)};
	std::vector<const dsrg_image *> images = {light, normal, height};
	for (const PointLightParams &p : params) {
		if (!p.cube) continue;
		CallMemory cube;
		cube.host = p.cube;
		cube.rowBytes = cube.strideBytes = (size_t)p.cubeWidth * 4;
		cube.rows = (size_t)p.cubeWidth * 6;
		cudaPointerAttributes a;
		cube.onDevice = cudaPointerGetAttributes(&a, p.cube) == cudaSuccess && a.type == cudaMemoryTypeDevice;
		cudaGetLastError();
		mem.push_back(cube);
		images.push_back(nullptr);
	}
	const int placed = place(ctx, mem);
	if (placed != DSRG_OK) return placed;
	for (size_t k = 0, c = 3; k < params.size(); k++)
		if (params[k].cube) params[k].cube = (const float *)mem[c++].device;
	// the light table travels in the context's table buffer
	const size_t bytes = params.size() * sizeof(PointLightParams);
	DSRG_CUDA_TRY(ctx, ctx->tables.reserve(bytes));
	DSRG_CUDA_TRY(ctx, ctx->lightTableHost.reserve(bytes));
	memcpy(ctx->lightTableHost.ptr, params.data(), bytes);
	DSRG_CUDA_TRY(ctx, cudaMemcpyAsync(ctx->tables.ptr, ctx->lightTableHost.ptr, bytes, cudaMemcpyHostToDevice, ctx->stream));
	PointFrame f;
	memcpy(f.toLight, view->screenDepthToLightSpace, sizeof(f.toLight));
	f.centerX = centerX;
	f.centerY = centerY;
	f.lightCount = (int32_t)params.size();
	f.lights = reinterpret_cast<const PointLightParams *>(ctx->tables.ptr);
	const dim3 grid((width + 255) / 256, (imageHeight + 7) / 8);
	light_points_kernel<<<grid, 256, 0, ctx->stream>>>((uint32_t *)mem[0].device, stride_of(mem[0]), (const uint32_t *)mem[1].device,
	                                                   stride_of(mem[1]), (const float *)mem[2].device, stride_of(mem[2]),
	                                                   width, imageHeight, f);
	add_launches(1);
	DSRG_CUDA_TRY(ctx, cudaGetLastError());
	return finish(ctx, mem, images.data(), wait);
}

int light_blend_impl(dsrg_context ctx, const dsrg_image *target, const dsrg_image *diffuse, const dsrg_image *light, bool wait) {
	if (!ctx) return DSRG_ERROR_INVALID_ARGUMENT;
	if (!valid_image(target) || !valid_image(diffuse) || !valid_image(light) || target->width != diffuse->width ||
	    target->height != diffuse->height || target->width != light->width || target->height != light->height ||
	    target->packOrder < 0 || target->packOrder > 3)
		return fail(ctx, DSRG_ERROR_INVALID_ARGUMENT, "dsrg_light_blend: target, diffuse and light must be images of one size");
	cudaSetDevice(ctx->device);
	std::vector<CallMemory> mem = {call_image(target, true), call_image(diffuse, false), call_image(light, false)};
	const dsrg_image *const images[3] = {target, diffuse, light};
	const int placed = place(ctx, mem);
	if (placed != DSRG_OK) return placed;
	const dim3 grid((target->width + 255) / 256, target->height);
	light_blend_kernel<<<grid, 256, 0, ctx->stream>>>((uint32_t *)mem[0].device, stride_of(mem[0]), target->packOrder,
	                                                  (const uint32_t *)mem[1].device, stride_of(mem[1]),
	                                                  (const uint32_t *)mem[2].device, stride_of(mem[2]), target->width,
	                                                  target->height);
	add_launches(1);
	DSRG_CUDA_TRY(ctx, cudaGetLastError());
	return finish(ctx, mem, images, wait);
}

int draw_higher_impl(dsrg_context ctx, const dsrg_image *targetHeight, const dsrg_image *targetA, const dsrg_image *targetB,
                     const dsrg_sprite *sprites, int32_t count, bool wait) {
	if (!ctx) return DSRG_ERROR_INVALID_ARGUMENT;
	if (count < 0 || (count > 0 && !sprites)) return fail(ctx, DSRG_ERROR_INVALID_ARGUMENT, "dsrg_draw_higher: null sprites");
	if (!valid_image(targetHeight) || !valid_image(targetA) || !valid_image(targetB) || targetHeight->width != targetA->width ||
	    targetHeight->height != targetA->height || targetHeight->width != targetB->width || targetHeight->height != targetB->height ||
	    targetA->packOrder < 0 || targetA->packOrder > 3 || targetB->packOrder < 0 || targetB->packOrder > 3)
		return fail(ctx, DSRG_ERROR_INVALID_ARGUMENT, "dsrg_draw_higher: targets must be images of one size");
	cudaSetDevice(ctx->device);
	if (count == 0) return DSRG_OK;
	std::vector<SpriteData> table(count);
	int32_t tallest = 1;
	for (int32_t i = 0; i < count; i++) {
		const dsrg_sprite &s = sprites[i];
		if (!sprite_ok(s)) return fail(ctx, DSRG_ERROR_INVALID_ARGUMENT, "dsrg_draw_higher: invalid sprite " + std::to_string(i));
		SpriteData &d = table[i];
		d.height = s.height; d.colorA = s.colorA; d.colorB = s.colorB;
		d.width = s.width; d.height_ = s.height_;
		d.heightStride = s.heightStrideBytes / 4; d.aStride = s.colorAStrideBytes / 4; d.bStride = s.colorBStrideBytes / 4;
		d.aPack = s.colorAPackOrder; d.bPack = s.colorBPackOrder;
		d.left = s.left; d.top = s.top; d.offset = s.offset;
		if (s.height_ > tallest) tallest = s.height_;
	}
	// the targets and every host sprite's three sources where the kernels reach them (device
	// sources are used as given)
	std::vector<CallMemory> mem = {call_image(targetHeight, true), call_image(targetA, true), call_image(targetB, true)};
	std::vector<const dsrg_image *> images = {targetHeight, targetA, targetB};
	for (int32_t i = 0; i < count; i++) {
		const dsrg_sprite &s = sprites[i];
		if (s.onDevice) continue;
		const void *sources[3] = {s.height, s.colorA, s.colorB};
		const int32_t strides[3] = {s.heightStrideBytes, s.colorAStrideBytes, s.colorBStrideBytes};
		for (int k = 0; k < 3; k++) {
			CallMemory m;
			m.host = sources[k];
			m.rowBytes = (size_t)s.width * 4;
			m.strideBytes = (size_t)strides[k];
			m.rows = (size_t)s.height_;
			m.onDevice = s.onDevice != 0;
			mem.push_back(m);
			images.push_back(nullptr);
		}
	}
	const int placed = place(ctx, mem);
	if (placed != DSRG_OK) return placed;
	for (int32_t i = 0, placedSprite = 0; i < count; i++) {
		if (sprites[i].onDevice) continue;
		SpriteData &d = table[i];
		const CallMemory *m = &mem[3 + 3 * (size_t)placedSprite++];
		d.height = (const float *)m[0].device; d.heightStride = stride_of(m[0]);
		d.colorA = (const uint32_t *)m[1].device; d.aStride = stride_of(m[1]);
		d.colorB = (const uint32_t *)m[2].device; d.bStride = stride_of(m[2]);
	}
	const int32_t width = targetHeight->width, height = targetHeight->height;
	const size_t pixels = (size_t)width * height;
	DSRG_CUDA_TRY(ctx, ctx->spriteKeys.reserve(pixels));
	DSRG_CUDA_TRY(ctx, ctx->spriteTables.reserve(sizeof(SpriteData) * table.size()));
	DSRG_CUDA_TRY(ctx, ctx->spriteTableHost.reserve(sizeof(SpriteData) * table.size()));
	memcpy(ctx->spriteTableHost.ptr, table.data(), sizeof(SpriteData) * table.size());
	DSRG_CUDA_TRY(ctx, cudaMemcpyAsync(ctx->spriteTables.ptr, ctx->spriteTableHost.ptr, sizeof(SpriteData) * table.size(), cudaMemcpyHostToDevice,
	                                   ctx->stream));
	DSRG_CUDA_TRY(ctx, cudaMemsetAsync(ctx->spriteKeys.ptr, 0, pixels * sizeof(unsigned long long), ctx->stream));
	const SpriteData *deviceTable = reinterpret_cast<const SpriteData *>(ctx->spriteTables.ptr);
	// about four rows per thread: 16 rows per block of 64 x 4 threads
	const int32_t blocksPerSprite = (tallest + 15) / 16 < 64 ? (tallest + 15) / 16 : 64;
	for (int32_t first = 0; first < count; first += 65535) { // grid y is limited to 65535 sprites per launch
		const int32_t n = count - first < 65535 ? count - first : 65535;
		higher_keys_kernel<<<dim3(blocksPerSprite, n), dim3(64, 4), 0, ctx->stream>>>(deviceTable, first, count, (const float *)mem[0].device,
		                                                                             stride_of(mem[0]), width, height, ctx->spriteKeys.ptr);
		add_launches(1);
	}
	const dim3 grid((width + 255) / 256, height);
	higher_resolve_kernel<<<grid, 256, 0, ctx->stream>>>(deviceTable, ctx->spriteKeys.ptr, (float *)mem[0].device, stride_of(mem[0]),
	                                                     (uint32_t *)mem[1].device, stride_of(mem[1]), targetA->packOrder,
	                                                     (uint32_t *)mem[2].device, stride_of(mem[2]), targetB->packOrder, width, height);
	add_launches(1);
	DSRG_CUDA_TRY(ctx, cudaGetLastError());
	return finish(ctx, mem, images.data(), wait);
}

// Where a shadow cube's words are for the kernels: device memory as given, page-locked memory
// through its device address; null for pageable memory.
const float *cube_in_place(const float *cube) {
	cudaPointerAttributes a;
	if (cudaPointerGetAttributes(&a, cube) == cudaSuccess && a.type == cudaMemoryTypeDevice) return cube;
	cudaGetLastError();
	void *mappedPointer = nullptr;
	return host_mapped(cube, &mappedPointer) ? (const float *)mappedPointer : nullptr;
}

// The steps of one sprite frame after its images were placed (see dsrg_sprite_frame).
// The clears, draw_higher and the directed light of a sprite frame: they touch neither the shadow
// cubes nor the buffers of the shadow batch.
int sprite_frame_images(dsrg_context ctx, const dsrg_sprite_frame_desc &d, const dsrg_image *img, const dsrg_sprite *sprites) {
	const dsrg_image &height = img[0], &diffuse = img[1], &normal = img[2], &light = img[3];
	uint32_t clearHeight;
	memcpy(&clearHeight, &d.clearHeight, 4);
	enqueue_fill_words(height.data, height.strideBytes / 4, height.width, height.height, clearHeight, ctx->stream);
	enqueue_fill_words(diffuse.data, diffuse.strideBytes / 4, diffuse.width, diffuse.height, d.clearDiffuse, ctx->stream);
	enqueue_fill_words(normal.data, normal.strideBytes / 4, normal.width, normal.height, d.clearNormal, ctx->stream);
	add_launches(3);
	DSRG_CUDA_TRY(ctx, cudaGetLastError());
	const int status = draw_higher_impl(ctx, &height, &diffuse, &normal, sprites, d.spriteCount, false);
	if (status != DSRG_OK) return status;
	return light_directed_impl(ctx, d.view, &light, &normal, d.sunDirection, d.sunIntensity, d.sunColor, 0, false);
}

int sprite_frame_steps(dsrg_context ctx, const dsrg_sprite_frame_desc &d, const dsrg_image *img, const dsrg_sprite *sprites,
                       const dsrg_point_light *lights) {
	const dsrg_image &height = img[0], &diffuse = img[1], &normal = img[2], &light = img[3], &output = img[4];
	int status = DSRG_OK;
	if (d.shadows) {
		// the sprite images on a second stream beside the shadow batch (whose short, latency-bound
		// launches leave most of the GPU's issue slots free), joined before the point lights
		if (!ctx->sideStream) {
			int leastPriority = 0, greatestPriority = 0;
			DSRG_CUDA_TRY(ctx, cudaDeviceGetStreamPriorityRange(&leastPriority, &greatestPriority));
			DSRG_CUDA_TRY(ctx, cudaStreamCreateWithPriority(&ctx->sideStream, cudaStreamNonBlocking, leastPriority));
			DSRG_CUDA_TRY(ctx, cudaEventCreateWithFlags(&ctx->sideStart, cudaEventDisableTiming));
			DSRG_CUDA_TRY(ctx, cudaEventCreateWithFlags(&ctx->sideDone, cudaEventDisableTiming));
		}
		cudaStream_t mainStream = ctx->stream;
		DSRG_CUDA_TRY(ctx, cudaEventRecord(ctx->sideStart, mainStream)); // after the frame's images were placed
		DSRG_CUDA_TRY(ctx, cudaStreamWaitEvent(ctx->sideStream, ctx->sideStart, 0));
		ctx->stream = ctx->sideStream;
		status = sprite_frame_images(ctx, d, img, sprites);
		ctx->stream = mainStream;
		// the main stream waits for the side stream whatever happens next, so that a wait for the
		// main stream covers both
		const cudaError_t recorded = cudaEventRecord(ctx->sideDone, ctx->sideStream);
		if (status == DSRG_OK && recorded == cudaSuccess) {
			batch_clear_depth(d.shadows);
			status = cudaGetLastError() == cudaSuccess ? dsrg_batch_render(d.shadows) // its host wait is for the main stream
			                                           : fail(ctx, DSRG_ERROR_CUDA, "sprite frame: clearing the shadow cubes failed");
		}
		const cudaError_t joined = recorded == cudaSuccess ? cudaStreamWaitEvent(mainStream, ctx->sideDone, 0) : recorded;
		if (status != DSRG_OK) return status;
		DSRG_CUDA_TRY(ctx, joined);
	} else {
		status = sprite_frame_images(ctx, d, img, sprites);
		if (status != DSRG_OK) return status;
	}
	status = light_points_impl(ctx, d.view, d.centerX, d.centerY, &light, &normal, &height, lights, d.lightCount, d.referenceThreads,
	                           false);
	if (status != DSRG_OK) return status;
	return light_blend_impl(ctx, &output, &diffuse, &light, false);
}

} // namespace

void enqueue_fill_words(void *image, int32_t strideWords, int32_t width, int32_t height, uint32_t value, cudaStream_t stream) {
	if (width <= 0 || height <= 0) return;
	for (int32_t first = 0; first < height; first += 65535) { // grid y is limited to 65535 rows per launch
		const int32_t rows = height - first < 65535 ? height - first : 65535;
		fill_words_kernel<<<dim3((width + 255) / 256, rows), 256, 0, stream>>>((uint32_t *)image + (size_t)first * strideWords,
		                                                                      strideWords, width, rows, value);
	}
}

extern "C" {

int dsrg_ortho_view_create(float cameraTilt, int32_t pixelsPerTile, int32_t index, dsrg_ortho_view *out) {
	if (!out || index < 0 || index > 7 || pixelsPerTile < 1) return DSRG_ERROR_INVALID_ARGUMENT;
	const float diag = 0.707106781f;
	// the reference's unqualified sqrt of a float argument resolves to the double overload
	const int32_t yPixelsPerTile = (int32_t)((double)(float)pixelsPerTile / sqrt((double)(cameraTilt * cameraTilt + 1)));
	const Vec3 forward[8] = {v3(diag, cameraTilt, diag), v3(-diag, cameraTilt, diag), v3(-diag, cameraTilt, -diag),
	                         v3(diag, cameraTilt, -diag), v3(0.0f, cameraTilt, 1.0f), v3(-1.0f, cameraTilt, 0.0f),
	                         v3(0.0f, cameraTilt, -1.0f), v3(1.0f, cameraTilt, 0.0f)};
	const M3 system = axis_system(forward[index], v3(0.0f, 1.0f, 0.0f));
	Vec3 normalDirection = system.z;
	normalDirection.y = 0.0f;
	const M3 normalToWorld = axis_system(normalDirection, v3(0.0f, 1.0f, 0.0f));
	// Camera::createOrthogonal(Transform3D(origin, system), ppt, ppt, 0.5) and worldToScreen of the x and z axes
	dsrg_camera cam;
	memset(&cam, 0, sizeof(cam));
	const float loc[12] = {0.0f, 0.0f, 0.0f, system.x.x, system.x.y, system.x.z, system.y.x, system.y.y, system.y.z,
	                       system.z.x, system.z.y, system.z.z};
	memcpy(cam.location, loc, sizeof(loc));
	cam.perspective = 0;
	cam.slope = 0.5f;
	cam.width = pixelsPerTile;
	cam.height = pixelsPerTile;
	const CameraData c = make_camera(cam);
	const float halfTile = (float)pixelsPerTile * 0.5f;
	const Projected px = camera_to_screen(c, world_to_camera(c, v3(1.0f, 0.0f, 0.0f)));
	const Projected pz = camera_to_screen(c, world_to_camera(c, v3(0.0f, 0.0f, 1.0f)));
	const int32_t xAxis[2] = {(int32_t)(px.isx - halfTile), (int32_t)(px.isy - halfTile)};
	const int32_t zAxis[2] = {(int32_t)(pz.isx - halfTile), (int32_t)(pz.isy - halfTile)};
	// OrthoView::OrthoView (orthoAPI.cpp:6-37)
	M3 tileToScreen;
	tileToScreen.x = v3((float)xAxis[0], (float)xAxis[1], 0.0f);
	tileToScreen.y = v3(0.0f, (float)(-yPixelsPerTile), 1.0f);
	tileToScreen.z = v3((float)zAxis[0], (float)zAxis[1], 0.0f);
	const M3 screenToTile = inverse_ref(tileToScreen);
	M3 toLight;
	toLight.x = transform_transposed_ref(normalToWorld, screenToTile.x);
	toLight.y = transform_transposed_ref(normalToWorld, screenToTile.y);
	toLight.z = transform_transposed_ref(normalToWorld, screenToTile.z);
	const M3 fromLight = inverse_ref(toLight);
	store_m3(normalToWorld, out->normalToWorld);
	store_m3(toLight, out->screenDepthToLightSpace);
	store_m3(fromLight, out->lightSpaceToScreenDepth);
	out->pixelOffsetPerTileX[0] = xAxis[0]; out->pixelOffsetPerTileX[1] = xAxis[1];
	out->pixelOffsetPerTileZ[0] = zAxis[0]; out->pixelOffsetPerTileZ[1] = zAxis[1];
	out->yPixelsPerTile = yPixelsPerTile;
	return DSRG_OK;
}

int dsrg_shadow_side_location(const float normalToWorld[9], int32_t side, float location[12]) {
	if (!normalToWorld || !location || side < 0 || side > 5) return DSRG_ERROR_INVALID_ARGUMENT;
	const Vec3 forward[6] = {v3(1.0f, 0.0f, 0.0f), v3(-1.0f, 0.0f, 0.0f), v3(0.0f, 1.0f, 0.0f),
	                         v3(0.0f, -1.0f, 0.0f), v3(0.0f, 0.0f, 1.0f), v3(0.0f, 0.0f, -1.0f)};
	const Vec3 up[6] = {v3(0.0f, 1.0f, 0.0f), v3(0.0f, 1.0f, 0.0f), v3(0.0f, 0.0f, 1.0f),
	                    v3(0.0f, 0.0f, 1.0f), v3(0.0f, 1.0f, 0.0f), v3(0.0f, 1.0f, 0.0f)};
	const M3 s = axis_system(forward[side], up[side]);
	const M3 n = load_m3(normalToWorld);
	M3 r; // FMatrix3x3 product (FMatrix3x3.h:50-52)
	r.x = transform_ref(n, s.x);
	r.y = transform_ref(n, s.y);
	r.z = transform_ref(n, s.z);
	location[0] = 0.0f; location[1] = 0.0f; location[2] = 0.0f;
	store_m3(r, location + 3);
	return DSRG_OK;
}

int dsrg_light_directed(dsrg_context ctx, const dsrg_ortho_view *view, const dsrg_image *light, const dsrg_image *normal,
                        const float direction[3], float intensity, const int32_t color[3], int32_t add) {
	return light_directed_impl(ctx, view, light, normal, direction, intensity, color, add, true);
}

int dsrg_light_points(dsrg_context ctx, const dsrg_ortho_view *view, int32_t centerX, int32_t centerY, const dsrg_image *light,
                      const dsrg_image *normal, const dsrg_image *height, const dsrg_point_light *lights, int32_t count,
                      int32_t referenceThreads) {
	return light_points_impl(ctx, view, centerX, centerY, light, normal, height, lights, count, referenceThreads, true);
}

int dsrg_light_blend(dsrg_context ctx, const dsrg_image *target, const dsrg_image *diffuse, const dsrg_image *light) {
	return light_blend_impl(ctx, target, diffuse, light, true);
}

int dsrg_draw_higher(dsrg_context ctx, const dsrg_image *targetHeight, const dsrg_image *targetA, const dsrg_image *targetB,
                     const dsrg_sprite *sprites, int32_t count) {
	return draw_higher_impl(ctx, targetHeight, targetA, targetB, sprites, count, true);
}

int dsrg_check_float_roots(dsrg_context ctx, uint32_t firstBits, uint32_t count, uint64_t *mismatches) {
	if (!ctx || !mismatches) return DSRG_ERROR_INVALID_ARGUMENT;
	cudaSetDevice(ctx->device);
	*mismatches = 0;
	if (count == 0) return DSRG_OK;
	DSRG_CUDA_TRY(ctx, ctx->tables.reserve(sizeof(unsigned long long)));
	unsigned long long *counter = reinterpret_cast<unsigned long long *>(ctx->tables.ptr);
	DSRG_CUDA_TRY(ctx, cudaMemsetAsync(counter, 0, sizeof(unsigned long long), ctx->stream));
	root_check_kernel<<<sm_count() * 8, 256, 0, ctx->stream>>>(firstBits, count, counter);
	add_launches(1);
	DSRG_CUDA_TRY(ctx, cudaGetLastError());
	unsigned long long found = 0;
	DSRG_CUDA_TRY(ctx, cudaMemcpyAsync(&found, counter, sizeof(found), cudaMemcpyDeviceToHost, ctx->stream));
	DSRG_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
	*mismatches = found;
	return DSRG_OK;
}

int dsrg_sprite_frame(dsrg_context ctx, const dsrg_sprite_frame_desc *frame) {
	if (!ctx) return DSRG_ERROR_INVALID_ARGUMENT;
	if (!frame || !frame->view) return fail(ctx, DSRG_ERROR_INVALID_ARGUMENT, "dsrg_sprite_frame: null argument");
	const dsrg_sprite_frame_desc &d = *frame;
	const dsrg_image *given[5] = {d.height, d.diffuse, d.normal, d.light, d.output};
	for (const dsrg_image *g : given)
		if (!valid_image(g) || g->width != d.height->width || g->height != d.height->height)
			return fail(ctx, DSRG_ERROR_INVALID_ARGUMENT, "dsrg_sprite_frame: height, diffuse, normal, light and output must be images of one size");
	if (d.spriteCount < 0 || (d.spriteCount > 0 && !d.sprites) || d.lightCount < 0 || (d.lightCount > 0 && !d.lights))
		return fail(ctx, DSRG_ERROR_INVALID_ARGUMENT, "dsrg_sprite_frame: null sprites or lights");
	for (int32_t i = 0; i < d.spriteCount; i++)
		if (!sprite_ok(d.sprites[i])) return fail(ctx, DSRG_ERROR_INVALID_ARGUMENT, "dsrg_sprite_frame: invalid sprite " + std::to_string(i));
	if (d.shadows && batch_context(d.shadows) != ctx)
		return fail(ctx, DSRG_ERROR_INVALID_ARGUMENT, "dsrg_sprite_frame: the shadow batch belongs to another context");
	cudaSetDevice(ctx->device);
	if (d.shadows && !batch_depth_in_place(d.shadows))
		return fail(ctx, DSRG_ERROR_INVALID_ARGUMENT, "dsrg_sprite_frame: shadow cubes must be device or page-locked memory");
	std::vector<dsrg_point_light> lights(d.lights, d.lights + d.lightCount);
	for (dsrg_point_light &l : lights) {
		if (!l.shadowCube) continue;
		l.shadowCube = cube_in_place(l.shadowCube);
		if (!l.shadowCube) return fail(ctx, DSRG_ERROR_INVALID_ARGUMENT, "dsrg_sprite_frame: shadow cubes must be device or page-locked memory");
	}
	// every image of the frame placed once: the five frame images (written) and each distinct sprite source (read)
	std::vector<CallMemory> mem;
	std::vector<const dsrg_image *> images;
	for (const dsrg_image *g : given) {
		mem.push_back(call_image(g, true));
		images.push_back(g);
	}
	std::vector<dsrg_sprite> sprites(d.sprites, d.sprites + d.spriteCount);
	// one block per distinct source (the same memory seen with the same size and stride)
	std::map<std::tuple<const void *, int32_t, int32_t, int32_t>, size_t> sourceBlock;
	std::vector<size_t> spriteBlocks(sprites.size() * 3);
	for (size_t i = 0; i < sprites.size(); i++) {
		const dsrg_sprite &s = sprites[i];
		if (s.onDevice) continue; // device sources are used as given
		const void *sources[3] = {s.height, s.colorA, s.colorB};
		const int32_t strides[3] = {s.heightStrideBytes, s.colorAStrideBytes, s.colorBStrideBytes};
		for (int k = 0; k < 3; k++) {
			const auto key = std::make_tuple(sources[k], s.width, s.height_, strides[k]);
			auto found = sourceBlock.find(key);
			if (found == sourceBlock.end()) {
				CallMemory m;
				m.host = sources[k];
				m.rowBytes = (size_t)s.width * 4;
				m.strideBytes = (size_t)(strides[k] > 0 ? strides[k] : 0);
				m.rows = (size_t)(s.height_ > 0 ? s.height_ : 0);
				m.onDevice = s.onDevice != 0;
				found = sourceBlock.emplace(key, mem.size()).first;
				mem.push_back(m);
				images.push_back(nullptr);
			}
			spriteBlocks[3 * i + k] = found->second;
		}
	}
	int status = place(ctx, mem);
	if (status != DSRG_OK) return status;
	dsrg_image placed[5];
	for (int i = 0; i < 5; i++) {
		placed[i] = *given[i];
		placed[i].data = mem[i].device;
		placed[i].strideBytes = (int32_t)mem[i].strideBytes;
		placed[i].onDevice = 1;
	}
	for (size_t i = 0; i < sprites.size(); i++) {
		dsrg_sprite &s = sprites[i];
		if (s.onDevice) continue;
		const CallMemory &h = mem[spriteBlocks[3 * i]], &a = mem[spriteBlocks[3 * i + 1]], &b = mem[spriteBlocks[3 * i + 2]];
		s.height = (const float *)h.device; s.heightStrideBytes = (int32_t)h.strideBytes;
		s.colorA = (const uint32_t *)a.device; s.colorAStrideBytes = (int32_t)a.strideBytes;
		s.colorB = (const uint32_t *)b.device; s.colorBStrideBytes = (int32_t)b.strideBytes;
		s.onDevice = 1;
	}
	status = sprite_frame_steps(ctx, d, placed, sprites.data(), lights.data());
	if (status != DSRG_OK) {
		cudaStreamSynchronize(ctx->stream); // nothing of the frame stays in flight
		cudaGetLastError();
		return status;
	}
	return finish(ctx, mem, images.data()); // the staged frame images back to the caller, and the frame's last wait
}

} // extern "C"
