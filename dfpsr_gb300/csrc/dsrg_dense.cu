// Dense models of the isometric sprite engine (SDK/SpriteEngine/spriteAPI.cpp:236-262, 1143-1327):
// DenseModel_create turns a model into vertex-coloured triangles with smooth normals, and
// renderDenseModel draws them into the sprite world's height, diffuse and normal images through
// an ortho view (drawModel at run time, the low-quality form; sprite generation, the high-quality
// form with normalized normals).
//
// The reference walks the triangles in order and writes a pixel when the new height is strictly
// above the stored one.  As in the triangle path, that result does not depend on the order if
// every candidate (height passing the initial image) competes for the pixel with a 64-bit key
// (ordered height, ~triangle index): the highest height wins, and among equal heights the earliest
// triangle, as the strict test keeps it.  dense_keys_kernel takes one triangle per thread and
// walks its bound; dense_resolve_kernel re-evaluates each pixel's winner and writes the three
// images.  Both evaluate the reference's expressions in its order (no contraction in this build),
// so the values are the reference's bit for bit.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "dsrg_internal.h"
#include "dsrg_raster.cuh"

using namespace dsrg;

struct dsrg_dense_model_s {
	dsrg_context context = nullptr;
	DeviceBuffer<float> triangles; // DENSE_FLOATS floats per triangle: colours (x 255), corners, normals
	int32_t count = 0;
	float minBound[3], maxBound[3]; // over the model's points (the model's bounding box)
};

namespace {

const int DENSE_FLOATS = 27;

struct V3 { float x, y, z; };
__host__ __device__ inline V3 v3(float x, float y, float z) { V3 r = {x, y, z}; return r; }
__host__ __device__ inline V3 add(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
__host__ __device__ inline V3 sub(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
// FVector.h:101-119: the cross product, and v / length(v) with length = sqrtf(squareLength(v))
__host__ __device__ inline V3 cross(V3 a, V3 b) { return v3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
__host__ __device__ inline V3 normalized(V3 v) {
	const float l = sqrtf(v.x * v.x + v.y * v.y + v.z * v.z);
	if (l == 0.0f) return v3(0.0f, 0.0f, 1.0f);
	return v3(v.x / l, v.y / l, v.z / l);
}
// FMatrix3x3::transform (FMatrix3x3.h:55-61), the matrix as x, y, z axes
struct M3 { V3 x, y, z; };
__host__ __device__ inline V3 transform(const M3 &m, V3 p) {
	return v3(p.x * m.x.x + p.y * m.y.x + p.z * m.z.x, p.x * m.x.y + p.y * m.y.y + p.z * m.z.y, p.x * m.x.z + p.y * m.y.z + p.z * m.z.z);
}
// FMatrix3x3 product (FMatrix3x3.h:78-80)
inline M3 product(const M3 &left, const M3 &right) {
	M3 r;
	r.x = transform(right, left.x);
	r.y = transform(right, left.y);
	r.z = transform(right, left.z);
	return r;
}

// The per-call transforms: object to screen (position, axes) and object normals to normal space,
// and the pixels the model can reach (its bounding box's screen bound, cut to the image), over
// which the key image is laid out.
struct DenseView {
	V3 position;
	M3 toScreen, toNormal;
	int32_t width, height;
	int32_t highQuality;
	int32_t rx0, ry0, rw, rh;
};

// (uint32_t)float of the reference's x86-64 build: a signed 64-bit truncation keeping the low 32 bits.
__device__ __forceinline__ uint32_t dense_u32(float x) { return (uint32_t)(int64_t)x; }

// min and max of base/noSimd.h:134-150 (the second operand when the comparison fails)
__device__ __forceinline__ float ref_min(float a, float b) { return a < b ? a : b; }
__device__ __forceinline__ float ref_max(float a, float b) { return a > b ? a : b; }

// One triangle's screen corners, bound (getBackCulledTriangleBound cut to the image) and the
// inverse of its corner offsets (FMatrix2x2.h:69-76).  False when nothing can be drawn.
struct DenseSetup {
	V3 a, b, c;
	float ixx, ixy, iyx, iyy;
	int32_t x0, y0, x1, y1;
};

__device__ __forceinline__ bool dense_setup(const float *t, const DenseView &v, DenseSetup &s) {
	s.a = add(transform(v.toScreen, v3(t[9], t[10], t[11])), v.position);
	s.b = add(transform(v.toScreen, v3(t[12], t[13], t[14])), v.position);
	s.c = add(transform(v.toScreen, v3(t[15], t[16], t[17])), v.position);
	const V3 a = s.a, b = s.b, c = s.c;
	if (((c.x - a.x) * (b.y - a.y)) + ((c.y - a.y) * (a.x - b.x)) >= 0.0f) return false; // back facing
	const float minX = ref_min(ref_min(a.x, b.x), c.x), minY = ref_min(ref_min(a.y, b.y), c.y);
	const float maxX = ref_max(ref_max(a.x, b.x), c.x), maxY = ref_max(ref_max(a.y, b.y), c.y);
	const int32_t left = (int32_t)minX, top = (int32_t)minY, right = (int32_t)maxX + 1, bottom = (int32_t)maxY + 1;
	if (!(left < v.width && right > 0 && top < v.height && bottom > 0)) return false;
	s.x0 = left > 0 ? left : 0;
	s.y0 = top > 0 ? top : 0;
	s.x1 = right < v.width ? right : v.width;
	s.y1 = bottom < v.height ? bottom : v.height;
	if (s.x1 <= s.x0 || s.y1 <= s.y0) return false;
	const float mxx = b.x - a.x, mxy = b.y - a.y, myx = c.x - a.x, myy = c.y - a.y;
	const float invDet = 1.0f / (mxx * myy - mxy * myx);
	s.ixx = myy * invDet; s.ixy = -mxy * invDet; s.iyx = -myx * invDet; s.iyy = mxx * invDet;
	return true;
}

// The affine weights of pixel (x, y) (its centre) and whether it is inside the triangle.
__device__ __forceinline__ bool dense_weights(const DenseSetup &s, int32_t x, int32_t y, float &wa, float &wb, float &wc) {
	const float ox = ((float)x + 0.5f) - s.a.x, oy = ((float)y + 0.5f) - s.a.y;
	wb = ox * s.ixx + oy * s.iyx;
	wc = ox * s.ixy + oy * s.iyy;
	wa = 1.0f - (wb + wc);
	return wa >= -0.00001f && wb >= -0.00001f && wc >= -0.00001f;
}

// One instance of a sequence drawn by one call: its model's triangles, its transforms and bound
// (in the view), and the sequence number of its first triangle.
struct DenseInstance {
	const float *triangles;
	uint32_t first, count;
	DenseView v;
};

// The instance holding sequence number t (instances sorted by first).
__device__ __forceinline__ uint32_t dense_instance_of(const DenseInstance *instances, uint32_t n, uint32_t t) {
	uint32_t lo = 0, hi = n;
	while (hi - lo > 1) {
		const uint32_t mid = (lo + hi) >> 1;
		if (instances[mid].first <= t) lo = mid; else hi = mid;
	}
	return lo;
}

// Keys of every instance's triangles (sequence number t = instance first + triangle): the
// highest height wins, among equal heights the earliest in the sequence, as the reference's
// strict test keeps it over consecutive calls.  The key image covers the rectangle (kx0, ky0, kw).
__global__ void dense_keys_kernel(const DenseInstance *__restrict__ instances, uint32_t instanceCount, uint32_t total,
                                  const float *__restrict__ height, int32_t heightStride, int32_t kx0, int32_t ky0, int32_t kw,
                                  unsigned long long *keys) {
	for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < total; t += gridDim.x * blockDim.x) {
		const DenseInstance &ins = instances[dense_instance_of(instances, instanceCount, t)];
		const DenseView &v = ins.v;
		DenseSetup s;
		if (!dense_setup(ins.triangles + (size_t)(t - ins.first) * DENSE_FLOATS, v, s)) continue;
		// inside the key image's bound (which holds every triangle bound; the cut only keeps
		// writes inside the buffer)
		const int32_t ya = max(s.y0, v.ry0), yb = min(s.y1, v.ry0 + v.rh), xa = max(s.x0, v.rx0), xb = min(s.x1, v.rx0 + v.rw);
		for (int32_t y = ya; y < yb; y++) {
			for (int32_t x = xa; x < xb; x++) {
				float wa, wb, wc;
				if (!dense_weights(s, x, y, wa, wb, wc)) continue;
				const float h = s.a.z * wa + s.b.z * wb + s.c.z * wc; // interpolateUsingAffineWeight (ITriangle2D.h:58-61)
				if (!(h > height[(size_t)y * heightStride + x])) continue;
				const unsigned long long key = ((unsigned long long)ordered_depth(h) << 32) | (unsigned long long)(~t);
				unsigned long long *k = &keys[(size_t)(y - ky0) * kw + (x - kx0)];
				if (key > *k) atomicMax(k, key);
			}
		}
	}
}

__global__ void dense_resolve_kernel(const DenseInstance *__restrict__ instances, uint32_t instanceCount, float *height,
                                     int32_t heightStride, uint32_t *diffuse, int32_t diffuseStride, uint32_t *normal,
                                     int32_t normalStride, int32_t kx0, int32_t ky0, int32_t kw, const unsigned long long *__restrict__ keys) {
	const int32_t x = kx0 + blockIdx.x * blockDim.x + threadIdx.x, y = ky0 + blockIdx.y;
	if (x >= kx0 + kw) return;
	const unsigned long long key = keys[(size_t)(y - ky0) * kw + (x - kx0)];
	if (key == 0ull) return;
	const uint32_t sequence = ~(uint32_t)(key & 0xFFFFFFFFull);
	const DenseInstance &ins = instances[dense_instance_of(instances, instanceCount, sequence)];
	const DenseView &v = ins.v;
	const float *t = ins.triangles + (size_t)(sequence - ins.first) * DENSE_FLOATS;
	DenseSetup s;
	dense_setup(t, v, s);
	float wa, wb, wc;
	dense_weights(s, x, y, wa, wb, wc);
	height[(size_t)y * heightStride + x] = s.a.z * wa + s.b.z * wb + s.c.z * wc;
	float col[3];
	for (int ch = 0; ch < 3; ch++) col[ch] = t[ch] * wa + t[3 + ch] * wb + t[6 + ch] * wc;
	const V3 na = transform(v.toNormal, v3(t[18], t[19], t[20]));
	const V3 nb = transform(v.toNormal, v3(t[21], t[22], t[23]));
	const V3 nc = transform(v.toNormal, v3(t[24], t[25], t[26]));
	V3 n = v3(na.x * wa + nb.x * wb + nc.x * wc, na.y * wa + nb.y * wb + nc.y * wc, na.z * wa + nb.z * wb + nc.z * wc);
	if (v.highQuality) n = normalized(n);
	const float nx = (n.x + 1.0f) * 127.5f, ny = (n.y + 1.0f) * 127.5f, nz = (n.z + 1.0f) * 127.5f;
	// written without saturation, as the reference does (colours are expected inside 0..255)
	diffuse[(size_t)y * diffuseStride + x] = dense_u32(col[0]) | (dense_u32(col[1]) << 8) | (dense_u32(col[2]) << 16) | (255u << 24);
	normal[(size_t)y * normalStride + x] = dense_u32(nx) | (dense_u32(ny) << 8) | (dense_u32(nz) << 16) | (255u << 24);
}

// A target in device memory: 4-byte pixels, rows at least as long as the image.
bool dense_image(const dsrg_image *img) {
	return img && img->data && img->onDevice && img->width > 0 && img->height > 0 && img->strideBytes >= img->width * 4 &&
	       img->strideBytes % 4 == 0;
}

} // namespace

extern "C" {

int dsrg_dense_model_create(dsrg_context ctx, const float *positions, int32_t pointCount, const int32_t *polygonIndices,
                            const float *colors, int32_t polygonCount, dsrg_dense_model *out) {
	if (!ctx || !out) return DSRG_ERROR_INVALID_ARGUMENT;
	*out = nullptr;
	if (pointCount < 0 || polygonCount < 0 || (pointCount > 0 && !positions) || (polygonCount > 0 && (!polygonIndices || !colors)))
		return fail(ctx, DSRG_ERROR_INVALID_ARGUMENT, "dsrg_dense_model_create: invalid arrays");
	int32_t count = 0;
	for (int32_t p = 0; p < polygonCount; p++) {
		const int32_t *idx = polygonIndices + p * 4;
		const int32_t corners = idx[3] < 0 ? 3 : 4;
		for (int32_t v = 0; v < corners; v++)
			if (idx[v] < 0 || idx[v] >= pointCount)
				return fail(ctx, DSRG_ERROR_INVALID_ARGUMENT, "dsrg_dense_model_create: point index out of range");
		count += corners - 2;
	}
	// DenseModelImpl::DenseModelImpl (spriteAPI.cpp:1189-1240): every polygon's normal (the
	// normalized sum of its fan triangles' normals, getAverageNormal at 1160-1171) is added to its
	// points, then each point's sum is normalized
	auto point = [&](int32_t i) { return v3(positions[i * 3], positions[i * 3 + 1], positions[i * 3 + 2]); };
	std::vector<V3> normals((size_t)(pointCount > 0 ? pointCount : 1), v3(0.0f, 0.0f, 0.0f));
	for (int32_t p = 0; p < polygonCount; p++) {
		const int32_t *idx = polygonIndices + p * 4;
		const int32_t corners = idx[3] < 0 ? 3 : 4;
		V3 sum = v3(0.0f, 0.0f, 0.0f);
		for (int32_t t = 0; t < corners - 2; t++)
			sum = add(sum, normalized(cross(sub(point(idx[t + 1]), point(idx[0])), sub(point(idx[t + 2]), point(idx[0])))));
		const V3 n = normalized(sum);
		for (int32_t v = 0; v < corners; v++) normals[idx[v]] = add(normals[idx[v]], n);
	}
	for (int32_t i = 0; i < pointCount; i++) normals[i] = normalized(normals[i]);
	float mn[3] = {0.0f, 0.0f, 0.0f}, mx[3] = {0.0f, 0.0f, 0.0f};
	for (int32_t i = 0; i < pointCount; i++)
		for (int c = 0; c < 3; c++) {
			const float q = positions[i * 3 + c];
			if (i == 0 || q < mn[c]) mn[c] = q;
			if (i == 0 || q > mx[c]) mx[c] = q;
		}
	std::vector<float> host((size_t)(count > 0 ? count : 1) * DENSE_FLOATS);
	size_t at = 0;
	for (int32_t p = 0; p < polygonCount; p++) {
		const int32_t *idx = polygonIndices + p * 4;
		const int32_t corners = idx[3] < 0 ? 3 : 4;
		for (int32_t vb = 1; vb < corners - 1; vb++) {
			const int32_t vert[3] = {0, vb, vb + 1};
			for (int k = 0; k < 3; k++) // FVector4Dto3D(colour) * 255.0f
				for (int ch = 0; ch < 3; ch++) host[at + k * 3 + ch] = colors[(p * 4 + vert[k]) * 4 + ch] * 255.0f;
			for (int k = 0; k < 3; k++) {
				const V3 q = point(idx[vert[k]]), n = normals[idx[vert[k]]];
				host[at + 9 + k * 3] = q.x; host[at + 10 + k * 3] = q.y; host[at + 11 + k * 3] = q.z;
				host[at + 18 + k * 3] = n.x; host[at + 19 + k * 3] = n.y; host[at + 20 + k * 3] = n.z;
			}
			at += DENSE_FLOATS;
		}
	}
	dsrg_dense_model m = new (std::nothrow) dsrg_dense_model_s();
	if (!m) return DSRG_ERROR_OUT_OF_MEMORY;
	m->context = ctx;
	m->count = count;
	for (int c = 0; c < 3; c++) { m->minBound[c] = mn[c]; m->maxBound[c] = mx[c]; }
	cudaSetDevice(ctx->device);
	cudaError_t e = m->triangles.reserve(host.size());
	if (e == cudaSuccess) e = cudaMemcpy(m->triangles.ptr, host.data(), host.size() * sizeof(float), cudaMemcpyHostToDevice);
	if (e != cudaSuccess) {
		delete m;
		return fail(ctx, DSRG_ERROR_CUDA, std::string("dsrg_dense_model_create: ") + cudaGetErrorString(e));
	}
	*out = m;
	return DSRG_OK;
}

int dsrg_dense_model_destroy(dsrg_dense_model m) {
	if (!m) return DSRG_ERROR_INVALID_ARGUMENT;
	cudaSetDevice(m->context->device);
	m->triangles.release();
	delete m;
	return DSRG_OK;
}

} // extern "C"

namespace {

// The transforms and reachable pixels of one instance (combineModelToScreenTransform,
// spriteAPI.cpp:29-35, with the product of Transform3D, Transform3D.h:56-58; tile to screen from
// the view's rounded axes, orthoAPI.cpp:9-13).  False when the instance cannot reach the image.
bool dense_view(const dsrg_dense_model_s *m, const dsrg_ortho_view *view, int32_t width, int32_t height, float originX, float originY,
                const float *modelToWorld, int32_t highQuality, DenseView &v) {
	M3 tileToScreen;
	tileToScreen.x = v3((float)view->pixelOffsetPerTileX[0], (float)view->pixelOffsetPerTileX[1], 0.0f);
	tileToScreen.y = v3(0.0f, (float)(-view->yPixelsPerTile), 1.0f);
	tileToScreen.z = v3((float)view->pixelOffsetPerTileZ[0], (float)view->pixelOffsetPerTileZ[1], 0.0f);
	M3 model;
	model.x = v3(modelToWorld[3], modelToWorld[4], modelToWorld[5]);
	model.y = v3(modelToWorld[6], modelToWorld[7], modelToWorld[8]);
	model.z = v3(modelToWorld[9], modelToWorld[10], modelToWorld[11]);
	v.position = add(transform(tileToScreen, v3(modelToWorld[0], modelToWorld[1], modelToWorld[2])), v3(originX, originY, 0.0f));
	v.toScreen = product(model, tileToScreen);
	const float *n = view->normalToWorld; // transpose(normalToWorldSpace) (FMatrix3x3.h:109-120)
	M3 transposed;
	transposed.x = v3(n[0], n[3], n[6]);
	transposed.y = v3(n[1], n[4], n[7]);
	transposed.z = v3(n[2], n[5], n[8]);
	v.toNormal = product(model, transposed);
	v.width = width;
	v.height = height;
	v.highQuality = highQuality ? 1 : 0;
	// The pixels the model can reach: its bounding box's corners through the same transform
	// (boundingBoxToRectangle, spriteAPI.cpp:1128-1141), widened by two pixels for the rounding
	// of points inside the box, cut to the image.  Nothing outside can be drawn, as in the
	// reference's early test.
	int64_t bx0 = 0, by0 = 0, bx1 = 0, by1 = 0;
	for (int k = 0; k < 8; k++) {
		const V3 corner = v3((k & 1) ? m->maxBound[0] : m->minBound[0], (k & 2) ? m->maxBound[1] : m->minBound[1],
		                     (k & 4) ? m->maxBound[2] : m->minBound[2]);
		const V3 s = add(transform(v.toScreen, corner), v.position);
		if (!(std::isfinite(s.x) && std::isfinite(s.y) && std::fabs(s.x) < 1.0e9f && std::fabs(s.y) < 1.0e9f)) {
			bx0 = by0 = -2000000000; bx1 = by1 = 2000000000; // no usable bound: the whole image
			break;
		}
		const int64_t px = (int32_t)s.x, py = (int32_t)s.y;
		if (k == 0 || px < bx0) bx0 = px;
		if (k == 0 || py < by0) by0 = py;
		if (k == 0 || px + 1 > bx1) bx1 = px + 1;
		if (k == 0 || py + 1 > by1) by1 = py + 1;
	}
	v.rx0 = (int32_t)std::max<int64_t>(bx0 - 2, 0);
	v.ry0 = (int32_t)std::max<int64_t>(by0 - 2, 0);
	const int32_t rx1 = (int32_t)std::min<int64_t>(bx1 + 2, width), ry1 = (int32_t)std::min<int64_t>(by1 + 2, height);
	if (rx1 <= v.rx0 || ry1 <= v.ry0 || m->count == 0) return false;
	v.rw = rx1 - v.rx0;
	v.rh = ry1 - v.ry0;
	return true;
}

// Draws the instances as consecutive renderDenseModel calls would, in two launches: keys of every
// instance's triangles over the union of their bounds, then one resolve over that union.
int dense_draw(dsrg_context ctx, const dsrg_dense_instance *instances, int32_t count, const dsrg_ortho_view *view, const dsrg_image *height,
               const dsrg_image *diffuse, const dsrg_image *normal, int32_t highQuality, const char *name) {
	if (!ctx || !view || count < 0 || (count > 0 && !instances)) return DSRG_ERROR_INVALID_ARGUMENT;
	if (!dense_image(height) || !dense_image(diffuse) || !dense_image(normal) || height->width != diffuse->width ||
	    height->height != diffuse->height || height->width != normal->width || height->height != normal->height)
		return fail(ctx, DSRG_ERROR_INVALID_ARGUMENT, std::string(name) + ": height, diffuse and normal must be device images of one size");
	std::vector<DenseInstance> table;
	table.reserve((size_t)count);
	uint64_t total = 0;
	int32_t kx0 = 0, ky0 = 0, kx1 = 0, ky1 = 0;
	for (int32_t i = 0; i < count; i++) {
		const dsrg_dense_instance &in = instances[i];
		if (!in.model || in.model->context != ctx) return fail(ctx, DSRG_ERROR_INVALID_ARGUMENT, std::string(name) + ": invalid model");
		DenseInstance d;
		if (!dense_view(in.model, view, height->width, height->height, in.originX, in.originY, in.modelToWorld, highQuality, d.v)) continue;
		d.triangles = in.model->triangles.ptr;
		d.first = (uint32_t)total;
		d.count = (uint32_t)in.model->count;
		total += (uint64_t)in.model->count;
		if (total >= 0xFFFFFFFFull) return fail(ctx, DSRG_ERROR_UNSUPPORTED, std::string(name) + ": more than 2^32 - 1 triangles in one call");
		if (table.empty()) { kx0 = d.v.rx0; ky0 = d.v.ry0; kx1 = d.v.rx0 + d.v.rw; ky1 = d.v.ry0 + d.v.rh; }
		kx0 = std::min(kx0, d.v.rx0); ky0 = std::min(ky0, d.v.ry0);
		kx1 = std::max(kx1, d.v.rx0 + d.v.rw); ky1 = std::max(ky1, d.v.ry0 + d.v.rh);
		table.push_back(d);
	}
	if (table.empty()) return DSRG_OK;
	const int32_t kw = kx1 - kx0, kh = ky1 - ky0;
	cudaSetDevice(ctx->device);
	const size_t tableBytes = table.size() * sizeof(DenseInstance);
	DSRG_CUDA_TRY(ctx, ctx->denseInstances.reserve(tableBytes));
	DSRG_CUDA_TRY(ctx, cudaMemcpyAsync(ctx->denseInstances.ptr, table.data(), tableBytes, cudaMemcpyHostToDevice, ctx->stream));
	const DenseInstance *deviceTable = reinterpret_cast<const DenseInstance *>(ctx->denseInstances.ptr);
	DSRG_CUDA_TRY(ctx, ctx->denseKeys.reserve((size_t)kw * kh));
	DSRG_CUDA_TRY(ctx, cudaMemsetAsync(ctx->denseKeys.ptr, 0, (size_t)kw * kh * sizeof(unsigned long long), ctx->stream));
	const uint64_t blocks64 = (total + 127) / 128;
	const int blocks = (int)std::min<uint64_t>(blocks64, (uint64_t)sm_count() * 64);
	dense_keys_kernel<<<blocks, 128, 0, ctx->stream>>>(deviceTable, (uint32_t)table.size(), (uint32_t)total,
	                                                   (const float *)height->data, height->strideBytes / 4, kx0, ky0, kw,
	                                                   ctx->denseKeys.ptr);
	const dim3 grid((kw + 127) / 128, kh);
	dense_resolve_kernel<<<grid, 128, 0, ctx->stream>>>(deviceTable, (uint32_t)table.size(), (float *)height->data,
	                                                    height->strideBytes / 4, (uint32_t *)diffuse->data, diffuse->strideBytes / 4,
	                                                    (uint32_t *)normal->data, normal->strideBytes / 4, kx0, ky0, kw,
	                                                    ctx->denseKeys.ptr);
	add_launches(2);
	DSRG_CUDA_TRY(ctx, cudaGetLastError());
	// the table's copy reads the host vector: wait before it goes
	DSRG_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
	return DSRG_OK;
}

} // namespace

extern "C" {

int dsrg_dense_render(dsrg_context ctx, dsrg_dense_model m, const dsrg_ortho_view *view, const dsrg_image *height,
                      const dsrg_image *diffuse, const dsrg_image *normal, float originX, float originY, const float *modelToWorld,
                      int32_t highQuality) {
	if (!ctx || !m || !view || !modelToWorld) return DSRG_ERROR_INVALID_ARGUMENT;
	dsrg_dense_instance instance;
	instance.model = m;
	instance.originX = originX;
	instance.originY = originY;
	memcpy(instance.modelToWorld, modelToWorld, sizeof(instance.modelToWorld));
	return dense_draw(ctx, &instance, 1, view, height, diffuse, normal, highQuality, "dsrg_dense_render");
}

int dsrg_dense_render_many(dsrg_context ctx, const dsrg_dense_instance *instances, int32_t count, const dsrg_ortho_view *view,
                           const dsrg_image *height, const dsrg_image *diffuse, const dsrg_image *normal, int32_t highQuality) {
	return dense_draw(ctx, instances, count, view, height, diffuse, normal, highQuality, "dsrg_dense_render_many");
}

} // extern "C"
