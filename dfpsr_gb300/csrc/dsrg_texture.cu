// Texture creation on the GPU: texture_create_RgbaU8(image, resolutions) (api/textureAPI.cpp:89-131)
// for any number of images at once.  The image is resized linearly to the next powers of two
// (filter_resize with Sampler::Linear, api/filterAPI.cpp:66-311, 852-859) straight into level 0 of
// the pyramid, and the pyramid is the integer 2x2 box average of texture_generatePyramid
// (textureAPI.cpp:44-87).  All textures of a call share each phase's launch: one for the
// horizontal half of two-step upscales, one for level 0, one per pyramid level; a work item is
// one texel of one texture, found by a binary search over the call's texel prefix sums.
#include <cuda_runtime.h>

#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "dsrg_internal.h"
#include "dsrg_shade.h"

using namespace dsrg;

namespace {

// One image-to-image resize (or copy) of one texture.
struct ResizeItem {
	const uint32_t *src;
	uint32_t *dst;
	int32_t srcStride, dstStride; // in texels
	int32_t srcWidth, srcHeight, width, height;
	int32_t mode;                 // RESIZE_*
	int32_t srcOrder;             // pack order of the source (the target is RGBA)
	uint32_t first;               // first work item (target texel) of this resize in the launch
};

// One pyramid level of one texture.
struct LevelItem {
	uint32_t *pixels;
	uint32_t srcOffset, dstOffset; // texel offsets of the source and target levels
	int32_t log2Width, log2Height; // of the target level
	uint32_t first;
};

enum ResizeMode { RESIZE_COPY = 0, RESIZE_VERTICAL = 1, RESIZE_HORIZONTAL = 2, RESIZE_BOTH = 3 };

// resize_optimized's choice for one step (filterAPI.cpp:157-260).
int resize_mode(int32_t srcWidth, int32_t srcHeight, int32_t width, int32_t height) {
	if (srcWidth == width && srcHeight == height) return RESIZE_COPY;
	if (srcWidth == width) return RESIZE_VERTICAL;
	if (srcHeight == height) return RESIZE_HORIZONTAL;
	return RESIZE_BOTH;
}

template <typename Item>
__device__ __forceinline__ int32_t find_item(const Item *items, int32_t count, uint32_t i) {
	int32_t lo = 0, hi = count - 1;
	while (lo < hi) {
		const int32_t mid = (lo + hi + 1) >> 1;
		if (items[mid].first <= i) lo = mid; else hi = mid - 1;
	}
	return lo;
}

__device__ __forceinline__ uint32_t read_clamped(const ResizeItem &r, int32_t x, int32_t y) { // image_readPixel_clamp
	x = x < 0 ? 0 : (x > r.srcWidth - 1 ? r.srcWidth - 1 : x);
	y = y < 0 ? 0 : (y > r.srcHeight - 1 ? r.srcHeight - 1 : y);
	return r.src[(size_t)y * r.srcStride + x];
}

__device__ __forceinline__ uint32_t channel(uint32_t c, int ch) { return (c >> (ch * 8)) & 0xFFu; }

// Channel ch (0 red .. 3 alpha) of a pixel packed in the given order (image_unpack).
__device__ __forceinline__ uint32_t channel_of(uint32_t c, int32_t order, int ch) { return (c >> pack_shift(order, ch)) & 0xFFu; }

// The 16.16 sampling position of target index i: start = offset / 2 - 32768 (Sampler::Linear),
// advanced by offset = 65536 * source / target per target pixel, clamped at 0.
__device__ __forceinline__ uint32_t sample_position(int32_t source, int32_t target, int32_t i) {
	const int32_t offset = (int32_t)((65536u * (uint32_t)source) / (uint32_t)target);
	const int32_t p = (int32_t)((uint32_t)(offset / 2) - 32768u + (uint32_t)i * (uint32_t)offset);
	return (uint32_t)(p < 0 ? 0 : p);
}

__global__ void resize_kernel(const ResizeItem *__restrict__ items, int32_t count, uint32_t total) {
	for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
		const ResizeItem r = items[find_item(items, count, i)];
		const uint32_t local = i - r.first;
		const int32_t x = (int32_t)(local % (uint32_t)r.width), y = (int32_t)(local / (uint32_t)r.width);
		uint32_t out = 0;
		if (r.mode == RESIZE_COPY) {
			// draw_copy, repacking another order channel by channel (imageImpl_drawCopy, drawAPI.cpp:498-520)
			const uint32_t c = r.src[(size_t)y * r.srcStride + x];
			for (int ch = 0; ch < 4; ch++) out |= channel_of(c, r.srcOrder, ch) << (ch * 8);
		} else if (r.mode == RESIZE_VERTICAL) {
			// mixColorsUniform with an 8-bit weight (the aligned branch of resize_optimized), on the
			// packed bytes as they lie: a source of another order keeps its byte order here
			const uint32_t sampleY = sample_position(r.srcHeight, r.height, y);
			uint32_t upperY = sampleY >> 16, lowerY = upperY + 1;
			if (upperY >= (uint32_t)r.srcHeight) upperY = (uint32_t)r.srcHeight - 1;
			if (lowerY >= (uint32_t)r.srcHeight) lowerY = (uint32_t)r.srcHeight - 1;
			const uint32_t ratio = (sampleY & 0xFFFFu) >> 8, inv = 256u - ratio;
			const uint32_t a = r.src[(size_t)upperY * r.srcStride + x], b = r.src[(size_t)lowerY * r.srcStride + x];
			for (int ch = 0; ch < 4; ch++) out |= ((channel(a, ch) * inv + channel(b, ch) * ratio) >> 8) << (ch * 8);
		} else if (r.mode == RESIZE_HORIZONTAL) {
			const uint32_t sampleX = sample_position(r.srcWidth, r.width, x);
			const uint32_t leftX = sampleX >> 16, rightRatio = sampleX & 0xFFFFu, leftRatio = 65536u - rightRatio;
			const uint32_t a = read_clamped(r, (int32_t)leftX, y), b = read_clamped(r, (int32_t)(leftX + 1), y);
			for (int ch = 0; ch < 4; ch++) {
				const uint32_t v = (channel_of(a, r.srcOrder, ch) * leftRatio + channel_of(b, r.srcOrder, ch) * rightRatio) >> 16;
				out |= (v > 255u ? 255u : v) << (ch * 8);
			}
		} else {
			// resize_reference with samplePixel<true>: bilinear, 16-bit weights
			const uint32_t sampleX = sample_position(r.srcWidth, r.width, x), sampleY = sample_position(r.srcHeight, r.height, y);
			const uint32_t leftX = sampleX >> 16, rightRatio = sampleX & 0xFFFFu, leftRatio = 65536u - rightRatio;
			const uint32_t upperY = sampleY >> 16, lowerRatio = sampleY & 0xFFFFu, upperRatio = 65536u - lowerRatio;
			const uint32_t ul = read_clamped(r, (int32_t)leftX, (int32_t)upperY), ur = read_clamped(r, (int32_t)(leftX + 1), (int32_t)upperY);
			const uint32_t ll = read_clamped(r, (int32_t)leftX, (int32_t)(upperY + 1));
			const uint32_t lr = read_clamped(r, (int32_t)(leftX + 1), (int32_t)(upperY + 1));
			for (int ch = 0; ch < 4; ch++) {
				const uint32_t upper = (channel_of(ul, r.srcOrder, ch) * leftRatio + channel_of(ur, r.srcOrder, ch) * rightRatio) >> 16;
				const uint32_t lower = (channel_of(ll, r.srcOrder, ch) * leftRatio + channel_of(lr, r.srcOrder, ch) * rightRatio) >> 16;
				const uint32_t v = (upper * upperRatio + lower * lowerRatio) >> 16;
				out |= (v > 255u ? 255u : v) << (ch * 8);
			}
		}
		r.dst[(size_t)y * r.dstStride + x] = out;
	}
}

// downsample (textureAPI.cpp:44-61): each channel the truncated mean of a 2x2 block of the level above.
__global__ void pyramid_kernel(const LevelItem *__restrict__ items, int32_t count, uint32_t total) {
	for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
		const LevelItem l = items[find_item(items, count, i)];
		const uint32_t local = i - l.first;
		const uint32_t x = local & ((1u << l.log2Width) - 1u), y = local >> l.log2Width;
		const uint32_t srcWidth = 2u << l.log2Width;
		const uint32_t *src = l.pixels + l.srcOffset + (size_t)(2u * y) * srcWidth + 2u * x;
		const uint2 upper = make_uint2(src[0], src[1]);
		const uint2 lower = make_uint2(src[srcWidth], src[srcWidth + 1]);
		uint32_t out = 0;
		for (int ch = 0; ch < 4; ch++)
			out |= ((channel(upper.x, ch) + channel(upper.y, ch) + channel(lower.x, ch) + channel(lower.y, ch)) / 4u) << (ch * 8);
		l.pixels[l.dstOffset + local] = out;
	}
}

int launch_grid(uint64_t n) {
	uint64_t blocks = (n + 255) / 256;
	const uint64_t cap = (uint64_t)sm_count() * 8;
	return (int)(blocks < cap ? (blocks > 0 ? blocks : 1) : cap);
}

// findLog2Size (textureAPI.cpp:30-40).
uint32_t find_log2_size(uint32_t size) {
	for (uint32_t l = 0; l < 15u; l++) if ((1u << l) >= size) return l;
	return 15u;
}

struct Plan {
	uint32_t lw, lh, maxMip, pixelCount, startOffset, highest;
	int32_t width, height;       // of level 0
	bool twoStep;
	size_t stagingOffset, tempOffset;
};

uint32_t layer_offset(const Plan &p, uint32_t mip) { return p.startOffset & ((p.highest - 1u) >> (mip << 1)); } // texture_getPixelOffsetToLayer

} // namespace

extern "C" {

int dsrg_texture_create_many(dsrg_context ctx, int32_t count, const dsrg_image *images, const int32_t *resolutions,
                             dsrg_texture *out) {
	if (!ctx || count < 0 || (count > 0 && (!images || !resolutions || !out))) return DSRG_ERROR_INVALID_ARGUMENT;
	for (int32_t i = 0; i < count; i++) out[i] = nullptr;
	std::vector<Plan> plans((size_t)count);
	size_t stagingTexels = 0, tempTexels = 0;
	for (int32_t i = 0; i < count; i++) {
		const dsrg_image &im = images[i];
		if (resolutions[i] < 1) return fail(ctx, DSRG_ERROR_INVALID_ARGUMENT, "Tried to create a texture without any resolutions stored, which would be empty!");
		if (im.width < 1 || im.height < 1 || !im.data)
			return fail(ctx, DSRG_ERROR_INVALID_ARGUMENT, "Tried to create a texture of an empty image!");
		if (im.width > 32768 || im.height > 32768)
			return fail(ctx, DSRG_ERROR_INVALID_ARGUMENT, "Tried to create a texture exceeding the maximum texture dimensions of 32768 x 32768 pixels!");
		if (im.packOrder < 0 || im.packOrder > 3) return fail(ctx, DSRG_ERROR_INVALID_ARGUMENT, "texture image: unknown pack order");
		if (im.strideBytes < im.width * 4 || (im.strideBytes & 3)) return fail(ctx, DSRG_ERROR_INVALID_ARGUMENT, "texture image: invalid stride");
		Plan &p = plans[i];
		p.lw = find_log2_size((uint32_t)im.width);
		p.lh = find_log2_size((uint32_t)im.height);
		// Texture constructor (implementation/image/Texture.h:66-101)
		p.maxMip = (uint32_t)(resolutions[i] - 1);
		if (p.maxMip > p.lw) p.maxMip = p.lw;
		if (p.maxMip > p.lh) p.maxMip = p.lh;
		if (p.maxMip > 15u) p.maxMip = 15u;
		p.highest = 1u << (p.lw + p.lh);
		uint64_t pixelCount = 0;
		uint32_t levelCount = p.highest;
		for (int32_t level = (int32_t)p.maxMip; level >= 0; level--) { pixelCount |= levelCount; levelCount >>= 2; }
		p.pixelCount = (uint32_t)pixelCount;
		p.startOffset = (uint32_t)pixelCount & ~p.highest;
		p.width = 1 << p.lw;
		p.height = 1 << p.lh;
		// resizeToTarget (filterAPI.cpp:298-314): wider and taller targets go through a horizontal step first
		p.twoStep = p.width != im.width && p.height > im.height;
		p.stagingOffset = stagingTexels;
		if (!im.onDevice) stagingTexels += (size_t)im.width * im.height;
		p.tempOffset = tempTexels;
		if (p.twoStep) tempTexels += (size_t)p.width * im.height;
	}
	if (count == 0) return DSRG_OK;
	cudaSetDevice(ctx->device);
	cudaStream_t stream = ctx->stream;
	std::vector<dsrg_texture> made;
	auto cleanup = [&](int status, const std::string &message) {
		cudaStreamSynchronize(stream);
		for (dsrg_texture t : made) { cudaFree(t->pixels); delete t; }
		for (int32_t i = 0; i < count; i++) out[i] = nullptr;
		return fail(ctx, status, message);
	};
	for (int32_t i = 0; i < count; i++) {
		dsrg_texture tex = new (std::nothrow) dsrg_texture_s();
		if (!tex) return cleanup(DSRG_ERROR_OUT_OF_MEMORY, "texture allocation failed");
		tex->context = ctx;
		made.push_back(tex);
		const Plan &p = plans[i];
		if (device_alloc((void **)&tex->pixels, sizeof(uint32_t) * p.pixelCount) != cudaSuccess)
			return cleanup(DSRG_ERROR_OUT_OF_MEMORY, "cudaMalloc failed for a texture pyramid");
		tex->pixelCount = p.pixelCount;
		const uint32_t f[9] = {p.lw, p.lh, p.maxMip, p.startOffset, p.highest - 1, (1u << (p.lw - p.maxMip)) - 1,
		                       (1u << (p.lh - p.maxMip)) - 1, (1u << p.lw) - 1, (1u << p.lh) - 1};
		memcpy(tex->fields, f, sizeof(f));
		TextureData &d = tex->data;
		memset(&d, 0, sizeof(d));
		d.pixels = tex->pixels;
		d.log2width = p.lw; d.log2height = p.lh; d.maxMipLevel = p.maxMip; d.startOffset = p.startOffset;
		d.maxLevelMask = p.highest - 1;
		d.maxWidthAndMask = (1u << p.lw) - 1; d.maxHeightAndMask = (1u << p.lh) - 1;
		d.floatMaxWidth = (float)(1u << p.lw); d.floatMaxHeight = (float)(1u << p.lh);
		d.exists = 1;
	}
	if (ctx->textureStaging.reserve(stagingTexels + tempTexels + 1) != cudaSuccess)
		return cleanup(DSRG_ERROR_OUT_OF_MEMORY, "texture staging allocation failed");
	uint32_t *staging = ctx->textureStaging.ptr, *temp = ctx->textureStaging.ptr + stagingTexels;
	// sources: host images are copied in, device images read where they are
	std::vector<const uint32_t *> source((size_t)count);
	std::vector<int32_t> sourceStride((size_t)count);
	for (int32_t i = 0; i < count; i++) {
		const dsrg_image &im = images[i];
		if (im.onDevice) {
			source[i] = (const uint32_t *)im.data;
			sourceStride[i] = im.strideBytes / 4;
		} else {
			uint32_t *dst = staging + plans[i].stagingOffset;
			if (cudaMemcpy2DAsync(dst, (size_t)im.width * 4, im.data, (size_t)im.strideBytes, (size_t)im.width * 4, (size_t)im.height,
			                      cudaMemcpyHostToDevice, stream) != cudaSuccess)
				return cleanup(DSRG_ERROR_CUDA, "texture upload failed");
			source[i] = dst;
			sourceStride[i] = im.width;
		}
	}
	// work tables: the horizontal steps, level 0, then every pyramid level
	std::vector<ResizeItem> horizontal, level0;
	uint32_t horizontalTotal = 0, level0Total = 0;
	uint32_t maxMip = 0;
	for (int32_t i = 0; i < count; i++) {
		const dsrg_image &im = images[i];
		const Plan &p = plans[i];
		uint32_t *level0Pixels = made[i]->pixels + layer_offset(p, 0);
		ResizeItem last;
		memset(&last, 0, sizeof(last));
		if (p.twoStep) {
			ResizeItem h;
			memset(&h, 0, sizeof(h));
			h.src = source[i]; h.srcStride = sourceStride[i]; h.srcWidth = im.width; h.srcHeight = im.height;
			h.dst = temp + p.tempOffset; h.dstStride = p.width; h.width = p.width; h.height = im.height;
			h.mode = resize_mode(im.width, im.height, p.width, im.height);
			h.srcOrder = im.packOrder;
			h.first = horizontalTotal;
			horizontalTotal += (uint32_t)(p.width * im.height);
			horizontal.push_back(h);
			last.src = h.dst; last.srcStride = p.width; last.srcWidth = p.width; last.srcHeight = im.height;
		} else {
			last.src = source[i]; last.srcStride = sourceStride[i]; last.srcWidth = im.width; last.srcHeight = im.height;
			last.srcOrder = im.packOrder; // a two-step upscale's second step reads the RGBA half (srcOrder 0)
		}
		last.dst = level0Pixels; last.dstStride = p.width; last.width = p.width; last.height = p.height;
		last.mode = resize_mode(last.srcWidth, last.srcHeight, p.width, p.height);
		last.first = level0Total;
		level0Total += (uint32_t)(p.width * p.height);
		level0.push_back(last);
		if (p.maxMip > maxMip) maxMip = p.maxMip;
	}
	std::vector<std::vector<LevelItem>> levels(maxMip + 1);
	std::vector<uint32_t> levelTotal(maxMip + 1, 0u);
	for (uint32_t level = 1; level <= maxMip; level++) {
		for (int32_t i = 0; i < count; i++) {
			const Plan &p = plans[i];
			if (p.maxMip < level) continue;
			LevelItem l;
			l.pixels = made[i]->pixels;
			l.srcOffset = layer_offset(p, level - 1);
			l.dstOffset = layer_offset(p, level);
			l.log2Width = (int32_t)(p.lw - level);
			l.log2Height = (int32_t)(p.lh - level);
			l.first = levelTotal[level];
			levelTotal[level] += 1u << (p.lw + p.lh - 2 * level);
			levels[level].push_back(l);
		}
	}
	// one table upload for the whole call
	std::vector<unsigned char> table;
	auto append = [&](const void *data, size_t bytes) {
		const size_t at = (table.size() + 15) & ~(size_t)15;
		table.resize(at + bytes);
		if (bytes) memcpy(table.data() + at, data, bytes);
		return at;
	};
	const size_t horizontalAt = append(horizontal.data(), horizontal.size() * sizeof(ResizeItem));
	const size_t level0At = append(level0.data(), level0.size() * sizeof(ResizeItem));
	std::vector<size_t> levelAt(maxMip + 1, 0);
	for (uint32_t level = 1; level <= maxMip; level++) levelAt[level] = append(levels[level].data(), levels[level].size() * sizeof(LevelItem));
	if (ctx->textureTables.reserve(table.size() + 16) != cudaSuccess) return cleanup(DSRG_ERROR_OUT_OF_MEMORY, "texture table allocation failed");
	unsigned char *tables = ctx->textureTables.ptr;
	if (cudaMemcpyAsync(tables, table.data(), table.size(), cudaMemcpyHostToDevice, stream) != cudaSuccess)
		return cleanup(DSRG_ERROR_CUDA, "texture table upload failed");
	if (!horizontal.empty()) {
		resize_kernel<<<launch_grid(horizontalTotal), 256, 0, stream>>>((const ResizeItem *)(tables + horizontalAt),
		                                                               (int32_t)horizontal.size(), horizontalTotal);
		add_launches(1);
	}
	resize_kernel<<<launch_grid(level0Total), 256, 0, stream>>>((const ResizeItem *)(tables + level0At), (int32_t)level0.size(),
	                                                           level0Total);
	add_launches(1);
	for (uint32_t level = 1; level <= maxMip; level++) {
		pyramid_kernel<<<launch_grid(levelTotal[level]), 256, 0, stream>>>((const LevelItem *)(tables + levelAt[level]),
		                                                                  (int32_t)levels[level].size(), levelTotal[level]);
		add_launches(1);
	}
	// the host tables and images may be reused by the caller, and a failure shows here
	const cudaError_t e = cudaStreamSynchronize(stream);
	if (e != cudaSuccess || cudaGetLastError() != cudaSuccess) return cleanup(DSRG_ERROR_CUDA, std::string("texture creation: ") + cudaGetErrorString(e));
	for (int32_t i = 0; i < count; i++) out[i] = made[i];
	return DSRG_OK;
}

int dsrg_texture_create(dsrg_context ctx, const uint32_t *pixels, int32_t width, int32_t height, int32_t resolutions,
                        dsrg_texture *out) {
	if (!ctx || !out) return DSRG_ERROR_INVALID_ARGUMENT;
	*out = nullptr;
	dsrg_image image;
	image.data = (void *)pixels;
	image.width = width;
	image.height = height;
	image.strideBytes = width * 4;
	image.packOrder = 0;
	image.onDevice = 0;
	return dsrg_texture_create_many(ctx, 1, &image, &resolutions, out);
}

int dsrg_texture_upload(dsrg_context ctx, const uint32_t *pyramid, uint32_t log2width, uint32_t log2height, uint32_t maxMipLevel,
                        dsrg_texture *out) {
	if (!ctx || !out || !pyramid) return DSRG_ERROR_INVALID_ARGUMENT;
	*out = nullptr;
	// the fields of the Texture constructor (implementation/image/Texture.h:66-101)
	if (log2width > 15u || log2height > 15u || maxMipLevel > log2width || maxMipLevel > log2height || maxMipLevel > 15u)
		return fail(ctx, DSRG_ERROR_INVALID_ARGUMENT, "dsrg_texture_upload: invalid pyramid dimensions");
	Plan p;
	memset(&p, 0, sizeof(p));
	p.lw = log2width; p.lh = log2height; p.maxMip = maxMipLevel;
	p.highest = 1u << (p.lw + p.lh);
	uint64_t pixelCount = 0;
	uint32_t levelCount = p.highest;
	for (int32_t level = (int32_t)p.maxMip; level >= 0; level--) { pixelCount |= levelCount; levelCount >>= 2; }
	p.pixelCount = (uint32_t)pixelCount;
	p.startOffset = (uint32_t)pixelCount & ~p.highest;
	cudaSetDevice(ctx->device);
	dsrg_texture tex = new (std::nothrow) dsrg_texture_s();
	if (!tex) return fail(ctx, DSRG_ERROR_OUT_OF_MEMORY, "texture allocation failed");
	tex->context = ctx;
	if (device_alloc((void **)&tex->pixels, sizeof(uint32_t) * p.pixelCount) != cudaSuccess) {
		delete tex;
		return fail(ctx, DSRG_ERROR_OUT_OF_MEMORY, "cudaMalloc failed for a texture pyramid");
	}
	tex->pixelCount = p.pixelCount;
	const uint32_t f[9] = {p.lw, p.lh, p.maxMip, p.startOffset, p.highest - 1, (1u << (p.lw - p.maxMip)) - 1,
	                       (1u << (p.lh - p.maxMip)) - 1, (1u << p.lw) - 1, (1u << p.lh) - 1};
	memcpy(tex->fields, f, sizeof(f));
	TextureData &d = tex->data;
	memset(&d, 0, sizeof(d));
	d.pixels = tex->pixels;
	d.log2width = p.lw; d.log2height = p.lh; d.maxMipLevel = p.maxMip; d.startOffset = p.startOffset;
	d.maxLevelMask = p.highest - 1;
	d.maxWidthAndMask = (1u << p.lw) - 1; d.maxHeightAndMask = (1u << p.lh) - 1;
	d.floatMaxWidth = (float)(1u << p.lw); d.floatMaxHeight = (float)(1u << p.lh);
	d.exists = 1;
	const cudaError_t e1 = cudaMemcpyAsync(tex->pixels, pyramid, sizeof(uint32_t) * p.pixelCount, cudaMemcpyHostToDevice, ctx->stream);
	const cudaError_t e2 = cudaStreamSynchronize(ctx->stream);
	if (e1 != cudaSuccess || e2 != cudaSuccess) {
		cudaFree(tex->pixels);
		delete tex;
		return fail(ctx, DSRG_ERROR_CUDA, std::string("dsrg_texture_upload: ") + cudaGetErrorString(e1 != cudaSuccess ? e1 : e2));
	}
	*out = tex;
	return DSRG_OK;
}

int dsrg_texture_destroy(dsrg_texture tex) {
	if (!tex) return DSRG_ERROR_INVALID_ARGUMENT;
	cudaSetDevice(tex->context->device);
	cudaStreamSynchronize(tex->context->stream);
	cudaFree(tex->pixels);
	delete tex;
	return DSRG_OK;
}

int dsrg_texture_read(dsrg_texture tex, uint32_t *pixels, int32_t maxPixels, uint32_t *fields, int32_t *count) {
	if (!tex) return DSRG_ERROR_INVALID_ARGUMENT;
	if (fields) memcpy(fields, tex->fields, sizeof(tex->fields));
	if (count) *count = (int32_t)tex->pixelCount;
	if (pixels && maxPixels > 0) {
		const size_t n = (size_t)maxPixels < tex->pixelCount ? (size_t)maxPixels : tex->pixelCount;
		dsrg_context ctx = tex->context;
		DSRG_CUDA_TRY(ctx, cudaMemcpyAsync(pixels, tex->pixels, n * sizeof(uint32_t), cudaMemcpyDeviceToHost, ctx->stream));
		DSRG_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
	}
	return DSRG_OK;
}

} // extern "C"
