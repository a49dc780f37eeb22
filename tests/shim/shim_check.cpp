// Drives the dsr::gpu shim with the reference's own objects and compares every result with the
// reference's own renderer on the same objects.  Test infrastructure: linked with the reference's
// library and either libdsrg.so or its oracle-backed test double (oracle_dsrg.cpp).
//
//   shim_check compare   every case below, byte for byte; exit status 0 when all are equal
//   shim_check context   one dsr::gpu call; prints what it threw (for a machine without a GPU)
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <stdexcept>
#include <string>

#include "DFPSR/includeFramework.h"
#include "dsr_gpu.h"

using namespace dsr;

namespace {

uint64_t g_state = 0x9E3779B97F4A7C15ull;
uint32_t next_u32() { // xorshift64*
	g_state ^= g_state >> 12;
	g_state ^= g_state << 25;
	g_state ^= g_state >> 27;
	return (uint32_t)((g_state * 0x2545F4914F6CDD1Dull) >> 32);
}
float uniform(float lo, float hi) { return lo + (hi - lo) * (float)(next_u32() >> 8) * (1.0f / 16777216.0f); }

TextureRgbaU8 noiseTexture(int32_t width, int32_t height, int32_t resolutions) {
	OrderedImageRgbaU8 image = image_create_RgbaU8(width, height);
	for (int32_t y = 0; y < height; y++) {
		uint32_t *row = image_getSafePointer<uint32_t>(image, y).getUnsafe();
		for (int32_t x = 0; x < width; x++) row[x] = next_u32();
	}
	return texture_create_RgbaU8(image, resolutions);
}

// count random triangles with vertices in [-1, 1]^3, random colours and texture coordinates, in one part.
void addRandomTriangles(Model &model, int32_t part, int32_t count, bool quads) {
	for (int32_t i = 0; i < count; i++) {
		const int32_t corners = quads ? 4 : 3;
		int32_t points[4];
		for (int32_t k = 0; k < corners; k++)
			points[k] = model_addPoint(model, FVector3D(uniform(-1.0f, 1.0f), uniform(-1.0f, 1.0f), uniform(-1.0f, 1.0f)));
		const int32_t polygon = quads ? model_addQuad(model, part, points[0], points[1], points[2], points[3])
		                              : model_addTriangle(model, part, points[0], points[1], points[2]);
		for (int32_t k = 0; k < corners; k++) {
			model_setTexCoord(model, part, polygon, k, FVector4D(uniform(0.0f, 1.0f), uniform(0.0f, 1.0f), uniform(0.0f, 1.0f), uniform(0.0f, 1.0f)));
			model_setVertexColor(model, part, polygon, k, FVector4D(uniform(0.0f, 1.0f), uniform(0.0f, 1.0f), uniform(0.0f, 1.0f), uniform(0.3f, 1.0f)));
		}
	}
}

Camera frontCamera(int32_t width, int32_t height, float x = 0.0f) {
	return Camera::createPerspective(Transform3D(FVector3D(x, 0.0f, -3.0f), FMatrix3x3()), (float)width, (float)height,
	                                 std::tan(30.0f * 3.14159265f / 180.0f));
}

bool sameImages(const ImageRgbaU8 &a, const ImageRgbaU8 &b) {
	if (image_exists(a) != image_exists(b)) return false;
	if (!image_exists(a)) return true;
	for (int32_t y = 0; y < image_getHeight(a); y++)
		if (std::memcmp(image_getSafePointer<uint32_t>(a, y).getUnsafe(), image_getSafePointer<uint32_t>(b, y).getUnsafe(),
		                sizeof(uint32_t) * image_getWidth(a)) != 0)
			return false;
	return true;
}
bool sameImages(const ImageF32 &a, const ImageF32 &b) {
	if (image_exists(a) != image_exists(b)) return false;
	if (!image_exists(a)) return true;
	for (int32_t y = 0; y < image_getHeight(a); y++)
		if (std::memcmp(image_getSafePointer<float>(a, y).getUnsafe(), image_getSafePointer<float>(b, y).getUnsafe(),
		                sizeof(float) * image_getWidth(a)) != 0)
			return false;
	return true;
}

ImageRgbaU8 colorTarget(int32_t width, int32_t height, PackOrderIndex order, uint32_t fill) {
	AlignedImageRgbaU8 image = image_create_RgbaU8_native(width, height, order);
	for (int32_t y = 0; y < height; y++) {
		uint32_t *row = image_getSafePointer<uint32_t>(image, y).getUnsafe();
		for (int32_t x = 0; x < width; x++) row[x] = fill ? (next_u32() | 0xFF000000u) : 0u;
	}
	return image;
}
ImageF32 depthTarget(int32_t width, int32_t height, bool prefill) {
	AlignedImageF32 image = image_create_F32(width, height);
	for (int32_t y = 0; y < height; y++) {
		float *row = image_getSafePointer<float>(image, y).getUnsafe();
		for (int32_t x = 0; x < width; x++) row[x] = prefill ? uniform(0.0f, 0.3f) : 0.0f;
	}
	return image;
}
ImageRgbaU8 copyOf(const ImageRgbaU8 &image) {
	if (!image_exists(image)) return ImageRgbaU8();
	ImageRgbaU8 out = image_create_RgbaU8_native(image_getWidth(image), image_getHeight(image), image_getPackOrderIndex(image));
	for (int32_t y = 0; y < image_getHeight(image); y++)
		std::memcpy(image_getSafePointer<uint32_t>(out, y).getUnsafe(), image_getSafePointer<uint32_t>(image, y).getUnsafe(),
		            sizeof(uint32_t) * image_getWidth(image));
	return out;
}
ImageF32 copyOf(const ImageF32 &image) {
	if (!image_exists(image)) return ImageF32();
	ImageF32 out = image_create_F32(image_getWidth(image), image_getHeight(image));
	for (int32_t y = 0; y < image_getHeight(image); y++)
		std::memcpy(image_getSafePointer<float>(out, y).getUnsafe(), image_getSafePointer<float>(image, y).getUnsafe(),
		            sizeof(float) * image_getWidth(image));
	return out;
}

int g_failures = 0;
void report(const char *name, bool colorSame, bool depthSame) {
	std::printf("%s: colour %s, depth %s\n", name, colorSame ? "equal" : "DIFFERS", depthSame ? "equal" : "DIFFERS");
	if (!colorSame || !depthSame) g_failures++;
}

// model_render through the reference and through dsr::gpu on copies of the same targets.
void compareModelRender(const char *name, const Model &model, const Camera &camera, ImageRgbaU8 color, ImageF32 depth,
                        const Transform3D &transform = Transform3D()) {
	ImageRgbaU8 refColor = copyOf(color), gpuColor = copyOf(color);
	ImageF32 refDepth = copyOf(depth), gpuDepth = copyOf(depth);
	dsr::model_render(model, transform, refColor, refDepth, camera);
	gpu::model_render(model, transform, gpuColor, gpuDepth, camera);
	report(name, sameImages(refColor, gpuColor), sameImages(refDepth, gpuDepth));
}

int compare() {
	const int32_t W = 800, H = 600;
	TextureRgbaU8 noise = noiseTexture(256, 256, 16), lightMap = noiseTexture(64, 32, 4), small = noiseTexture(100, 60, 16);
	// 1. the 800x600 configuration: 20,000 random triangles, a 256x256 mip-mapped texture
	Model c0 = model_create();
	const int32_t part0 = model_addEmptyPart(c0, U"triangles");
	model_setDiffuseMap(c0, part0, noise);
	addRandomTriangles(c0, part0, 20000, false);
	compareModelRender("model_render 800x600 20k", c0, frontCamera(W, H), colorTarget(W, H, PackOrderIndex::RGBA, 0), depthTarget(W, H, false));
	// 2. BGRA and ARGB targets of odd size, prefilled, depth-only and colour-only targets
	compareModelRender("model_render BGRA 199x151 prefilled", c0, frontCamera(199, 151), colorTarget(199, 151, PackOrderIndex::BGRA, 1),
	                   depthTarget(199, 151, true));
	compareModelRender("model_render ARGB colour only", c0, frontCamera(203, 77), colorTarget(203, 77, PackOrderIndex::ARGB, 1), ImageF32());
	compareModelRender("model_render depth only", c0, frontCamera(203, 77), ImageRgbaU8(), depthTarget(203, 77, true));
	// 3. two parts (triangles with a diffuse map, quads with diffuse and light maps), moved by a transform
	Model parts = model_create();
	const int32_t a = model_addEmptyPart(parts, U"a"), b = model_addEmptyPart(parts, U"b");
	model_setDiffuseMap(parts, a, small);
	model_setDiffuseMap(parts, b, noise);
	model_setLightMap(parts, b, lightMap);
	addRandomTriangles(parts, a, 1500, false);
	addRandomTriangles(parts, b, 1500, true);
	const Transform3D moved(FVector3D(0.2f, -0.1f, 0.4f), FMatrix3x3());
	compareModelRender("model_render two parts", parts, frontCamera(320, 240), colorTarget(320, 240, PackOrderIndex::RGBA, 0),
	                   depthTarget(320, 240, false), moved);
	// 4. an alpha-filtered model over prefilled targets; an orthogonal camera
	Model glass = model_create();
	const int32_t g = model_addEmptyPart(glass, U"glass");
	model_setDiffuseMap(glass, g, small);
	model_setFilter(glass, Filter::Alpha);
	addRandomTriangles(glass, g, 800, false);
	compareModelRender("model_render alpha", glass, frontCamera(256, 192), colorTarget(256, 192, PackOrderIndex::RGBA, 1),
	                   depthTarget(256, 192, true));
	const Camera ortho = Camera::createOrthogonal(Transform3D(FVector3D(0.0f, 0.0f, -3.0f), FMatrix3x3()), 256.0f, 200.0f, 1.3f);
	compareModelRender("model_render orthogonal", parts, ortho, colorTarget(256, 200, PackOrderIndex::RGBA, 0), depthTarget(256, 200, false));
	// 5. model_renderDepth
	{
		ImageF32 refDepth = depthTarget(320, 240, true), gpuDepth = copyOf(refDepth);
		dsr::model_renderDepth(c0, Transform3D(), refDepth, frontCamera(320, 240));
		gpu::model_renderDepth(c0, Transform3D(), gpuDepth, frontCamera(320, 240));
		report("model_renderDepth", true, sameImages(refDepth, gpuDepth));
	}
	// 6. the renderer: an occluding box, three tasks (one alpha-filtered), single triangles, the
	//    occlusion grid from the tasks given so far, a box test and the debug wireframe
	{
		const int32_t w = 400, h = 300;
		const Camera camera = frontCamera(w, h, 0.1f);
		ImageRgbaU8 refColor = colorTarget(w, h, PackOrderIndex::RGBA, 0), gpuColor = copyOf(refColor);
		ImageF32 refDepth = depthTarget(w, h, false), gpuDepth = copyOf(refDepth);
		dsr::Renderer ref = dsr::renderer_create();
		gpu::Renderer dev = gpu::renderer_create();
		const FVector3D boxLo(-0.3f, -0.3f, 0.5f), boxHi(0.3f, 0.3f, 0.9f);
		bool visibleRef = false, visibleGpu = false;
		ProjectedPoint points[50][3];
		FVector4D colors[50][3], coords[50][3];
		for (int t = 0; t < 50; t++) {
			for (int k = 0; k < 3; k++) {
				points[t][k] = camera.worldToScreen(FVector3D(uniform(-1.0f, 1.0f), uniform(-1.0f, 1.0f), uniform(-1.5f, 1.0f)));
				colors[t][k] = FVector4D(uniform(0.0f, 1.0f), uniform(0.0f, 1.0f), uniform(0.0f, 1.0f), 1.0f);
				coords[t][k] = FVector4D(uniform(0.0f, 1.0f), uniform(0.0f, 1.0f), uniform(0.0f, 1.0f), uniform(0.0f, 1.0f));
			}
		}
		for (int pass = 0; pass < 2; pass++) {
			const bool isRef = pass == 0;
			ImageRgbaU8 &color = isRef ? refColor : gpuColor;
			ImageF32 &depth = isRef ? refDepth : gpuDepth;
			if (isRef) dsr::renderer_begin(ref, color, depth); else gpu::renderer_begin(dev, color, depth);
			if (isRef) dsr::renderer_occludeFromBox(ref, boxLo, boxHi, Transform3D(), camera, true);
			else gpu::renderer_occludeFromBox(dev, boxLo, boxHi, Transform3D(), camera, true);
			if (isRef) { dsr::renderer_giveTask(ref, parts, moved, camera); dsr::renderer_giveTask(ref, c0, Transform3D(), camera); }
			else { gpu::renderer_giveTask(dev, parts, moved, camera); gpu::renderer_giveTask(dev, c0, Transform3D(), camera); }
			for (int t = 0; t < 50; t++) {
				const ProjectedPoint *p = points[t];
				const FVector4D *colorK = colors[t], *coordK = coords[t];
				if (isRef) dsr::renderer_giveTask_triangle(ref, p[0], p[1], p[2], colorK[0], colorK[1], colorK[2], coordK[0], coordK[1], coordK[2],
				                                           noise, lightMap, Filter::Solid, camera);
				else gpu::renderer_giveTask_triangle(dev, p[0], p[1], p[2], colorK[0], colorK[1], colorK[2], coordK[0], coordK[1], coordK[2],
				                                     noise, lightMap, Filter::Solid, camera);
			}
			if (isRef) { dsr::renderer_occludeFromExistingTriangles(ref); visibleRef = dsr::renderer_isBoxVisible(ref, boxLo, boxHi, Transform3D(), camera); }
			else { gpu::renderer_occludeFromExistingTriangles(dev); visibleGpu = gpu::renderer_isBoxVisible(dev, boxLo, boxHi, Transform3D(), camera); }
			if (isRef) dsr::renderer_giveTask(ref, glass, Transform3D(), camera); else gpu::renderer_giveTask(dev, glass, Transform3D(), camera);
			if (isRef) dsr::renderer_end(ref, true); else gpu::renderer_end(dev, true);
		}
		report("renderer occluders, tasks, triangles, alpha, wireframe", sameImages(refColor, gpuColor) && visibleRef == visibleGpu,
		       sameImages(refDepth, gpuDepth));
		// the reference's call-order errors arrive as the same exceptions
		std::string refMessage, gpuMessage;
		try { dsr::renderer_end(ref); } catch (const std::exception &e) { refMessage = e.what(); }
		try { gpu::renderer_end(dev); } catch (const std::exception &e) { gpuMessage = e.what(); }
		const bool sameError = !refMessage.empty() && gpuMessage.find(refMessage.substr(0, refMessage.find('\n'))) != std::string::npos;
		std::printf("renderer_end without renderer_begin: reference \"%s\", dsr::gpu \"%s\"\n",
		            refMessage.substr(0, refMessage.find('\n')).c_str(), gpuMessage.substr(0, gpuMessage.find('\n')).c_str());
		if (!sameError) g_failures++;
	}
	gpu::forget_all();
	std::printf("%s\n", g_failures == 0 ? "all equal" : "MISMATCH");
	return g_failures == 0 ? 0 : 1;
}

} // namespace

DSR_MAIN_CALLER(dsrMain)
void dsrMain(List<String> args) {
	if (args.length() > 1 && string_match(args[1], U"context")) {
		try {
			gpu::Renderer r = gpu::renderer_create();
			std::printf("created\n");
		} catch (const std::exception &e) {
			std::printf("threw: %s\n", e.what());
		}
		return;
	}
	const int status = compare();
	heap_terminatingApplication();
	std::fflush(stdout);
	std::_Exit(status);
}
