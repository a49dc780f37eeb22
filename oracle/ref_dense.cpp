// Test infrastructure only: the UNMODIFIED reference's renderDenseModel and DenseModel_create
// (Source/SDK/SpriteEngine/spriteAPI.cpp:1174-1327), reached by compiling spriteAPI.cpp into this
// translation unit, because renderDenseModel is file-static there.  Built by oracle/Makefile.ref
// into the reference harness library; never part of the product.
#include "SDK/SpriteEngine/spriteAPI.cpp"

#include <cstring>

using namespace dsr;

extern "C" {

// A model of triangles and quads (polyIndices: polyCount x 4, index 3 = -1 for a triangle; colors:
// polyCount x 4 x 4 floats) made dense and drawn with renderDenseModel<highQuality> into
// width x heightPx images (height F32, diffuse and normal RGBA as raw 32-bit words, no padding),
// seen through OrthoSystem(cameraTilt, pixelsPerTile).view[viewIndex].
void refh_dense_render(const float *positions, int pointCount, const int *polyIndices, const float *colors, int polyCount,
                       float cameraTilt, int pixelsPerTile, int viewIndex, float *height, uint32_t *diffuse, uint32_t *normal,
                       int width, int heightPx, float originX, float originY, const float *modelToWorld, int highQuality) {
	Model model = model_create();
	const int part = model_addEmptyPart(model, U"part");
	for (int p = 0; p < pointCount; p++) model_addPoint(model, FVector3D(positions[p * 3], positions[p * 3 + 1], positions[p * 3 + 2]));
	for (int p = 0; p < polyCount; p++) {
		const int *idx = polyIndices + p * 4;
		const int corners = idx[3] < 0 ? 3 : 4;
		const int poly = corners == 3 ? model_addTriangle(model, part, idx[0], idx[1], idx[2])
		                              : model_addQuad(model, part, idx[0], idx[1], idx[2], idx[3]);
		for (int v = 0; v < corners; v++) {
			const float *co = colors + (p * 4 + v) * 4;
			model_setVertexColor(model, part, poly, v, FVector4D(co[0], co[1], co[2], co[3]));
		}
	}
	DenseModel dense = DenseModel_create(model);
	OrthoSystem system(cameraTilt, pixelsPerTile);
	AlignedImageF32 heightImage = image_create_F32(width, heightPx);
	OrderedImageRgbaU8 diffuseImage = image_create_RgbaU8(width, heightPx);
	OrderedImageRgbaU8 normalImage = image_create_RgbaU8(width, heightPx);
	for (int y = 0; y < heightPx; y++) {
		std::memcpy(image_getSafePointer<float>(heightImage, y).getUnsafe(), height + (size_t)y * width, sizeof(float) * width);
		std::memcpy(image_getSafePointer<uint32_t>(diffuseImage, y).getUnsafe(), diffuse + (size_t)y * width, sizeof(uint32_t) * width);
		std::memcpy(image_getSafePointer<uint32_t>(normalImage, y).getUnsafe(), normal + (size_t)y * width, sizeof(uint32_t) * width);
	}
	const Transform3D transform(FVector3D(modelToWorld[0], modelToWorld[1], modelToWorld[2]),
	  FMatrix3x3(FVector3D(modelToWorld[3], modelToWorld[4], modelToWorld[5]), FVector3D(modelToWorld[6], modelToWorld[7], modelToWorld[8]),
	             FVector3D(modelToWorld[9], modelToWorld[10], modelToWorld[11])));
	if (highQuality)
		renderDenseModel<true>(dense, system.view[viewIndex], heightImage, diffuseImage, normalImage, FVector2D(originX, originY), transform);
	else
		renderDenseModel<false>(dense, system.view[viewIndex], heightImage, diffuseImage, normalImage, FVector2D(originX, originY), transform);
	for (int y = 0; y < heightPx; y++) {
		std::memcpy(height + (size_t)y * width, image_getSafePointer<float>(heightImage, y).getUnsafe(), sizeof(float) * width);
		std::memcpy(diffuse + (size_t)y * width, image_getSafePointer<uint32_t>(diffuseImage, y).getUnsafe(), sizeof(uint32_t) * width);
		std::memcpy(normal + (size_t)y * width, image_getSafePointer<uint32_t>(normalImage, y).getUnsafe(), sizeof(uint32_t) * width);
	}
}

} // extern "C"
