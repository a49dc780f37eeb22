// dsr::gpu -- the reference's model and renderer API (Source/DFPSR/api/modelAPI.h:285-301,
// Source/DFPSR/api/rendererAPI.h:46-135) drawn on the GPU through the dsrg C ABI (include/dsrg.h).
//
// Every function keeps the signature, argument meaning and call protocol of its dsr:: namesake, and
// reports failures the way the reference does, through dsr::throwError (api/stringAPI.cpp:1470-1488):
// a std::runtime_error by default.  A program switches by replacing `dsr::model_render(...)` with
// `dsr::gpu::model_render(...)` and `dsr::Renderer` with `dsr::gpu::Renderer`; models, textures,
// images and cameras stay the reference's own objects.
//
// Compiled against the reference's headers (Source/ on the include path) and linked with the
// reference's library and libdsrg.so; C++14 like the reference.
//
// What moves to the GPU, and when:
//   - A model is copied to the GPU the first time it is drawn: its points, every part's polygons,
//     texture coordinates and vertex colours, its bounding box and its filter, one dsrg model per
//     part (drawn in part order, as ModelImpl::render walks them).  Its textures are copied the
//     same way, pyramid as they are.  The copies are kept, and the model and its textures are held
//     by handle, until model_forget / texture_forget / forget_all: call them after editing a model
//     or a texture that was already drawn.
//   - Target images stay in the reference's host memory.  Each call copies them to the GPU and back
//     (the library stages pageable memory); images whose buffers are page-locked are drawn in place.
//   - Cameras are read whole on every call (Camera::createPerspective / createOrthogonal cameras).
//
// Threading follows the reference: one thread drives a renderer; model_render is synchronous.
#ifndef DFPSR_GB300_DSR_GPU_H
#define DFPSR_GB300_DSR_GPU_H

#include <cstdint>
#include <memory>

#include "DFPSR/api/modelAPI.h"
#include "DFPSR/api/rendererAPI.h"

namespace dsr {
namespace gpu {

// The GPU the following calls draw on (default 0).  Takes effect before the first GPU call only.
void setDevice(int32_t device);

// model_render (api/modelAPI.h:285): draws the model into the colour and depth images, either of
// which may be empty.
void model_render(const Model& model, const Transform3D &modelToWorldTransform, ImageRgbaU8& colorBuffer,
                  ImageF32& depthBuffer, const Camera &camera);
// model_renderDepth (api/modelAPI.h:291).
void model_renderDepth(const Model& model, const Transform3D &modelToWorldTransform, ImageF32& depthBuffer,
                       const Camera &camera);

// Drops the GPU copy of a model or texture (and the handle kept with it); the next draw copies it again.
void model_forget(const Model& model);
void texture_forget(const TextureRgbaU8& texture);
// Drops every GPU copy and the GPU context.
void forget_all();

// renderer_* (api/rendererAPI.h:46-135, api/modelAPI.h:299-301).
struct RendererImpl;
using Renderer = std::shared_ptr<RendererImpl>;
Renderer renderer_create();
bool renderer_exists(const Renderer& renderer);
void renderer_begin(Renderer& renderer, ImageRgbaU8& colorBuffer, ImageF32& depthBuffer);
ImageRgbaU8 renderer_getColorBuffer(const Renderer& renderer);
ImageF32 renderer_getDepthBuffer(const Renderer& renderer);
bool renderer_takesTriangles(const Renderer& renderer);
void renderer_occludeFromBox(Renderer& renderer, const FVector3D& minimum, const FVector3D& maximum,
                             const Transform3D &modelToWorldTransform, const Camera &camera, bool debugSilhouette = false);
void renderer_occludeFromTopRows(Renderer& renderer, const Camera &camera);
bool renderer_hasOccluders(const Renderer& renderer);
bool renderer_isBoxVisible(const Renderer& renderer, const FVector3D &minimum, const FVector3D &maximum,
                           const Transform3D &modelToWorldTransform, const Camera &camera);
void renderer_giveTask_triangle(Renderer& renderer,
  const ProjectedPoint &posA, const ProjectedPoint &posB, const ProjectedPoint &posC,
  const FVector4D &colorA, const FVector4D &colorB, const FVector4D &colorC,
  const FVector4D &texCoordA, const FVector4D &texCoordB, const FVector4D &texCoordC,
  const TextureRgbaU8& diffuseMap, const TextureRgbaU8& lightMap,
  Filter filter, const Camera &camera);
void renderer_occludeFromExistingTriangles(Renderer& renderer);
void renderer_end(Renderer& renderer, bool debugWireframe = false);
// renderer_giveTask / model_render_threaded (api/modelAPI.h:295-301).
void renderer_giveTask(Renderer& renderer, const Model& model, const Transform3D &modelToWorldTransform, const Camera &camera);
void model_render_threaded(const Model& model, const Transform3D &modelToWorldTransform, Renderer& renderer, const Camera &camera);

}
}

#endif
