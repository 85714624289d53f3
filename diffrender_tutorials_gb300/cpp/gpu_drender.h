// GPU implementations of the reference renderer's C++ interfaces.
//
// For code written against FROL256/diffrender_tutorials: IDiffRender
// (src/virtual_drender.h:14-26) and IOptimizer (src/optimizer.h:52-61) over
// the drgb C ABI (include/drgb.h).  Compile gpu_drender.cpp together with the
// reference's sources (it includes their headers) and link libdrgb.so; then
//
//   auto r = diff_render::MakeGpuDifferentialRenderer(settings);   // instead of MakeDifferentialRenderer
//   auto o = diff_render::CreateGpuOptimizer();                     // instead of CreateSimpleOptimizer
//
// Semantics follow the reference: render() writes into caller-sized images;
// d_render() accumulates into the DScene, d_render_and_compare() clears it
// first and returns the MSE divided by views*W*H; a renderer refuses to render
// a scene other than the one last committed.  Errors are printed and the call
// returns, as the reference does (src/drender.h:103-107); the C ABI's error
// code and message are available from last_error().
//
// The reference's own CPU optimiser (OptSimple) also accepts the renderer
// returned here, since it only calls IDiffRender::d_render_and_compare.
#pragma once
#include <memory>
#include <string>

#include "optimizer.h"
#include "virtual_drender.h"

namespace diff_render {

// Renderer on CUDA device `device`.  Models: SILHOUETTE, VERTEX_COLOR,
// TEXTURE_COLOR, LAMBERT, PHONG, GGX and PATH_TEST (the reference's
// numbering; PATH_TEST draws from a counter-based generator in place of
// rand(), so its images agree with the reference's in expectation), and the
// point-light vertex-albedo (16) and diffuse path (17) models that have no
// reference counterpart.  Any other number prints an error and the renderer
// stays unusable.
std::shared_ptr<IDiffRender> MakeGpuDifferentialRenderer(const DiffRenderSettings& settings, int device = 0);

// OptSimple's loop with every iteration (render, loss, gradients, update,
// scene refit) on the GPU, replayed from a CUDA graph.
std::shared_ptr<IOptimizer> CreateGpuOptimizer(int device = 0);

// Code and message of the last failed drgb call made by these classes on this
// thread (0 and "" after a successful call).
int last_error(std::string* message = nullptr);

}  // namespace diff_render
