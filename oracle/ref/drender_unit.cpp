// The reference's src/drender.cpp compiled together with the point-light
// model of ref_pointlight.h, so that DiffRender<> can be instantiated for it:
// drender.cpp defines edge_grad as an inline function that only its own
// translation unit sees.  Test infrastructure; built by build_ref.py in place
// of drender.cpp (the reference file is included where it lies, unchanged).
#include "ref_pointlight.h"

#include "drender.cpp"

namespace diff_render {

std::shared_ptr<IDiffRender> MakePointLightRenderer(const DiffRenderSettings& settings) {
  auto impl = std::make_shared<DiffRender<kPointLightVColor>>();
  impl->init(settings);
  impl->mode = SHADING_MODEL::VERTEX_COLOR;  // the gradient layout with the albedo (colour) block
  return impl;
}

}  // namespace diff_render
