// The point-light vertex-albedo shading model for the reference's own
// DiffRender<> template (src/drender.h:74-425), so that the reference's
// render loop, interior and edge derivatives and optimiser run the benchmark
// workload unchanged.  The reference has no such model (its LAMBERT,
// src/shade_lambert.cpp:7-35, uses a directional light and a texture); this
// restates the oracle's (oracle/oracle.c, lpv_factor / shade / shade_grad)
// with the reference's types and operation order.  Test infrastructure and
// CPU-baseline timing only.
//
// Constants are the workload's: light at (3,3,3), intensity 10, ambient 0.1.
// The albedo is the per-vertex colour, so gradients use the VERTEX_COLOR
// DScene layout (positions, colours, transforms).
#pragma once
#include <algorithm>

#include "dmodels.h"

namespace diff_render {

constexpr SHADING_MODEL kPointLightVColor = (SHADING_MODEL)16;

// vis * I * max(0, n.l) / d^2 + ambient at a camera hit
static inline float point_light_factor(const Scene& scene, IRayTracer* tracer, const SurfaceInfo& s, unsigned A,
                                       unsigned B, unsigned C, float3 ray_pos, float3 ray_dir) {
  const float3 light_pos(3.0f, 3.0f, 3.0f);
  const float intensity = 10.0f, ambient = 0.1f;
  const float u = s.u, v = s.v;
  const float3 n = scene.get_norm(A) * (1.0f - u - v) + scene.get_norm(B) * v + scene.get_norm(C) * u;
  const float3 p = ray_pos + ray_dir * (s.t - 1e-5f);
  const float3 L = light_pos - p;
  const float d2 = dot(L, L);
  const float dist = sqrtf(d2);
  const float3 l = L / dist;
  const float ndl = std::max(0.0f, dot(n, l));
  // the lit term is 0 when n.l <= 0 whatever the visibility
  const float vis = (ndl > 0.0f && tracer->GetNearestHit(p, l, 0.0f, dist).primId != unsigned(-1)) ? 0.0f : 1.0f;
  return vis * intensity * ndl / d2 + ambient;
}

template <>
inline float3 shade<kPointLightVColor>(const Scene& scene, IRayTracer* tracer, const float2 screen_pos) {
  float3 ray_pos = {0, 0, 0}, ray_dir = {0, 0, 0};
  SurfaceInfo s = tracer->CastSingleRay(screen_pos.x, screen_pos.y, &ray_pos, &ray_dir);
  if (s.primId == unsigned(-1)) return float3(0, 0, 0);
  const auto A = scene.get_index(s.geomId, s.instId, s.primId * 3 + 0);
  const auto B = scene.get_index(s.geomId, s.instId, s.primId * 3 + 1);
  const auto C = scene.get_index(s.geomId, s.instId, s.primId * 3 + 2);
  const float u = s.u, v = s.v;
  const float3 albedo = scene.get_color(A) * (1.0f - u - v) + scene.get_color(B) * v + scene.get_color(C) * u;
  return albedo * point_light_factor(scene, tracer, s, A, B, C, ray_pos, ray_dir);
}

// d colour / d albedo of the three vertices (the lighting factor is held
// fixed, as the reference's shade_grad models hold it).
template <>
inline void shade_grad<kPointLightVColor>(const Scene& scene, IRayTracer* tracer, const float2 screen_pos,
                                          const float3 val, const AuxData aux, DScene& grad) {
  (void)aux;
  float3 ray_pos = {0, 0, 0}, ray_dir = {0, 0, 0};
  SurfaceInfo s = tracer->CastSingleRay(screen_pos.x, screen_pos.y, &ray_pos, &ray_dir);
  if (s.primId == unsigned(-1)) return;
  DMesh* dm = grad.get_dmesh(s.geomId);
  if (!dm || !dm->color(0)) return;
  const auto A = scene.get_index(s.geomId, s.instId, s.primId * 3 + 0);
  const auto B = scene.get_index(s.geomId, s.instId, s.primId * 3 + 1);
  const auto C = scene.get_index(s.geomId, s.instId, s.primId * 3 + 2);
  const float k = point_light_factor(scene, tracer, s, A, B, C, ray_pos, ray_dir);
  const float u = s.u, v = s.v;
  const auto a = scene.get_vertex_n(s.geomId, s.primId * 3 + 0);
  const auto b = scene.get_vertex_n(s.geomId, s.primId * 3 + 1);
  const auto c = scene.get_vertex_n(s.geomId, s.primId * 3 + 2);
  const float3 ca = val * ((1.0f - u - v) * k), cb = val * (v * k), cc = val * (u * k);
  float* pa = dm->color(a);
  float* pb = dm->color(b);
  float* pc = dm->color(c);
  pa[0] += ca.x; pa[1] += ca.y; pa[2] += ca.z;
  pb[0] += cb.x; pb[1] += cb.y; pb[2] += cb.z;
  pc[0] += cc.x; pc[1] += cc.y; pc[2] += cc.z;
}

}  // namespace diff_render
