// Shading models and the two traversal policies they run on.
//
// Per-ray policy (WARP = false): each thread traverses the LBVH on its own
// (trace<ANY>).  Used where a warp's rays are unrelated -- the edge-sample
// pass, which draws samples at random over all edges.
//
// Warp-coherent policy (WARP = true): the 32 rays of a warp traverse the
// LBVH together (trace_warp<ANY>).  Used by the pixel kernel, whose warps
// hold the samples of one or two adjacent pixels, so their camera rays,
// shadow rays and re-traced adjoint rays visit nearly the same nodes.  The
// node to visit is the same for the whole warp (one broadcast load), a child
// is entered when any lane's ray reaches it before that lane's current hit
// distance, the order of two hit children follows the majority of lanes,
// and the traversal stack lives one entry per lane, read back with a
// shuffle.  Every lane still tests every leaf its own ray reaches, so the
// result per lane is the same as with the per-ray policy.
//
// The shading code below is written in masked form: lanes without a hit
// carry an inactive flag through the traversal calls instead of leaving
// early, so that in the warp policy all 32 lanes reach every traversal call.
#pragma once

namespace drgb {

template <bool ANY>
__device__ DRGB_TRACE_ATTR bool trace_warp(const JobDev& J, f3 o, f3 d, float tNear, float tFar, bool active,
                                           Hit& best) {
  best.t = tFar;
  best.tri = -1;
  best.u = 0.0f;
  best.v = 0.0f;
  const unsigned FULL = 0xffffffffu;
  if (J.n_tris <= 0) return false;
  if (J.trace_bruteforce) return active ? trace<ANY>(J, o, d, tNear, tFar, best) : false;
  bool live = active;
  if (!__any_sync(FULL, live)) return false;
  const int lane = threadIdx.x & 31;
  const f3 inv = mk(safe_inv(d.x), safe_inv(d.y), safe_inv(d.z));
  const f3 oi = mk(o.x * inv.x, o.y * inv.y, o.z * inv.z);
  const float lo_t = tNear - fabsf(tNear) * 4e-6f - 1e-6f;
  unsigned n_box = 0, n_tri = 0;
  int s0 = 0, s1 = 0;  // stack entry i is held by lane i%32 in slot i/32
  int sp = 0;
  int node = J.root;
  int guard = 0;
  while (true) {
    if (node >= 0) {
      const float4 n0 = __ldg(J.nodes + 4 * node + 0);
      const float4 n1 = __ldg(J.nodes + 4 * node + 1);
      const float4 n2 = __ldg(J.nodes + 4 * node + 2);
      const float4 n3 = __ldg(J.nodes + 4 * node + 3);
      bool h0 = false, h1 = false;
      float t0 = 0.0f, t1 = 0.0f;
      if (live) {
        const float hi_t = cull_bound(best.t);
        t0 = slab(n0.x, n0.y, n0.z, n0.w, n2.x, n2.y, inv, oi, lo_t, hi_t);
        t1 = slab(n1.x, n1.y, n1.z, n1.w, n2.z, n2.w, inv, oi, lo_t, hi_t);
        h0 = t0 <= hi_t;
        h1 = t1 <= hi_t;
        n_box += 2;
      }
      const int c0 = __float_as_int(n3.x), c1 = __float_as_int(n3.y);
      const unsigned b0 = __ballot_sync(FULL, h0), b1 = __ballot_sync(FULL, h1);
      if (b0 && b1) {
        const unsigned p0 = __ballot_sync(FULL, h0 && (!h1 || t0 <= t1));
        const bool first0 = 2 * __popc(p0) >= __popc(b0 | b1);
        if (sp >= 64) {
          if (lane == 0) atomicOr(J.err, ERR_STACK_OVERFLOW);
          break;
        }
        const int far = first0 ? c1 : c0;
        if (lane == (sp & 31)) {
          if (sp < 32) s0 = far;
          else s1 = far;
        }
        sp++;
        node = first0 ? c0 : c1;
        continue;
      } else if (b0) {
        node = c0;
        continue;
      } else if (b1) {
        node = c1;
        continue;
      }
    } else {
      const int k = ~node;
      const float4 a = __ldg(J.tri + 3 * k), e1 = __ldg(J.tri + 3 * k + 1), e2 = __ldg(J.tri + 3 * k + 2);
      const int id = __float_as_int(a.w);
      if (live) {
        float t, u, v;
        n_tri++;
        if (mt_test(o, d, f4to3(a), f4to3(e1), f4to3(e2), tNear, t, u, v) &&
            (t < best.t || (t == best.t && id < best.tri))) {
          best.t = t;
          best.u = u;
          best.v = v;
          best.tri = id;
          if (ANY) live = false;
        }
      }
      if (ANY && !__any_sync(FULL, live)) break;
    }
    if (sp == 0) break;
    sp--;
    node = __shfl_sync(FULL, sp < 32 ? s0 : s1, sp & 31);
    if (++guard > J.trace_limit) {
      if (lane == 0) atomicOr(J.err, ERR_TRAVERSAL_LIMIT);
      break;
    }
  }
  if (active) add_work(J, n_box, n_tri);
  return best.tri >= 0;
}

// Traversal under a policy; inactive lanes report a miss.
template <bool ANY, bool WARP>
__device__ __forceinline__ bool trace_p(const JobDev& J, f3 o, f3 d, float tNear, float tFar, bool active, Hit& h,
                                        int seed = -1) {
  if (WARP) return trace_warp<ANY>(J, o, d, tNear, tFar, active, h);
  if (!active) {
    h.t = tFar;
    h.tri = -1;
    h.u = h.v = 0.0f;
    return false;
  }
  return trace<ANY>(J, o, d, tNear, tFar, h, seed);
}

// Surface record of a camera ray (SurfaceInfo, raytrace.h:21-29, plus ids).
// Without a hit the vertex ids are 0, so masked loads stay in bounds.
struct Surf {
  Hit h;
  int A, B, C;  // global vertex ids
  int block;
  f3 ro, rd;
};

template <bool WARP>
__device__ __forceinline__ bool cast_p(const JobDev& J, const CamDev& cam, float x, float y, bool active, Surf& s,
                                       int seed = -1) {
  camera_ray(cam, x, y, s.ro, s.rd);
  const bool hit = trace_p<false, WARP>(J, s.ro, s.rd, 0.0f, 1e9f, active, s.h, seed);
  s.A = s.B = s.C = 0;
  s.block = 0;
  if (hit) {
    const int4 tv = __ldg(J.tri_v + s.h.tri);
    s.A = tv.x;
    s.B = tv.y;
    s.C = tv.z;
    s.block = tv.w;
  }
  return hit;
}

// The camera ray of a sample whose nearest hit the raster pass found:
// hit = {t, u, v, triangle bits} (triangle -1: none), the values the
// reference's ray/triangle test computed for that ray.  uv != null: the
// record is the point-light model's, hit = {shading point, triangle bits}
// and *uv = {u, v}; the surface is then returned with ro = that point,
// rd = 0 and t = 1e-5, so that ro + rd * (t - 1e-5), the shader's point,
// is the stored point.  ray = false: the model reads no ray (its
// interpolation uses u, v only) and none is built.
__device__ __forceinline__ bool cast_vis(const JobDev& J, const CamDev& cam, float x, float y, bool active,
                                         float4 hit, Surf& s, const float2* uv = nullptr, bool ray = true) {
  if (ray && !uv) {
    camera_ray(cam, x, y, s.ro, s.rd);
  } else {
    s.ro = mk(hit.x, hit.y, hit.z);
    s.rd = mk(0.0f, 0.0f, 0.0f);
  }
  s.h.t = 1e9f;
  s.h.tri = -1;
  s.h.u = s.h.v = 0.0f;
  s.A = s.B = s.C = 0;
  s.block = 0;
  if (active) add_list_work(J, true, 0, 0);
  const int id = __float_as_int(hit.w);
  if (!active || id < 0) return false;
  if (id >= J.n_tris) {
    atomicOr(J.err, ERR_VISIBILITY);
    return false;
  }
  if (uv) {
    const float2 q = *uv;
    s.h.t = 1e-5f;
    s.h.u = q.x;
    s.h.v = q.y;
  } else {
    s.h.t = hit.x;
    s.h.u = hit.y;
    s.h.v = hit.z;
  }
  s.h.tri = id;
  const int4 tv = __ldg(J.tri_v + id);
  s.A = tv.x;
  s.B = tv.y;
  s.C = tv.z;
  s.block = tv.w;
  return true;
}

// Lists of at most this many entries are sorted by their distance bound
// (k_sort_lists): a query stops at the first entry whose bound it beats.
constexpr uint32_t kSortedList = 64;

// Screen tile of image position (x, y) in `view` (index into ra_tiles).
__device__ __forceinline__ int tile_of(const JobDev& J, int view, float x, float y) {
  const int tx = min(J.ra_ntx - 1, (int)x / J.ra_tw), ty = min(J.ra_nty - 1, (int)y / J.ra_th);
  return (view * J.ra_nty + ty) * J.ra_ntx + tx;
}

// Whether a camera ray of `view` at image position (x, y) uses the raster
// pass's tile lists (built for this call's geometry; the footprints are
// clipped to the image, so only positions inside it): only where the
// tile's list is sorted.  A single query against a long unsorted list reads
// every entry and costs more than the traversal (dense meshes: 200k
// triangles at 512x512 doubled the edge pass).
__device__ __forceinline__ bool tiles_usable(const JobDev& J, const CamDev& cam, int view, float x, float y) {
  if (!(J.ra_tiles && (*J.ra_state & 2u) && x >= 0.0f && x < cam.width && y >= 0.0f && y < cam.height))
    return false;
  const int b = tile_of(J, view, x, y);
  return __ldg(J.ra_tiles + b + 1) - __ldg(J.ra_tiles + b) <= kSortedList;
}

// The nearest hit of the camera ray of `view` at (x, y) among the triangles
// of its screen tile: the reference's test on each footprint holding the
// point, the smallest {t, flattened triangle} kept (the traversal's tie
// rule); t, u, v are those the test computed.
__device__ __forceinline__ bool cast_tiles(const JobDev& J, const CamDev& cam, int view, float x, float y,
                                           bool active, Surf& s) {
  camera_ray(cam, x, y, s.ro, s.rd);
  s.h.t = 1e9f;
  s.h.tri = -1;
  s.h.u = s.h.v = 0.0f;
  s.A = s.B = s.C = 0;
  s.block = 0;
  if (!active) return false;
  const int b = tile_of(J, view, x, y);
  const uint32_t i0 = __ldg(J.ra_tiles + b), i1 = __ldg(J.ra_tiles + b + 1);
  const bool sorted = i1 - i0 <= kSortedList;
  unsigned long long best = ~0ull;
  float bu = 0.0f, bv = 0.0f;
  unsigned n_tri = 0, n_fp = 0;
  for (uint32_t i = i0; i < i1; i++) {
    const int j = __ldg(J.ra_list + i);
    const float4 q0 = __ldg(J.ra_rec + 4 * j + 1);
    // no hit on it can be nearer than the best so far (none yet: NaN
    // compares false), nor on the entries after it in a sorted list
    if (q0.w > __uint_as_float((uint32_t)(best >> 32))) {
      if (sorted) break;
      continue;
    }
    n_fp++;
    const float4 box = __ldg(J.ra_rec + 4 * j);
    if (!(x >= box.x && x <= box.y && y >= box.z && y <= box.w)) continue;
    const float4 q1 = __ldg(J.ra_rec + 4 * j + 2), q2 = __ldg(J.ra_rec + 4 * j + 3);
    if (!(q0.x * x + q0.y * y + q0.z >= 0.0f && q1.x * x + q1.y * y + q1.z >= 0.0f &&
          q2.x * x + q2.y * y + q2.z >= 0.0f))
      continue;
    const int k = j - view * J.n_tris;
    const float4 a = __ldg(J.tri + 3 * k), e1 = __ldg(J.tri + 3 * k + 1), e2 = __ldg(J.tri + 3 * k + 2);
    float t, u, v;
    n_tri++;
    if (mt_test(s.ro, s.rd, f4to3(a), f4to3(e1), f4to3(e2), 0.0f, t, u, v) && t < 1e9f) {
      const unsigned long long key = ((unsigned long long)__float_as_uint(t) << 32) | (uint32_t)__float_as_int(a.w);
      if (key < best) {
        best = key;
        bu = u;
        bv = v;
      }
    }
  }
  add_list_work(J, true, n_fp, n_tri);
  if (best == ~0ull) return false;
  s.h.t = __uint_as_float((uint32_t)(best >> 32));
  s.h.u = bu;
  s.h.v = bv;
  s.h.tri = (int)(uint32_t)best;
  const int4 tv = __ldg(J.tri_v + s.h.tri);
  s.A = tv.x;
  s.B = tv.y;
  s.C = tv.z;
  s.block = tv.w;
  return true;
}

__device__ __forceinline__ bool cast(const JobDev& J, const CamDev& cam, float x, float y, Surf& s) {
  return cast_p<false>(J, cam, x, y, true, s);
}

// sample_bilinear_clamp_3f (shade_common.cpp:3-21)
__device__ __forceinline__ f3 sample_bilinear(float tx, float ty, int w, int h, const float* data) {
  tx = ref_clamp(tx, 0.0f, 1.0f);
  ty = ref_clamp(ty, 0.0f, 1.0f);
  tx *= (float)w;
  ty *= (float)h;
  const int ix = (int)tx, iy = (int)ty;
  const int x0 = clampi(ix, 0, w - 1), y0 = clampi(iy, 0, h - 1);
  const int x1 = clampi(ix + 1, 0, w - 1), y1 = clampi(iy + 1, 0, h - 1);
  const float dx = tx - (float)x0, dy = ty - (float)y0;
  const float* p00 = data + 3 * (y0 * w + x0);
  const float* p01 = data + 3 * (y1 * w + x0);
  const float* p10 = data + 3 * (y0 * w + x1);
  const float* p11 = data + 3 * (y1 * w + x1);
  float r[3];
#pragma unroll
  for (int i = 0; i < 3; i++)
    r[i] = (1 - dx) * (1 - dy) * __ldg(p00 + i) + (1 - dx) * dy * __ldg(p01 + i) + dx * (1 - dy) * __ldg(p10 + i) +
           dx * dy * __ldg(p11 + i);
  return mk(r[0], r[1], r[2]);
}

__device__ __forceinline__ float2 interp_tc(const JobDev& J, const Surf& s) {
  const float2 a = __ldg(J.tc + s.A), b = __ldg(J.tc + s.B), c = __ldg(J.tc + s.C);
  const float w0 = 1.0f - s.h.u - s.h.v;
  return make_float2((a.x * w0 + b.x * s.h.v) + s.h.u * c.x, (a.y * w0 + b.y * s.h.v) + s.h.u * c.y);
}

// Lighting factor of the point-light vertex-albedo model:
// vis * I * max(0, n.l) / d^2 + ambient, with the reference Lambert's bias.
// With n.l <= 0 the lit term is 0 whatever the visibility: no shadow ray.
// One out-of-line copy for the forward and adjoint passes (+2 % on GB300;
// -DDRGB_LPV_INLINE inlines it).
#ifdef DRGB_LPV_INLINE
#define DRGB_LPV_ATTR __forceinline__
#else
#define DRGB_LPV_ATTR __noinline__
#endif
// Grid coordinates of a point in the light's view (LightGrid).
__device__ __forceinline__ void light_project(const LightGrid& g, f3 q, float& a, float& b) {
  const float dx = q.x - g.lx, dy = q.y - g.ly, dz = q.z - g.lz;
  const float z = dx * g.wx + dy * g.wy + dz * g.wz;
  a = (dx * g.ux + dy * g.uy + dz * g.uz) / z * g.scale + g.half;
  b = (dx * g.vx + dy * g.vy + dz * g.vz) / z * g.scale + g.half;
}

// Whether the shadow ray (p, l) toward the point light meets a triangle at
// 0 < t < tfar: the reference's test (mt_test, any hit) on the triangles
// whose light-space footprint holds p's grid position.  Every point of the
// segment from p to the light has that grid position, so the triangles the
// segment crosses are all among them (the footprints carry a margin of
// 0.125 cells for rounding).  The caller checks that the grid is usable.
__device__ __forceinline__ bool light_occluded(const JobDev& J, f3 p, f3 l, float tfar) {
  const LightGrid& g = *J.sh_grid;
  float a, b;
  light_project(g, p, a, b);
  const int cx = min(g.G - 1, max(0, (int)a)), cy = min(g.G - 1, max(0, (int)b));
  const int c = cy * g.G + cx;
  const uint32_t i0 = __ldg(J.sh_cells + c), i1 = __ldg(J.sh_cells + c + 1);
  const bool sorted = i1 - i0 <= kSortedList;
  unsigned n_tri = 0, n_fp = 0;
  bool occ = false;
  for (uint32_t i = i0; i < i1 && !occ; i++) {
    const int k = __ldg(J.sh_list + i);
    const float4 q0 = __ldg(J.sh_rec + 4 * k + 1);
    if (q0.w >= tfar) {  // no nearer to the light than p: not between them
      if (sorted) break;  // nor is any later entry of a sorted list
      continue;
    }
    n_fp++;
    const float4 box = __ldg(J.sh_rec + 4 * k);
    if (!(a >= box.x && a <= box.y && b >= box.z && b <= box.w)) continue;
    const float4 q1 = __ldg(J.sh_rec + 4 * k + 2), q2 = __ldg(J.sh_rec + 4 * k + 3);
    if (!(q0.x * a + q0.y * b + q0.z >= 0.0f && q1.x * a + q1.y * b + q1.z >= 0.0f &&
          q2.x * a + q2.y * b + q2.z >= 0.0f))
      continue;
    const float4 A = __ldg(J.tri + 3 * k), e1 = __ldg(J.tri + 3 * k + 1), e2 = __ldg(J.tri + 3 * k + 2);
    float t, u, v;
    n_tri++;
    occ = mt_test(p, l, f4to3(A), f4to3(e1), f4to3(e2), 0.0f, t, u, v) && t < tfar;
  }
  add_list_work(J, true, n_fp, n_tri);
  return occ;
}

// Shadow ray toward the point light: the light-space cells when they hold
// the current geometry, else the hierarchy.
template <bool WARP>
__device__ __forceinline__ bool point_shadow(const JobDev& J, f3 p, f3 l, float tfar, bool active) {
  if (!WARP && J.sh_grid && J.sh_grid->valid) return active && light_occluded(J, p, l, tfar);
  Hit sh;
  return trace_p<true, WARP>(J, p, l, 0.0f, tfar, active, sh);
}

template <bool WARP>
__device__ DRGB_LPV_ATTR float lpv_factor_p(const JobDev& J, const Surf& s, bool hit) {
  f3 p = mk(0.0f, 0.0f, 0.0f), l = mk(0.0f, 0.0f, 1.0f);
  float d2 = 1.0f, dist = 0.0f, ndl = 0.0f;
  if (hit) {
    const float u = s.h.u, v = s.h.v;
    const f3 n = interp(ld3(J.nrm, s.A), ld3(J.nrm, s.B), ld3(J.nrm, s.C), u, v);
    p = s.ro + s.rd * (s.h.t - 1e-5f);
    const f3 L = mk(J.mp.light_pos[0], J.mp.light_pos[1], J.mp.light_pos[2]) - p;
    d2 = dot(L, L);
    dist = sqrtf(d2);
    l = L / dist;
    ndl = ref_max(0.0f, dot(n, l));
  }
  const float vis = point_shadow<WARP>(J, p, l, dist, hit && ndl > 0.0f) ? 0.0f : 1.0f;
  return vis * J.mp.light_intensity * ndl / d2 + J.mp.ambient;
}

__device__ __forceinline__ float lpv_factor(const JobDev& J, const Surf& s) { return lpv_factor_p<false>(J, s, true); }

// Counter-based hash for the path model.
__device__ __forceinline__ uint32_t pcg_hash(uint32_t x) {
  uint32_t state = x * 747796405u + 2891336453u;
  uint32_t word = ((state >> ((state >> 28u) + 4u)) ^ state) * 277803737u;
  return (word >> 22u) ^ word;
}
__device__ __forceinline__ float rnd01(uint32_t a, uint32_t b, uint32_t c) {
  uint32_t h = pcg_hash(a ^ pcg_hash(b ^ pcg_hash(c)));
  return (float)(h >> 8) * (1.0f / 16777216.0f);
}

// sin and cos of 2*pi*x for x in [0, 1) (the bounce azimuth).  x*4 and its
// nearest integer q are exact, so is f = 4x - q in [-1/2, 1/2]; a = f*pi/2
// then lies in [-pi/4, pi/4], where the Taylor series of sin to a^9 and of
// cos to a^10 are accurate to 2e-9, and the quadrant q turns (sin a, cos a)
// into (sin, cos) of the full angle.  Plain multiplies and adds in a fixed
// order (no contraction): the oracle evaluates the same sequence, so both
// sides draw bit-identical bounce directions, which the math library's
// sinf/cosf (different on host and device) would not give.
// sin and cos of a in [-pi/4, pi/4] by those two series.
__device__ __forceinline__ void sincos_small(float a, float* ps, float* pc) {
  const float a2 = a * a;
  *ps = a * (1.0f + a2 * (-1.66666672e-1f + a2 * (8.33333377e-3f + a2 * (-1.98412701e-4f + a2 * 2.75573188e-6f))));
  *pc = 1.0f + a2 * (-0.5f + a2 * (4.16666679e-2f + a2 * (-1.38888892e-3f + a2 * (2.48015876e-5f +
                                                                                a2 * -2.75573188e-7f))));
}
__device__ __forceinline__ void sincos_turns(float x, float* s, float* c) {
  const float x4 = x * 4.0f;
  const float q = rintf(x4);
  float ps, pc;
  sincos_small((x4 - q) * 1.57079633f, &ps, &pc);
  switch (((int)q) & 3) {
    case 0: *s = ps; *c = pc; break;
    case 1: *s = pc; *c = -ps; break;
    case 2: *s = -ps; *c = -pc; break;
    default: *s = -pc; *c = ps; break;
  }
}

// Fixed-depth diffuse path tracer (same definition as the oracle's
// path_diffuse): point light, Lambert BRDF, cosine-weighted bounces.
// `alive` = the camera ray hit; the bounce loop runs the same number of
// times on every lane.
template <bool WARP>
__device__ inline f3 path_diffuse_p(const JobDev& J, const Surf& first, uint32_t key, bool alive, f3* d_alb0) {
  const f3 lp = mk(J.mp.light_pos[0], J.mp.light_pos[1], J.mp.light_pos[2]);
  const float I = J.mp.light_intensity;
  f3 L = mk(0, 0, 0), beta = mk(1, 1, 1), beta_na = mk(1, 1, 1), dL0 = mk(0, 0, 0);
  Surf sf = first;
  f3 ro = first.ro, rd = first.rd;
  for (int bounce = 0; bounce <= J.mp.path_depth; bounce++) {
    bool hitb = alive;
    if (bounce > 0) {
      Hit hh;
      hitb = trace_p<false, WARP>(J, ro, rd, 0.0f, 1e9f, alive, hh);
      if (alive && !hitb) {
        L = L + beta * J.mp.ambient;
        dL0 = dL0 + beta_na * J.mp.ambient;
      }
      if (hitb) {
        sf.h = hh;
        const int4 tv = __ldg(J.tri_v + hh.tri);
        sf.A = tv.x;
        sf.B = tv.y;
        sf.C = tv.z;
      }
    }
    f3 alb = mk(0, 0, 0), n = mk(0, 0, 1), p = mk(0, 0, 0), l = mk(0, 0, 1);
    float d2 = 1.0f, dist = 0.0f, ndl = 0.0f;
    if (hitb) {
      const float u = sf.h.u, v = sf.h.v;
      alb = interp(ld3(J.col, sf.A), ld3(J.col, sf.B), ld3(J.col, sf.C), u, v);
      n = normalize(interp(ld3(J.nrm, sf.A), ld3(J.nrm, sf.B), ld3(J.nrm, sf.C), u, v));
      const f3 pa = ld3(J.pos, sf.A);
      const f3 ng = normalize(cross(ld3(J.pos, sf.B) - pa, ld3(J.pos, sf.C) - pa));
      if (dot(ng, rd) > 0.0f) n = n * -1.0f;
      const f3 ngf = dot(ng, n) < 0.0f ? ng * -1.0f : ng;
      p = (ro + rd * sf.h.t) + ngf * 1e-4f;
      const f3 Lv = lp - p;
      d2 = dot(Lv, Lv);
      dist = sqrtf(d2);
      l = Lv / dist;
      ndl = ref_max(0.0f, dot(n, l));
    }
    const bool occluded = point_shadow<WARP>(J, p, l, dist, hitb && ndl > 0.0f);
    if (hitb && ndl > 0.0f && !occluded) {
      const float k = I * ndl / (d2 * 3.14159265f);
      L = L + (beta * alb) * k;
      dL0 = dL0 + (bounce == 0 ? beta_na : beta_na * alb) * k;
    }
    if (bounce == J.mp.path_depth) break;
    if (hitb) {
      const float r1 = rnd01(key, (uint32_t)bounce, J.mp.seed);
      const float r2 = rnd01(key, (uint32_t)bounce + 1000u, J.mp.seed);
      float sphi, cphi;
      sincos_turns(r1, &sphi, &cphi);  // azimuth 2*pi*r1
      const float sr = sqrtf(r2);
      const f3 a = fabsf(n.x) > 0.5f ? mk(0, 1, 0) : mk(1, 0, 0);
      const f3 ex = normalize(cross(a, n));
      const f3 ey = cross(n, ex);
      const float lx = sr * cphi, ly = sr * sphi, lz = sqrtf(ref_max(0.0f, 1.0f - r2));
      rd = normalize((ex * lx + ey * ly) + n * lz);
      ro = p;
      beta_na = bounce == 0 ? beta_na : beta_na * alb;
      beta = beta * alb;
    }
    alive = hitb;
  }
  if (d_alb0) *d_alb0 = dL0;
  return L;
}

// ConcentricSampleDisk (shade_path_test.cpp:77-95; Shirley and Chiu's
// concentric map of the square onto the disk).  The angle of either wedge is
// reduced to [-pi/4, pi/4] (cos(pi/2 - b) = sin b, sin(pi/2 - b) = cos b) and
// evaluated by sincos_small, so the oracle draws the same directions.
__device__ __forceinline__ float2 concentric_disk(float u0, float u1) {
  const float ox = 2.0f * u0 - 1.0f, oy = 2.0f * u1 - 1.0f;
  if (ox == 0.0f && oy == 0.0f) return make_float2(0.0f, 0.0f);
  float sn, cs;
  if (fabsf(ox) > fabsf(oy)) {
    sincos_small(0.785398163f * (oy / ox), &sn, &cs);
    return make_float2(ox * cs, ox * sn);
  }
  sincos_small(0.785398163f * (ox / oy), &sn, &cs);
  return make_float2(oy * sn, oy * cs);
}

// Luminance of the throughput (intensity(), shade_path_test.cpp:75: double
// weights, rounded to float).
__device__ __forceinline__ float path_luminance(f3 c) {
  return (float)(0.2126 * (double)c.x + 0.7152 * (double)c.y + 0.0722 * (double)c.z);
}

// shade<PATH_TEST> (shade_path_test.cpp:183-282): up to 8 bounces with
// Russian roulette after the fourth, texture albedo, next-event estimation
// toward the point light of colour normalize(1,0.8,0.5) x 2 (PointLight
// normalises its colour, scene.h:77-82) at (0,0.7,0.7) jittered
// by +-0.1 per axis, ambient 0.5 for rays that leave the scene.  The shading
// frame is the interpolated (unnormalised) normal n and
// e_x = normalize(n x tangent), e_y = normalize(n x e_x); bounces are
// cosine-sampled in it and weighted by max(0, n_geom . dir) / pdf; a shadow
// ray counts every hit along its whole line (GetNearestHit without a far
// limit).  The reference draws from the shared rand(); here sample `key`,
// bounce b and the job seed index a counter-based hash: draws 8b..8b+2
// jitter the light, 8b+3 and 8b+4 pick the bounce, 8b+5 decides the
// roulette.  A path whose throughput is exactly zero stops (its further
// terms are all zero).  `alive` = the camera ray hit; every lane makes the
// same traversal calls until the whole warp's paths have ended.
template <bool WARP>
__device__ inline f3 path_test_p(const JobDev& J, const Surf& first, uint32_t key, bool alive) {
  constexpr float kPi = 3.14159265358979323846f;
  f3 L = mk(0.0f, 0.0f, 0.0f), beta = mk(1.0f, 1.0f, 1.0f);
  Surf sf = first;
  f3 ro = first.ro, rd = first.rd;
  for (int bounce = 0; bounce < 8; bounce++) {
    bool hitb = alive;
    if (bounce > 0) {
      Hit hh;
      hitb = trace_p<false, WARP>(J, ro, rd, 0.0f, 1e9f, alive, hh);
      if (alive && !hitb) L = L + beta * 0.5f;
      if (hitb) {
        sf.h = hh;
        const int4 tv = __ldg(J.tri_v + hh.tri);
        sf.A = tv.x;
        sf.B = tv.y;
        sf.C = tv.z;
        sf.block = tv.w;
      }
    }
    f3 p = mk(0.0f, 0.0f, 0.0f), l = mk(0.0f, 0.0f, 1.0f), n = mk(0.0f, 0.0f, 1.0f), ng = n, alb = n;
    f3 ex = mk(1.0f, 0.0f, 0.0f), ey = mk(0.0f, 1.0f, 0.0f);
    float ld = 1.0f;
    const uint32_t r0 = 8u * (uint32_t)bounce;
    if (hitb) {
      const float u = sf.h.u, v = sf.h.v;
      const MeshDev& m = J.meshes[J.blocks[sf.block].mesh];
      const float2 tc = interp_tc(J, sf);
      n = interp(ld3(J.nrm, sf.A), ld3(J.nrm, sf.B), ld3(J.nrm, sf.C), u, v);
      const f3 tg = interp(ld3(J.tan, sf.A), ld3(J.tan, sf.B), ld3(J.tan, sf.C), u, v);
      const f3 pa = ld3(J.pos, sf.A);
      ng = normalize(cross(ld3(J.pos, sf.B) - pa, ld3(J.pos, sf.C) - pa));
      p = (ro + rd * sf.h.t) + ng * 1e-4f;
      ex = normalize(cross(n, tg));
      ey = normalize(cross(n, ex));
      alb = sample_bilinear(tc.x, tc.y, m.tex_w, m.tex_h, m.tex);
      const f3 jit = mk(2.0f * rnd01(key, r0, J.mp.seed) - 1.0f, 2.0f * rnd01(key, r0 + 1u, J.mp.seed) - 1.0f,
                        2.0f * rnd01(key, r0 + 2u, J.mp.seed) - 1.0f);
      const f3 lv = (mk(0.0f, 0.7f, 0.7f) + jit * 0.1f) - p;
      ld = dot(lv, lv);
      l = lv / sqrtf(ld);
    }
    Hit sh;
    const bool occ = trace_p<true, WARP>(J, p, l, 0.0f, 1e9f, hitb, sh);
    if (hitb && !occ) {
      const f3 Li = (normalize(mk(1.0f, 0.8f, 0.5f)) * 2.0f) / ld;  // PointLight normalises its colour
      L = L + beta * (Li * ((alb / kPi) * ref_max(0.0f, dot(n, l))));
    }
    if (hitb) {
      const f3 wo = normalize(rd * -1.0f);
      const float woz = dot(wo, n);
      const float2 d = concentric_disk(rnd01(key, r0 + 3u, J.mp.seed), rnd01(key, r0 + 4u, J.mp.seed));
      float wz = sqrtf(ref_max(0.0f, 1.0f - d.x * d.x - d.y * d.y));
      if (woz < 0.0f) wz = -wz;
      const float pdf = woz * wz > 0.0f ? fabsf(wz) / kPi : 1e9f;
      const f3 nd = mk(ex.x * d.x + ey.x * d.y + n.x * wz, ex.y * d.x + ey.y * d.y + n.y * wz,
                       ex.z * d.x + ey.z * d.y + n.z * wz);
      beta = beta * (((alb / kPi) * ref_max(0.0f, dot(ng, nd))) / pdf);
      rd = nd;
      ro = p;
      if (bounce > 3) {
        const float q = ref_max(0.05f, 1.0f - path_luminance(beta));
        if (rnd01(key, r0 + 5u, J.mp.seed) < q) hitb = false;
        else beta = beta / (1.0f - q);
      }
      if (beta.x == 0.0f && beta.y == 0.0f && beta.z == 0.0f) hitb = false;
    }
    alive = hitb;
    if (WARP ? !__any_sync(0xffffffffu, alive) : !alive) break;
  }
  return L;
}

// Out of line for the generic shader, whose other models would otherwise
// share its register allocation.
static __device__ __noinline__ f3 path_test_call(const JobDev& J, const Surf& first, uint32_t key, bool alive) {
  return path_test_p<false>(J, first, key, alive);
}

// shade<M> for every model (shade_simple.cpp, shade_lambert.cpp).  MODE != 0
// compiles a single model (no code, hence no registers, for the others);
// MODE == 0 switches on the job's model at run time.  Inactive lanes return
// the background.
// Lit term of shade<PHONG> (shade_lambert.cpp:45-77): Kd*max(0,n.-L) +
// Ks*pow(max(0,n.r),32).  The reference's unqualified pow(float, int)
// resolves to pow(double, double), so the sum is formed in double and
// rounded to float where it multiplies the light colour.
__device__ __forceinline__ float phong_term(f3 n, f3 light_dir) {
  const float ndl = ref_max(0.0f, dot(n, light_dir * -1.0f));
  const f3 refl = light_dir - n * (2.0f * dot(n, light_dir));
  const double spec = pow((double)ref_max(0.0f, dot(n, refl)), 32.0);
  return (float)((double)(1.0f * ndl) + (double)1.0f * spec);
}

// LightingFuncGGX (shade_lambert.cpp:90-124) with the reference's float /
// double promotions: the D denominator and the Fresnel term are evaluated in
// double (double literals and pow) and stored to float.
__device__ __forceinline__ float ggx_specular(f3 N, f3 V, f3 L, float roughness, float F0) {
  const float alpha = roughness * roughness;
  const f3 H = normalize(V + L);
  const float dotNL = ref_max(0.0f, ref_min(1.0f, dot(N, L)));
  const float dotNV = ref_max(0.0f, ref_min(1.0f, dot(N, V)));
  const float dotNH = ref_max(0.0f, ref_min(1.0f, dot(N, H)));
  const float dotLH = ref_max(0.0f, ref_min(1.0f, dot(L, H)));
  const float alphaSqr = alpha * alpha;
  const float pi = 3.14159f;
  const float denom = (float)((double)(dotNH * dotNH) * ((double)alphaSqr - 1.0) + 1.0);
  const float D = alphaSqr / (pi * denom * denom);
  const float dotLH5 = (float)pow((double)(1.0f - dotLH), 5.0);
  const float F = (float)((double)F0 + (1.0 - (double)F0) * (double)dotLH5);
  const float k = alpha / 2.0f;
  const float vis = (1.0f / (dotNL * (1.0f - k) + k)) * (1.0f / (dotNV * (1.0f - k) + k));
  return dotNL * D * F * vis;
}

// Lit term of shade<GGX> (shade_lambert.cpp:128-161): max(0,n.-L) + GGX.
__device__ __forceinline__ float ggx_term(f3 n, f3 ray_dir, f3 light_dir) {
  const float ggx = ggx_specular(n, ray_dir * -1.0f, light_dir * -1.0f, 0.2f, 0.8f);
  return ref_max(0.0f, dot(n, light_dir * -1.0f)) + ggx;
}

// hit_tri (may be null) receives the camera ray's triangle, -1 on a miss.
// use_vis (uniform over the launch): the camera ray's hit is the sample's
// rasterised hit record vkey instead of a traversal (vkey is not read
// otherwise).
// view >= 0: the camera ray may come from the raster pass's tile lists of
// that view (see tiles_usable).
template <int MODE, bool WARP>
__device__ inline f3 shade_p(const JobDev& J, const CamDev& cam, float x, float y, uint32_t key, bool active,
                             int* hit_tri = nullptr, bool use_vis = false,
                             float4 vkey = float4{0.0f, 0.0f, 0.0f, 0.0f}, int view = -1,
                             const float2* vuv = nullptr) {
  const int mode = MODE ? MODE : J.mode;
  Surf s;
  const bool hit = use_vis ? cast_vis(J, cam, x, y, active, vkey, s, vuv, model_reads_ray(MODE))
                   : (!WARP && view >= 0 && tiles_usable(J, cam, view, x, y)) ? cast_tiles(J, cam, view, x, y, active, s)
                                                                       : cast_p<WARP>(J, cam, x, y, active, s);
  if (hit_tri) *hit_tri = hit ? s.h.tri : -1;
  const float u = s.h.u, v = s.h.v;
  switch (mode) {
    case SILHOUETTE:
      return hit ? mk(1.0f, 1.0f, 1.0f) : mk(0.0f, 0.0f, 0.0f);
    case VERTEX_COLOR:
      return hit ? interp(ld3(J.col, s.A), ld3(J.col, s.B), ld3(J.col, s.C), u, v) : mk(0.0f, 0.0f, 0.0f);
    case TEXTURE_COLOR: {
      if (!hit) return mk(0.0f, 0.0f, 0.0f);
      const MeshDev& m = J.meshes[J.blocks[s.block].mesh];
      const float2 tc = interp_tc(J, s);
      return sample_bilinear(tc.x, tc.y, m.tex_w, m.tex_h, m.tex);
    }
    case LAMBERT: {
      // light_dir = normalize(-1,-1,0), colour (1,0.5,0.2), ambient 0.1, BIAS 1e-5
      const f3 light_dir = normalize(mk(-1.0f, -1.0f, 0.0f));
      const f3 to_light = light_dir * -1.0f;
      f3 diffuse = mk(0.0f, 0.0f, 0.0f), surf_pos = mk(0.0f, 0.0f, 0.0f);
      float ndl = 0.0f;
      if (hit) {
        const MeshDev& m = J.meshes[J.blocks[s.block].mesh];
        const float2 tc = interp_tc(J, s);
        const f3 n = interp(ld3(J.nrm, s.A), ld3(J.nrm, s.B), ld3(J.nrm, s.C), u, v);
        diffuse = sample_bilinear(tc.x, tc.y, m.tex_w, m.tex_h, m.tex);
        surf_pos = s.ro + s.rd * (s.h.t - 1e-5f);
        ndl = ref_max(0.0f, dot(n, to_light));
      }
      // (colour * vis) * 0 is 0 for either visibility: trace only when lit
      Hit sh;
      const bool occ = trace_p<true, WARP>(J, surf_pos, to_light, 0.0f, 1e9f, hit && ndl > 0.0f, sh);
      if (!hit) return mk(0.0f, 0.0f, 0.0f);
      const f3 lit = (mk(1.0f, 0.5f, 0.2f) * (occ ? 0.0f : 1.0f)) * ndl;
      return (lit + mk(1.0f, 1.0f, 1.0f) * 0.1f) * diffuse;
    }
    case PHONG:
    case GGX: {
      // shade<PHONG> / shade<GGX>: light direction, colour (1,0.5,0.2),
      // ambient Ka*(1,1,1), shadow ray toward the light, times the texture
      const bool phong = mode == PHONG;
      const f3 light_dir = phong ? normalize(mk(0.0f, -0.25f, -1.0f)) : normalize(mk(0.15f, 0.0f, -1.0f));
      const f3 to_light = light_dir * -1.0f;
      f3 diffuse = mk(0.0f, 0.0f, 0.0f), surf_pos = mk(0.0f, 0.0f, 0.0f);
      float term = 0.0f;
      if (hit) {
        const MeshDev& m = J.meshes[J.blocks[s.block].mesh];
        const float2 tc = interp_tc(J, s);
        const f3 n = interp(ld3(J.nrm, s.A), ld3(J.nrm, s.B), ld3(J.nrm, s.C), u, v);
        diffuse = sample_bilinear(tc.x, tc.y, m.tex_w, m.tex_h, m.tex);
        surf_pos = s.ro + s.rd * (s.h.t - 1e-5f);
        term = phong ? phong_term(n, light_dir) : ggx_term(n, s.rd, light_dir);
      }
      // (colour * vis) * 0 is 0 for either visibility: trace only when lit
      Hit sh;
      const bool occ = trace_p<true, WARP>(J, surf_pos, to_light, 0.0f, 1e9f, hit && term != 0.0f, sh);
      if (!hit) return mk(0.0f, 0.0f, 0.0f);
      const f3 lit = (mk(1.0f, 0.5f, 0.2f) * (occ ? 0.0f : 1.0f)) * term;
      return (lit + mk(1.0f, 1.0f, 1.0f) * (phong ? 0.1f : 0.01f)) * diffuse;
    }
    case LAMBERT_POINT_VCOLOR: {
      const float k = lpv_factor_p<WARP>(J, s, hit);
      if (!hit) return mk(0.0f, 0.0f, 0.0f);
      return interp(ld3(J.col, s.A), ld3(J.col, s.B), ld3(J.col, s.C), u, v) * k;
    }
    case PATH_DIFFUSE: {
      const f3 r = path_diffuse_p<WARP>(J, s, key, hit, nullptr);
      return hit ? r : mk(J.mp.ambient, J.mp.ambient, J.mp.ambient);
    }
    case PATH_TEST: {
      const f3 r = (MODE == 0 && !WARP) ? path_test_call(J, s, key, hit) : path_test_p<WARP>(J, s, key, hit);
      return hit ? r : mk(0.5f, 0.5f, 0.5f);
    }
    default:
      return mk(0.0f, 0.0f, 0.0f);
  }
}

template <int MODE = 0>
__device__ inline f3 shade(const JobDev& J, const CamDev& cam, float x, float y, uint32_t key) {
  return shade_p<MODE, false>(J, cam, x, y, key, true);
}

// The generic shader as one out-of-line function (callers that shade
// several points keep a single copy of every model's code).
#ifdef DRGB_EDGE_SHADE_NOINLINE
static __device__ __noinline__ f3 shade_generic(const JobDev& J, const CamDev& cam, float x, float y, uint32_t key,
                                                int view = -1) {
  return shade_p<0, false>(J, cam, x, y, key, true, nullptr, false, float4{0.0f, 0.0f, 0.0f, 0.0f}, view);
}
#else
static __device__ __forceinline__ f3 shade_generic(const JobDev& J, const CamDev& cam, float x, float y,
                                                   uint32_t key, int view = -1) {
  return shade_p<0, false>(J, cam, x, y, key, true, nullptr, false, float4{0.0f, 0.0f, 0.0f, 0.0f}, view);
}
#endif

}  // namespace drgb
