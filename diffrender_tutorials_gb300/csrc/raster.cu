// Primary visibility by tile rasterisation (DRGB_OPT_PRIMARY_RASTER).
//
// The forward grid samples and the adjoint Hammersley samples of every
// pixel are camera rays whose nearest hit the reference finds with its
// brute-force caster (src/raytrace3d_bf.cpp:102-156).  Instead of tracing
// each through the hierarchy, triangles are binned to screen tiles and each
// tile resolves its samples against its own short list:
//
//   bin     : per (view, triangle) a conservative screen footprint -- the
//             projected triangle grown by RA_MARGIN pixels -- and the tiles
//             its box overlaps; per tile a count, an exclusive scan, then
//             the lists (view, triangle) filled through per-tile cursors;
//   resolve : one block per (view, tile).  The tile's triangles are staged
//             in shared memory with the screen edge lines the binning pass
//             stored for them; every thread
//             takes samples of the tile, builds the sample's camera ray once
//             (camera_ray, the reference's arithmetic) and runs the
//             reference's Moller-Trumbore test (mt_test) on each staged
//             triangle whose footprint holds the sample, keeping the minimum
//             {t bits, flattened triangle}: t > 0 orders as its float bits,
//             equal t keeps the lowest triangle -- the brute-force loop's
//             tie rule.  The hit {t, u, v, triangle} is written once per
//             sample (no atomics), and the pixel kernel shades from it.
// A hit that lies on its triangle projects inside it up to float rounding,
// far below the margin, so every such hit is among the candidates and the
// winner is the caster's nearest hit.  Not among them: the caster's
// clamped-determinant hits (|det| < 1e-6, reported at t = |(o-A).N|/1e-6,
// off the triangle), which a hierarchy does not find either.
//
// The lists live in a buffer of fixed capacity; a call whose lists do not
// fit sets the state word, the resolve pass then writes nothing and the
// pixel kernel traces its samples (same results), and the renderer doubles
// the capacity for the next call.
#include <cmath>

#include "engine.h"

namespace drgb {

constexpr float RA_MARGIN = 0.125f;  // pixels around the projected triangle
#ifndef DRGB_RA_THREADS
#define DRGB_RA_THREADS 256
#endif
constexpr int RA_THREADS = DRGB_RA_THREADS;  // threads of a resolve block, samples of a tile
constexpr int RA_STAGE = 64;         // triangles staged in shared memory at a time

struct RaTri {
  float x0, x1, y0, y1;     // footprint box in pixels (margin included, clipped to the image)
  bool edge_test;            // the three edge lines below are usable
  float nx[3], ny[3], c[3];  // inside (up to the margin) iff nx*x + ny*y + c >= 0 for all three
};

// Screen-space footprint of leaf triangle `leaf` in view `cam`.  false: no
// camera ray can hit it (entirely behind the camera, or off the image).
__device__ __forceinline__ bool ra_setup(const JobDev& J, const CamDev& cam, int leaf, RaTri& r) {
  const float W = cam.width, H = cam.height;
  const float4 a = __ldg(J.tri + 3 * leaf), e1 = __ldg(J.tri + 3 * leaf + 1), e2 = __ldg(J.tri + 3 * leaf + 2);
  const f3 P[3] = {f4to3(a), mk(a.x + e1.x, a.y + e1.y, a.z + e1.z), mk(a.x + e2.x, a.y + e2.y, a.z + e2.z)};
  const float* m = cam.wvp;
  float sx[3], sy[3];
  int behind = 0;
#pragma unroll
  for (int i = 0; i < 3; i++) {
    const float cw = P[i].x * m[3] + P[i].y * m[7] + P[i].z * m[11] + m[15];
    if (!(cw > 1e-6f)) {
      behind++;
      sx[i] = sy[i] = 0.0f;
      continue;
    }
    const float cx = P[i].x * m[0] + P[i].y * m[4] + P[i].z * m[8] + m[12];
    const float cy = P[i].x * m[1] + P[i].y * m[5] + P[i].z * m[9] + m[13];
    sx[i] = (cx / cw * 0.5f + 0.5f) * W;
    sy[i] = (-cy / cw * 0.5f + 0.5f) * H;
  }
  r.edge_test = false;
#pragma unroll
  for (int e = 0; e < 3; e++) r.nx[e] = r.ny[e] = r.c[e] = 0.0f;
  if (behind == 3) return false;  // a camera ray meets it at t < 0 only
  if (behind > 0) {  // crosses the camera plane: every sample is a candidate
    r.x0 = 0.0f; r.x1 = W; r.y0 = 0.0f; r.y1 = H;
    return true;
  }
  r.x0 = fmaxf(0.0f, fminf(sx[0], fminf(sx[1], sx[2])) - RA_MARGIN);
  r.x1 = fminf(W, fmaxf(sx[0], fmaxf(sx[1], sx[2])) + RA_MARGIN);
  r.y0 = fmaxf(0.0f, fminf(sy[0], fminf(sy[1], sy[2])) - RA_MARGIN);
  r.y1 = fminf(H, fmaxf(sy[0], fmaxf(sy[1], sy[2])) + RA_MARGIN);
  if (!(r.x0 <= r.x1 && r.y0 <= r.y1)) return false;  // off the image (or NaN)
  const float area2 = (sx[1] - sx[0]) * (sy[2] - sy[0]) - (sy[1] - sy[0]) * (sx[2] - sx[0]);
  const float big = 1e6f;
  const bool finite = fabsf(sx[0]) < big && fabsf(sx[1]) < big && fabsf(sx[2]) < big && fabsf(sy[0]) < big &&
                      fabsf(sy[1]) < big && fabsf(sy[2]) < big;
  if (finite && fabsf(area2) > 1e-3f) {
    const float s = area2 > 0.0f ? 1.0f : -1.0f;
    r.edge_test = true;
#pragma unroll
    for (int i = 0; i < 3; i++) {
      const int j = i == 2 ? 0 : i + 1;
      const float dx = sx[j] - sx[i], dy = sy[j] - sy[i];
      const float inv = 1.0f / sqrtf(dx * dx + dy * dy);
      r.nx[i] = -dy * inv * s;
      r.ny[i] = dx * inv * s;
      r.c[i] = -(r.nx[i] * sx[i] + r.ny[i] * sy[i]) + RA_MARGIN;
    }
  }
  return true;
}

// A lower bound on the distance from `o` of any point of triangle P: the
// distance to its centroid less its largest vertex distance, shrunk by a
// relative 1e-5 and 1e-6 for rounding (0 when o is that close).  A hit on
// the triangle at ray parameter t (unit direction) has t >= this bound, so a
// query that already holds a hit nearer than the bound can skip it.
__device__ __forceinline__ float dist_lower_bound(const f3 P[3], float ox, float oy, float oz) {
  const float cx = (P[0].x + P[1].x + P[2].x) * (1.0f / 3.0f), cy = (P[0].y + P[1].y + P[2].y) * (1.0f / 3.0f),
              cz = (P[0].z + P[1].z + P[2].z) * (1.0f / 3.0f);
  float rb = 0.0f;
#pragma unroll
  for (int i = 0; i < 3; i++) {
    const float dx = P[i].x - cx, dy = P[i].y - cy, dz = P[i].z - cz;
    rb = fmaxf(rb, sqrtf(dx * dx + dy * dy + dz * dz));
  }
  const float dx = cx - ox, dy = cy - oy, dz = cz - oz;
  const float lb = sqrtf(dx * dx + dy * dy + dz * dz) - rb * 1.0001f;
  return lb > 0.0f ? lb * (1.0f - 1e-5f) - 1e-6f : 0.0f;
}

// Orders each list (lengths 2..64; longer ones stay unsorted) by the lower
// bound in rec[4 * entry + 1].w, nearest first, so the queries meet the
// triangles that can win first and skip the rest by one comparison.  One
// warp per list, two entries per lane: an entry's place is the number of
// entries before it in the order (key, position in the list), counted
// against every key broadcast by shuffle; the keys compare as their bits
// mapped to an unsigned order (a total order, NaN included, so the places
// are distinct).  The queries' results do not depend on how equal keys are
// ordered.
__device__ __forceinline__ uint32_t key_order(float k) {
  const uint32_t u = __float_as_uint(k);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

__global__ void k_sort_lists(const uint32_t* offs, int n_lists, int* list, const float4* rec, uint32_t cap) {
  const int w = (int)(((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
  if (w >= n_lists || offs[n_lists] > cap) return;  // lists that did not fit were not filled
  const uint32_t i0 = offs[w], n = offs[w + 1] - i0;
  if (n < 2 || n > kSortedList) return;  // warp-uniform
  int* L = list + i0;
  const uint32_t ia = lane, ib = lane + 32;
  const int ea = ia < n ? L[ia] : 0, eb = ib < n ? L[ib] : 0;
  const uint32_t ka = ia < n ? key_order(rec[4 * ea + 1].w) : 0u;
  const uint32_t kb = ib < n ? key_order(rec[4 * eb + 1].w) : 0u;
  uint32_t ra = 0, rb = 0;
  for (uint32_t j = 0; j < n; j++) {
    const uint32_t kj = __shfl_sync(0xffffffffu, j < 32 ? ka : kb, (int)(j & 31));
    ra += (kj < ka || (kj == ka && j < ia)) ? 1u : 0u;
    rb += (kj < kb || (kj == kb && j < ib)) ? 1u : 0u;
  }
  __syncwarp();  // every lane has read its entries before any is moved
  if (ia < n) L[ra] = ea;
  if (ib < n) L[rb] = eb;
}

// Tile range of a footprint (tiles of tw x th pixels, ntx x nty per view).
__device__ __forceinline__ void ra_tiles(const RaTri& r, int tw, int th, int ntx, int nty, int& tx0, int& tx1,
                                         int& ty0, int& ty1) {
  tx0 = max(0, (int)floorf(r.x0) / tw);
  tx1 = min(ntx - 1, (int)floorf(r.x1) / tw);
  ty0 = max(0, (int)floorf(r.y0) / th);
  ty1 = min(nty - 1, (int)floorf(r.y1) / th);
}

// A footprint as the resolve pass reads it: box, then the three edge lines
// (all zero when unusable: 0 >= 0 holds), 16 floats.
struct __align__(16) RaRec {
  float4 box;         // x0, x1, y0, y1
  float4 l0, l1, l2;  // nx, ny, c; l0.w: lower bound on the hit distance (dist_lower_bound)
};

// PASS 0: each (view, leaf slot) thread j (view-major) stores its footprint
// record in `rec[j]` and counts itself in every tile its box overlaps;
// PASS 1: fills the lists with j.  `tiles` = per view ntx*nty counters, then
// (scanned) offsets with the total at [n_tiles]; `cursor` per tile; `list`
// of `cap` slots; `state` bit 0 set when the lists do not fit.
// One warp per (view, leaf): its lanes share the tiles of large footprints.
template <int PASS>
__global__ void k_bin(const JobDev* jobs, int tw, int th, int ntx, int nty, uint32_t* tiles, uint32_t* cursor,
                      int* list, uint32_t cap, uint32_t* state, RaRec* rec) {
  const JobDev& J = jobs[0];
  const int j = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (j >= J.n_views * J.n_tris) return;
  const int view = j / J.n_tris, leaf = j - view * J.n_tris;
  const int n_tiles = J.n_views * ntx * nty;
  if (PASS == 1 && tiles[n_tiles] > cap) {
    if (j == 0 && lane == 0) atomicOr(state, 1u);
    return;
  }
  RaTri r;
  const CamDev& cam = J.cams[view];
  const bool ok = ra_setup(J, cam, leaf, r);
  if (PASS == 0) {
    const float4 a = __ldg(J.tri + 3 * leaf), e1 = __ldg(J.tri + 3 * leaf + 1), e2 = __ldg(J.tri + 3 * leaf + 2);
    const f3 P[3] = {f4to3(a), mk(a.x + e1.x, a.y + e1.y, a.z + e1.z), mk(a.x + e2.x, a.y + e2.y, a.z + e2.z)};
    // the camera rays start at wv_inv * (0,0,0,1) (camera_ray)
    const float lb = dist_lower_bound(P, cam.wv_inv[12], cam.wv_inv[13], cam.wv_inv[14]);
    RaRec q;
    q.box = ok ? make_float4(r.x0, r.x1, r.y0, r.y1) : make_float4(1.0f, 0.0f, 1.0f, 0.0f);
    q.l0 = make_float4(r.nx[0], r.ny[0], r.c[0], lb);
    q.l1 = make_float4(r.nx[1], r.ny[1], r.c[1], 0.0f);
    q.l2 = make_float4(r.nx[2], r.ny[2], r.c[2], 0.0f);
    if (lane == 0) rec[j] = q;
  }
  if (!ok) return;
  int tx0, tx1, ty0, ty1;
  ra_tiles(r, tw, th, ntx, nty, tx0, tx1, ty0, ty1);
  const int base = view * ntx * nty;
  const int nx = tx1 - tx0 + 1, n = nx * (ty1 - ty0 + 1);
  for (int q = lane; q < n; q += 32) {
    const int ty = ty0 + q / nx, tx = tx0 + q % nx;
    const int t = base + ty * ntx + tx;
    if (PASS == 0) {
      atomicAdd(tiles + t, 1u);
    } else {
      const uint32_t pos = tiles[t] + atomicAdd(cursor + t, 1u);
      list[pos] = j;
    }
  }
}

// Sample s of a tile in pass `pass`: its pixel, index and position (the
// pixel kernel's float operations).
__device__ __forceinline__ bool ra_sample(const JobDev& J, int pass, int s, int tile_samples, int tx, int ty,
                                          int tw, int th, int W, int H, int& px, int& py, int& k, float& x,
                                          float& y) {
  const int S = J.S, sq = J.sq;
  const int p = s / S;
  k = s - p * S;
  px = tx * tw + p % tw;
  py = ty * th + p / tw;
  x = y = 0.0f;
  if (!(s < tile_samples && px < W && py < H)) return false;
  if (pass == 0) {
    const int dy = k / sq, dx = k - dy * sq;
    x = (float)px + (dx + 0.5f) / (float)sq;
    y = (float)py + (dy + 0.5f) / (float)sq;
  } else {
    x = (float)px + __ldg(J.ham + 2 * k);
    y = (float)py + __ldg(J.ham + 2 * k + 1);
  }
  return true;
}

// Nearest-hit update of one sample against staged triangle c.
__device__ __forceinline__ void ra_test(const float4* s_a, const float4* s_e1, const float4* s_e2,
                                        const RaRec* s_rec, int c, bool act, float x, float y, f3 ro, f3 rd,
                                        unsigned long long& best, float& bu, float& bv, unsigned& n_tests,
                                        unsigned& n_fp) {
  if (!act) return;
  const RaRec& q = s_rec[c];
  // no hit on this triangle can be nearer than the best so far (~0: none yet, NaN compares false)
  if (q.l0.w > __uint_as_float((uint32_t)(best >> 32))) return;
  n_fp++;
  if (!(x >= q.box.x && x <= q.box.y && y >= q.box.z && y <= q.box.w)) return;
  if (!(q.l0.x * x + q.l0.y * y + q.l0.z >= 0.0f && q.l1.x * x + q.l1.y * y + q.l1.z >= 0.0f &&
        q.l2.x * x + q.l2.y * y + q.l2.z >= 0.0f))
    return;
  const float4 a = s_a[c];
  float tt, u, v;
  n_tests++;
  if (mt_test(ro, rd, f4to3(a), f4to3(s_e1[c]), f4to3(s_e2[c]), 0.0f, tt, u, v) && tt < 1e9f) {
    const unsigned long long key = ((unsigned long long)__float_as_uint(tt) << 32) | (uint32_t)__float_as_int(a.w);
    if (key < best) {
      best = key;
      bu = u;
      bv = v;
    }
  }
}

// The hit record of a sample's best key: {t, u, v, triangle bits}, or a
// miss {1e9, 0, 0, -1}.
__device__ __forceinline__ float4 ra_hit(unsigned long long best, float u, float v) {
  if (best == ~0ull) return make_float4(1e9f, 0.0f, 0.0f, __int_as_float(-1));
  return make_float4(__uint_as_float((uint32_t)(best >> 32)), u, v, __int_as_float((int)(uint32_t)best));
}

// The point-light model's record: the shading point ro + rd * (t - 1e-5)
// (lpv_factor_p's arithmetic on the sample's own camera ray), the triangle,
// and u, v beside it.
__device__ __forceinline__ void ra_point(unsigned long long best, float u, float v, f3 ro, f3 rd, float4* rec,
                                         float2* uv) {
  if (best == ~0ull) {
    *rec = make_float4(0.0f, 0.0f, 0.0f, __int_as_float(-1));
    *uv = make_float2(0.0f, 0.0f);
    return;
  }
  const f3 p = ro + rd * (__uint_as_float((uint32_t)(best >> 32)) - 1e-5f);
  *rec = make_float4(p.x, p.y, p.z, __int_as_float((int)(uint32_t)best));
  *uv = make_float2(u, v);
}

// One block per (view, tile): the nearest hit of every forward (passes & 1)
// and adjoint (passes & 2) sample of the tile's pixels.  The tile's
// triangles are staged once per RA_STAGE for both passes; a thread holds
// one forward and one adjoint sample (tiles of at most RA_THREADS samples),
// whose two independent tests interleave.  Larger tiles (more than
// RA_THREADS samples per pixel) take their samples RA_THREADS at a time.
// Four resident blocks (64 registers): the unconstrained allocation (94
// registers, two blocks) ran the icosphere workload at 170.5 against 192.5
// iterations/s on GB300.
#ifndef DRGB_RESOLVE_MIN_BLOCKS
#define DRGB_RESOLVE_MIN_BLOCKS 4
#endif
__global__ void __launch_bounds__(RA_THREADS, DRGB_RESOLVE_MIN_BLOCKS) k_resolve(const JobDev* jobs, int passes, int tw, int th, int ntx,
                                                        int nty, const uint32_t* tiles, const int* list,
                                                        const uint32_t* state, const RaRec* rec) {
  __shared__ float4 s_a[RA_STAGE], s_e1[RA_STAGE], s_e2[RA_STAGE];  // A | id bits, e1, e2
  __shared__ RaRec s_rec[RA_STAGE];
  if (*state & 1u) return;  // lists did not fit: the pixel kernel traces
  const JobDev& J = jobs[0];
  const int b = blockIdx.x;
  const int per_view = ntx * nty;
  const int view = b / per_view, t = b - view * per_view;
  const int ty = t / ntx, tx = t - ty * ntx;
  const CamDev& cam = J.cams[view];
  const int W = (int)cam.width, H = (int)cam.height;
  const int S = J.S;
  const uint32_t l0 = tiles[b], l1 = tiles[b + 1];
  const int n_list = (int)(l1 - l0);
  const bool sorted = n_list <= RA_STAGE;  // k_sort_lists orders lists of up to 64
  const int64_t vbase = J.img_off[view];
  const int tile_samples = tw * th * S;
  const bool fwd = passes & 1, adj = (passes >> 1) & 1;
  for (int s0 = 0; s0 < tile_samples; s0 += RA_THREADS) {
    const int s = s0 + threadIdx.x;
    int px0, py0, k0, px1, py1, k1;
    float x0, y0, x1, y1;
    const bool a0 = fwd && ra_sample(J, 0, s, tile_samples, tx, ty, tw, th, W, H, px0, py0, k0, x0, y0);
    const bool a1 = adj && ra_sample(J, 1, s, tile_samples, tx, ty, tw, th, W, H, px1, py1, k1, x1, y1);
    f3 ro0 = mk(0.0f, 0.0f, 0.0f), rd0 = mk(0.0f, 0.0f, 1.0f), ro1 = ro0, rd1 = rd0;
    if (n_list > 0) {
      if (a0) camera_ray(cam, x0, y0, ro0, rd0);
      if (a1) camera_ray(cam, x1, y1, ro1, rd1);
    }
    unsigned long long b0 = ~0ull, b1 = ~0ull;
    float u0 = 0.0f, v0 = 0.0f, u1 = 0.0f, v1 = 0.0f;
    unsigned n_tests = 0, n_fp = 0;
    for (int c0 = 0; c0 < n_list; c0 += RA_STAGE) {
      const int nc = min(RA_STAGE, n_list - c0);
      if (c0 > 0 || s0 > 0) __syncthreads();  // the previous stage is no longer read
      if ((int)threadIdx.x < nc) {
        const int j = list[l0 + c0 + threadIdx.x];
        const int leaf = j - view * J.n_tris;
        s_a[threadIdx.x] = __ldg(J.tri + 3 * leaf);
        s_e1[threadIdx.x] = __ldg(J.tri + 3 * leaf + 1);
        s_e2[threadIdx.x] = __ldg(J.tri + 3 * leaf + 2);
        s_rec[threadIdx.x] = rec[j];
      }
      __syncthreads();
      for (int c = 0; c < nc; c++) {
        // a sorted list (one stage): once both samples hold hits nearer than
        // this entry's bound, no later entry can win either (no best yet:
        // NaN, the comparison fails)
        if (sorted) {
          const float lb = s_rec[c].l0.w;
          if ((!a0 || lb > __uint_as_float((uint32_t)(b0 >> 32))) &&
              (!a1 || lb > __uint_as_float((uint32_t)(b1 >> 32))))
            break;
        }
        ra_test(s_a, s_e1, s_e2, s_rec, c, a0, x0, y0, ro0, rd0, b0, u0, v0, n_tests, n_fp);
        ra_test(s_a, s_e1, s_e2, s_rec, c, a1, x1, y1, ro1, rd1, b1, u1, v1, n_tests, n_fp);
      }
    }
    // every sample of the tile is written, a miss too
    const int64_t i0 = (vbase + (int64_t)py0 * W + px0) * S + k0, i1 = (vbase + (int64_t)py1 * W + px1) * S + k1;
    if (J.vis_uv_fwd) {  // shading point + u, v (the same arithmetic as the shader's)
      if (a0) ra_point(b0, u0, v0, ro0, rd0, J.vis_fwd + i0, J.vis_uv_fwd + i0);
      if (a1) ra_point(b1, u1, v1, ro1, rd1, J.vis_adj + i1, J.vis_uv_adj + i1);
    } else {
      if (a0) J.vis_fwd[i0] = ra_hit(b0, u0, v0);
      if (a1) J.vis_adj[i1] = ra_hit(b1, u1, v1);
    }
    if (J.work && n_list > 0 && (a0 || a1)) {
      atomicAdd(J.work + 0, (unsigned long long)(a0 + a1));  // the samples' camera rays
      atomicAdd(J.work + 2, (unsigned long long)n_tests);
      atomicAdd(J.work + 3, (unsigned long long)n_fp);
    }
  }
}

// ---------------------------------------------------------------------------
// Shadow rays toward the point light (LAMBERT_POINT_VCOLOR, PATH_DIFFUSE).
// Every shadow ray runs from a surface point p to the light, so in a view
// from the light the whole segment sits at p's grid position: the triangles
// it can meet are those whose light-space footprint holds that position.
// The grid covers the scene's bounding sphere (from the leaf triangles); a
// light inside or near the sphere leaves the grid unusable (ok = 0) and the
// rays are traced.  Lists per cell as for the camera tiles.
// ---------------------------------------------------------------------------
constexpr int SH_THREADS = 1024;

__global__ void __launch_bounds__(SH_THREADS) k_light_grid(const JobDev* jobs, LightGrid* g, int G) {
  __shared__ float red[6][SH_THREADS / 32];
  const JobDev& J = jobs[0];
  const float inf = __int_as_float(0x7f800000);
  float lo[3] = {inf, inf, inf}, hi[3] = {-inf, -inf, -inf};
  for (int k = threadIdx.x; k < J.n_tris; k += SH_THREADS) {
    const float4 a = __ldg(J.tri + 3 * k), e1 = __ldg(J.tri + 3 * k + 1), e2 = __ldg(J.tri + 3 * k + 2);
    const float P[3][3] = {{a.x, a.y, a.z}, {a.x + e1.x, a.y + e1.y, a.z + e1.z}, {a.x + e2.x, a.y + e2.y, a.z + e2.z}};
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int c = 0; c < 3; c++) {
        lo[c] = fminf(lo[c], P[i][c]);
        hi[c] = fmaxf(hi[c], P[i][c]);
      }
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int c = 0; c < 3; c++) {
    for (int o = 16; o > 0; o >>= 1) {
      lo[c] = fminf(lo[c], __shfl_xor_sync(0xffffffffu, lo[c], o));
      hi[c] = fmaxf(hi[c], __shfl_xor_sync(0xffffffffu, hi[c], o));
    }
    if (lane == 0) {
      red[c][warp] = lo[c];
      red[3 + c][warp] = hi[c];
    }
  }
  __syncthreads();
  if (threadIdx.x != 0) return;
  for (int w = 1; w < SH_THREADS / 32; w++)
    for (int c = 0; c < 3; c++) {
      red[c][0] = fminf(red[c][0], red[c][w]);
      red[3 + c][0] = fmaxf(red[3 + c][0], red[3 + c][w]);
    }
  LightGrid q;
  q.lx = J.mp.light_pos[0];
  q.ly = J.mp.light_pos[1];
  q.lz = J.mp.light_pos[2];
  const float cx = 0.5f * (red[0][0] + red[3][0]), cy = 0.5f * (red[1][0] + red[4][0]),
              cz = 0.5f * (red[2][0] + red[5][0]);
  const float ex = red[3][0] - red[0][0], ey = red[4][0] - red[1][0], ez = red[5][0] - red[2][0];
  const float r = 0.5f * sqrtf(ex * ex + ey * ey + ez * ez) * 1.001f + 1e-6f;
  float wx = cx - q.lx, wy = cy - q.ly, wz = cz - q.lz;
  const float d = sqrtf(wx * wx + wy * wy + wz * wz);
  q.G = G;
  q.valid = 0;
  q.overflow = 0;
  q.ok = J.n_tris > 0 && d > 1.05f * r && isfinite(d);
  if (q.ok) {
    wx /= d; wy /= d; wz /= d;
    // u = normalize(up x w), v = w x u, up the axis least aligned with w
    const bool yup = fabsf(wy) < 0.9f;
    const float upx = yup ? 0.0f : 1.0f, upy = yup ? 1.0f : 0.0f;
    float ux = upy * wz, uy = -upx * wz, uz = upx * wy - upy * wx;
    const float ul = sqrtf(ux * ux + uy * uy + uz * uz);
    ux /= ul; uy /= ul; uz /= ul;
    q.ux = ux; q.uy = uy; q.uz = uz;
    q.vx = wy * uz - wz * uy; q.vy = wz * ux - wx * uz; q.vz = wx * uy - wy * ux;
    q.wx = wx; q.wy = wy; q.wz = wz;
    const float sn = r / d;
    const float tn = sn / sqrtf(1.0f - sn * sn) * 1.02f;  // tangent of the cone around the sphere
    q.half = 0.5f * (float)G;
    q.scale = q.half / tn;
  } else {
    q.ux = q.uy = q.uz = q.vx = q.vy = q.vz = q.wx = q.wy = q.wz = 0.0f;
    q.half = q.scale = 0.0f;
  }
  *g = q;
}

// PASS 0: footprint record of leaf k and its cell counts; PASS 1: the
// lists.  One warp per leaf.
template <int PASS>
__global__ void k_light_bin(const JobDev* jobs, LightGrid* g, uint32_t* cells, uint32_t* cursor, int* list,
                            uint32_t cap, float4* rec) {
  const JobDev& J = jobs[0];
  const int k = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (k >= J.n_tris || !g->ok) return;
  const int G = g->G;
  if (PASS == 1 && cells[G * G] > cap) {
    if (k == 0 && lane == 0) g->overflow = 1;
    return;
  }
  const float4 a = __ldg(J.tri + 3 * k), e1 = __ldg(J.tri + 3 * k + 1), e2 = __ldg(J.tri + 3 * k + 2);
  const f3 P[3] = {f4to3(a), mk(a.x + e1.x, a.y + e1.y, a.z + e1.z), mk(a.x + e2.x, a.y + e2.y, a.z + e2.z)};
  float sa[3], sb[3];
#pragma unroll
  for (int i = 0; i < 3; i++) light_project(*g, P[i], sa[i], sb[i]);
  const float x0 = fminf(sa[0], fminf(sa[1], sa[2])) - RA_MARGIN, x1 = fmaxf(sa[0], fmaxf(sa[1], sa[2])) + RA_MARGIN;
  const float y0 = fminf(sb[0], fminf(sb[1], sb[2])) - RA_MARGIN, y1 = fmaxf(sb[0], fmaxf(sb[1], sb[2])) + RA_MARGIN;
  if (PASS == 0) {
    float4 L[3] = {make_float4(0, 0, 0, 0), make_float4(0, 0, 0, 0), make_float4(0, 0, 0, 0)};
    const float area2 = (sa[1] - sa[0]) * (sb[2] - sb[0]) - (sb[1] - sb[0]) * (sa[2] - sa[0]);
    if (fabsf(area2) > 1e-6f) {
      const float sg = area2 > 0.0f ? 1.0f : -1.0f;
#pragma unroll
      for (int i = 0; i < 3; i++) {
        const int j = i == 2 ? 0 : i + 1;
        const float dx = sa[j] - sa[i], dy = sb[j] - sb[i];
        const float inv = 1.0f / sqrtf(dx * dx + dy * dy);
        const float nx = -dy * inv * sg, ny = dx * inv * sg;
        L[i] = make_float4(nx, ny, -(nx * sa[i] + ny * sb[i]) + RA_MARGIN, 0.0f);
      }
    }
    // shadow rays end at the light: a triangle no nearer to it than the ray's origin is not in the way
    L[0].w = dist_lower_bound(P, g->lx, g->ly, g->lz);
    if (lane == 0) {
      rec[4 * k + 0] = make_float4(x0, x1, y0, y1);
      rec[4 * k + 1] = L[0];
      rec[4 * k + 2] = L[1];
      rec[4 * k + 3] = L[2];
    }
  }
  const int cx0 = min(G - 1, max(0, (int)floorf(x0))), cx1 = min(G - 1, max(0, (int)floorf(x1)));
  const int cy0 = min(G - 1, max(0, (int)floorf(y0))), cy1 = min(G - 1, max(0, (int)floorf(y1)));
  const int nx = cx1 - cx0 + 1, n = nx * (cy1 - cy0 + 1);
  for (int q = lane; q < n; q += 32) {
    const int c = (cy0 + q / nx) * G + cx0 + q % nx;
    if (PASS == 0) {
      atomicAdd(cells + c, 1u);
    } else {
      const uint32_t pos = cells[c] + atomicAdd(cursor + c, 1u);
      list[pos] = k;
    }
  }
}

__global__ void k_light_valid(LightGrid* g) { g->valid = g->ok && !g->overflow; }

// Light-space cells of the current geometry (grid G x G).
void launch_light_grid(const JobDev* d_job, const Job& J, int G, cudaStream_t s) {
  LightGrid* g = J.sh_grid.p;
  const int n_cells = G * G;
  DRGB_CUDA(cudaMemsetAsync(J.sh_cells.p, 0, sizeof(uint32_t) * (n_cells + 1), s));
  DRGB_CUDA(cudaMemsetAsync(J.sh_cursor.p, 0, sizeof(uint32_t) * n_cells, s));
  k_light_grid<<<1, SH_THREADS, 0, s>>>(d_job, g, G);
  const int grid = (int)(((int64_t)J.n_tris * 32 + 255) / 256);
  k_light_bin<0><<<grid, 256, 0, s>>>(d_job, g, J.sh_cells.p, J.sh_cursor.p, J.sh_list.p, (uint32_t)J.sh_list.n,
                                      J.sh_rec.p);
  launch_rs_scan(J.sh_cells.p, n_cells + 1, s);
  k_light_bin<1><<<grid, 256, 0, s>>>(d_job, g, J.sh_cells.p, J.sh_cursor.p, J.sh_list.p, (uint32_t)J.sh_list.n,
                                      J.sh_rec.p);
  k_sort_lists<<<(int)(((int64_t)n_cells * 32 + 255) / 256), 256, 0, s>>>(J.sh_cells.p, n_cells, J.sh_list.p, J.sh_rec.p,
                                                      (uint32_t)J.sh_list.n);
  k_light_valid<<<1, 1, 0, s>>>(g);
  count_launch(5);
}

// Cells per side of the light grid for n triangles (a few cells each).
int light_grid_size(int n_tris) {
  int G = (int)(2.0 * std::sqrt((double)std::max(1, n_tris)));
  return std::min(1024, std::max(32, (G + 7) / 8 * 8));
}

// The lists hold the current geometry unless they did not fit.
__global__ void k_tiles_valid(uint32_t* state) {
  if (!(*state & 1u)) *state |= 2u;
}

// Tile shape for S samples per pixel: square, at most RA_THREADS samples.
void raster_tile(int S, int& tw, int& th) {
  int d = 1;
  while ((d + 1) * (d + 1) * S <= RA_THREADS) d++;
  tw = th = d;
}

void launch_raster(const JobDev* d_job, const Job& J, int passes, int ntx, int nty, int tw, int th,
                   cudaStream_t s) {
  const int n_tiles = J.n_views * ntx * nty;
  const int tasks = J.n_views * J.n_tris;
  uint32_t* tiles = J.ra_tiles.p;
  uint32_t* cursor = J.ra_cursor.p;
  uint32_t* state = J.ra_state.p;
  DRGB_CUDA(cudaMemsetAsync(tiles, 0, sizeof(uint32_t) * (n_tiles + 1), s));
  DRGB_CUDA(cudaMemsetAsync(cursor, 0, sizeof(uint32_t) * n_tiles, s));
  DRGB_CUDA(cudaMemsetAsync(state, 0, sizeof(uint32_t), s));
  const int grid = (int)(((int64_t)tasks * 32 + 255) / 256);
  RaRec* rec = reinterpret_cast<RaRec*>(J.ra_rec.p);
  k_bin<0><<<grid, 256, 0, s>>>(d_job, tw, th, ntx, nty, tiles, cursor, J.ra_list.p, (uint32_t)J.ra_list.n, state,
                                rec);
  launch_rs_scan(tiles, n_tiles + 1, s);
  k_bin<1><<<grid, 256, 0, s>>>(d_job, tw, th, ntx, nty, tiles, cursor, J.ra_list.p, (uint32_t)J.ra_list.n, state,
                                rec);
  k_sort_lists<<<(int)(((int64_t)n_tiles * 32 + 255) / 256), 256, 0, s>>>(tiles, n_tiles, J.ra_list.p, J.ra_rec.p,
                                                     (uint32_t)J.ra_list.n);
  k_resolve<<<n_tiles, RA_THREADS, 0, s>>>(d_job, passes, tw, th, ntx, nty, tiles, J.ra_list.p, state, rec);
  k_tiles_valid<<<1, 1, 0, s>>>(state);
  count_launch(5);
}

}  // namespace drgb
