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
//             the lists (triangle leaf slots) filled through per-tile cursors;
//   resolve : one block per (view, tile).  The tile's triangles are staged
//             in shared memory with their screen edge lines; every thread
//             takes samples of the tile, builds the sample's camera ray once
//             (camera_ray, the reference's arithmetic) and runs the
//             reference's Moller-Trumbore test (mt_test) on each staged
//             triangle whose footprint holds the sample, keeping the minimum
//             {t bits, flattened triangle}: t > 0 orders as its float bits,
//             equal t keeps the lowest triangle -- the brute-force loop's
//             tie rule.  The key is written once per sample (no atomics).
//
// The pixel kernel then re-runs mt_test on the winning triangle for t, u, v.
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
#include "engine.h"

namespace drgb {

constexpr float RA_MARGIN = 0.125f;  // pixels around the projected triangle
constexpr int RA_THREADS = 256;
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

// Tile range of a footprint (tiles of tw x th pixels, ntx x nty per view).
__device__ __forceinline__ void ra_tiles(const RaTri& r, int tw, int th, int ntx, int nty, int& tx0, int& tx1,
                                         int& ty0, int& ty1) {
  tx0 = max(0, (int)floorf(r.x0) / tw);
  tx1 = min(ntx - 1, (int)floorf(r.x1) / tw);
  ty0 = max(0, (int)floorf(r.y0) / th);
  ty1 = min(nty - 1, (int)floorf(r.y1) / th);
}

// PASS 0: count triangles per tile; PASS 1: fill the lists.  Thread j =
// (view, leaf slot), view-major.  `tiles` = per view ntx*nty counters, then
// (scanned) offsets with the total at [n_tiles]; `cursor` per tile; `list`
// of `cap` slots; `state` bit 0 set when the lists do not fit.
template <int PASS>
__global__ void k_bin(const JobDev* jobs, int tw, int th, int ntx, int nty, uint32_t* tiles, uint32_t* cursor,
                      int* list, uint32_t cap, uint32_t* state) {
  const JobDev& J = jobs[0];
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= J.n_views * J.n_tris) return;
  const int view = j / J.n_tris, leaf = j - view * J.n_tris;
  const int n_tiles = J.n_views * ntx * nty;
  if (PASS == 1 && tiles[n_tiles] > cap) {
    if (j == 0) atomicOr(state, 1u);
    return;
  }
  RaTri r;
  if (!ra_setup(J, J.cams[view], leaf, r)) return;
  int tx0, tx1, ty0, ty1;
  ra_tiles(r, tw, th, ntx, nty, tx0, tx1, ty0, ty1);
  const int base = view * ntx * nty;
  for (int ty = ty0; ty <= ty1; ty++)
    for (int tx = tx0; tx <= tx1; tx++) {
      const int t = base + ty * ntx + tx;
      if (PASS == 0) {
        atomicAdd(tiles + t, 1u);
      } else {
        const uint32_t pos = tiles[t] + atomicAdd(cursor + t, 1u);
        list[pos] = leaf;
      }
    }
}

// One block per (view, tile): the nearest hit of every forward (passes & 1)
// and adjoint (passes & 2) sample of the tile's pixels.
__global__ void __launch_bounds__(RA_THREADS) k_resolve(const JobDev* jobs, int passes, int tw, int th, int ntx,
                                                        int nty, const uint32_t* tiles, const int* list,
                                                        const uint32_t* state) {
  __shared__ float4 s_a[RA_STAGE], s_e1[RA_STAGE], s_e2[RA_STAGE];  // A | id bits, e1, e2
  __shared__ float s_box[RA_STAGE][4];
  __shared__ float s_lin[RA_STAGE][9];
  __shared__ int s_lines[RA_STAGE];
  if (*state & 1u) return;  // lists did not fit: the pixel kernel traces
  const JobDev& J = jobs[0];
  const int b = blockIdx.x;
  const int per_view = ntx * nty;
  const int view = b / per_view, t = b - view * per_view;
  const int ty = t / ntx, tx = t - ty * ntx;
  const CamDev& cam = J.cams[view];
  const int W = (int)cam.width, H = (int)cam.height;
  const int S = J.S, sq = J.sq;
  const uint32_t l0 = tiles[b], l1 = tiles[b + 1];
  const int n_list = (int)(l1 - l0);
  const int64_t vbase = J.img_off[view];
  const int tile_samples = tw * th * S;
  for (int pass = 0; pass < 2; pass++) {
    if (!((passes >> pass) & 1)) continue;
    unsigned long long* vis = pass == 0 ? J.vis_fwd : J.vis_adj;
    // every sample of the tile is written: a miss as ~0
    for (int s0 = 0; s0 < tile_samples; s0 += RA_THREADS) {
      const int s = s0 + threadIdx.x;
      const int p = s / S, k = s - p * S;
      const int px = tx * tw + p % tw, py = ty * th + p / tw;
      const bool act = s < tile_samples && px < W && py < H;
      float x = 0.0f, y = 0.0f;
      if (act) {
        if (pass == 0) {
          const int dy = k / sq, dx = k - dy * sq;
          x = (float)px + (dx + 0.5f) / (float)sq;  // the pixel kernel's grid position
          y = (float)py + (dy + 0.5f) / (float)sq;
        } else {
          x = (float)px + __ldg(J.ham + 2 * k);
          y = (float)py + __ldg(J.ham + 2 * k + 1);
        }
      }
      f3 ro = mk(0.0f, 0.0f, 0.0f), rd = mk(0.0f, 0.0f, 1.0f);
      if (act && n_list > 0) camera_ray(cam, x, y, ro, rd);
      unsigned long long best = ~0ull;
      unsigned n_tests = 0;
      for (int c0 = 0; c0 < n_list; c0 += RA_STAGE) {
        const int nc = min(RA_STAGE, n_list - c0);
        __syncthreads();  // the previous stage is no longer read
        if ((int)threadIdx.x < nc) {
          const int leaf = list[l0 + c0 + threadIdx.x];
          RaTri r;
          const bool ok = ra_setup(J, cam, leaf, r);
          s_a[threadIdx.x] = __ldg(J.tri + 3 * leaf);
          s_e1[threadIdx.x] = __ldg(J.tri + 3 * leaf + 1);
          s_e2[threadIdx.x] = __ldg(J.tri + 3 * leaf + 2);
          // an empty box (x0 > x1) for a footprint that turned out empty
          s_box[threadIdx.x][0] = ok ? r.x0 : 1.0f;
          s_box[threadIdx.x][1] = ok ? r.x1 : 0.0f;
          s_box[threadIdx.x][2] = ok ? r.y0 : 1.0f;
          s_box[threadIdx.x][3] = ok ? r.y1 : 0.0f;
          s_lines[threadIdx.x] = ok && r.edge_test;
#pragma unroll
          for (int e = 0; e < 3; e++) {
            s_lin[threadIdx.x][3 * e + 0] = r.nx[e];
            s_lin[threadIdx.x][3 * e + 1] = r.ny[e];
            s_lin[threadIdx.x][3 * e + 2] = r.c[e];
          }
        }
        __syncthreads();
        if (act) {
          for (int c = 0; c < nc; c++) {
            if (!(x >= s_box[c][0] && x <= s_box[c][1] && y >= s_box[c][2] && y <= s_box[c][3])) continue;
            if (s_lines[c]) {
              const float* L = s_lin[c];
              if (!(L[0] * x + L[1] * y + L[2] >= 0.0f && L[3] * x + L[4] * y + L[5] >= 0.0f &&
                    L[6] * x + L[7] * y + L[8] >= 0.0f))
                continue;
            }
            const float4 a = s_a[c];
            float tt, u, v;
            n_tests++;
            if (mt_test(ro, rd, f4to3(a), f4to3(s_e1[c]), f4to3(s_e2[c]), 0.0f, tt, u, v) && tt < 1e9f) {
              const unsigned long long key =
                  ((unsigned long long)__float_as_uint(tt) << 32) | (uint32_t)__float_as_int(a.w);
              best = key < best ? key : best;
            }
          }
        }
      }
      if (act) vis[(vbase + (int64_t)py * W + px) * S + k] = best;
      if (J.work && act && n_list > 0) {
        atomicAdd(J.work + 0, 1ull);  // the sample's camera ray
        atomicAdd(J.work + 2, (unsigned long long)n_tests);
      }
    }
  }
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
  const int grid = (tasks + 255) / 256;
  k_bin<0><<<grid, 256, 0, s>>>(d_job, tw, th, ntx, nty, tiles, cursor, J.ra_list.p, (uint32_t)J.ra_list.n, state);
  launch_rs_scan(tiles, n_tiles + 1, s);
  k_bin<1><<<grid, 256, 0, s>>>(d_job, tw, th, ntx, nty, tiles, cursor, J.ra_list.p, (uint32_t)J.ra_list.n, state);
  k_resolve<<<n_tiles, RA_THREADS, 0, s>>>(d_job, passes, tw, th, ntx, nty, tiles, J.ra_list.p, state);
  count_launch(3);
}

}  // namespace drgb
