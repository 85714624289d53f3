// Fused pixel kernel: forward render, MSE loss with its adjoint, and the
// interior adjoint, one tile of pixels per work item.
//
//  * forward: DiffRender::render (src/drender.h:98-141) -- the sq x sq grid
//    of sub-pixel centres, colours summed in the reference's order;
//  * loss: LossAndDiffLoss (src/utils.cpp:15-27) -- adjoint 2*(I-T), squared
//    error accumulated in double;
//  * interior adjoint: interior_derivatives (src/drender.h:197-233) with
//    shade_grad<M> -- the first S Hammersley points of planeHammersley(spp),
//    visibility re-traced rather than stored.
//
// The pixel's adjoint is known as soon as its forward samples are summed,
// so the interior pass runs in the same block right after the forward pass.
// Vertex-colour gradients are summed per triangle across the warp before
// one lane issues the global atomics.  Work items are taken from an atomic
// queue by a persistent grid, so one launch covers any number of jobs,
// views and tile shapes.
#include "engine.h"

namespace drgb {

constexpr int PX_THREADS = 256;

// Traversal policy of the pixel kernel: per-ray by default (measured faster
// on GB300 for the icosphere workload: 78 vs 73 iterations/s); build with
// -DDRGB_PIXEL_WARP_TRACE for the warp-coherent traversal.
#ifdef DRGB_PIXEL_WARP_TRACE
constexpr bool kPixelWarp = true;
#else
constexpr bool kPixelWarp = false;
#endif

// Warp-aggregated scatter of per-vertex colour gradients.  All 32 lanes
// must call it; lanes without a contribution pass tri = -1.  The lanes that
// hit one triangle form a group; for each group (in order of its lowest
// lane) lanes 0-8 each sum one of the 9 values over the group's lanes in
// lane order, then add it with one atomic each (or, in deterministic mode,
// lane 0 writes the group's 3 records at rec_base + rec_n; rec_n: records of
// this work item so far, warp-uniform).
template <bool DET>
__device__ __forceinline__ void scatter_vertex_colors(const JobDev& J, int tri, int gA, int gB, int gC,
                                                      const float c[9], float* wscr, int64_t rec_base, int& rec_n) {
  const int lane = threadIdx.x & 31;
  const unsigned peers = __match_any_sync(0xffffffffu, tri);
#pragma unroll
  for (int i = 0; i < 9; i++) wscr[i * 32 + lane] = c[i];
  __syncwarp();
  unsigned leaders = __ballot_sync(0xffffffffu, tri >= 0 && lane == __ffs(peers) - 1);
  while (leaders) {
    const int ld = __ffs(leaders) - 1;
    leaders &= leaders - 1;
    const unsigned group = __shfl_sync(0xffffffffu, peers, ld);
    const int t = __shfl_sync(0xffffffffu, tri, ld);
    const int vA = __shfl_sync(0xffffffffu, gA, ld), vB = __shfl_sync(0xffffffffu, gB, ld);
    const int vC = __shfl_sync(0xffffffffu, gC, ld);
    float sum = 0.0f;
    if (lane < 9) {
      unsigned m = group;
      while (m) {
        const int l = __ffs(m) - 1;
        m &= m - 1;
        sum += wscr[lane * 32 + l];
      }
    }
    const int b = __ldg(J.tri_v + t).w;
    const BlockDev bd = J.blocks[b];
    const MeshDev& md = J.meshes[bd.mesh];
    if (md.dslot < 0) continue;  // warp-uniform: the group's mesh
    float* g = J.grad + md.g_base + md.color_off;
    const int vert = (lane < 3 ? vA : lane < 6 ? vB : vC) - bd.vert_off;
    if (DET && J.det) {
      float v[9];
#pragma unroll
      for (int i = 0; i < 9; i++) v[i] = __shfl_sync(0xffffffffu, sum, i);
      if (lane == 0) {
        const int64_t slot = rec_base + rec_n;
        const uint32_t k0 = (uint32_t)(g - J.grad);
        J.rec_key[slot + 0] = k0 + 3 * (vA - bd.vert_off);
        J.rec_val[slot + 0] = make_float4(v[0], v[1], v[2], 0.0f);
        J.rec_key[slot + 1] = k0 + 3 * (vB - bd.vert_off);
        J.rec_val[slot + 1] = make_float4(v[3], v[4], v[5], 0.0f);
        J.rec_key[slot + 2] = k0 + 3 * (vC - bd.vert_off);
        J.rec_val[slot + 2] = make_float4(v[6], v[7], v[8], 0.0f);
      }
      rec_n += 3;
    } else if (lane < 9) {
      atomicAdd(g + 3 * vert + lane % 3, sum);
    }
  }
  __syncwarp();
}

// sample_bilinear_clamp_3f_grad (shade_common.cpp:23-46): the four taps
// and their weights; data points at the texture's gradient block.
__device__ __forceinline__ void texture_taps(f3 val, float tx, float ty, int w, int h, int idx[4], f3 v[4]) {
  const float px = tx * (float)w, py = ty * (float)h;
  const int ix = (int)px, iy = (int)py;
  const int x0 = clampi(ix, 0, w - 1), y0 = clampi(iy, 0, h - 1);
  const int x1 = clampi(ix + 1, 0, w - 1), y1 = clampi(iy + 1, 0, h - 1);
  const float dx = px - (float)x0, dy = py - (float)y0;
  idx[0] = 3 * (y0 * w + x0);
  idx[1] = 3 * (y1 * w + x0);
  idx[2] = 3 * (y0 * w + x1);
  idx[3] = 3 * (y1 * w + x1);
  const float w00 = (1 - dx) * (1 - dy), w01 = (1 - dx) * dy, w10 = dx * (1 - dy), w11 = dx * dy;
  v[0] = val * w00;
  v[1] = val * w01;
  v[2] = val * w10;
  v[3] = val * w11;
}

// All 32 lanes call it; lanes with g == nullptr contribute nothing.
template <bool DET>
__device__ __forceinline__ void texture_grad(const JobDev& J, float* g, f3 val, float tx, float ty, int w, int h,
                                             int64_t rec_base, int& rec_n) {
  const int lane = threadIdx.x & 31;
  int idx[4];
  f3 v[4];
  if (g) texture_taps(val, tx, ty, w, h, idx, v);
  if (DET && J.det) {
    const unsigned writers = __ballot_sync(0xffffffffu, g != nullptr);
    if (g) {
      const int64_t slot = rec_base + rec_n + 4 * __popc(writers & ((1u << lane) - 1u));
      const uint32_t k0 = (uint32_t)(g - J.grad);
#pragma unroll
      for (int k = 0; k < 4; k++) {
        J.rec_key[slot + k] = k0 + idx[k];
        J.rec_val[slot + k] = make_float4(v[k].x, v[k].y, v[k].z, 0.0f);
      }
    }
    rec_n += 4 * __popc(writers);
  } else if (g) {
#pragma unroll
    for (int k = 0; k < 4; k++) {
      atomicAdd(g + idx[k] + 0, v[k].x);
      atomicAdd(g + idx[k] + 1, v[k].y);
      atomicAdd(g + idx[k] + 2, v[k].z);
    }
  }
}

// shade_grad<M> for one sample; every lane of the warp must call it.  MODE
// as for shade().
// HITS: the sample's primary hit comes from the stored hit buffer (written by
// a PX_HIT_STORE launch) instead of being traced again.
template <int MODE, bool DET, bool HITS>
__device__ __forceinline__ void shade_grad(const JobDev& J, const CamDev& cam, bool active, float x, float y, f3 val,
                                           uint32_t key, float* wscr, int64_t rec_base, int& rec_n,
                                           const float4* stored, int seed, bool use_vis, float4 vkey,
                                           const float2* vuv) {
  const int mode = MODE ? MODE : J.mode;
  Surf s;
  bool hit;
  if (HITS) {
    camera_ray(cam, x, y, s.ro, s.rd);
    const float4 hb = *stored;
    s.h.t = hb.x;
    s.h.u = hb.y;
    s.h.v = hb.z;
    s.h.tri = __float_as_int(hb.w);
    hit = active && s.h.tri >= 0;
    s.A = s.B = s.C = s.block = 0;
    if (hit) {
      const int4 tv = __ldg(J.tri_v + s.h.tri);
      s.A = tv.x;
      s.B = tv.y;
      s.C = tv.z;
      s.block = tv.w;
    }
  } else if (use_vis) {
    // the gradients of the vertex-colour and texture models read u, v only
    hit = cast_vis(J, cam, x, y, active, vkey, s, vuv,
                   MODE == 0 || mode == LAMBERT_POINT_VCOLOR || mode == PATH_DIFFUSE);
  } else {
    hit = cast_p<kPixelWarp>(J, cam, x, y, active, s, seed);
  }
  if (model_has_color(mode)) {
    float c[9];
    int tri = -1, gA = 0, gB = 0, gC = 0;
#pragma unroll
    for (int i = 0; i < 9; i++) c[i] = 0.0f;
    // warp-collective traversals first, then the per-lane arithmetic
    float k = 1.0f;
    f3 d0 = mk(0.0f, 0.0f, 0.0f);
    if (mode == LAMBERT_POINT_VCOLOR) k = lpv_factor_p<kPixelWarp>(J, s, hit);
    if (mode == PATH_DIFFUSE) path_diffuse_p<kPixelWarp>(J, s, key, hit, &d0);
    if (hit) {
      const float u = s.h.u, v = s.h.v;
      f3 ca, cb, cc;
      if (mode == VERTEX_COLOR) {
        ca = val * (1.0f - u - v);
        cb = val * v;
        cc = val * u;
      } else if (mode == LAMBERT_POINT_VCOLOR) {
        ca = val * ((1.0f - u - v) * k);
        cb = val * (v * k);
        cc = val * (u * k);
      } else {
        const f3 vd = val * d0;
        ca = vd * (1.0f - u - v);
        cb = vd * v;
        cc = vd * u;
      }
      c[0] = ca.x; c[1] = ca.y; c[2] = ca.z;
      c[3] = cb.x; c[4] = cb.y; c[5] = cb.z;
      c[6] = cc.x; c[7] = cc.y; c[8] = cc.z;
      tri = s.h.tri;
      gA = s.A; gB = s.B; gC = s.C;
    }
    scatter_vertex_colors<DET>(J, tri, gA, gB, gC, c, wscr, rec_base, rec_n);
  } else if (model_has_tex(mode)) {
    float* g = nullptr;
    float2 tc = make_float2(0.0f, 0.0f);
    int tw = 0, th = 0;
    if (hit) {
      const BlockDev bd = J.blocks[s.block];
      const MeshDev& md = J.meshes[bd.mesh];
      if (md.dslot >= 0 && md.tex_off >= 0) {
        tc = interp_tc(J, s);
        g = J.grad + md.g_base + md.tex_off;
        tw = md.tex_w;
        th = md.tex_h;
      }
    }
    texture_grad<DET>(J, g, val, tc.x, tc.y, tw, th, rec_base, rec_n);
  }
}

// One warp per work item: a tile of tile_w x tile_h pixels whose samples
// fill at most 64 lanes (two passes of 32).  Warps take items from an atomic
// queue on their own and synchronise only within themselves, so no warp
// waits for a slower one.
constexpr int PX_WARPS = PX_THREADS / 32;
constexpr int PX_MAX_SAMPLES = 64;

// DET: the deterministic-mode variant (gradient records instead of atomics
// for jobs that have record buffers).  HITS: the adjoint's primary hits are
// written to (PX_HIT_STORE) or read from (PX_HIT_LOAD) the job's hit buffer,
// one float4 {t, u, v, triangle} per adjoint sample, instead of re-traced.
// Resident blocks per SM the register allocation must allow (the kernel is
// latency bound: more warps hide more of it; values from timing on GB300).
#ifndef DRGB_PX_MIN_BLOCKS
#define DRGB_PX_MIN_BLOCKS 4
#endif
#ifndef DRGB_PX_MIN_BLOCKS_PATH
#define DRGB_PX_MIN_BLOCKS_PATH 4
#endif
// The record-writing (deterministic) variants: 4 blocks as well (99 -> 64
// registers for the point-light model; 85.5 -> 96.3 deterministic
// iterations/s on the icosphere).
#ifndef DRGB_PX_MIN_BLOCKS_DET
#define DRGB_PX_MIN_BLOCKS_DET 4
#endif
constexpr int px_min_blocks(int mode, bool det, bool hits) {
  (void)hits;  // the stored-hit variants get the same budget, for a like-for-like comparison
  return mode == 0 ? 1 : det ? DRGB_PX_MIN_BLOCKS_DET : model_is_path(mode) ? DRGB_PX_MIN_BLOCKS_PATH : DRGB_PX_MIN_BLOCKS;
}
template <int MODE, bool DET, bool HITS>
__global__ void __launch_bounds__(PX_THREADS, px_min_blocks(MODE, DET, HITS)) k_pixels(const JobDev* __restrict__ jobs, const int4* __restrict__ items,
                                                       int n_items, int* counter, const int flags) {
  // Shared memory per block stays small: what the block does not take
  // stays L1 for the traversal's node and triangle loads (shared memory and
  // L1 are one array per SM).  The forward colours and the adjoint's scatter
  // scratch are never live together, so they share one buffer; the
  // Hammersley points are read through L1.
  constexpr int kWarpScratch = PX_MAX_SAMPLES * 3 > 9 * 32 ? PX_MAX_SAMPLES * 3 : 9 * 32;
  __shared__ JobDev sJ_all[PX_WARPS];
  __shared__ CamDev sC_all[PX_WARPS];
  __shared__ float4 s_adj_all[PX_WARPS][32];
  __shared__ float s_buf_all[PX_WARPS][kWarpScratch];
#ifdef DRGB_SEED_HITS
  __shared__ int s_hit_all[PX_WARPS][PX_MAX_SAMPLES];  // forward hit triangle of each sample
#endif
  stage_top_nodes(jobs[0]);  // a single job's top levels (none for a batch)

  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  JobDev& J = sJ_all[warp];
  CamDev& C = sC_all[warp];
  float4* s_adj = s_adj_all[warp];
  float* s_col = s_buf_all[warp];  // forward: sample colours
  float* wscr = s_buf_all[warp];   // adjoint: scatter scratch
#ifdef DRGB_SEED_HITS
  int* s_hit = s_hit_all[warp];
#endif
  int cur_job = -1, cur_view = -1;
  for (;;) {
    int it = 0;
    if (lane == 0) it = atomicAdd(counter, 1);
    it = __shfl_sync(0xffffffffu, it, 0);
    if (it >= n_items) break;
    const int4 item = items[it];
    if (item.x != cur_job) {
      const int* src = reinterpret_cast<const int*>(jobs + item.x);
      int* dst = reinterpret_cast<int*>(&J);
      for (int i = lane; i < (int)(sizeof(JobDev) / sizeof(int)); i += 32) dst[i] = src[i];
      __syncwarp();
      cur_job = item.x;
      cur_view = -1;
    }
    if (item.y != cur_view) {
      const int* src = reinterpret_cast<const int*>(J.cams + item.y);
      int* dst = reinterpret_cast<int*>(&C);
      for (int i = lane; i < (int)(sizeof(CamDev) / sizeof(int)); i += 32) dst[i] = src[i];
      cur_view = item.y;
    }
    __syncwarp();
    // the item's job had its raster pass resolve this launch's camera samples
    const bool vis_ok = (flags & PX_VIS) && J.ra_state && !(*J.ra_state & 1u);
    const int view = item.y, x0 = item.z, y0 = item.w;
    const int W = (int)C.width, H = (int)C.height;
    const int tw = J.tile_w;
    const int P = tw * J.tile_h;
    const int S = J.S, sq = J.sq;
    const int NS = P * S;
    if (flags & PX_FWD) {
      for (int base = 0; base < NS; base += 32) {
        const int s = base + lane;
        const int p = s / S, k = s - p * S;
        const int px = x0 + p % tw, py = y0 + p / tw;
        f3 c = mk(0.0f, 0.0f, 0.0f);
        const bool act = s < NS && px < W && py < H;
        float fx = 0.0f, fy = 0.0f;
        uint32_t key = 0;
        if (act) {
          const int dy = k / sq, dx = k - dy * sq;
          const float xoff = (dx + 0.5f) / (float)sq;
          const float yoff = (dy + 0.5f) / (float)sq;
          const int64_t pix = (int64_t)py * W + px;
          key = ((uint32_t)view * 0x9E3779B9u) ^ ((uint32_t)(pix * 64 + dy * sq + dx) * 2654435761u);
          fx = (float)px + xoff;
          fy = (float)py + yoff;
        }
        // every lane calls it (required by the warp-coherent policy)
#ifdef DRGB_SEED_HITS
        int ht = -1;
        const f3 sc = shade_p<MODE, kPixelWarp>(J, C, fx, fy, key, act, &ht);
        if (s < NS) s_hit[s] = act ? ht : -1;
#else
        const bool use_vis = vis_ok && J.vis_fwd != nullptr;
        const int64_t vi = (J.img_off[view] + (int64_t)py * W + px) * S + k;
        const float4 vk = act && use_vis ? J.vis_fwd[vi] : make_float4(0.0f, 0.0f, 0.0f, __int_as_float(-1));
        const float2* vuv = use_vis && J.vis_uv_fwd ? J.vis_uv_fwd + (act ? vi : 0) : nullptr;
        const f3 sc = shade_p<MODE, kPixelWarp>(J, C, fx, fy, key, act, nullptr, use_vis, vk, -1, vuv);
#endif
        if (act) c = sc / (float)S;
        if (s < NS) {
          s_col[3 * s + 0] = c.x;
          s_col[3 * s + 1] = c.y;
          s_col[3 * s + 2] = c.z;
        }
      }
      __syncwarp();
      double lsum = 0.0;
      if (lane < P) {
        const int qx = x0 + lane % tw, qy = y0 + lane / tw;
        if (qx < W && qy < H) {
          float ax = 0.0f, ay = 0.0f, az = 0.0f;
          for (int j = 0; j < S; j++) {  // the reference's summation order
            ax += s_col[3 * (lane * S + j) + 0];
            ay += s_col[3 * (lane * S + j) + 1];
            az += s_col[3 * (lane * S + j) + 2];
          }
          const int64_t q = (int64_t)qy * W + qx;
          if ((flags & PX_IMG) && J.images) {
            float* o = J.images + 3 * (J.img_off[view] + q);
            o[0] = ax; o[1] = ay; o[2] = az;
          }
          if (flags & PX_LOSS) {
            const float* t = J.targets + 3 * (J.img_off[view] + q);
            const float dx = ax - t[0], dy = ay - t[1], dz = az - t[2];
            const float4 a = make_float4(2.0f * dx, 2.0f * dy, 2.0f * dz, 0.0f);
            s_adj[lane] = a;
            J.adj[(int64_t)view * J.W * J.H + q] = a;
            lsum = (double)(dx * dx + dy * dy + dz * dz);
          }
        }
      }
      if (flags & PX_LOSS) {
        // pixel order within the tile
        double acc = 0.0;
        for (int j = 0; j < P; j++) acc += __shfl_sync(0xffffffffu, lsum, j);
        if (lane == 0) J.loss_part[it - J.item_base] = acc;
      }
    }
    if (flags & PX_ADJ) {
      const bool store_hits = HITS && (flags & PX_HIT_STORE);
      if (!(flags & PX_LOSS) && !store_hits) {
        if (lane < P) {
          const int qx = x0 + lane % tw, qy = y0 + lane / tw;
          float4 a = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
          if (qx < W && qy < H) {
            const float* src = J.adj_in + 3 * ((int64_t)view * J.W * J.H + (int64_t)qy * W + qx);
            a = make_float4(src[0], src[1], src[2], 0.0f);
          }
          s_adj[lane] = a;
        }
      }
      __syncwarp();
      const int64_t rec_base = (int64_t)(it - J.item_base) * J.rec_item_cap;
      int rec_n = 0;
      for (int base = 0; base < NS; base += 32) {
        const int s = base + lane;
        const int p = s / S, k = s - p * S;
        const int px = x0 + p % tw, py = y0 + p / tw;
        f3 val = mk(0.0f, 0.0f, 0.0f);
        bool act = false;
        float sx = 0.0f, sy = 0.0f;
        uint32_t key = 0;
        if (s < NS && px < W && py < H) {
          if (store_hits) {
            act = true;  // the adjoint is not known yet: every sample is traced
          } else {
            const float4 a = s_adj[p];
            val = mk(a.x, a.y, a.z) / (float)S;
            act = !(val.x == 0.0f && val.y == 0.0f && val.z == 0.0f);
          }
          sx = (float)px + __ldg(J.ham + 2 * k);
          sy = (float)py + __ldg(J.ham + 2 * k + 1);
          const int64_t pix = (int64_t)py * W + px;
          key = ((uint32_t)view * 0x9E3779B9u) ^ 0x5bd1e995u ^ ((uint32_t)(pix * 64 + k) * 2654435761u);
        }
        // one hit-buffer slot per adjoint sample of the item
        const float4* hslot = HITS ? J.hit_buf + ((int64_t)(it - J.item_base) * NS + min(s, NS - 1)) : nullptr;
        if (store_hits) {
          Surf sf;
          const bool h = cast_p<kPixelWarp>(J, C, sx, sy, act, sf);
          if (s < NS)
            const_cast<float4*>(hslot)[0] = make_float4(sf.h.t, sf.h.u, sf.h.v, __int_as_float(h ? sf.h.tri : -1));
          continue;
        }
        // -DDRGB_SEED_HITS: test first the forward hit of the grid sample whose
        // cell holds this point (bit-identical results; 3 % slower on GB300
        // for the point-light sphere, so off)
        int seed = -1;
#ifdef DRGB_SEED_HITS
        if ((flags & PX_FWD) && act) {
          const int gx = min(sq - 1, (int)(__ldg(J.ham + 2 * k) * (float)sq));
          const int gy = min(sq - 1, (int)(__ldg(J.ham + 2 * k + 1) * (float)sq));
          seed = s_hit[p * S + gy * sq + gx];
        }
#endif
        const bool use_vis = vis_ok && J.vis_adj != nullptr;
        const int64_t vi = (J.img_off[view] + (int64_t)py * W + px) * S + k;
        const float4 vk = act && use_vis ? J.vis_adj[vi] : make_float4(0.0f, 0.0f, 0.0f, __int_as_float(-1));
        const float2* vuv = use_vis && J.vis_uv_adj ? J.vis_uv_adj + (act ? vi : 0) : nullptr;
        shade_grad<MODE, DET, HITS>(J, C, act, sx, sy, val, key, wscr, rec_base, rec_n, hslot, seed, use_vis, vk,
                                    vuv);
      }
      if (DET && J.det && lane == 0 && !store_hits) J.rec_count[it - J.item_base] = rec_n;
    }
    __syncwarp();
  }
}

// LossAndDiffLoss (utils.cpp:15-27) summed as d_render_and_compare does
// (drender.h:183-189): a double sum per view, cast to float, views added in
// order, divided by views*W*H.  The per-item double partials of a view are
// summed by kLossBlocks blocks over fixed contiguous chunks, each in a fixed
// tree order; the block of a job that finishes last (completion ticket) adds
// the chunk sums of each view in chunk order.  The association is fixed, so
// the loss does not depend on scheduling; FP64 work is spread over
// kLossBlocks SMs (GB300's FP64 rate is 1/32 of FP32).
constexpr int LOSS_THREADS = 256;
__global__ void __launch_bounds__(LOSS_THREADS) k_loss_finalize(const JobDev* jobs, int n_jobs) {
  __shared__ double red[LOSS_THREADS];
  __shared__ bool last;
  const int j = blockIdx.y;
  if (j >= n_jobs) return;
  const JobDev& J = jobs[j];
  const int b = blockIdx.x, tid = threadIdx.x;
  const int per_view = J.n_views > 0 ? J.item_count / J.n_views : 0;
  const int cs = (per_view + kLossBlocks - 1) / kLossBlocks;
  const int lo = b * cs, hi = min(per_view, lo + cs);
  for (int v = 0; v < J.n_views; v++) {
    double acc = 0.0;
    for (int i = lo + tid; i < hi; i += LOSS_THREADS) acc += J.loss_part[(int64_t)v * per_view + i];
    red[tid] = acc;
    __syncthreads();
    for (int h = LOSS_THREADS / 2; h > 0; h >>= 1) {
      if (tid < h) red[tid] += red[tid + h];
      __syncthreads();
    }
    if (tid == 0) J.loss_blk[v * kLossBlocks + b] = red[0];
    __syncthreads();
  }
  if (tid == 0) {
    __threadfence();
    last = (atomicAdd(J.loss_ticket, 1u) % kLossBlocks) == kLossBlocks - 1;
  }
  __syncthreads();
  if (!last || tid != 0) return;
  __threadfence();
  float mse = 0.0f;
  for (int v = 0; v < J.n_views; v++) {
    double sum = 0.0;
    for (int k = 0; k < kLossBlocks; k++) sum += __ldcg(J.loss_blk + v * kLossBlocks + k);
    mse += (float)sum;
  }
  J.loss_out[0] = mse / (float)(J.n_views * J.W * J.H);
}

// Caller-supplied adjoint images (3 floats per pixel) -> float4 adjoint.
__global__ void k_adj_convert(const JobDev* jobs, int64_t n) {
  const JobDev& J = jobs[0];
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  J.adj[i] = make_float4(J.adj_in[3 * i], J.adj_in[3 * i + 1], J.adj_in[3 * i + 2], 0.0f);
}

void launch_adj_convert(const JobDev* d_job, int64_t n_pixels, cudaStream_t s) {
  if (n_pixels <= 0) return;
  k_adj_convert<<<(unsigned)((n_pixels + 255) / 256), 256, 0, s>>>(d_job, n_pixels);
  count_launch();
}

// IRayTracer::CastSingleRay for a list of pixel positions: SurfaceInfo fields.
__global__ void k_cast(const JobDev* jobs, const CamDev* cam, const float* xy, int64_t n, uint32_t* prim,
                       uint32_t* inst, uint32_t* geom, float* t, float* u, float* v) {
  const JobDev& J = jobs[0];
  stage_top_nodes(J);
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  Surf s;
  if (cast(J, *cam, xy[2 * i], xy[2 * i + 1], s)) {
    const BlockDev bd = J.blocks[s.block];
    prim[i] = (uint32_t)(s.h.tri - bd.tri_off);
    inst[i] = (uint32_t)bd.inst;
    geom[i] = (uint32_t)bd.mesh;
  } else {
    prim[i] = inst[i] = geom[i] = kNoHit;
  }
  t[i] = s.h.t;
  u[i] = s.h.u;
  v[i] = s.h.v;
}

void launch_cast(const JobDev* d_job, const CamDev* d_cam, const float* d_xy, int64_t n, uint32_t* prim,
                 uint32_t* inst, uint32_t* geom, float* t, float* u, float* v, cudaStream_t s) {
  k_cast<<<(unsigned)((n + 127) / 128), 128, 0, s>>>(d_job, d_cam, d_xy, n, prim, inst, geom, t, u, v);
  count_launch();
}

// `mode` selects the kernel compiled for one shading model; 0 (a launch whose
// jobs mix models) runs the generic kernel that switches per job.  `det`
// selects the deterministic-mode variants.
template <bool DET>
static void launch_pixels_t(const JobDev* d_jobs, const int4* d_items, int n_items, int* d_counter, int flags,
                            int grid, cudaStream_t s, int mode) {
  switch (mode) {
    case SILHOUETTE: k_pixels<SILHOUETTE, DET, false><<<grid, PX_THREADS, 0, s>>>(d_jobs, d_items, n_items, d_counter, flags); break;
    case VERTEX_COLOR: k_pixels<VERTEX_COLOR, DET, false><<<grid, PX_THREADS, 0, s>>>(d_jobs, d_items, n_items, d_counter, flags); break;
    case TEXTURE_COLOR: k_pixels<TEXTURE_COLOR, DET, false><<<grid, PX_THREADS, 0, s>>>(d_jobs, d_items, n_items, d_counter, flags); break;
    case LAMBERT: k_pixels<LAMBERT, DET, false><<<grid, PX_THREADS, 0, s>>>(d_jobs, d_items, n_items, d_counter, flags); break;
    case PHONG: k_pixels<PHONG, DET, false><<<grid, PX_THREADS, 0, s>>>(d_jobs, d_items, n_items, d_counter, flags); break;
    case GGX: k_pixels<GGX, DET, false><<<grid, PX_THREADS, 0, s>>>(d_jobs, d_items, n_items, d_counter, flags); break;
    case LAMBERT_POINT_VCOLOR:
      k_pixels<LAMBERT_POINT_VCOLOR, DET, false><<<grid, PX_THREADS, 0, s>>>(d_jobs, d_items, n_items, d_counter, flags);
      break;
    case PATH_DIFFUSE: k_pixels<PATH_DIFFUSE, DET, false><<<grid, PX_THREADS, 0, s>>>(d_jobs, d_items, n_items, d_counter, flags); break;
    case PATH_TEST: k_pixels<PATH_TEST, DET, false><<<grid, PX_THREADS, 0, s>>>(d_jobs, d_items, n_items, d_counter, flags); break;
    default: k_pixels<0, DET, false><<<grid, PX_THREADS, 0, s>>>(d_jobs, d_items, n_items, d_counter, flags); break;
  }
}

// Stored-hit variants: specialised for the vertex-colour, point-light and
// path models, the generic kernel otherwise.
template <bool DET>
static void launch_pixels_hits(const JobDev* d_jobs, const int4* d_items, int n_items, int* d_counter, int flags,
                               int grid, cudaStream_t s, int mode) {
  switch (mode) {
    case VERTEX_COLOR: k_pixels<VERTEX_COLOR, DET, true><<<grid, PX_THREADS, 0, s>>>(d_jobs, d_items, n_items, d_counter, flags); break;
    case LAMBERT_POINT_VCOLOR:
      k_pixels<LAMBERT_POINT_VCOLOR, DET, true><<<grid, PX_THREADS, 0, s>>>(d_jobs, d_items, n_items, d_counter, flags);
      break;
    case PATH_DIFFUSE: k_pixels<PATH_DIFFUSE, DET, true><<<grid, PX_THREADS, 0, s>>>(d_jobs, d_items, n_items, d_counter, flags); break;
    default: k_pixels<0, DET, true><<<grid, PX_THREADS, 0, s>>>(d_jobs, d_items, n_items, d_counter, flags); break;
  }
}

void launch_pixels(const JobDev* d_jobs, const int4* d_items, int n_items, int* d_counter, int flags, int grid,
                   cudaStream_t s, int mode, bool det) {
  if (n_items <= 0) return;
  if ((flags & PX_LOSS) && !(flags & PX_FWD)) throw CudaError("loss needs the forward pass", DRGB_ERR_INVALID);
  DRGB_CUDA(cudaMemsetAsync(d_counter, 0, sizeof(int), s));
  if (grid <= 0 || grid > n_items) grid = n_items;
  // records are only written by the adjoint pass
  const bool rec = det && (flags & PX_ADJ) && !(flags & PX_HIT_STORE);
  if (flags & (PX_HIT_STORE | PX_HIT_LOAD)) {
    if (!(flags & PX_ADJ)) throw CudaError("stored hits belong to the adjoint pass", DRGB_ERR_INVALID);
    if (rec) launch_pixels_hits<true>(d_jobs, d_items, n_items, d_counter, flags, grid, s, mode);
    else launch_pixels_hits<false>(d_jobs, d_items, n_items, d_counter, flags, grid, s, mode);
  } else if (rec) {
    launch_pixels_t<true>(d_jobs, d_items, n_items, d_counter, flags, grid, s, mode);
  } else {
    launch_pixels_t<false>(d_jobs, d_items, n_items, d_counter, flags, grid, s, mode);
  }
  count_launch();
}

int pixel_blocks_resident(int mode) {
  int n = 0;
  const void* f = nullptr;
  switch (mode) {
    case SILHOUETTE: f = (const void*)k_pixels<SILHOUETTE, false, false>; break;
    case VERTEX_COLOR: f = (const void*)k_pixels<VERTEX_COLOR, false, false>; break;
    case TEXTURE_COLOR: f = (const void*)k_pixels<TEXTURE_COLOR, false, false>; break;
    case LAMBERT: f = (const void*)k_pixels<LAMBERT, false, false>; break;
    case PHONG: f = (const void*)k_pixels<PHONG, false, false>; break;
    case GGX: f = (const void*)k_pixels<GGX, false, false>; break;
    case LAMBERT_POINT_VCOLOR: f = (const void*)k_pixels<LAMBERT_POINT_VCOLOR, false, false>; break;
    case PATH_DIFFUSE: f = (const void*)k_pixels<PATH_DIFFUSE, false, false>; break;
    case PATH_TEST: f = (const void*)k_pixels<PATH_TEST, false, false>; break;
    default: f = (const void*)k_pixels<0, false, false>; break;
  }
  DRGB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, f, PX_THREADS, 0));
  return std::max(1, n);
}

void launch_loss_finalize(const JobDev* d_jobs, int n_jobs, cudaStream_t s) {
  k_loss_finalize<<<dim3(kLossBlocks, n_jobs), LOSS_THREADS, 0, s>>>(d_jobs, n_jobs);
  count_launch();
}

}  // namespace drgb
